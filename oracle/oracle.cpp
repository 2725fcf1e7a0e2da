// CPU oracle for the warporacer3d rollout hot path. TEST INFRASTRUCTURE ONLY:
// the parity tests, the smoke check and the CPU-baseline leg of the benchmark
// call it as the checker; no product code path links or calls it.
//
// A line-by-line restatement of the reference's per-index kernels:
//   racer/sim.mojo:59-152  Surface, Spot, Map (header, at, probe, surface,
//                          waypoint, progress)
//   racer/sim.mojo:155-167 derivative (slope bicycle with a friction circle)
//   racer/sim.mojo:170-181 spawn
//   racer/sim.mojo:184-235 advance (4 RK4 substeps, crash, reward, respawn)
//   racer/sim.mojo:238-266 scan (sphere-traced planar lidar)
//   racer/sim.mojo:323-348 Sim.sample
//   racer/ppo.mojo:40-44,68-138 Policy init / forward / backward
//   racer/ppo.mojo:218-230 GAE, :276-304 minibatch gather and loss,
//                          :317-337 Adam
// The order of every floating-point operation follows the Mojo source
// (left-to-right associativity; SIMD reduce_add as a halving tree). It is
// compiled with -ffp-contract=off. sin/cos/exp/log come from the project's
// rmath.h and random numbers from philox.h (the reference's Mojo stdlib
// functions are not in its checkout), so the CUDA kernels, built without
// contraction, can be compared with it bit for bit.
//
// CPU schedule mirrors racer/device.mojo:56-80: a parallel-for over cars for
// physics, a parallel-for over cars with a serial beam loop for the lidar.
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../warporacer3d_gb300/csrc/philox.h"
#include "../warporacer3d_gb300/csrc/rmath.h"

namespace {

// racer/sim.mojo:15-56
const float WHEELBASE = 0.3302f, HALF_DIAG = 0.3f, GRIP = 1.05f, G = 9.81f;
const float STEER_MAX = 0.4189f, STEER_RATE = 3.2f, ACCEL_MAX = 9.51f, SPEED_MAX = 5.0f;
const int SUBSTEPS = 4;
const float DT = (float)(1.0 / 240);
const int HORIZON = 3000;
const float RANGE = 10.0f, FOV = 4.71238898f;
const float MOUNT_X = 0.27f, MOUNT_Z = 0.23f;
enum { X = 0, Y, Z, HEADING, SPEED, STEER, STEPS, PROGRESS, EPISODE, FRICTION, RETURN, STATE };
const int OUT = 3;
const int CRASH = 1, TIMEOUT = 2;
const int HEADER = 12;
enum { CLEARANCE = 0, HEIGHT = 1, NEAREST = 2 };
const float PI_F = 3.14159274f;      // Float32(pi)
const float TWO_PI_F = 6.28318548f;  // Float32(2 * pi)

// racer/ppo.mojo:17-31
const int H = 64, HA = H + 1;
const float GAMMA = 0.99f, LAMBDA = 0.95f, CLIP = 0.2f, LR = 3e-4f, MAX_NORM = 0.5f;

float hl2p() { return (float)(0.5 * log(2.0 * M_PI)); }

float clampf_(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

struct Spot {
  int layer;
  float clearance, height;
};
struct Surface {
  float height, sx, sy;
  // racer/sim.mojo:65-69
  void slopes(float heading, float* along, float* across) const {
    float s, c;
    rmath::sincosf_(heading, &s, &c);
    *along = sx * c + sy * s;
    *across = -sx * s + sy * c;
  }
};

// racer/sim.mojo:81-152
struct Map {
  int nx, ny, waypoints, layers;
  float x0, y0, cell, spacing, slope;
  long route;
  const float* d;

  explicit Map(const float* data) : d(data) {
    nx = (int)d[0];
    ny = (int)d[1];
    x0 = d[2];
    y0 = d[3];
    cell = d[4];
    waypoints = (int)d[5];
    spacing = d[6];
    layers = (int)d[7];
    slope = d[8];
    route = HEADER + 3L * layers * nx * ny;
  }
  long grid(int layer, int which) const { return HEADER + (long)(3 * layer + which) * nx * ny; }

  // Nearest cell; off the map every grid reads -1 (racer/sim.mojo:108-114).
  // Non-finite coordinates count as off the map.
  float at(int layer, int which, float x, float y) const {
    float fx = floorf((x - x0) / cell + 0.5f);
    float fy = floorf((y - y0) / cell + 0.5f);
    if (!(fx >= 0.0f && fx < (float)nx && fy >= 0.0f && fy < (float)ny)) return -1.0f;
    return d[grid(layer, which) + (long)fy * nx + (long)fx];
  }
  // racer/sim.mojo:116-124: the drivable layer nearest z; strict < keeps the lower layer on ties.
  Spot probe(float x, float y, float z) const {
    Spot best = {0, -1.0f, at(0, HEIGHT, x, y)};
    float gap = 1e30f;
    for (int l = 0; l < layers; ++l) {
      Spot spot = {l, at(l, CLEARANCE, x, y), at(l, HEIGHT, x, y)};
      if (spot.clearance > 0.0f && fabsf(spot.height - z) < gap) {
        best = spot;
        gap = fabsf(spot.height - z);
      }
    }
    return best;
  }
  // racer/sim.mojo:126-140: bilinear height and gradient.
  Surface surface(int layer, float x, float y) const {
    float fx = (x - x0) / cell;
    float fy = (y - y0) / cell;
    float flx = floorf(fx), fly = floorf(fy);
    int ix = flx >= 0.0f ? (flx <= (float)(nx - 2) ? (int)flx : nx - 2) : 0;
    int iy = fly >= 0.0f ? (fly <= (float)(ny - 2) ? (int)fly : ny - 2) : 0;
    float tx = clampf_(fx - (float)ix, 0.0f, 1.0f);
    float ty = clampf_(fy - (float)iy, 0.0f, 1.0f);
    long k = grid(layer, HEIGHT) + (long)iy * nx + ix;
    float h0 = d[k], h1 = d[k + 1], h2 = d[k + nx], h3 = d[k + nx + 1];
    float w0 = (1 - tx) * (1 - ty), w1 = tx * (1 - ty), w2 = (1 - tx) * ty, w3 = tx * ty;
    Surface s;
    s.height = (h0 * w0 + h2 * w2) + (h1 * w1 + h3 * w3);  // reduce_add halving tree
    s.sx = ((h1 - h0) * (1 - ty) + (h3 - h2) * ty) / cell;
    s.sy = ((h2 - h0) * (1 - tx) + (h3 - h1) * tx) / cell;
    return s;
  }
  float waypoint(long w, int field) const { return d[route + 4 * w + field]; }
  // racer/sim.mojo:146-152. w = -1 (off the map) reads d[route - 4 + field], as the reference does.
  float progress(int layer, float x, float y) const {
    long w = (long)at(layer, NEAREST, x, y);
    float heading = waypoint(w, 3);
    float s, c;
    rmath::sincosf_(heading, &s, &c);
    float along = (x - waypoint(w, 0)) * c + (y - waypoint(w, 1)) * s;
    return (float)w + along / spacing;
  }
};

struct Vec4 {
  float v[4];
};

// racer/sim.mojo:155-167
Vec4 derivative(const Vec4& p, float steer, float accel, float grip, float along, float across) {
  float nz = 1.0f / sqrtf((1.0f + along * along) + across * across);
  float load = (grip * G) * nz;
  float v = fmaxf(fabsf(p.v[3]), 0.5f) * (p.v[3] >= 0.0f ? 1.0f : -1.0f);
  float slide = (G * across) * nz;
  float ss, cs;
  rmath::sincosf_(steer, &ss, &cs);
  float lateral = clampf_((((v * p.v[3]) * ss) / cs) / WHEELBASE + slide, -load, load);
  float yaw = (lateral - slide) / v;
  float longitudinal = sqrtf(fmaxf(load * load - lateral * lateral, 0.0f));
  float dv = clampf_(accel, -longitudinal, longitudinal) - (G * along) * nz;
  float sh, ch;
  rmath::sincosf_(p.v[2], &sh, &ch);
  Vec4 r = {{p.v[3] * ch, p.v[3] * sh, yaw, dv}};
  return r;
}

Vec4 axpy(const Vec4& p, const Vec4& k, float h) {
  Vec4 r;
  for (int j = 0; j < 4; ++j) r.v[j] = p.v[j] + k.v[j] * h;
  return r;
}

inline float& S(float* s, int n, int row, int i) { return s[(long)row * n + i]; }

// racer/sim.mojo:170-181
void spawn(float* s, int n, const Map& map, int i, uint64_t seed) {
  float episode = S(s, n, EPISODE, i) + 1.0f;
  float r[4];
  philox::uniform4(seed, (uint64_t)i, (uint64_t)episode, r);
  int w = std::min((int)(r[0] * (float)map.waypoints), map.waypoints - 1);
  for (int row = 0; row < STATE; ++row) S(s, n, row, i) = 0.0f;
  S(s, n, X, i) = map.waypoint(w, 0);
  S(s, n, Y, i) = map.waypoint(w, 1);
  S(s, n, Z, i) = map.waypoint(w, 2);
  S(s, n, HEADING, i) = map.waypoint(w, 3);
  S(s, n, PROGRESS, i) = (float)w;
  S(s, n, EPISODE, i) = episode;
  S(s, n, FRICTION, i) = 0.85f + 0.3f * r[1];
}

// racer/sim.mojo:184-235. obs is [IN, n] with IN = beams + 5; row OBS = beams + 4 is the bias.
void advance(float* s, const float* act, float* reward, float* done, float* obs, int n, int beams, const Map& map,
             int i, uint64_t seed) {
  const int OBS = 4 + beams;
  Vec4 p = {{S(s, n, X, i), S(s, n, Y, i), S(s, n, HEADING, i), S(s, n, SPEED, i)}};
  Spot spot = map.probe(p.v[0], p.v[1], S(s, n, Z, i));
  Surface ground = map.surface(spot.layer, p.v[0], p.v[1]);
  float steer = S(s, n, STEER, i);
  float rate = clampf_(act[i], -1.0f, 1.0f) * STEER_RATE;
  float accel = clampf_(act[n + i], -1.0f, 1.0f) * ACCEL_MAX;
  float grip = GRIP * S(s, n, FRICTION, i);
  bool crashed = false;
  const float half_dt = DT / 2.0f, sixth_dt = DT / 6.0f;
  for (int sub = 0; sub < SUBSTEPS; ++sub) {
    float along, across;
    ground.slopes(p.v[2], &along, &across);
    float mid = steer + (rate * DT) / 2.0f;
    Vec4 k1 = derivative(p, steer, accel, grip, along, across);
    Vec4 k2 = derivative(axpy(p, k1, half_dt), mid, accel, grip, along, across);
    Vec4 k3 = derivative(axpy(p, k2, half_dt), mid, accel, grip, along, across);
    Vec4 k4 = derivative(axpy(p, k3, DT), steer + rate * DT, accel, grip, along, across);
    for (int j = 0; j < 4; ++j) p.v[j] = p.v[j] + ((k1.v[j] + 2.0f * (k2.v[j] + k3.v[j])) + k4.v[j]) * sixth_dt;
    p.v[3] = clampf_(p.v[3], -SPEED_MAX, SPEED_MAX);
    steer = clampf_(steer + rate * DT, -STEER_MAX, STEER_MAX);
    spot = map.probe(p.v[0], p.v[1], spot.height);
    ground = map.surface(spot.layer, p.v[0], p.v[1]);
    crashed = crashed || spot.clearance < HALF_DIAG || ground.sx * ground.sx + ground.sy * ground.sy > 1.0f;
  }
  if (p.v[2] > PI_F) p.v[2] -= TWO_PI_F;
  if (p.v[2] < -PI_F) p.v[2] += TWO_PI_F;
  float progress = map.progress(spot.layer, p.v[0], p.v[1]);
  float dp = progress - S(s, n, PROGRESS, i);
  float half = (float)map.waypoints / 2.0f;
  dp = dp > half ? dp - 2.0f * half : (dp < -half ? dp + 2.0f * half : dp);
  float score = crashed ? -2.0f : ((10.0f * dp) * map.spacing - (0.001f * steer) * steer);
  float steps = S(s, n, STEPS, i) + 1.0f;
  float reason = (float)(crashed ? CRASH : (steps >= (float)HORIZON ? TIMEOUT : 0));
  S(s, n, X, i) = p.v[0];
  S(s, n, Y, i) = p.v[1];
  S(s, n, Z, i) = spot.height;
  S(s, n, HEADING, i) = p.v[2];
  S(s, n, SPEED, i) = p.v[3];
  S(s, n, STEER, i) = steer;
  S(s, n, STEPS, i) = steps;
  S(s, n, PROGRESS, i) = progress;
  S(s, n, RETURN, i) = S(s, n, RETURN, i) + score;
  reward[i] = score;
  done[i] = reason;
  if (reason > 0.0f) {
    spawn(s, n, map, i, seed);
    ground = map.surface(map.probe(S(s, n, X, i), S(s, n, Y, i), S(s, n, Z, i)).layer, S(s, n, X, i), S(s, n, Y, i));
  }
  float along, across;
  ground.slopes(S(s, n, HEADING, i), &along, &across);
  obs[i] = S(s, n, STEER, i) / STEER_MAX;
  obs[(long)n + i] = S(s, n, SPEED, i) / SPEED_MAX;
  obs[2L * n + i] = along;
  obs[3L * n + i] = across;
  obs[(long)OBS * n + i] = 1.0f;
}

// racer/sim.mojo:238-266. Returns the range in metres; *iters counts probe iterations.
float scan(const Map& map, const float* s, const float* obs, int n, int beams, int i, int beam, int* iters) {
  float heading = S(const_cast<float*>(s), n, HEADING, i);
  float sh, ch;
  rmath::sincosf_(heading, &sh, &ch);
  float fwd[3] = {ch, sh, obs[2L * n + i]};
  float left[3] = {-sh, ch, obs[3L * n + i]};
  float azimuth = -FOV / 2.0f + (float)beam * (FOV / (float)(beams - 1));
  float sa, ca;
  rmath::sincosf_(azimuth, &sa, &ca);
  float dir[3];
  for (int j = 0; j < 3; ++j) dir[j] = ca * fwd[j] + sa * left[j];
  float norm = sqrtf((dir[0] * dir[0] + dir[2] * dir[2]) + (dir[1] * dir[1] + 0.0f));
  for (int j = 0; j < 3; ++j) dir[j] = dir[j] / norm;
  float ox = (S(const_cast<float*>(s), n, X, i) + MOUNT_X * fwd[0]) + 0.0f;
  float oy = (S(const_cast<float*>(s), n, Y, i) + MOUNT_X * fwd[1]) + 0.0f;
  float oz = (S(const_cast<float*>(s), n, Z, i) + MOUNT_X * fwd[2]) + MOUNT_Z;
  float horizontal = sqrtf(dir[0] * dir[0] + dir[1] * dir[1]);
  float descent = (1.5f * map.slope) * horizontal + fmaxf(-dir[2], 0.0f);
  float t = 0.0f, last = 0.0f, last_floor = 0.0f;
  int count = 0;
  while (t < RANGE) {
    ++count;
    float px = ox + t * dir[0], py = oy + t * dir[1], pz = oz + t * dir[2];
    Spot spot = map.probe(px, py, pz);
    float floor_ = (pz - spot.height) - 0.03f;
    if (floor_ < 0.0f) {
      *iters = count;
      return fminf(last + ((t - last) * last_floor) / (last_floor - floor_), RANGE);
    }
    float step = fminf(spot.clearance - map.cell, floor_ / descent);
    if (step < 0.5f * map.cell) break;
    last = t;
    last_floor = floor_;
    t += step;
  }
  *iters = count;
  return fminf(t, RANGE);
}

void set_threads(int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
}

}  // namespace

extern "C" {

float orc_half_log_2pi() { return hl2p(); }

// ---- Map queries (racer/sim.mojo:108-152) ----
void orc_probe(const float* d, float x, float y, float z, int* layer, float* clearance, float* height) {
  Map map(d);
  Spot s = map.probe(x, y, z);
  *layer = s.layer;
  *clearance = s.clearance;
  *height = s.height;
}
void orc_surface(const float* d, int layer, float x, float y, float* out3) {
  Map map(d);
  Surface s = map.surface(layer, x, y);
  out3[0] = s.height;
  out3[1] = s.sx;
  out3[2] = s.sy;
}
float orc_progress(const float* d, int layer, float x, float y) { return Map(d).progress(layer, x, y); }
float orc_at(const float* d, int layer, int which, float x, float y) { return Map(d).at(layer, which, x, y); }
void orc_derivative(const float* p4, float steer, float accel, float grip, float along, float across, float* out4) {
  Vec4 p = {{p4[0], p4[1], p4[2], p4[3]}};
  Vec4 r = derivative(p, steer, accel, grip, along, across);
  for (int j = 0; j < 4; ++j) out4[j] = r.v[j];
}
void orc_sincos(const float* x, int count, float* s, float* c) {
  for (int i = 0; i < count; ++i) rmath::sincosf_(x[i], &s[i], &c[i]);
}
void orc_exp(const float* x, int count, float* y) {
  for (int i = 0; i < count; ++i) y[i] = rmath::expf_(x[i]);
}
void orc_log(const float* x, int count, float* y) {
  for (int i = 0; i < count; ++i) y[i] = rmath::logf_(x[i]);
}
void orc_philox(uint64_t seed, uint64_t subsequence, uint64_t offset, uint32_t* out4) {
  philox::block(seed, subsequence, offset, out4);
}

// ---- Sim (racer/sim.mojo:291-321) ----
// Sim.reset's spawn kernel: spawn every car, zero its actions (racer/sim.mojo:299-304).
void orc_sim_spawn(const float* d, int n, uint64_t seed, float* state, float* actions, int threads) {
  Map map(d);
  set_threads(threads);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    spawn(state, n, map, i, seed);
    actions[i] = 0.0f;
    actions[(long)n + i] = 0.0f;
  }
}

// Sim.step's physics launch (racer/sim.mojo:314-315,320).
void orc_sim_physics(const float* d, int n, int beams, uint64_t seed, float* state, const float* actions,
                     float* reward, float* done, float* obs, int threads) {
  Map map(d);
  set_threads(threads);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) advance(state, actions, reward, done, obs, n, beams, map, i, seed);
}

// Sim.step's lidar launch (racer/sim.mojo:317-318,321); iters (optional, [beams, n]) gets
// the probe iterations of every beam.
void orc_sim_lidar(const float* d, int n, int beams, const float* state, float* obs, int* iters, int threads) {
  Map map(d);
  set_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; ++i) {
    for (int b = 0; b < beams; ++b) {
      int it = 0;
      float r = scan(map, state, obs, n, beams, i, b, &it);
      obs[(long)(4 + b) * n + i] = r / RANGE;
      if (iters) iters[(long)b * n + i] = it;
    }
  }
}

// Sim.sample (racer/sim.mojo:323-348). output is [3, n].
void orc_sim_sample(int n, uint64_t seed, const float* output, const float* log_std, float* actions, float* logp,
                    float* value, int deterministic, int64_t step) {
  const float half_log_2pi = hl2p();
  for (int i = 0; i < n; ++i) {
    float noise[4];
    philox::normal4(seed + 1, (uint64_t)i, (uint64_t)step, noise);
    float probability = 0.0f;
    for (int a = 0; a < 2; ++a) {
      float z = deterministic ? 0.0f : noise[a];
      actions[(long)a * n + i] = output[(long)a * n + i] + rmath::expf_(log_std[a]) * z;
      probability -= ((0.5f * z) * z + log_std[a]) + half_log_2pi;
    }
    logp[i] = probability;
    value[i] = output[2L * n + i];
  }
}

// ---- Policy (racer/ppo.mojo:68-138) ----
// theta layout: W0 [H, IN] | W1 [H, HA] | W2 [OUT, HA] | logstd [2].
int orc_policy_size(int in) { return H * in + H * HA + OUT * HA + 2; }

// racer/ppo.mojo:74-89, including its use of the absolute index i in `i % HA`.
void orc_policy_init(int in, uint64_t seed, float* theta) {
  const int obs = in - 1;
  const int w1 = H * in, w2 = w1 + H * HA, logstd = w2 + OUT * HA, p = logstd + 2;
  for (int i = 0; i < p; ++i) {
    float scale = 0.0f;
    if (i < w1) {
      scale = (i % in < obs) ? sqrtf(2.0f / (float)obs) : 0.0f;
    } else if (i < w2) {
      scale = (i % HA < H) ? sqrtf(1.0f / (float)H) : 0.0f;
    } else if (i < logstd) {
      scale = (i % HA < H) ? ((i - w2) / HA < 2 ? 0.00125f : 0.125f) : 0.0f;
    } else {
      theta[i] = -0.5f;
      continue;
    }
    float z[4];
    philox::normal4(seed, (uint64_t)i, 0, z);
    theta[i] = scale * z[0];
  }
}

// c[rows, cols] = act(w[rows, k] @ b[k, cols]) with b row-major [k, cols]; blocked over
// columns, float accumulation in k order.
static void gemm_rows(const float* w, int rows, int k, const float* b, int cols, float* c, bool squash) {
  const int BLOCK = 64;
  int nblocks = (cols + BLOCK - 1) / BLOCK;
#pragma omp parallel for schedule(static)
  for (int blk = 0; blk < nblocks; ++blk) {
    int j0 = blk * BLOCK, j1 = std::min(cols, j0 + BLOCK);
    float acc[BLOCK];
    for (int r = 0; r < rows; ++r) {
      for (int j = j0; j < j1; ++j) acc[j - j0] = 0.0f;
      const float* wr = w + (long)r * k;
      for (int kk = 0; kk < k; ++kk) {
        float a = wr[kk];
        const float* br = b + (long)kk * cols;
        for (int j = j0; j < j1; ++j) acc[j - j0] += a * br[j];
      }
      for (int j = j0; j < j1; ++j) c[(long)r * cols + j] = squash ? tanhf(acc[j - j0]) : acc[j - j0];
    }
  }
}

// Policy.forward (racer/ppo.mojo:108-111): h1 [HA, cols] and h2 [HA, cols] keep row H = 1.
void orc_policy_forward(int in, const float* theta, const float* x, int cols, float* h1, float* h2, float* o,
                        int threads) {
  set_threads(threads);
  const int w1 = H * in, w2 = w1 + H * HA;
  gemm_rows(theta, H, in, x, cols, h1, true);
  for (int j = 0; j < cols; ++j) h1[(long)H * cols + j] = 1.0f;
  gemm_rows(theta + w1, H, HA, h1, cols, h2, true);
  for (int j = 0; j < cols; ++j) h2[(long)H * cols + j] = 1.0f;
  gemm_rows(theta + w2, OUT, HA, h2, cols, o, false);
}

// Policy.backward (racer/ppo.mojo:113-138): d3 [OUT, cols] -> d2, d1 [HA, cols] and the
// W0/W1/W2 entries of grad (accumulated in double, written as float).
void orc_policy_backward(int in, const float* theta, const float* x, int cols, const float* h1, const float* h2,
                         const float* d3, float* d2, float* d1, float* grad, int threads) {
  set_threads(threads);
  const int w1 = H * in, w2 = w1 + H * HA;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < cols; ++j) {
    for (int k = 0; k < HA; ++k) {  // d2 = (W2^T d3) * (1 - h2^2)
      float acc = 0.0f;
      for (int r = 0; r < OUT; ++r) acc += theta[w2 + r * HA + k] * d3[(long)r * cols + j];
      float a = h2[(long)k * cols + j];
      d2[(long)k * cols + j] = acc * (1.0f - a * a);
    }
    for (int k = 0; k < HA; ++k) {  // d1 = (W1^T d2[:H]) * (1 - h1^2)
      float acc = 0.0f;
      for (int r = 0; r < H; ++r) acc += theta[w1 + r * HA + k] * d2[(long)r * cols + j];
      float a = h1[(long)k * cols + j];
      d1[(long)k * cols + j] = acc * (1.0f - a * a);
    }
  }
  // weight gradients: gW0 = d1[:H] x^T, gW1 = d2[:H] h1^T, gW2 = d3 h2^T
#pragma omp parallel for schedule(static)
  for (int r = 0; r < H; ++r) {
    for (int k = 0; k < in; ++k) {
      double acc = 0.0;
      for (int j = 0; j < cols; ++j) acc += (double)d1[(long)r * cols + j] * x[(long)k * cols + j];
      grad[r * in + k] = (float)acc;
    }
    for (int k = 0; k < HA; ++k) {
      double acc = 0.0;
      for (int j = 0; j < cols; ++j) acc += (double)d2[(long)r * cols + j] * h1[(long)k * cols + j];
      grad[w1 + r * HA + k] = (float)acc;
    }
  }
  for (int r = 0; r < OUT; ++r)
    for (int k = 0; k < HA; ++k) {
      double acc = 0.0;
      for (int j = 0; j < cols; ++j) acc += (double)d3[(long)r * cols + j] * h2[(long)k * cols + j];
      grad[w2 + r * HA + k] = (float)acc;
    }
}

// ---- Trainer pieces (racer/ppo.mojo:218-337) ----
// GAE per car (racer/ppo.mojo:218-230); last_value is the bootstrap value row [n].
void orc_gae(int n, int rollout, const float* reward, const float* done, const float* value, const float* last_value,
             float* advantage) {
  for (int i = 0; i < n; ++i) {
    float next = last_value[i];
    float running = 0.0f;
    for (int t = rollout - 1; t >= 0; --t) {
      long k = (long)t * n + i;
      float alive = done[k] == 0.0f ? 1.0f : 0.0f;
      float delta = (reward[k] + (GAMMA * alive) * next) - value[k];
      running = delta + ((GAMMA * LAMBDA) * alive) * running;
      advantage[k] = running;
      next = value[k];
    }
  }
}

// minibatch gather (racer/ppo.mojo:276-279): x [IN, batch] from rollout obs [(R+1), IN, n].
void orc_gather(int in, int n, int batch, int minibatches, int m, const float* obs, float* x) {
#pragma omp parallel for schedule(static)
  for (int b = 0; b < batch; ++b) {
    long s = (long)b * minibatches + m;
    for (int r = 0; r < in; ++r) x[(long)r * batch + b] = obs[((s / n) * in + r) * n + s % n];
  }
}

// minibatch loss derivatives (racer/ppo.mojo:281-304): d3 [OUT + 3, batch].
void orc_loss(int n, int batch, int minibatches, int m, const float* actions, const float* logp, const float* value,
              const float* advantage, const float* o, const float* log_std, float adv_mean, float adv_scale,
              float* d3) {
  const float half_log_2pi = hl2p();
  for (int b = 0; b < batch; ++b) {
    long s = (long)b * minibatches + m;
    long t = s / n, i = s % n;
    float new_logp = 0.0f, error[2], invvar[2];
    for (int a = 0; a < 2; ++a) {
      error[a] = actions[(t * 2 + a) * n + i] - o[(long)a * batch + b];
      invvar[a] = rmath::expf_(-2.0f * log_std[a]);
      new_logp -= (((0.5f * error[a]) * error[a]) * invvar[a] + log_std[a]) + half_log_2pi;
    }
    float logratio = new_logp - logp[s];
    float ratio = rmath::expf_(logratio);
    float a_hat = (advantage[s] - adv_mean) * adv_scale;
    float dlogp = (-a_hat * ratio) / (float)batch;
    if ((a_hat >= 0.0f && ratio > 1.0f + CLIP) || (a_hat < 0.0f && ratio < 1.0f - CLIP)) dlogp = 0.0f;
    for (int a = 0; a < 2; ++a) {
      d3[(long)a * batch + b] = (dlogp * error[a]) * invvar[a];
      d3[(long)(OUT + a) * batch + b] = dlogp * ((error[a] * error[a]) * invvar[a] - 1.0f);
    }
    d3[2L * batch + b] = (0.5f * clampf_((o[2L * batch + b] - value[s]) - advantage[s], -1.0f, 1.0f)) / (float)batch;
    d3[(long)(OUT + 2) * batch + b] = (ratio - 1.0f) - logratio;
  }
}

// Trainer.adam (racer/ppo.mojo:317-337); norm2 is the squared gradient norm.
void orc_adam(int p, int logstd, int step, float norm2, float* theta, const float* grad, float* first,
              float* second) {
  float scale = fminf(1.0f, MAX_NORM / (sqrtf(norm2) + 1e-8f));
  float c1 = 1.0f - powf(0.9f, (float)step), c2 = 1.0f - powf(0.999f, (float)step);
  for (int i = 0; i < p; ++i) {
    float g = grad[i] * scale;
    float m = 0.9f * first[i] + 0.1f * g;
    float v = 0.999f * second[i] + (0.001f * g) * g;
    first[i] = m;
    second[i] = v;
    float m_hat = m / c1, v_hat = v / c2;
    float value = theta[i] - (LR * m_hat) / (sqrtf(v_hat) + 1e-5f);
    theta[i] = i >= logstd ? fminf(fmaxf(value, -2.0f), 0.0f) : value;
  }
}

}  // extern "C"
