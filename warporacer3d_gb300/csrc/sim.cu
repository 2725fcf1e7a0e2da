// Simulator kernels: spawn, physics (RK4 bicycle, crash, reward, respawn),
// sphere-traced lidar and Gaussian action sampling.
//
// Reference behaviour: racer/sim.mojo:59-348 (Map lookups :108-152,
// derivative :155-167, spawn :170-181, advance :184-235, scan :238-266,
// Sim.reset/step/sample :291-348).
//
// This translation unit is compiled with --fmad=false and IEEE division and
// square root, and every transcendental comes from rmath.h, so each kernel is
// the same sequence of binary32 operations as the CPU restatement (fused
// multiply-adds appear only as explicit intrinsics where a proof shows the
// same result): layer, waypoint and crash outputs, the state and the ranges
// match it bit for bit.
//
// Layout in HBM (feature-major, as the reference): state [11, n],
// actions [2, n], reward [n], done [n], obs [beams + 5, n]. The track array is
// kept unchanged and, for the probes, repacked per cell as
// [ny * nx][layers] float2 (clearance, height): one 16-byte load answers a
// two-layer probe.
#include <string.h>

#include "common.cuh"
#include "fwd_tc.cuh"
#include "kernels.h"
#include "philox.h"
#include "rmath.h"
#include "sample.cuh"

namespace racer {
namespace {

struct Spot {
  int layer;
  float clearance, height;
};
struct Surface {
  float height, sx, sy;
};

__device__ __forceinline__ float clampf_(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

__device__ __forceinline__ void slopes(const Surface& g, float heading, float* along, float* across) {
  float s, c;
  rmath::sincosf_(heading, &s, &c);
  *along = g.sx * c + g.sy * s;
  *across = -g.sx * s + g.sy * c;
}

// floor((v - v0) / cell + 0.5), the reference's nearest-cell coordinate
// (racer/sim.mojo:110-111), without the division in almost every case:
// u' = (v - v0) * RN(1/cell) + 0.5 differs from the exact u by less than
// delta = (|u'| + 1) * 2^-20 (the two quotients are within 3 * 2^-24 |q| of
// each other and each + 0.5 rounds by half an ulp), so when u' is farther
// than delta from an integer both floors agree; inside that band the IEEE
// division decides. The result is bit-identical to the division form.
__device__ __forceinline__ float cell_coord(float v, float v0, float cell, float inv_cell) {
  float d = v - v0;
  float u = d * inv_cell + 0.5f;
  float fl = floorf(u);
  float g = u - fl;
  float delta = (fabsf(u) + 1.0f) * 9.5367431640625e-07f;
  if (g > delta && g < 1.0f - delta) return fl;
  return floorf(d / cell + 0.5f);
}

// Nearest-cell index (racer/sim.mojo:108-114); false off the map or for
// non-finite coordinates. The reference computes u = RN(RN(RN(x - x0) / h)
// + 0.5) (h = cell) and takes floor(u); the fast path computes
// v = RN(x * r + c) in one fused multiply-add, with r = RN(1 / h) and
// c = RN(-x0 * r) (TrackDev.cx, cy), and takes the nearest integer of v.
// With e = 2^-24, w = (x - x0) / h exactly, D = |w| and X = |x0| / h:
// |u - (w + 0.5)| <= e (2.0001 D + 1.0001 |u|) and |v - w| <= e (|x| / h +
// 2.0001 X + 1.0001 |v|). Where |v| <= M + 2 (M = max(nx, ny)) that gives
// |u - (v + 0.5)| <= e (5.0003 M + 3.0001 X + 12.02), so with the band delta
// = e (5.001 M + 4.001 X + 16), which also covers the rounding of v - rint(v),
// a v farther than delta from every half-integer has floor(u) = rint(v);
// farther out both are off the map (the error is at most 6 e |v| + e (4 X +
// 3) there). Inside the band, and for NaN and infinities, the division
// decides.
__device__ __forceinline__ bool cell_of(const TrackDev& t, float x, float y, long* idx) {
  const float vx = __fmaf_rn(x, t.inv_cell, t.cx), vy = __fmaf_rn(y, t.inv_cell, t.cy);
  const float rx = rintf(vx), ry = rintf(vy);
  if (fabsf(vx - rx) < t.band && fabsf(vy - ry) < t.band) {
    const int ix = (int)rx, iy = (int)ry;  // saturating conversion: far off the map stays off it
    if ((unsigned)ix >= (unsigned)t.nx || (unsigned)iy >= (unsigned)t.ny) return false;
    *idx = (long)(iy * t.nx + ix);
    return true;
  }
  float fx = cell_coord(x, t.x0, t.cell, t.inv_cell);
  float fy = cell_coord(y, t.y0, t.cell, t.inv_cell);
  if (!(fx >= 0.0f && fx < t.nxf && fy >= 0.0f && fy < t.nyf)) return false;
  *idx = (long)((int)fy * t.nx + (int)fx);
  return true;
}

// The cell of the march's probe at tt along a ray among the lidar's cells
// (TrackDev.lc), decided as cell_of decides it for the probe point px =
// RN(ox + RN(tt dx)), py alike, with every off-map point sent to the border
// column or row. Fast path: v = RN(tt ax + bx) in one fused multiply-add, with
// ax = RN(dx r), bx = RN(ox r + cx) held per beam (r = RN(1 / cell), cx =
// RN(-x0 r)). With e = 2^-24, w = (px - x0) / cell exactly, D = |w|, X =
// |x0| / cell and T = tt |dx| <= RANGE, the roundings of r, cx, ax, bx and v
// and those of the product and sum in px give |v - w| <= e (3 D + 3 T / cell
// + 2 X + |v|) to first order, and the reference's u = RN(RN(RN(px - x0) /
// cell) + 0.5) has |u - (w + 0.5)| <= e (2.0001 D + 1.0001 |u|). Where |v| <=
// M + 2 (M = max(nx, ny)) that is |u - (v + 0.5)| <= e (7.0002 M + 3 T / cell
// + 2 X + 14.6), inside mdelta = e (7.001 M + 2.001 X + 3.001 RANGE / cell +
// 16) (TrackDev.mband = 0.5 - mdelta): a v farther than mdelta from every
// half-integer has floor(u) = rint(v), and farther out both are off the map.
// Inside the band, and for NaN and infinities, the point's own coordinates
// go through cell_coord.
// The nearest integer comes from adding and subtracting 1.5 * 2^23 (exactly
// rint(v) for |v| < 2^22) and the cell from the sum's bits less those of
// 1.5 * 2^23, in unsigned arithmetic: for |v| >= 2^22 that is >= 2^22 > nx,
// so such points are off the map on either path, as they are for the
// reference. The unsigned column clamped to nx and row to ny then land
// off-map points on a border cell: no conversion, compare or select on the
// common path.
__device__ __forceinline__ unsigned lidar_cell(const TrackDev& t, float vx, float vy, float tt, float ox, float oy,
                                               float dx, float dy) {
  constexpr float MAGIC = 12582912.0f;  // 1.5 * 2^23
  const float mx = vx + MAGIC, my = vy + MAGIC;
  const float rx = mx - MAGIC, ry = my - MAGIC;
  unsigned ix, iy;
  if (fabsf(vx - rx) < t.mband && fabsf(vy - ry) < t.mband) {
    ix = (unsigned)__float_as_int(mx) - 0x4B400000u, iy = (unsigned)__float_as_int(my) - 0x4B400000u;
  } else {
    const float px = ox + tt * dx, py = oy + tt * dy;
    const float fx = cell_coord(px, t.x0, t.cell, t.inv_cell), fy = cell_coord(py, t.y0, t.cell, t.inv_cell);
    const bool on = fx >= 0.0f && fx < t.nxf && fy >= 0.0f && fy < t.nyf;
    ix = on ? (unsigned)(int)fx : 0xFFFFFFFFu, iy = on ? (unsigned)(int)fy : 0xFFFFFFFFu;
  }
  return min(iy, (unsigned)t.ny) * (unsigned)t.lw + min(ix, (unsigned)t.nx);
}

// racer/sim.mojo:116-124. LAYERS = 0 reads the layer count from the track.
// The first drivable layer is taken only if |height - z| < 1e30 (the initial
// gap). GUARD = false drops that test where it cannot fail: grid heights are
// finite with |h| <= 1e6 (checked on upload) and the caller knows |z| <= 1e20
// + 10, so the result is the same.
template <int LAYERS, bool GUARD = true>
__device__ __forceinline__ Spot probe(const TrackDev& t, float x, float y, float z) {
  long idx;
  if (!cell_of(t, x, y, &idx)) return Spot{0, -1.0f, -1.0f};  // off the map every grid reads -1
  Spot best;
  float gap = 1e30f;
  if (LAYERS == 2) {
    float4 v = __ldg(reinterpret_cast<const float4*>(t.cl) + idx);
    best = Spot{0, -1.0f, v.y};
    if (v.x > 0.0f && (!GUARD || fabsf(v.y - z) < gap)) {
      best = Spot{0, v.x, v.y};
      gap = fabsf(v.y - z);
    }
    if (v.z > 0.0f && fabsf(v.w - z) < gap) best = Spot{1, v.z, v.w};
  } else if (LAYERS == 1) {
    float2 v = __ldg(t.cl + idx);
    best = Spot{0, -1.0f, v.y};
    if (v.x > 0.0f && (!GUARD || fabsf(v.y - z) < gap)) best = Spot{0, v.x, v.y};
  } else {
    const int L = t.layers;
    const float2* p = t.cl + idx * L;
    float2 v0 = __ldg(p);
    best = Spot{0, -1.0f, v0.y};
    for (int l = 0; l < L; ++l) {
      float2 v = __ldg(p + l);
      if (v.x > 0.0f && fabsf(v.y - z) < gap) {
        best = Spot{l, v.x, v.y};
        gap = fabsf(v.y - z);
      }
    }
  }
  return best;
}

// probe<LAYERS, false>'s (clearance - cell, height - z) for one or two layers
// at the march's point (lidar_cell's arguments, height z), from the lidar's
// cells: RN(height - z), the negation of the reference's RN(z - height), which
// the layer choice computes anyway. Per cell they hold (c0 - cell, h0, c1 - cell, h1), the clearance of
// an undrivable layer as -1; slot 1 holds layer 1 only where both layers are
// drivable and a NaN height otherwise, which never compares nearer, and a
// cell where only layer 1 is drivable holds it in slot 0. So layer 1 is taken
// exactly where probe takes it: where both are drivable and |h1 - z| <
// |h0 - z|, or where only it is (probe's test |h1 - z| < 1e30 cannot fail
// with |z| <= 1e20 + 10 and |h1| <= 1e6). The border cells read clearance and
// height -1, as off the map.
template <int LAYERS>
__device__ __forceinline__ float2 lidar_probe(const TrackDev& t, float vx, float vy, float tt, float ox, float oy,
                                              float dx, float dy, float z) {
  const unsigned idx = lidar_cell(t, vx, vy, tt, ox, oy, dx, dy);
  if (LAYERS == 2) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(t.lc) + idx);
    const float d0 = v.y - z, d1 = v.w - z;
    return fabsf(d1) < fabsf(d0) ? make_float2(v.z, d1) : make_float2(v.x, d0);
  }
  const float2 v = __ldg(reinterpret_cast<const float2*>(t.lc) + idx);
  return make_float2(v.x, v.y - z);
}

// racer/sim.mojo:126-140: bilinear height and its gradient, in two parts: the
// cell and weights (independent of the layer) and the corner heights.
struct SurfaceCell {
  long base;  // offset of corner (ix, iy) within a layer's height grid
  float tx, ty;
};

__device__ __forceinline__ SurfaceCell surface_cell(const TrackDev& t, float x, float y) {
  float fx = (x - t.x0) / t.cell;
  float fy = (y - t.y0) / t.cell;
  float flx = floorf(fx), fly = floorf(fy);
  int ix = flx >= 0.0f ? (flx <= (float)(t.nx - 2) ? (int)flx : t.nx - 2) : 0;
  int iy = fly >= 0.0f ? (fly <= (float)(t.ny - 2) ? (int)fly : t.ny - 2) : 0;
  return SurfaceCell{(long)iy * t.nx + ix, clampf_(fx - (float)ix, 0.0f, 1.0f), clampf_(fy - (float)iy, 0.0f, 1.0f)};
}

__device__ __forceinline__ float4 surface_corners(const TrackDev& t, int layer, long base) {
  const float* hp = t.d + HEADER + (long)(3 * layer + 1) * t.nx * t.ny + base;
  return make_float4(__ldg(hp), __ldg(hp + 1), __ldg(hp + t.nx), __ldg(hp + t.nx + 1));
}

__device__ __forceinline__ Surface surface_blend(const TrackDev& t, const SurfaceCell& c, float4 h) {
  const float tx = c.tx, ty = c.ty;
  float w0 = (1.0f - tx) * (1.0f - ty), w1 = tx * (1.0f - ty), w2 = (1.0f - tx) * ty, w3 = tx * ty;
  Surface s;
  s.height = (h.x * w0 + h.z * w2) + (h.y * w1 + h.w * w3);
  s.sx = ((h.y - h.x) * (1.0f - ty) + (h.w - h.z) * ty) / t.cell;
  s.sy = ((h.z - h.x) * (1.0f - tx) + (h.w - h.y) * tx) / t.cell;
  return s;
}

__device__ __forceinline__ Surface surface(const TrackDev& t, int layer, float x, float y) {
  const SurfaceCell c = surface_cell(t, x, y);
  return surface_blend(t, c, surface_corners(t, layer, c.base));
}

// Probe and the surface under the chosen layer. With two layers the corner
// heights of both layers are loaded alongside the probe and those of the
// chosen layer blended, so the loads do not wait for the layer.
template <int LAYERS>
__device__ __forceinline__ Surface probe_surface(const TrackDev& t, float x, float y, float z, Spot* spot) {
  if (LAYERS == 2) {
    const SurfaceCell c = surface_cell(t, x, y);
    const float4 h0 = surface_corners(t, 0, c.base), h1 = surface_corners(t, 1, c.base);
    *spot = probe<LAYERS>(t, x, y, z);
    return surface_blend(t, c, spot->layer ? h1 : h0);
  }
  *spot = probe<LAYERS>(t, x, y, z);
  return surface(t, spot->layer, x, y);
}

__device__ __forceinline__ float waypoint(const TrackDev& t, long w, int field) {
  return __ldg(t.d + t.route + 4 * w + field);
}

// racer/sim.mojo:146-152. Off the map the nearest grid reads -1 and the
// route lookup lands on d[route - 4 + field], as in the reference.
__device__ __forceinline__ float progress(const TrackDev& t, int layer, float x, float y) {
  long idx;
  long w = -1;
  if (cell_of(t, x, y, &idx)) w = (long)__ldg(t.d + HEADER + (long)(3 * layer + 2) * t.nx * t.ny + idx);
  float heading = waypoint(t, w, 3);
  float s, c;
  rmath::sincosf_(heading, &s, &c);
  float along = (x - waypoint(t, w, 0)) * c + (y - waypoint(t, w, 1)) * s;
  return (float)w + along / t.spacing;
}

struct V4 {
  float x, y, h, s;  // position, heading, speed
};

// racer/sim.mojo:155-167
__device__ __forceinline__ V4 derivative(const V4& p, float steer, float accel, float grip, float along,
                                         float across) {
  float nz = 1.0f / sqrtf((1.0f + along * along) + across * across);
  float load = (grip * GRAV) * nz;
  float v = fmaxf(fabsf(p.s), 0.5f) * (p.s >= 0.0f ? 1.0f : -1.0f);
  float slide = (GRAV * across) * nz;
  float ss, cs;
  rmath::sincosf_(steer, &ss, &cs);
  float lateral = clampf_((((v * p.s) * ss) / cs) / WHEELBASE + slide, -load, load);
  float yaw = (lateral - slide) / v;
  float longitudinal = sqrtf(fmaxf(load * load - lateral * lateral, 0.0f));
  float dv = clampf_(accel, -longitudinal, longitudinal) - (GRAV * along) * nz;
  float sh, ch;
  rmath::sincosf_(p.h, &sh, &ch);
  return V4{p.s * ch, p.s * sh, yaw, dv};
}

__device__ __forceinline__ V4 axpy(const V4& p, const V4& k, float h) {
  return V4{p.x + k.x * h, p.y + k.y * h, p.h + k.h * h, p.s + k.s * h};
}

// racer/sim.mojo:170-181. `local` is the car's index within its track's
// segment (its Philox counter); i is its column in the batch. Returns the
// pose written (x, y, z, heading).
__device__ float4 spawn(const TrackDev& t, float* s, int n, int i, int local, uint64_t seed) {
  float episode = s[(long)EPISODE * n + i] + 1.0f;
  float r[4];
  philox::uniform4(seed, (uint64_t)local, (uint64_t)episode, r);
  int w = min((int)(r[0] * (float)t.waypoints), t.waypoints - 1);
  const float4 pose = make_float4(waypoint(t, w, 0), waypoint(t, w, 1), waypoint(t, w, 2), waypoint(t, w, 3));
  for (int row = 0; row < STATE; ++row) s[(long)row * n + i] = 0.0f;
  s[(long)X * n + i] = pose.x;
  s[(long)Y * n + i] = pose.y;
  s[(long)Z * n + i] = pose.z;
  s[(long)HEADING * n + i] = pose.w;
  s[(long)PROGRESS * n + i] = (float)w;
  s[(long)EPISODE * n + i] = episode;
  s[(long)FRICTION * n + i] = 0.85f + 0.3f * r[1];
  return pose;
}

// Segment of car i (segments are few; a short scan).
__device__ __forceinline__ int segment_of(const Segments& g, int i) {
  int k = 0;
  while (k + 1 < g.count && i >= g.car0[k + 1]) ++k;
  return k;
}

__global__ void k_spawn(const __grid_constant__ Segments g, float* state, float* actions, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = segment_of(g, i);
  spawn(g.t[k], state, n, i, i - g.car0[k], g.seed[k]);
  actions[i] = 0.0f;
  actions[(long)n + i] = 0.0f;
}

// racer/sim.mojo:184-235: one 60 Hz step of car i (segment index local).
template <int LAYERS>
__device__ __forceinline__ void advance_car(const TrackDev& t, float* s, const float* act, float* reward, float* done,
                                            float* obs, int n, int beams, uint64_t seed, float4* ray, int i,
                                            int local) {
  V4 p{s[(long)X * n + i], s[(long)Y * n + i], s[(long)HEADING * n + i], s[(long)SPEED * n + i]};
  Spot spot;
  Surface ground = probe_surface<LAYERS>(t, p.x, p.y, s[(long)Z * n + i], &spot);
  float steer = s[(long)STEER * n + i];
  float rate = clampf_(act[i], -1.0f, 1.0f) * STEER_RATE;
  float accel = clampf_(act[(long)n + i], -1.0f, 1.0f) * ACCEL_MAX;
  float grip = GRIP * s[(long)FRICTION * n + i];
  bool crashed = false;
  const float half_dt = DT / 2.0f, sixth_dt = DT / 6.0f;
#pragma unroll 1
  for (int sub = 0; sub < SUBSTEPS; ++sub) {
    float along, across;
    slopes(ground, p.h, &along, &across);
    float mid = steer + (rate * DT) / 2.0f;
    V4 k1 = derivative(p, steer, accel, grip, along, across);
    V4 k2 = derivative(axpy(p, k1, half_dt), mid, accel, grip, along, across);
    V4 k3 = derivative(axpy(p, k2, half_dt), mid, accel, grip, along, across);
    V4 k4 = derivative(axpy(p, k3, DT), steer + rate * DT, accel, grip, along, across);
    p.x = p.x + ((k1.x + 2.0f * (k2.x + k3.x)) + k4.x) * sixth_dt;
    p.y = p.y + ((k1.y + 2.0f * (k2.y + k3.y)) + k4.y) * sixth_dt;
    p.h = p.h + ((k1.h + 2.0f * (k2.h + k3.h)) + k4.h) * sixth_dt;
    p.s = p.s + ((k1.s + 2.0f * (k2.s + k3.s)) + k4.s) * sixth_dt;
    p.s = clampf_(p.s, -SPEED_MAX, SPEED_MAX);
    steer = clampf_(steer + rate * DT, -STEER_MAX, STEER_MAX);
    ground = probe_surface<LAYERS>(t, p.x, p.y, spot.height, &spot);
    crashed = crashed || spot.clearance < HALF_DIAG || ground.sx * ground.sx + ground.sy * ground.sy > 1.0f;
  }
  if (p.h > PI_F) p.h -= TWO_PI_F;
  if (p.h < -PI_F) p.h += TWO_PI_F;
  float prog = progress(t, spot.layer, p.x, p.y);
  float dp = prog - s[(long)PROGRESS * n + i];
  float half = (float)t.waypoints / 2.0f;
  dp = dp > half ? dp - 2.0f * half : (dp < -half ? dp + 2.0f * half : dp);
  float score = crashed ? -2.0f : ((10.0f * dp) * t.spacing - (0.001f * steer) * steer);
  float steps = s[(long)STEPS * n + i] + 1.0f;
  float reason = (float)(crashed ? CRASH : (steps >= (float)HORIZON ? TIMEOUT : 0));
  s[(long)X * n + i] = p.x;
  s[(long)Y * n + i] = p.y;
  s[(long)Z * n + i] = spot.height;
  s[(long)HEADING * n + i] = p.h;
  s[(long)SPEED * n + i] = p.s;
  s[(long)STEER * n + i] = steer;
  s[(long)STEPS * n + i] = steps;
  s[(long)PROGRESS * n + i] = prog;
  s[(long)RETURN * n + i] = s[(long)RETURN * n + i] + score;
  reward[i] = score;
  done[i] = reason;
  float heading = p.h, speed = p.s;
  // the pose the lidar frame starts from: the one just stored, and the layer
  // the last probe chose (a probe at this cell with the height it returned
  // selects that layer again)
  float fx = p.x, fy = p.y, fz = spot.height;
  int layer = spot.layer;
  if (reason > 0.0f) {
    const float4 pose = spawn(t, s, n, i, local, seed);
    fx = pose.x, fy = pose.y, fz = pose.z, heading = pose.w;
    layer = probe<LAYERS>(t, fx, fy, fz).layer;
    ground = surface(t, layer, fx, fy);
    speed = 0.0f;
    steer = 0.0f;
  }
  float along, across;
  slopes(ground, heading, &along, &across);
  obs[i] = steer / STEER_MAX;
  obs[(long)n + i] = speed / SPEED_MAX;
  obs[2L * n + i] = along;
  obs[3L * n + i] = across;
  obs[(long)(beams + 4) * n + i] = 1.0f;
  // The lidar's per-car frame (racer/sim.mojo:243-249), from the values just
  // written: origin = position + MOUNT_X forward + MOUNT_Z up, and the
  // heading's cos/sin with the slopes that tilt the body plane; .w of the
  // second half carries the car's layer (surrogate input).
  float ch, sh;
  rmath::sincosf_(heading, &sh, &ch);
  ray[i] = make_float4((fx + MOUNT_X * ch) + 0.0f, (fy + MOUNT_X * sh) + 0.0f, (fz + MOUNT_X * along) + MOUNT_Z, ch);
  ray[n + i] = make_float4(sh, along, across, (float)layer);
}

// With eval_reward set, each car also adds its reward (FP64) and a crash
// count to its own accumulators (racer eval's sums, kept on the device).
__global__ void k_advance(const __grid_constant__ Segments g, float* s, const float* act, float* reward, float* done,
                          float* obs, int n, int beams, float4* ray, double* eval_reward, int* eval_crash, int c0,
                          int c1) {
  const int i = c0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= c1) return;
  const int k = segment_of(g, i);
  const TrackDev& t = g.t[k];
  if (t.layers == 1)
    advance_car<1>(t, s, act, reward, done, obs, n, beams, g.seed[k], ray, i, i - g.car0[k]);
  else if (t.layers == 2)
    advance_car<2>(t, s, act, reward, done, obs, n, beams, g.seed[k], ray, i, i - g.car0[k]);
  else
    advance_car<0>(t, s, act, reward, done, obs, n, beams, g.seed[k], ray, i, i - g.car0[k]);
  if (eval_reward) {
    eval_reward[i] += (double)reward[i];
    eval_crash[i] += done[i] == (float)CRASH;
  }
}

// FP64 re-integration of racer/sim.mojo:189-213 (the 4 RK4 substeps) for
// the accuracy audit: the same ODE and parameters in double precision with
// CUDA's double sin/cos/sqrt; map lookups stay binary32 at the rounded
// position, as the map itself is binary32.
__device__ void derivative64(const double* p, double steer, double accel, double grip, double along,
                             double across, double* out) {
  const double G = (double)GRAV, WB = (double)WHEELBASE;
  const double nz = 1.0 / sqrt((1.0 + along * along) + across * across);
  const double load = (grip * G) * nz;
  const double v = fmax(fabs(p[3]), 0.5) * (p[3] >= 0.0 ? 1.0 : -1.0);
  const double slide = (G * across) * nz;
  const double lateral = fmin(fmax((((v * p[3]) * sin(steer)) / cos(steer)) / WB + slide, -load), load);
  const double yaw = (lateral - slide) / v;
  const double longitudinal = sqrt(fmax(load * load - lateral * lateral, 0.0));
  const double dv = fmin(fmax(accel, -longitudinal), longitudinal) - (G * along) * nz;
  out[0] = p[3] * cos(p[2]);
  out[1] = p[3] * sin(p[2]);
  out[2] = yaw;
  out[3] = dv;
}

// Per car that did not end its episode this step: |position|, |heading| and
// |speed| differences between the FP32 step (next) and the FP64 re-integration
// from the same state (prev) and actions. stats: [0] count, [1..3] sums,
// [4..6] maxima (as doubles).
template <int LAYERS>
__device__ void rk4_f64_car(const TrackDev& t, const float* prev, const float* act, const float* next, int n,
                            double* stats, int i) {
  double p[4] = {prev[(long)X * n + i], prev[(long)Y * n + i], prev[(long)HEADING * n + i],
                 prev[(long)SPEED * n + i]};
  Spot spot = probe<LAYERS>(t, (float)p[0], (float)p[1], prev[(long)Z * n + i]);
  Surface ground = surface(t, spot.layer, (float)p[0], (float)p[1]);
  double steer = prev[(long)STEER * n + i];
  const double rate = (double)(clampf_(act[i], -1.0f, 1.0f) * STEER_RATE);
  const double accel = (double)(clampf_(act[(long)n + i], -1.0f, 1.0f) * ACCEL_MAX);
  const double grip = (double)(GRIP * prev[(long)FRICTION * n + i]);
  const double dt = 1.0 / 240.0;
  for (int sub = 0; sub < SUBSTEPS; ++sub) {
    const double c = cos(p[2]), s = sin(p[2]);
    const double along = (double)ground.sx * c + (double)ground.sy * s;
    const double across = -(double)ground.sx * s + (double)ground.sy * c;
    double k1[4], k2[4], k3[4], k4[4], q[4];
    derivative64(p, steer, accel, grip, along, across, k1);
    for (int j = 0; j < 4; ++j) q[j] = p[j] + k1[j] * (dt / 2);
    derivative64(q, steer + rate * dt / 2, accel, grip, along, across, k2);
    for (int j = 0; j < 4; ++j) q[j] = p[j] + k2[j] * (dt / 2);
    derivative64(q, steer + rate * dt / 2, accel, grip, along, across, k3);
    for (int j = 0; j < 4; ++j) q[j] = p[j] + k3[j] * dt;
    derivative64(q, steer + rate * dt, accel, grip, along, across, k4);
    for (int j = 0; j < 4; ++j) p[j] += (k1[j] + 2 * (k2[j] + k3[j]) + k4[j]) * (dt / 6);
    p[3] = fmin(fmax(p[3], -(double)SPEED_MAX), (double)SPEED_MAX);
    steer = fmin(fmax(steer + rate * dt, -(double)STEER_MAX), (double)STEER_MAX);
    spot = probe<LAYERS>(t, (float)p[0], (float)p[1], spot.height);
    ground = surface(t, spot.layer, (float)p[0], (float)p[1]);
  }
  const double pi = 3.141592653589793;
  double dh = (double)next[(long)HEADING * n + i] - p[2];
  dh -= 2 * pi * rint(dh / (2 * pi));
  const double dx = (double)next[(long)X * n + i] - p[0], dy = (double)next[(long)Y * n + i] - p[1];
  const double e[3] = {sqrt(dx * dx + dy * dy), fabs(dh), fabs((double)next[(long)SPEED * n + i] - p[3])};
  atomicAdd(stats, 1.0);
  for (int k = 0; k < 3; ++k) {
    atomicAdd(stats + 1 + k, e[k]);
    unsigned long long* mx = reinterpret_cast<unsigned long long*>(stats + 4 + k);
    atomicMax(mx, (unsigned long long)__double_as_longlong(e[k]));  // nonnegative doubles order as integers
  }
}

__global__ void k_rk4_f64(const __grid_constant__ Segments g, const float* prev, const float* act, const float* next,
                          const float* done, int n, double* stats) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || done[i] != 0.0f) return;
  const TrackDev& t = g.t[segment_of(g, i)];
  if (t.layers == 1)
    rk4_f64_car<1>(t, prev, act, next, n, stats, i);
  else if (t.layers == 2)
    rk4_f64_car<2>(t, prev, act, next, n, stats, i);
  else
    rk4_f64_car<0>(t, prev, act, next, n, stats, i);
}

// The lidar frame of a car at rest on a layer (racer/sim.mojo:229-234,
// 243-249): pose (x, y, heading, layer) -> z = the layer's bilinear height,
// the slopes along and across the heading, and the same frame k_advance
// writes. Used to label surrogate training poses with the exact tracer.
__global__ void k_pose_frames(TrackDev t, const float4* __restrict__ poses, int count, float4* ray) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float4 p = poses[i];
  const int layer = (int)p.w;
  const Surface g = surface(t, layer, p.x, p.y);
  float along, across;
  slopes(g, p.z, &along, &across);
  float ch, sh;
  rmath::sincosf_(p.z, &sh, &ch);
  ray[i] = make_float4((p.x + MOUNT_X * ch) + 0.0f, (p.y + MOUNT_X * sh) + 0.0f, (g.height + MOUNT_X * along) + MOUNT_Z,
                       ch);
  ray[count + i] = make_float4(sh, along, across, (float)layer);
}

// racer/sim.mojo:238-266: the sphere-traced lidar, one thread per (car, beam).
// A block holds a few warps; each warp marches 32 consecutive beams of one
// car, so its lanes start at one origin and probe neighbouring cells (L1
// reuse) and finish after similar numbers of probes. The per-car
// frame comes from the physics kernel (`ray`). Every result of a beam is the
// reference's: its operations are the reference's, in its order, except
// where another sequence provably gives the same bits: the nearest-cell
// index (cell_of, and along the ray lidar_cell: one fused multiply-add, the
// division only near a cell boundary), the probe's layer choice (lidar_probe:
// folded into the lidar's own cells where it does not depend on the ray),
// the probe count (dropped where its bound cannot end the march) and
// floor/descent (quotient: two residual corrections of the reciprocal; the
// guarded march divides only where min() can select it).
template <int LAYERS, bool NC = true>
__device__ __forceinline__ void trace(const TrackDev& t, const float4* ray, float* obs, int n,
                                      const float2* __restrict__ beam_dir, int max_iters, int* iters, int car,
                                      int beam);

// The lidar grid: the blocks of the segment in slot j of the launch order are
// [block0[j], block0[j + 1]), each covering `cars` consecutive cars of it.
struct LidarGrid {
  int order[MAX_SEGMENTS];
  int block0[MAX_SEGMENTS + 1];
};

__device__ __forceinline__ void trace_any(const TrackDev& t, const float4* __restrict__ ray, float* obs, int n,
                                          const float2* __restrict__ beam_dir, int max_iters, int* iters, int car,
                                          int beam) {
  if (t.layers == 1)
    trace<1>(t, ray, obs, n, beam_dir, max_iters, iters, car, beam);
  else if (t.layers == 2)
    trace<2>(t, ray, obs, n, beam_dir, max_iters, iters, car, beam);
  else
    trace<0>(t, ray, obs, n, beam_dir, max_iters, iters, car, beam);
}

// Resident blocks per SM a lidar kernel is compiled for: all 64 warp slots
// (32 registers a thread) or, for the wide variant, 48 of them (40 registers).
constexpr int lidar_min_blocks(int cars, bool wide) {
  return (wide ? 48 : 64) / cars < 32 ? (wide ? 48 : 64) / cars : 32;
}

// One track (cars [c0, c1) of the batch): its fields are kernel parameters,
// read as constant operands. CARS warps per block (one car each): small
// blocks release their slot as soon as their few cars finish.
template <int LAYERS, int CARS, bool WIDE, bool LIST>
__global__ void __launch_bounds__(CARS * 32, lidar_min_blocks(CARS, WIDE))
    k_lidar_track(TrackDev t, int max_iters, const float4* __restrict__ ray, float* obs, int n, int c0, int c1,
                  int beams, const float2* __restrict__ beam_dir, int* iters, const int* __restrict__ list,
                  const int* list_count) {
  const int beam = blockIdx.y * 32 + (threadIdx.x & 31);
  if (beam >= beams) return;
  if (LIST) {  // only the listed cars (surrogate fallback), grid-stride over the list
    const int count = *list_count;
    for (int q = blockIdx.x * CARS + (threadIdx.x >> 5); q < count; q += gridDim.x * CARS) {
      const int car = list[q];
      if (car < n) trace<LAYERS>(t, ray, obs, n, beam_dir, max_iters, iters, car, beam);
    }
    return;
  }
  const int car = c0 + (int)blockIdx.x * CARS + (int)(threadIdx.x >> 5);
  if (car < c1) trace<LAYERS>(t, ray, obs, n, beam_dir, max_iters, iters, car, beam);
}

// One track with the (car, beam) items of cars [c0, c0 + items / beams) in
// car-major order, 32 consecutive items per warp: a warp may hold the last
// beams of one car and the first of the next, so no lane idles at the end of
// a car's beams when the beam count is not a multiple of 32 (108 beams fill
// 3.375 warps a car). Each beam is traced exactly as in k_lidar_track.
template <int LAYERS, int CARS, bool WIDE>
__global__ void __launch_bounds__(CARS * 32, lidar_min_blocks(CARS, WIDE))
    k_lidar_flat(TrackDev t, int max_iters, const float4* __restrict__ ray, float* obs, int n, int c0,
                 unsigned items, int beams, const float2* __restrict__ beam_dir, int* iters) {
  const unsigned item = (blockIdx.x * CARS + (threadIdx.x >> 5)) * 32u + (threadIdx.x & 31);
  if (item >= items) return;
  const unsigned car = item / (unsigned)beams;
  trace<LAYERS>(t, ray, obs, n, beam_dir, max_iters, iters, c0 + (int)car, (int)(item - car * (unsigned)beams));
}

// Dynamic variant of k_lidar_track: a persistent grid whose warps take
// (car, 32-beam group) units from `counter` (zero at launch) one at a time,
// so no warp holds a block slot waiting for a sibling and the last wave has
// no tail of idle slots.
// With LIST, the cars are list[0 .. *list_count) (the surrogate's fallback
// cars, counted on the device), whatever their number.
template <int LAYERS, bool WIDE, bool LIST>
__global__ void __launch_bounds__(128, lidar_min_blocks(4, WIDE))
    k_lidar_dynamic(TrackDev t, int max_iters, const float4* __restrict__ ray, float* obs, int n, int c0, int c1,
                    int beams, const float2* __restrict__ beam_dir, int* iters, unsigned* counter,
                    const int* __restrict__ list, const int* list_count) {
  const int groups = (beams + 31) >> 5;
  const unsigned cars = LIST ? (unsigned)min(max(*list_count, 0), n) : (unsigned)(c1 - c0);
  const unsigned total = cars * (unsigned)groups;
  const int lane = threadIdx.x & 31;
  // the next unit is claimed before the current one is traced, so the atomic's
  // round trip overlaps the march
  unsigned next = 0;
  if (lane == 0) next = atomicAdd(counter, 1u);
  unsigned unit = __shfl_sync(0xffffffffu, next, 0);
  while (unit < total) {
    if (lane == 0) next = atomicAdd(counter, 1u);
    const int car = LIST ? list[unit / (unsigned)groups] : c0 + (int)(unit / (unsigned)groups);
    const int beam = (int)(unit % (unsigned)groups) * 32 + lane;
    if (beam < beams && (unsigned)car < (unsigned)n) trace<LAYERS>(t, ray, obs, n, beam_dir, max_iters, iters, car, beam);
    unit = __shfl_sync(0xffffffffu, next, 0);
  }
}

// Several tracks: a block's segment depends on blockIdx only, so the track's
// fields are block-uniform.
template <int CARS, bool WIDE>
__global__ void __launch_bounds__(CARS * 32, lidar_min_blocks(CARS, WIDE))
    k_lidar_segments(const __grid_constant__ Segments g, const __grid_constant__ LidarGrid lg,
                     const float4* __restrict__ ray, float* obs, int n, int beams,
                     const float2* __restrict__ beam_dir, int* iters) {
  const int beam = blockIdx.y * 32 + (threadIdx.x & 31);
  if (beam >= beams) return;
  int j = 0;
  while (j + 1 < g.count && (int)blockIdx.x >= lg.block0[j + 1]) ++j;
  const int k = lg.order[j];
  const int car = g.car0[k] + ((int)blockIdx.x - lg.block0[j]) * CARS + (int)(threadIdx.x >> 5);
  if (car < g.car0[k + 1]) trace_any(g.t[k], ray, obs, n, beam_dir, g.max_iters[k], iters, car, beam);
}

template <int LAYERS, bool GUARD, bool COUNTED = true>
__device__ __forceinline__ float march(const TrackDev& t, float ox, float oy, float oz, float dx, float dy, float dz,
                                       float descent, float inv_descent, int max_iters, int* count_out);

// The range of one beam (racer/sim.mojo:240-266); `count` gets its probes.
// NC: the ray frames are read-only for the whole launch (the read-only data
// path); the fused rollout, which rewrites them every step, loads them
// through L2 instead, where the block's own writes before a barrier are seen.
template <int LAYERS, bool NC = true>
__device__ __forceinline__ float beam_range(const TrackDev& t, const float4* ray, int n,
                                            const float2* __restrict__ beam_dir, int max_iters, bool counted,
                                            int car, int beam, int* count_out);

__device__ __forceinline__ float quotient(float a, float b, float y, float q0);

// RN(a / b) for b normal and a zero or normal of either sign, from y = RN(1 / b):
// the quotient's residual corrections (a sign-symmetric computation), with a
// zero returned as itself so that -0 / b stays -0.
__device__ __forceinline__ float div_by(float a, float b, float y) { return a == 0.0f ? a : quotient(a, b, y, a * y); }

// range / RANGE for a range in [0, RANGE] (the march's result): below 2^-60
// the IEEE division; above, the corrections with RN(1 / 10) = 0.1f, whose
// steps scale with the dividend's exponent there (no subnormal intermediate),
// so one binade checked exhaustively (tests/test_cell_index.py) covers them all.
__device__ __forceinline__ float range_obs(float range) {
  static_assert(RANGE == 10.0f, "range_obs divides by 10");
  return range < 8.67361738e-19f ? range / RANGE : quotient(range, RANGE, 0.1f, range * 0.1f);
}

template <int LAYERS, bool NC>
__device__ __forceinline__ void trace(const TrackDev& t, const float4* ray, float* obs, int n,
                                      const float2* __restrict__ beam_dir, int max_iters, int* iters, int car,
                                      int beam) {
  int count = 0;
  const float range = beam_range<LAYERS, NC>(t, ray, n, beam_dir, max_iters, iters != nullptr, car, beam, &count);
  obs[(long)(4 + beam) * n + car] = range_obs(range);
  if (iters) iters[(long)beam * n + car] = count;
}

template <int LAYERS, bool NC>
__device__ __forceinline__ float beam_range(const TrackDev& t, const float4* ray, int n,
                                            const float2* __restrict__ beam_dir, int max_iters, bool counted,
                                            int car, int beam, int* count_out) {
  // (ox, oy, oz, cos h), (sin h, along, across)
  const float4 r0 = NC ? __ldg(ray + car) : __ldcg(ray + car), r1 = NC ? __ldg(ray + n + car) : __ldcg(ray + n + car);
  const float2 az = __ldg(beam_dir + beam);                        // (cos azimuth, sin azimuth)
  float dx = az.x * r0.w + az.y * -r1.x;
  float dy = az.x * r1.x + az.y * r0.w;
  float dz = az.x * r1.y + az.y * r1.z;
  const float norm = sqrtf((dx * dx + dz * dz) + (dy * dy + 0.0f));
  // the reference's three divisions by norm, a normal number (at least about
  // 1: the heading rotation keeps dx^2 + dy^2 near 1) unless the frame holds a
  // NaN or an infinity, which take the IEEE divisions
  if (norm <= 3.40282347e38f) {
    const float rnorm = 1.0f / norm;
    dx = div_by(dx, norm, rnorm);
    dy = div_by(dy, norm, rnorm);
    dz = div_by(dz, norm, rnorm);
  } else {
    dx = dx / norm;
    dy = dy / norm;
    dz = dz / norm;
  }
  const float ox = r0.x, oy = r0.y, oz = r0.z;
  const float descent = (1.5f * t.slope) * sqrtf(dx * dx + dy * dy) + fmaxf(-dz, 0.0f);
  const float inv_descent = 1.0f / descent;
  int count = 0;
  // every probe height lies within RANGE of the origin's (|dz| <= 1): with
  // |oz| <= 1e20 the probe's height guard cannot fail (NaN takes the guarded loop)
  // the unguarded march also needs a descent of 0 or a normal number (its quotient; see march)
  // where the probe bound provably never ends the march first (TrackDev.free_march)
  // and no count is asked for, the loop tests tt < RANGE alone, as the reference does
  float range;
  if (!(fabsf(oz) <= 1e20f && (descent == 0.0f || descent >= 1.17549435e-38f)))
    range = march<LAYERS, true>(t, ox, oy, oz, dx, dy, dz, descent, inv_descent, max_iters, &count);
  else if (counted || !t.free_march)
    range = march<LAYERS, false>(t, ox, oy, oz, dx, dy, dz, descent, inv_descent, max_iters, &count);
  else
    range = march<LAYERS, false, false>(t, ox, oy, oz, dx, dy, dz, descent, inv_descent, max_iters, &count);
  *count_out = count;
  return range;
}

// RN(a / b) from y = RN(1 / b) and q0 = RN(a * y), by two residual
// corrections (Markstein, IBM J. Res. Dev. 34(1), 1990): r = a - b q is exact
// in one fused multiply-add when q is within a few ulps of a / b, and
// RN(q + r y) is then the correctly rounded quotient once q is faithful,
// which the first correction makes it. For the march's operands (0 <= a,
// b >= 0, neither subnormal) this is the IEEE quotient whenever that is
// finite; for b = 0, an overflowing product or a NaN it gives NaN or +inf.
// Checked against IEEE division on random and near-midpoint quotients
// (tests/test_cell_index.py) and by the bit-exact lidar tests.
__device__ __forceinline__ float quotient(float a, float b, float y, float q0) {
  const float q1 = __fmaf_rn(__fmaf_rn(-q0, b, a), y, q0);
  return __fmaf_rn(__fmaf_rn(-q1, b, a), y, q1);
}

// The march of one beam (racer/sim.mojo:252-266); returns the range.
template <int LAYERS, bool GUARD, bool COUNTED>
__device__ __forceinline__ float march(const TrackDev& t, float ox, float oy, float oz, float dx, float dy, float dz,
                                       float descent, float inv_descent, int max_iters, int* count_out) {
  const float cell = t.cell, min_step = 0.5f * t.cell;
  float tt = 0.0f, last = 0.0f, last_floor = 0.0f, range = -1.0f;
  int count = 0;
  if (!GUARD) {
    // descent is 0 or normal here: the quotient is RN(fl / descent) whenever
    // it is finite and below the clearance term; otherwise it is >= that term
    // or NaN (fl / 0, or a product that overflowed), and fminf returns the
    // clearance term as for the reference's min(a, inf) or min(a, NaN). The
    // step is computed before the ground test and unused once the ground is
    // crossed, so one branch ends the march on either condition.
    constexpr bool CELLS = LAYERS == 1 || LAYERS == 2;  // the lidar's cells (lidar_probe)
    const float ax = CELLS ? dx * t.inv_cell : 0.0f, ay = CELLS ? dy * t.inv_cell : 0.0f;
    const float bx = CELLS ? __fmaf_rn(ox, t.inv_cell, t.cx) : 0.0f, by = CELLS ? __fmaf_rn(oy, t.inv_cell, t.cy) : 0.0f;
    // The loop enters with tt = 0 < RANGE; one exit test a probe covers the
    // ground crossed, a step below the minimum and the next probe at or past
    // RANGE (or past the probe bound), where the reference's loop test would
    // fail after tt += step.
    float fl, step, next;
    for (;;) {
      if (COUNTED) ++count;
      const float pz = oz + tt * dz;
      float2 spot;  // (clearance - cell, height - pz)
      if (CELLS) {
        spot = lidar_probe<LAYERS>(t, __fmaf_rn(tt, ax, bx), __fmaf_rn(tt, ay, by), tt, ox, oy, dx, dy, pz);
      } else {
        const Spot s = probe<LAYERS, false>(t, ox + tt * dx, oy + tt * dy, pz);
        spot = make_float2(s.clearance - cell, s.height - pz);
      }
      fl = -spot.y - 0.03f;  // the reference's (pz - height) - 0.03: RN(pz - h) = -RN(h - pz)
      step = fminf(spot.x, quotient(fl, descent, inv_descent, fl * inv_descent));
      next = tt + step;
      if (fl < 0.0f || step < min_step || !(next < RANGE) || (COUNTED && count >= max_iters)) break;
      last = tt;
      last_floor = fl;
      tt = next;
    }
    *count_out = count;
    if (fl < 0.0f) return fminf(last + ((tt - last) * last_floor) / (last_floor - fl), RANGE);
    return fminf(step < min_step ? tt : next, RANGE);
  }
  while (tt < RANGE && count < max_iters) {
    ++count;
    const float px = ox + tt * dx, py = oy + tt * dy, pz = oz + tt * dz;
    const Spot spot = probe<LAYERS, GUARD>(t, px, py, pz);
    const float fl = (pz - spot.height) - 0.03f;
    if (fl < 0.0f) {
      range = fminf(last + ((tt - last) * last_floor) / (last_floor - fl), RANGE);
      break;
    }
    const float a = spot.clearance - cell;
    if (a < min_step) break;  // min(a, fl / descent) <= a < min_step
    // fl * RN(1/descent) is within (1 + 2^-23) of the exact fl / descent, so
    // a product above a * (1 + 2^-20) proves the correctly rounded quotient
    // is >= a and min() returns a: the division is needed only when the
    // floor term may win.
    float step = a;
    if (!(fl * inv_descent > a * 1.00000095f)) step = fminf(a, fl / descent);
    if (step < min_step) break;
    last = tt;
    last_floor = fl;
    tt += step;
  }
  *count_out = count;
  return range < 0.0f ? fminf(tt, RANGE) : range;
}

// racer/sim.mojo:323-348. step = *step_base (if given) + step_add.
__global__ void k_sample(int n, uint64_t seed, const float* output, const float* log_std, float* actions, float* logp,
                         float* value, int deterministic, const int64_t* step_base, int64_t step_add) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t step = (step_base ? *step_base : 0) + step_add;
  sample_car(n, i, seed, output[i], output[(long)n + i], output[2L * n + i], log_std, actions, logp, value,
             deterministic, step);
}

__global__ void k_add_i64(int64_t* p, int64_t v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p += v;
}

}  // namespace

// ---- host launchers ----
Segments single_segment(const TrackDev& t, int n, uint64_t seed) {
  Segments g{};
  g.count = 1;
  g.car0[0] = 0;
  g.car0[1] = n;
  g.max_iters[0] = lidar_max_iters(t);
  g.seed[0] = seed;
  g.t[0] = t;
  return g;
}

void launch_spawn(const Segments& g, float* state, float* actions, int n, cudaStream_t st) {
  k_spawn<<<(n + 127) / 128, 128, 0, st>>>(g, state, actions, n);
}

void launch_advance(const Segments& g, float* state, const float* actions, float* reward, float* done, float* obs,
                    int n, int beams, float4* ray, cudaStream_t st, double* eval_reward, int* eval_crash, int c0,
                    int c1) {
  if (c1 < 0) c1 = n;
  if (c1 <= c0) return;
  k_advance<<<(c1 - c0 + 127) / 128, 128, 0, st>>>(g, state, actions, reward, done, obs, n, beams, ray, eval_reward,
                                                   eval_crash, c0, c1);
}



int lidar_max_iters(const TrackDev& t) { return (int)ceilf(RANGE / (0.5f * t.cell)) + 2; }

// Slots in the shape's order (invalid or repeated entries skipped, missing
// segments appended in index order) and their block ranges.
static LidarGrid lidar_grid(const Segments& g, const LidarShape& shape) {
  LidarGrid lg{};
  bool used[MAX_SEGMENTS] = {};
  int slots = 0;
  for (int j = 0; j < MAX_SEGMENTS; ++j) {
    const int k = shape.order[j];
    if (k >= 0 && k < g.count && !used[k]) used[k] = true, lg.order[slots++] = k;
  }
  for (int k = 0; k < g.count; ++k)
    if (!used[k]) lg.order[slots++] = k;
  lg.block0[0] = 0;
  for (int j = 0; j < g.count; ++j) {
    const int k = lg.order[j];
    lg.block0[j + 1] = lg.block0[j] + (g.car0[k + 1] - g.car0[k] + shape.cars - 1) / shape.cars;
  }
  for (int j = g.count; j < MAX_SEGMENTS; ++j) lg.block0[j + 1] = lg.block0[g.count];
  return lg;
}

template <int LAYERS, int CARS, bool WIDE>
static void lidar_track(const TrackDev& t, int max_iters, const float4* ray, float* obs, int n, int c0, int c1,
                        int beams, const float2* beam_dir, int* iters, cudaStream_t st, bool flat = false) {
  const long items = (long)(c1 - c0) * beams;
  if (flat && items > 0 && items < (1L << 31)) {
    const unsigned blocks = (unsigned)((items + 32 * CARS - 1) / (32 * CARS));
    k_lidar_flat<LAYERS, CARS, WIDE><<<blocks, CARS * 32, 0, st>>>(t, max_iters, ray, obs, n, c0, (unsigned)items,
                                                                   beams, beam_dir, iters);
    return;
  }
  dim3 grid((c1 - c0 + CARS - 1) / CARS, (beams + 31) / 32);
  if (grid.x == 0) return;
  k_lidar_track<LAYERS, CARS, WIDE, false>
      <<<grid, CARS * 32, 0, st>>>(t, max_iters, ray, obs, n, c0, c1, beams, beam_dir, iters, nullptr, nullptr);
}

template <int LAYERS, bool WIDE>
static void lidar_dynamic(const TrackDev& t, int max_iters, const float4* ray, float* obs, int n, int c0, int c1,
                          int beams, const float2* beam_dir, int* iters, unsigned* counter, int sms,
                          cudaStream_t st) {
  const long units = (long)(c1 - c0) * ((beams + 31) / 32);
  if (units <= 0) return;
  const long blocks = std::min<long>((long)sms * lidar_min_blocks(4, WIDE), (units + 3) / 4);
  cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
  k_lidar_dynamic<LAYERS, WIDE, false><<<(unsigned)blocks, 128, 0, st>>>(t, max_iters, ray, obs, n, c0, c1, beams,
                                                                          beam_dir, iters, counter, nullptr, nullptr);
}

template <int CARS, bool WIDE>
static void lidar_segment(const Segments& g, int k, const float4* ray, float* obs, int n, int beams,
                          const float2* beam_dir, int* iters, cudaStream_t st, const LidarShape& shape) {
  const TrackDev& t = g.t[k];
  const int c0 = g.car0[k], c1 = g.car0[k + 1];
  if (shape.dynamic && shape.counters) {
    unsigned* counter = shape.counters + k;
    if (t.layers == 1)
      lidar_dynamic<1, WIDE>(t, g.max_iters[k], ray, obs, n, c0, c1, beams, beam_dir, iters, counter, shape.sms, st);
    else if (t.layers == 2)
      lidar_dynamic<2, WIDE>(t, g.max_iters[k], ray, obs, n, c0, c1, beams, beam_dir, iters, counter, shape.sms, st);
    else
      lidar_dynamic<0, WIDE>(t, g.max_iters[k], ray, obs, n, c0, c1, beams, beam_dir, iters, counter, shape.sms, st);
    return;
  }
  const bool flat = shape.flat == 1;
  if (t.layers == 1)
    lidar_track<1, CARS, WIDE>(t, g.max_iters[k], ray, obs, n, c0, c1, beams, beam_dir, iters, st, flat);
  else if (t.layers == 2)
    lidar_track<2, CARS, WIDE>(t, g.max_iters[k], ray, obs, n, c0, c1, beams, beam_dir, iters, st, flat);
  else
    lidar_track<0, CARS, WIDE>(t, g.max_iters[k], ray, obs, n, c0, c1, beams, beam_dir, iters, st, flat);
}

template <int CARS, bool WIDE>
static void lidar_shape(const Segments& g, const LidarShape& shape, const float4* ray, float* obs, int n, int beams,
                        const float2* beam_dir, int* iters, cudaStream_t st) {
  if (g.count == 1) {
    lidar_segment<CARS, WIDE>(g, 0, ray, obs, n, beams, beam_dir, iters, st, shape);
    return;
  }
  const LidarGrid lg = lidar_grid(g, shape);
  dim3 grid(lg.block0[g.count], (beams + 31) / 32);
  k_lidar_segments<CARS, WIDE><<<grid, CARS * 32, 0, st>>>(g, lg, ray, obs, n, beams, beam_dir, iters);
}

bool lidar_shape_ok(const LidarShape& shape) {
  return (shape.cars == 2 || shape.cars == 4 || shape.cars == 8) && (shape.wide == 0 || shape.wide == 1) &&
         (shape.flat == 0 || shape.flat == 1);
}

void launch_lidar(const Segments& g, const LidarShape& shape, const float4* ray, float* obs, int n, int beams,
                  const float2* beam_dir, int* iters, cudaStream_t st) {
  if (g.count < 1 || g.car0[g.count] == 0) return;
  const bool wide = shape.wide == 1;
  if (shape.cars == 2)
    wide ? lidar_shape<2, true>(g, shape, ray, obs, n, beams, beam_dir, iters, st)
         : lidar_shape<2, false>(g, shape, ray, obs, n, beams, beam_dir, iters, st);
  else if (shape.cars == 8)
    wide ? lidar_shape<8, true>(g, shape, ray, obs, n, beams, beam_dir, iters, st)
         : lidar_shape<8, false>(g, shape, ray, obs, n, beams, beam_dir, iters, st);
  else
    wide ? lidar_shape<4, true>(g, shape, ray, obs, n, beams, beam_dir, iters, st)
         : lidar_shape<4, false>(g, shape, ray, obs, n, beams, beam_dir, iters, st);
}

void launch_lidar_segment(const Segments& g, int k, const LidarShape& shape, const float4* ray, float* obs, int n,
                          int beams, const float2* beam_dir, int* iters, cudaStream_t st) {
  if (k < 0 || k >= g.count) return;
  const bool wide = shape.wide == 1;
  if (shape.cars == 2)
    wide ? lidar_segment<2, true>(g, k, ray, obs, n, beams, beam_dir, iters, st, shape)
         : lidar_segment<2, false>(g, k, ray, obs, n, beams, beam_dir, iters, st, shape);
  else if (shape.cars == 8)
    wide ? lidar_segment<8, true>(g, k, ray, obs, n, beams, beam_dir, iters, st, shape)
         : lidar_segment<8, false>(g, k, ray, obs, n, beams, beam_dir, iters, st, shape);
  else
    wide ? lidar_segment<4, true>(g, k, ray, obs, n, beams, beam_dir, iters, st, shape)
         : lidar_segment<4, false>(g, k, ray, obs, n, beams, beam_dir, iters, st, shape);
}

void launch_lidar_cars(const Segments& g, const LidarShape& shape, int c0, int c1, const float4* ray, float* obs,
                       int n, int beams, const float2* beam_dir, int* iters, cudaStream_t st) {
  if (g.count != 1 || c1 <= c0) return;
  const TrackDev& t = g.t[0];
  const bool wide = shape.wide == 1;
  const bool flat = shape.flat == 1;
#define RACER_LIDAR_CARS(CARS, WIDE)                                                                         \
  if (t.layers == 1)                                                                                          \
    lidar_track<1, CARS, WIDE>(t, g.max_iters[0], ray, obs, n, c0, c1, beams, beam_dir, iters, st, flat);   \
  else if (t.layers == 2)                                                                                     \
    lidar_track<2, CARS, WIDE>(t, g.max_iters[0], ray, obs, n, c0, c1, beams, beam_dir, iters, st, flat);   \
  else                                                                                                        \
    lidar_track<0, CARS, WIDE>(t, g.max_iters[0], ray, obs, n, c0, c1, beams, beam_dir, iters, st, flat);
  if (shape.cars == 2) {
    if (wide) { RACER_LIDAR_CARS(2, true) } else { RACER_LIDAR_CARS(2, false) }
  } else if (shape.cars == 8) {
    if (wide) { RACER_LIDAR_CARS(8, true) } else { RACER_LIDAR_CARS(8, false) }
  } else {
    if (wide) { RACER_LIDAR_CARS(4, true) } else { RACER_LIDAR_CARS(4, false) }
  }
#undef RACER_LIDAR_CARS
}

void launch_lidar(const TrackDev& t, const float4* ray, float* obs, int n, int beams, const float2* beam_dir,
                  int* iters, cudaStream_t st) {
  launch_lidar(single_segment(t, n, 0), LidarShape{}, ray, obs, n, beams, beam_dir, iters, st);
}

void launch_lidar_list(const TrackDev& t, const float4* ray, float* obs, int n, int beams, const float2* beam_dir,
                       const int* list, const int* list_count, int list_max, unsigned* counter, int sms,
                       cudaStream_t st) {
  const long units = (long)list_max * ((beams + 31) / 32);
  if (units <= 0) return;
  // the 40-register variant: no spills with the list indirection
  const long blocks = std::min<long>((long)sms * lidar_min_blocks(4, true), (units + 3) / 4);
  const int max_iters = lidar_max_iters(t);
  cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
  if (t.layers == 1)
    k_lidar_dynamic<1, true, true><<<(unsigned)blocks, 128, 0, st>>>(t, max_iters, ray, obs, n, 0, n, beams, beam_dir,
                                                                     nullptr, counter, list, list_count);
  else if (t.layers == 2)
    k_lidar_dynamic<2, true, true><<<(unsigned)blocks, 128, 0, st>>>(t, max_iters, ray, obs, n, 0, n, beams, beam_dir,
                                                                     nullptr, counter, list, list_count);
  else
    k_lidar_dynamic<0, true, true><<<(unsigned)blocks, 128, 0, st>>>(t, max_iters, ray, obs, n, 0, n, beams, beam_dir,
                                                                     nullptr, counter, list, list_count);
}

// Spot check of a learned prediction: beams offset, offset + stride, ... of
// every car traced exactly (beam_range, the reference's range) and compared
// with the predicted obs rows pred [beams, n] (range / RANGE); a car with a
// beam off by more than tol (obs units) gets minr = 0, which puts it on the
// exact-fallback list (k_select_cars). One thread per (car, checked beam).
// The offset is (*step_base + step_add) % stride, so it moves on with the
// step in replays of a captured rollout.
template <int LAYERS>
__global__ void k_lidar_spot(TrackDev t, int max_iters, const float4* __restrict__ ray, const float* __restrict__ pred,
                             int n, int beams, const float2* __restrict__ beam_dir, int stride,
                             const int64_t* step_base, int64_t step_add, int per_car, float tol, unsigned* minr) {
  const long item = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= (long)n * per_car) return;
  const int64_t step = (step_base ? *step_base : 0) + step_add;
  const int offset = (int)(((step % stride) + stride) % stride);
  const int car = (int)(item / per_car), beam = offset + (int)(item % per_car) * stride;
  if (beam >= beams) return;
  int count = 0;
  const float range = beam_range<LAYERS>(t, ray, n, beam_dir, max_iters, false, car, beam, &count);
  if (!(fabsf(range / RANGE - __ldg(pred + (long)beam * n + car)) <= tol)) atomicMin(minr + car, 0u);
}

// ---- the fused persistent rollout: policy forward, sampling, physics and lidar ----
//
// One CTA owns cars [c0, c1) (at most 128) for all `steps` Runner steps
// (main.mojo:40-48), whose phases run one after the other, separated by block
// barriers: the BF16 policy forward on tcgen05 with the fused sampling, the
// physics of each car (one thread each), the lidar (a warp marches 32 beams of
// one car at a time). Cars never interact, so no grid-wide synchronisation is
// needed, and every result is the chained graph's: the same device functions
// (advance_car, trace) and the same forward (k-blocks, MMAs, epilogue) as
// mlp_tc.cu's register-staged kernel. Two CTAs share an SM, so one's forward or
// physics, latency-bound, runs beside the other's lidar.
// Data the kernel rewrites every step (obs, the ray frames, actions) is read
// with coherent loads (never the read-only path); the block's barrier orders
// its writes before the next phase's reads.
struct FusedRolloutCfg {
  static constexpr int GROUPS = 2;              // forward producer groups of four warps, one stage each
  static constexpr int MMA_WARP = GROUPS * 4;  // warp 8: layer 1's MMAs
  static constexpr int THREADS = 16 * 32;       // every warp marches beams
  static constexpr int OFF_A = 0;               // GROUPS x A; H = [h | 1 | 0] reuses A[0], A[1]
  static constexpr int OFF_B = OFF_A + GROUPS * A_BYTES;
  static constexpr int OFF_W1 = OFF_B + GROUPS * B_BYTES;
  static constexpr int OFF_W2 = OFF_W1 + 2 * B_BYTES;
  static constexpr int OFF_BAR = OFF_W2 + 2 * 16 * 128;
  // + barriers, + alignment slack, + 16 KB so every descriptor-addressed read stays inside the allocation
  static constexpr int SMEM_BYTES = OFF_BAR + 128 + 1024 + 16384;
  static_assert((2 * GROUPS + 3) * 8 + 8 <= 128, "barriers, the TMEM slot and the abort word fit their 128 bytes");
};
static_assert(2 * FusedRolloutCfg::SMEM_BYTES <= 227 * 1024, "two CTAs per SM");

template <int LAYERS>
__global__ void __launch_bounds__(FusedRolloutCfg::THREADS, 2)
    k_rollout_fused(const __grid_constant__ Segments g, float* s, float* act, float* reward, float* done_rows,
                    float* obs, int n, int beams, float4* ray, const float2* __restrict__ beam_dir, int cars_per_cta,
                    int steps, const uint4* __restrict__ w0s, int kblocks, const uint4* __restrict__ w1s,
                    const uint4* __restrict__ w2s, float* og, SampleArgs sa, int* err) {
  using C = FusedRolloutCfg;
  constexpr int GROUPS = C::GROUPS, MMA_WARP = C::MMA_WARP;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* empty = full + GROUPS;
  uint64_t* done = empty + GROUPS;
  uint64_t* drain = done + 1;  // [2]: thread 0's and the MMA lane's final commits after a timeout
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 2);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);  // set by a timed-out wait
  constexpr uint32_t limit = tc::WAIT_LIMIT;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r = tid & (TILE - 1);  // sample row of a producer or epilogue thread
  const int c0 = (int)blockIdx.x * cars_per_cta, c1 = min(n, c0 + cars_per_cta);
  const int in = beams + 5;
  const TrackDev& t = g.t[0];

  if (tid == 0) {
    for (int q = 0; q < GROUPS; ++q) {
      tc::mbar_init(&full[q], TILE);
      tc::mbar_init(&empty[q], 1);
    }
    tc::mbar_init(done, 1);
    tc::mbar_init(&drain[0], 1);
    tc::mbar_init(&drain[1], 1);
    *abort = 0;
    tc::fence_barrier_init();
  }
  if (warp == MMA_WARP) {
    tc::tmem_alloc(tslot, 64);
    tc::tmem_relinquish();
  }
  {  // W1 (2 x 8 KB) and W2 (2 x 2 KB), resident for the whole rollout
    uint4* w1 = reinterpret_cast<uint4*>(smem + C::OFF_W1);
    uint4* w2 = reinterpret_cast<uint4*>(smem + C::OFF_W2);
    for (int e = tid; e < 2 * B_BYTES / 16; e += C::THREADS) w1[e] = __ldg(w1s + e);
    for (int e = tid; e < 2 * 16 * 128 / 16; e += C::THREADS) w2[e] = __ldg(w2s + e);
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t id64 = tc::idesc_bf16(TILE, 64);
  bool ok = true;
  bool issued = false;  // this thread issued an MMA
  const int beam_groups = (beams + 31) >> 5;

  for (int step = 0; step < steps; ++step) {
    // ---- policy forward on the cars' observations, with the sampling in the epilogue ----
    const int c = c0 + r;
    const bool live = c < c1;
    if (warp < MMA_WARP) {
      const int q = warp >> 2;                               // producer group: k-blocks q, q + GROUPS, ...
      const uint32_t uses = (kblocks - q + GROUPS - 1) / GROUPS;  // uses of its stage in a step
      uint8_t* A = smem + C::OFF_A + q * A_BYTES;
      uint4* B = reinterpret_cast<uint4*>(smem + C::OFF_B + q * B_BYTES);
      for (int j = 0;; ++j) {
        const int kb = q + GROUPS * j;
        if (kb >= kblocks) break;
        const uint32_t use = (uint32_t)step * uses + (uint32_t)j;
        uint4 wb[4];
        const uint4* src = w0s + (long)kb * (B_BYTES / 16);
#pragma unroll
        for (int e = 0; e < 4; ++e) wb[e] = __ldg(src + r + e * TILE);
        if (use >= 1 && !tc::mbar_wait_abort(&empty[q], (use - 1) & 1, abort, limit)) ok = false;
        // the k-block's 64 inputs of this row in four chunks of 16 (the same BF16 operand as mlp_tc.cu's
        // producers write; fewer live registers)
#pragma unroll 1
        for (int h = 0; h < 4; ++h) {
          float v[16];
#pragma unroll
          for (int f = 0; f < 16; ++f) {
            const int row = kb * 64 + 16 * h + f;
            v[f] = (live && row < in) ? __ldcg(obs + (long)row * n + c) : 0.0f;
          }
#pragma unroll
          for (int f = 0; f < 2; ++f) {
            const int chunk = 2 * h + f;
            const uint4 pk = make_uint4(tc::pack_bf16(v[8 * f], v[8 * f + 1]), tc::pack_bf16(v[8 * f + 2], v[8 * f + 3]),
                                        tc::pack_bf16(v[8 * f + 4], v[8 * f + 5]),
                                        tc::pack_bf16(v[8 * f + 6], v[8 * f + 7]));
            *reinterpret_cast<uint4*>(A + r * 128 + ((chunk ^ (r & 7)) << 4)) = pk;
          }
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) B[r + e * TILE] = wb[e];
        tc::fence_proxy_async_smem();
        tc::mbar_arrive(&full[q]);
      }
    } else if (warp == MMA_WARP && lane == 0) {
      for (int kb = 0; kb < kblocks; ++kb) {
        const int q = kb % GROUPS;
        const uint32_t uses = (kblocks - q + GROUPS - 1) / GROUPS;
        const uint32_t use = (uint32_t)step * uses + (uint32_t)(kb / GROUPS);
        if (!tc::mbar_wait_abort(&full[q], use & 1, abort, limit)) ok = false;
        if (*abort) continue;  // issue nothing after a timeout
        issued = true;
        tc::tc_fence_after();
        const uint32_t a = tc::smem_u32(smem + C::OFF_A + q * A_BYTES), b = tc::smem_u32(smem + C::OFF_B + q * B_BYTES);
#pragma unroll
        for (int k = 0; k < 4; ++k)
          tc::mma_bf16(tmem, tc::sdesc_sw128(a + 32 * k), tc::sdesc_sw128(b + 32 * k), id64, (kb | k) ? 1u : 0u);
        tc::mma_commit(&empty[q]);
      }
      if (!*abort) tc::mma_commit(done);
    }
    if (warp < 4) {
      SampleArgs sk = sa;
      sk.step_add = sa.step_add + step;
      if (!fwd_epilogue(smem, C::OFF_A, C::OFF_W1, C::OFF_W2, tmem, done, 3u * (uint32_t)step, r, live, c, n, nullptr,
                        nullptr, og, 0, sk, abort, limit, &issued))
        ok = false;
    }
    tc::tc_fence_before();
    __syncthreads();  // the actions of this step are written
    // ---- physics: one thread per car ----
    for (int i = c0 + tid; i < c1; i += C::THREADS)
      advance_car<LAYERS>(t, s, act, reward, done_rows, obs, n, beams, g.seed[0], ray, i, i);
    __syncthreads();  // frames and obs rows 0-3 written
    // ---- lidar: (car, 32-beam group) units over the warps ----
    const int units = (c1 - c0) * beam_groups;
    for (int u = warp; u < units; u += C::THREADS / 32) {
      const int car = c0 + u / beam_groups, beam = (u % beam_groups) * 32 + lane;
      if (beam < beams) trace<LAYERS, false>(t, ray, obs, n, beam_dir, g.max_iters[0], nullptr, car, beam);
    }
    tc::tc_fence_before();
    __syncthreads();  // obs complete before the next step's forward reads it
  }
  if (*abort) {  // the MMAs issued before a timeout complete before the TMEM is freed
    if (issued) {
      uint64_t* mine = &drain[tid == 0 ? 0 : 1];
      tc::mma_commit(mine);
      if (!tc::mbar_wait(mine, 0, tc::WAIT_LIMIT)) ok = false;
    }
    tc::tc_fence_before();
    __syncthreads();
  }
  __syncwarp();
  if (warp == MMA_WARP) tc::tmem_dealloc(tmem, 64);
  if (!ok) atomicExch(err, 1);
}

__global__ void k_select_cars(const unsigned* minr, int n, unsigned threshold_bits, int* list, int* count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && minr[i] < threshold_bits) list[atomicAdd(count, 1)] = i;
}

void launch_lidar_spot(const TrackDev& t, const float4* ray, const float* pred, int n, int beams,
                       const float2* beam_dir, int stride, const int64_t* step_base, int64_t step_add, float tol,
                       unsigned* minr, cudaStream_t st) {
  if (stride < 1 || n < 1) return;
  const int per_car = (beams + stride - 1) / stride;  // the most any offset checks
  const long items = (long)n * per_car;
  const unsigned blocks = (unsigned)((items + 127) / 128);
  const int mi = lidar_max_iters(t);
#define RACER_SPOT(L)                                                                                            \
  k_lidar_spot<L><<<blocks, 128, 0, st>>>(t, mi, ray, pred, n, beams, beam_dir, stride, step_base, step_add, per_car, \
                                          tol, minr)
  if (t.layers == 1)
    RACER_SPOT(1);
  else if (t.layers == 2)
    RACER_SPOT(2);
  else
    RACER_SPOT(0);
#undef RACER_SPOT
}

// The fused rollout's cars per CTA: two CTAs per SM over all cars, at most 128
// (one MMA tile); at least 1.
int rollout_fused_cars_per_cta(int n, int sms) {
  const int ctas = 2 * (sms > 0 ? sms : 1);
  const int per = (n + ctas - 1) / ctas;
  return per < 1 ? 1 : (per > TILE ? TILE : per);
}

cudaError_t launch_rollout_fused(const Segments& g, float* state, float* actions, float* reward, float* done,
                                 float* obs, int n, int beams, float4* ray, const float2* beam_dir, int steps,
                                 const uint8_t* pack, float* og, const SampleArgs& sa, int* err, int sms,
                                 cudaStream_t st) {
  static unsigned long long configured = 0;  // per device
  cudaError_t e = once_per_device(&configured, [] {
    for (auto* k : {k_rollout_fused<0>, k_rollout_fused<1>, k_rollout_fused<2>}) {
      cudaError_t a = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, FusedRolloutCfg::SMEM_BYTES);
      if (a != cudaSuccess) return a;
    }
    return cudaSuccess;
  });
  if (e != cudaSuccess) return e;
  if (g.count != 1 || n < 1 || steps < 1) return cudaErrorInvalidValue;
  const int kb = (beams + 5 + 63) / 64;
  const uint4* w0 = reinterpret_cast<const uint4*>(pack);
  const uint4* w1 = reinterpret_cast<const uint4*>(pack + (size_t)kb * 8192);
  const uint4* w2 = reinterpret_cast<const uint4*>(pack + (size_t)kb * 8192 + 2 * 8192);
  const int per = rollout_fused_cars_per_cta(n, sms);
  const unsigned blocks = (unsigned)((n + per - 1) / per);
  const int layers = g.t[0].layers;
#define RACER_FUSED(L)                                                                                              \
  k_rollout_fused<L><<<blocks, FusedRolloutCfg::THREADS, FusedRolloutCfg::SMEM_BYTES, st>>>(                        \
      g, state, actions, reward, done, obs, n, beams, ray, beam_dir, per, steps, w0, kb, w1, w2, og, sa, err)
  if (layers == 1)
    RACER_FUSED(1);
  else if (layers == 2)
    RACER_FUSED(2);
  else
    RACER_FUSED(0);
#undef RACER_FUSED
  return cudaGetLastError();
}

void launch_select_cars(const unsigned* minr, int n, float threshold, int* list, int* count, cudaStream_t st) {
  unsigned bits;
  memcpy(&bits, &threshold, sizeof bits);
  k_select_cars<<<(n + 255) / 256, 256, 0, st>>>(minr, n, bits, list, count);
}

void launch_rk4_audit(const Segments& g, const float* prev, const float* actions, const float* next,
                      const float* done, int n, double* stats, cudaStream_t st) {
  k_rk4_f64<<<(n + 127) / 128, 128, 0, st>>>(g, prev, actions, next, done, n, stats);
}

void launch_pose_frames(const TrackDev& t, const float4* poses, int count, float4* ray, cudaStream_t st) {
  k_pose_frames<<<(count + 127) / 128, 128, 0, st>>>(t, poses, count, ray);
}

void launch_sample(int n, uint64_t seed, const float* output, const float* log_std, float* actions, float* logp,
                   float* value, int deterministic, const int64_t* step_base, int64_t step_add, cudaStream_t st) {
  k_sample<<<(n + 127) / 128, 128, 0, st>>>(n, seed, output, log_std, actions, logp, value, deterministic,
                                            step_base, step_add);
}

void launch_add_i64(int64_t* p, int64_t v, cudaStream_t st) { k_add_i64<<<1, 32, 0, st>>>(p, v); }

// Per-beam (cos, sin) of the azimuth -FOV/2 + b * FOV/(beams-1), computed with
// the same binary32 operations as racer/sim.mojo:246-247.
void beam_table(int beams, float2* out) {
  for (int b = 0; b < beams; ++b) {
    float az = -FOV / 2.0f + (float)b * (FOV / (float)(beams - 1));
    float s, c;
    rmath::sincosf_(az, &s, &c);
    out[b] = make_float2(c, s);
  }
}

}  // namespace racer
