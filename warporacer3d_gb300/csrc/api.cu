// C ABI of the warporacer3d GB300 library (declared in include/racer.h).
//
// Host-side objects mirror the reference's Mojo structs: racer_sim owns the
// buffers of Sim (racer/sim.mojo:269-289), racer_policy the parameters of
// Policy (racer/ppo.mojo:63-90), racer_acts an Activations
// (racer/ppo.mojo:47-60), racer_trainer the rollout storage, minibatch
// scratch and Adam state of Trainer (racer/ppo.mojo:141-185). Every method
// enqueues CUDA kernels on the object's stream; nothing runs on the CPU.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <limits>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/racer.h"
#include "common.cuh"
#include "kernels.h"
#include "objects.h"
#include "policy_fwd.h"
#include "surrogate.h"
#include "tma.h"

namespace racer_host {
static thread_local std::string g_error;
void set_error(const std::string& msg) { g_error = msg; }
const char* get_error() { return g_error.c_str(); }
}  // namespace racer_host

using namespace racer;
using racer_host::set_error;

#define RACER_ARG(cond, msg)   \
  do {                         \
    if (!(cond)) {             \
      set_error(msg);          \
      return 1;                \
    }                          \
  } while (0)

#define RACER_LAUNCHED()                                                                            \
  do {                                                                                              \
    cudaError_t err_ = cudaGetLastError();                                                          \
    if (err_ != cudaSuccess) {                                                                      \
      set_error(std::string("kernel launch: ") + cudaGetErrorString(err_));                         \
      return 2;                                                                                     \
    }                                                                                               \
  } while (0)

namespace {

template <typename T>
int dalloc(T** p, size_t count, int fill_byte = 0) {
  RACER_TRY(cudaMalloc((void**)p, count * sizeof(T) + 16));
  RACER_TRY(cudaMemset(*p, fill_byte, count * sizeof(T) + 16));
  return 0;
}

// A stream the library may capture: NULL (the legacy default stream) becomes
// an owned blocking stream, which stays ordered with default-stream work.
int own_stream(void* given, cudaStream_t* out, bool* owned) {
  if (given) {
    *out = (cudaStream_t)given;
    *owned = false;
    return 0;
  }
  RACER_TRY(cudaStreamCreate(out));
  *owned = true;
  return 0;
}

__global__ void k_fill(float* p, long count, float v) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) p[i] = v;
}
__global__ void k_set_i64(int64_t* p, int64_t v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p = v;
}

}  // namespace

struct racer_acts {
  int cols = 0;
  float *h1 = nullptr, *h2 = nullptr, *o = nullptr;
};

struct racer_trainer {
  int n = 0, beams = 0, in_rows = 0, rollout = 0, batch = 0, step = 0;
  float *obs = nullptr, *actions = nullptr, *logp = nullptr, *value = nullptr, *reward = nullptr, *done = nullptr,
        *advantage = nullptr;
  float *x = nullptr, *d3 = nullptr, *d2 = nullptr, *d1 = nullptr, *grad = nullptr, *first = nullptr,
        *second = nullptr, *stats = nullptr, *red = nullptr;
  racer_acts* acts = nullptr;
  cudaStream_t st = nullptr;
  bool owned = false;
  // The update as a CUDA graph: captured on the second update of a policy
  // generation (the first runs eagerly and sets up the policy's workspaces),
  // replayed after that; Adam's bias corrections of its 16 steps come from
  // c12_host (pinned), copied inside the graph.
  float *c12_dev = nullptr, *c12_host = nullptr;
  // BF16 copy of the four minibatches' inputs [4][IN][xld], written by the gather, and its
  // tensor maps: the BF16 backward's operand for the layer-0 weight gradient
  void* xb = nullptr;
  int xld = 0;
  CUtensorMap xmaps[MINIBATCHES];
  cudaGraphExec_t update_exec = nullptr;
  racer_policy* update_policy = nullptr;
  int update_generation = -1;
  bool update_warm = false;
  bool graphs = true;
  // rollouts with the learned lidar (racer_trainer_set_surrogate)
  racer_surrogate* sur = nullptr;
  int audit_every = 16;
  float fallback = 0.05f;  // obs units (range / RANGE)
};

extern "C" {

const char* racer_last_error(void) { return racer_host::get_error(); }
int racer_version(void) { return 1; }

int racer_alloc(size_t bytes, void** dev) {
  RACER_ARG(dev, "racer_alloc: null output");
  RACER_TRY(cudaMalloc(dev, bytes ? bytes : 1));
  RACER_TRY(cudaMemset(*dev, 0, bytes ? bytes : 1));
  return 0;
}
int racer_free(void* dev) {
  if (dev) RACER_TRY(cudaFree(dev));
  return 0;
}
int racer_upload(void* dev, const void* host, size_t bytes, void* stream) {
  RACER_TRY(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  RACER_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return 0;
}
int racer_download(void* host, const void* dev, size_t bytes, void* stream) {
  RACER_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  RACER_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return 0;
}
int racer_synchronize(void* stream) {
  RACER_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return 0;
}

// ---------------- Sim ----------------

// Checks the track array against its header (racer/track.py:15-18,123-125;
// racer/sim.mojo:96-102 only requires 12 floats, the GPU needs every grid in
// bounds): positive finite cell, grid sizes, and every nearest-waypoint entry
// an integer in [0, waypoints).
static int check_track(const float* d, size_t len) {
  RACER_ARG(d, "track: null pointer");
  RACER_ARG(len >= 12, "not a track array (fewer than 12 header floats)");
  for (int k = 0; k < 9; ++k) RACER_ARG(isfinite(d[k]), "track header holds a non-finite value");
  RACER_ARG(d[0] >= 2 && d[1] >= 2 && d[0] == floorf(d[0]) && d[1] == floorf(d[1]), "track: bad grid size");
  RACER_ARG(d[4] > 0, "track: cell size must be positive");
  RACER_ARG(d[5] >= 1 && d[5] == floorf(d[5]), "track: bad waypoint count");
  RACER_ARG(d[7] >= 1 && d[7] <= 16 && d[7] == floorf(d[7]), "track: bad layer count");
  RACER_ARG(d[6] > 0, "track: waypoint spacing must be positive");
  size_t nx = (size_t)d[0], ny = (size_t)d[1], w = (size_t)d[5], L = (size_t)d[7];
  RACER_ARG(len == 12 + 3 * L * nx * ny + 4 * w, "track array length does not match its header");
  for (size_t l = 0; l < L; ++l) {
    const float* near = d + 12 + (3 * l + 2) * nx * ny;
    for (size_t k = 0; k < nx * ny; ++k) {
      float v = near[k];
      RACER_ARG(v >= 0 && v < (float)w && v == floorf(v), "track: nearest-waypoint grid out of range");
    }
    // the lidar's probe relies on finite heights of at most 1e6 m (sim.cu, probe)
    const float* height = d + 12 + (3 * l + 1) * nx * ny;
    for (size_t k = 0; k < nx * ny; ++k)
      RACER_ARG(fabsf(height[k]) <= 1e6f, "track: heights must be finite and within 1e6 m");
  }
  return 0;
}

// Uploads one track (the array unchanged plus the per-cell float2 repack) and
// fills its device view.
static int upload_track(const float* track, size_t len, float** d_track, float2** d_cl, TrackDev* t) {
  int nx = (int)track[0], ny = (int)track[1], L = (int)track[7];
  const size_t cells = (size_t)nx * ny;
  // the lidar's cells follow the per-cell repack in the same allocation
  const size_t lidar = L <= 2 ? (size_t)(nx + 1) * (ny + 1) * L : 0;
  std::vector<float2> cl(cells * L + lidar);
  for (int l = 0; l < L; ++l) {
    const float* c = track + 12 + (size_t)(3 * l) * nx * ny;
    const float* h = c + cells;
    for (size_t k = 0; k < cells; ++k) cl[k * L + l] = make_float2(c[k], h[k]);
  }
  // Per cell of the unguarded march's probe (sim.cu, lidar_probe), which
  // keeps layer 1 only where it is drivable and nearer the ray than layer 0:
  // (clearance - cell, height) per slot, the clearance of an undrivable
  // layer (not > 0) read as -1, in binary32 as the march subtracts it. Where
  // one layer alone is drivable it takes slot 0 and slot 1's height is NaN
  // (it never compares nearer); where neither is, slot 0 is layer 0. The
  // border column and row read clearance and height -1, as off the map.
  if (lidar) {
    float2* lc = cl.data() + cells * L;
    const float cell = track[4], nan = std::numeric_limits<float>::quiet_NaN();
    const float off = -1.0f - cell;
    auto slot = [&](float2 v) { return make_float2((v.x > 0.0f ? v.x : -1.0f) - cell, v.y); };
    for (size_t k = 0; k < lidar; ++k) lc[k] = make_float2(off, L == 2 && k % 2 == 1 ? nan : -1.0f);
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const size_t k = (size_t)y * nx + x, q = ((size_t)y * (nx + 1) + x) * L;
        const float2 v0 = cl[k * L];
        if (L == 1) {
          lc[q] = slot(v0);
          continue;
        }
        const float2 v1 = cl[k * L + 1];
        const bool d0 = v0.x > 0.0f, d1 = v1.x > 0.0f;
        lc[q] = slot(d0 || !d1 ? v0 : v1);
        lc[q + 1] = d0 && d1 ? slot(v1) : make_float2(off, nan);
      }
  }
  if (int rc = dalloc(d_track, len)) return rc;
  if (int rc = dalloc(d_cl, cl.size())) return rc;
  RACER_TRY(cudaMemcpy(*d_track, track, len * sizeof(float), cudaMemcpyHostToDevice));
  RACER_TRY(cudaMemcpy(*d_cl, cl.data(), cl.size() * sizeof(float2), cudaMemcpyHostToDevice));
  t->d = *d_track;
  t->cl = *d_cl;
  t->lc = lidar ? reinterpret_cast<const float*>(*d_cl + cells * L) : nullptr;
  t->lw = nx + 1;
  t->nx = nx;
  t->ny = ny;
  t->waypoints = (int)track[5];
  t->layers = L;
  t->x0 = track[2];
  t->y0 = track[3];
  t->cell = track[4];
  t->inv_cell = 1.0f / track[4];
  {
    // the nearest-cell shortcut (sim.cu, cell_of): v = RN(x * inv_cell + cx) with
    // cx = RN(-x0 * inv_cell); rint(v) is the reference's cell whenever |v - rint(v)| < band
    t->cx = -t->x0 * t->inv_cell;
    t->cy = -t->y0 * t->inv_cell;
    const double X = ceil(std::max(fabs((double)t->x0), fabs((double)t->y0)) / (double)track[4]);
    const double delta = (5.001 * (nx > ny ? nx : ny) + 4.001 * X + 16.0) * 0x1p-24;
    t->band = delta < 0.25 ? (float)(0.5 - delta * (1.0 + 0x1p-20)) : 0.0f;  // 0: every lookup divides
    // the march's probe takes v = RN(tt * RN(d * inv_cell) + RN(o * inv_cell + cx)) along the ray,
    // with tt |d| <= RANGE: a wider band (sim.cu, lidar_cell)
    const double mdelta = (7.001 * (nx > ny ? nx : ny) + 2.001 * X + 3.001 * (double)RANGE / track[4] + 16.0) * 0x1p-24;
    t->mband = mdelta < 0.25 ? (float)(0.5 - mdelta * (1.0 + 0x1p-20)) : 0.0f;
  }
  t->spacing = track[6];
  t->slope = track[8];
  t->nxf = (float)nx;
  t->nyf = (float)ny;
  t->route = 12 + 3L * L * nx * ny;
  {
    // Every probe the march continues from adds a step >= m = 0.5 cell, and
    // RN(tt + step) >= (tt + m)(1 - 2^-24), so after k probes tt >= m k
    // (1 - 2^-24)^k. Where that reaches RANGE at k = max_iters the loop's
    // `tt < RANGE` test always ends it first, and the probe count is not needed.
    const float m = 0.5f * t->cell;
    const int k = lidar_max_iters(*t);
    t->free_march = (double)m * k * pow(1.0 - 0x1p-24, k) >= (double)RANGE * (1.0 + 1e-9) ? 1 : 0;
  }
  return 0;
}

int racer_sim_create_segments(int count, const float* const* tracks, const size_t* lens, const int* cars,
                              const uint64_t* seeds, int beams, void* stream, racer_sim** out) {
  RACER_ARG(out, "racer_sim_create: null output");
  RACER_ARG(count >= 1 && count <= MAX_SEGMENTS, "racer_sim_create_segments: 1 to 8 segments");
  RACER_ARG(tracks && lens && cars && seeds, "racer_sim_create_segments: null argument");
  RACER_ARG(beams >= 2, "racer_sim_create: beams must be at least 2");
  long total = 0;
  for (int k = 0; k < count; ++k) {
    RACER_ARG(cars[k] >= 1, "racer_sim_create: every segment needs at least one car");
    total += cars[k];
    if (int rc = check_track(tracks[k], lens[k])) return rc;
  }
  RACER_ARG(total <= (1L << 30), "racer_sim_create: too many cars");
  const int n = (int)total;
  racer_sim* s = new racer_sim();
  s->n = n;
  s->beams = beams;
  s->in_rows = beams + 5;
  s->seed = seeds[0];
  s->track_len = lens[0];
  int rc = 0;
  if ((rc = own_stream(stream, &s->st, &s->owned))) { delete s; return rc; }
  s->seg.count = count;
  s->seg.car0[0] = 0;
  s->seg_track.assign(count, nullptr);
  s->seg_cl.assign(count, nullptr);
  for (int k = 0; k < count && !rc; ++k) {
    rc = upload_track(tracks[k], lens[k], &s->seg_track[k], &s->seg_cl[k], &s->seg.t[k]);
    s->seg.car0[k + 1] = s->seg.car0[k] + cars[k];
    s->seg.seed[k] = seeds[k];
    s->seg.max_iters[k] = lidar_max_iters(s->seg.t[k]);
  }
  for (int k = count; k < MAX_SEGMENTS; ++k) s->seg.car0[k + 1] = n;
  if (rc) {
    racer_sim_destroy(s);
    return rc;
  }
  s->t = s->seg.t[0];
  s->d_track = s->seg_track[0];
  s->d_cl = s->seg_cl[0];
  std::vector<float2> dirs(beams);
  beam_table(beams, dirs.data());
  if ((rc = dalloc(&s->beam_dir, beams)) || (rc = dalloc(&s->state, (size_t)STATE * n)) ||
      (rc = dalloc(&s->obs, (size_t)s->in_rows * n)) || (rc = dalloc(&s->actions, 2 * (size_t)n)) ||
      (rc = dalloc(&s->reward, n)) || (rc = dalloc(&s->done, n)) || (rc = dalloc(&s->step_base, 1)) ||
      (rc = dalloc(&s->ray, 2 * (size_t)n))) {
    racer_sim_destroy(s);
    return rc;
  }
  if ((rc = dalloc(&s->counters, MAX_SEGMENTS))) {
    racer_sim_destroy(s);
    return rc;
  }
  int device = 0;
  if (cudaGetDevice(&device) == cudaSuccess)
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
  cudaError_t err = cudaMemcpy(s->beam_dir, dirs.data(), beams * sizeof(float2), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    set_error(std::string("racer_sim_create upload: ") + cudaGetErrorString(err));
    racer_sim_destroy(s);
    return 2;
  }
  *out = s;
  return 0;
}

int racer_sim_create(const float* track, size_t len, int n, uint64_t seed, int beams, void* stream,
                     racer_sim** out) {
  RACER_ARG(n >= 1, "racer_sim_create: n must be positive");
  return racer_sim_create_segments(1, &track, &len, &n, &seed, beams, stream, out);
}

int racer_sim_destroy(racer_sim* s) {
  if (!s) return 0;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  for (auto& kv : s->surrogate_graphs) cudaGraphExecDestroy(kv.second);
  cudaFree(s->counters);
  for (cudaStream_t c : s->chain_st) cudaStreamDestroy(c);
  for (cudaEvent_t e : s->chain_join) cudaEventDestroy(e);
  if (s->chain_fork) cudaEventDestroy(s->chain_fork);
  for (auto& kv : s->eval_graphs) cudaGraphExecDestroy(kv.second);
  cudaFree(s->eval_reward);
  cudaFree(s->eval_crash);
  cudaFree(s->eval_total);
  cudaFree(s->snapshot);
  for (cudaStream_t a : s->aux) cudaStreamDestroy(a);
  for (cudaEvent_t e : s->join) cudaEventDestroy(e);
  if (s->fork) cudaEventDestroy(s->fork);
  for (float* p : s->seg_track) cudaFree(p);
  for (float2* p : s->seg_cl) cudaFree(p);
  cudaFree(s->beam_dir);
  cudaFree(s->ray);
  cudaFree(s->state);
  cudaFree(s->obs);
  cudaFree(s->actions);
  cudaFree(s->reward);
  cudaFree(s->done);
  cudaFree(s->step_base);
  if (s->owned && s->st) cudaStreamDestroy(s->st);
  delete s;
  return 0;
}

int racer_sim_get_buffers(racer_sim* s, racer_sim_buffers* out) {
  RACER_ARG(s && out, "racer_sim_get_buffers: null argument");
  out->state = s->state;
  out->obs = s->obs;
  out->actions = s->actions;
  out->reward = s->reward;
  out->done = s->done;
  out->track = s->d_track;
  return 0;
}

// Launch order of the segments under `shape` (a permutation; entries out of
// range or repeated are skipped and missing segments appended).
static void segment_order(const racer_sim* s, const LidarShape& shape, int* order) {
  bool used[MAX_SEGMENTS] = {};
  int slots = 0;
  for (int j = 0; j < MAX_SEGMENTS; ++j) {
    const int k = shape.order[j];
    if (k >= 0 && k < s->seg.count && !used[k]) used[k] = true, order[slots++] = k;
  }
  for (int k = 0; k < s->seg.count; ++k)
    if (!used[k]) order[slots++] = k;
}

// The lidar over every segment: one segment-table launch, or (split) each
// segment's one-track kernel on its own stream, forked from and joined back
// into `st` (parallel branches when captured into a graph).
static int lidar_on(racer_sim* s, const LidarShape& given, float* obs, int32_t* iters, cudaStream_t st) {
  LidarShape shape = given;
  shape.counters = s->counters;
  shape.sms = s->sms;
  if (s->seg.count == 1 || !shape.split) {
    launch_lidar(s->seg, shape, s->ray, obs, s->n, s->beams, s->beam_dir, iters, st);
    RACER_LAUNCHED();
    return 0;
  }
  const int extra = s->seg.count - 1;
  if ((int)s->aux.size() < extra) {
    if (!s->fork) RACER_TRY(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming));
    while ((int)s->aux.size() < extra) {
      cudaStream_t a;
      cudaEvent_t e;
      RACER_TRY(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
      s->aux.push_back(a);
      RACER_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      s->join.push_back(e);
    }
  }
  int order[MAX_SEGMENTS];
  segment_order(s, shape, order);
  RACER_TRY(cudaEventRecord(s->fork, st));
  launch_lidar_segment(s->seg, order[0], shape, s->ray, obs, s->n, s->beams, s->beam_dir, iters, st);
  for (int j = 1; j <= extra; ++j) {
    RACER_TRY(cudaStreamWaitEvent(s->aux[j - 1], s->fork, 0));
    launch_lidar_segment(s->seg, order[j], shape, s->ray, obs, s->n, s->beams, s->beam_dir, iters, s->aux[j - 1]);
    RACER_TRY(cudaEventRecord(s->join[j - 1], s->aux[j - 1]));
  }
  for (int j = 1; j <= extra; ++j) RACER_TRY(cudaStreamWaitEvent(st, s->join[j - 1], 0));
  RACER_LAUNCHED();
  return 0;
}

static int sim_step_on(racer_sim* s, const float* actions, float* reward, float* done, float* obs, int32_t* iters,
                       cudaStream_t st, bool eval = false) {
  launch_advance(s->seg, s->state, actions, reward, done, obs, s->n, s->beams, s->ray, st,
                 eval ? s->eval_reward : nullptr, eval ? s->eval_crash : nullptr);
  RACER_LAUNCHED();
  return lidar_on(s, s->shape, obs, iters, st);
}

int racer_sim_reset(racer_sim* s) {
  RACER_ARG(s, "racer_sim_reset: null sim");
  launch_spawn(s->seg, s->state, s->actions, s->n, s->st);
  return sim_step_on(s, s->actions, s->reward, s->done, s->obs, nullptr, s->st);
}

int racer_sim_step(racer_sim* s, const float* actions, float* reward, float* done, float* obs) {
  RACER_ARG(s && actions && reward && done && obs, "racer_sim_step: null argument");
  return sim_step_on(s, actions, reward, done, obs, nullptr, s->st);
}

int racer_sim_step_counted(racer_sim* s, const float* actions, float* reward, float* done, float* obs,
                           int32_t* iters) {
  RACER_ARG(s && actions && reward && done && obs && iters, "racer_sim_step_counted: null argument");
  return sim_step_on(s, actions, reward, done, obs, iters, s->st);
}

int racer_sim_sample(racer_sim* s, const float* output, const float* log_std, float* actions, float* logp,
                     float* value, int deterministic, int64_t step) {
  RACER_ARG(s && output && log_std && actions && logp && value, "racer_sim_sample: null argument");
  launch_sample(s->n, s->seed, output, log_std, actions, logp, value, deterministic, nullptr, step, s->st);
  RACER_LAUNCHED();
  return 0;
}

// ---------------- Policy ----------------

int racer_policy_create(int beams, uint64_t seed, void* stream, racer_policy** out) {
  RACER_ARG(out, "racer_policy_create: null output");
  RACER_ARG(beams >= 2, "racer_policy_create: beams must be at least 2");
  racer_policy* p = nullptr;
  int rc = policy_new(beams + 5, stream, &p);
  if (rc) return rc;
  launch_policy_init(beams + 5, seed, policy_theta(p), policy_stream(p));
  RACER_LAUNCHED();
  if ((rc = policy_refresh(p))) {
    policy_delete(p);
    return rc;
  }
  *out = p;
  return 0;
}

int racer_policy_destroy(racer_policy* p) {
  policy_delete(p);
  return 0;
}

int racer_policy_theta(racer_policy* p, float** theta, int* count) {
  RACER_ARG(p, "racer_policy_theta: null policy");
  if (theta) *theta = policy_theta(p);
  if (count) *count = policy_params(p);
  return 0;
}

int racer_policy_set_precision(racer_policy* p, int bf16) {
  RACER_ARG(p, "racer_policy_set_precision: null policy");
  return policy_set_precision(p, bf16);
}

int racer_policy_sync(racer_policy* p) {
  RACER_ARG(p, "racer_policy_sync: null policy");
  return policy_refresh(p);
}

int racer_acts_create(racer_policy* p, int cols, racer_acts** out) {
  RACER_ARG(p && out, "racer_acts_create: null argument");
  RACER_ARG(cols >= 1, "racer_acts_create: cols must be positive");
  racer_acts* a = new racer_acts();
  a->cols = cols;
  int rc;
  if ((rc = dalloc(&a->h1, (size_t)HA * cols)) || (rc = dalloc(&a->h2, (size_t)HA * cols)) ||
      (rc = dalloc(&a->o, (size_t)OUT * cols))) {
    racer_acts_destroy(a);
    return rc;
  }
  long count = (long)HA * cols;
  k_fill<<<(unsigned)((count + 255) / 256), 256>>>(a->h1, count, 1.0f);
  k_fill<<<(unsigned)((count + 255) / 256), 256>>>(a->h2, count, 1.0f);
  RACER_TRY(cudaDeviceSynchronize());
  *out = a;
  return 0;
}

int racer_acts_destroy(racer_acts* a) {
  if (!a) return 0;
  cudaFree(a->h1);
  cudaFree(a->h2);
  cudaFree(a->o);
  delete a;
  return 0;
}

int racer_acts_buffers(racer_acts* a, float** h1, float** h2, float** o) {
  RACER_ARG(a, "racer_acts_buffers: null acts");
  if (h1) *h1 = a->h1;
  if (h2) *h2 = a->h2;
  if (o) *o = a->o;
  return 0;
}

static int forward_on(racer_policy* p, const float* x, racer_acts* a, cudaStream_t st,
                      const SampleArgs* sa = nullptr, int write_hidden = 1, int c0 = 0, int c1 = -1) {
  return policy_forward(p, x, a->cols, a->h1, a->h2, a->o, write_hidden, sa, st, c0, c1);
}

int racer_policy_status(racer_policy* p, int* code) {
  RACER_ARG(p && code, "racer_policy_status: null argument");
  return policy_status(p, code);
}

int racer_policy_wait_test(racer_policy* p, int polls) {
  RACER_ARG(p && polls >= 1, "racer_policy_wait_test: null policy or a poll count below 1");
  return policy_wait_probe(p, (uint32_t)polls);
}

int racer_policy_forward(racer_policy* p, const float* x, racer_acts* a) {
  RACER_ARG(p && x && a, "racer_policy_forward: null argument");
  return forward_on(p, x, a, policy_stream(p));
}

int racer_policy_backward(racer_policy* p, const float* x, racer_acts* a, const float* d3, float* d2, float* d1,
                          float* grad) {
  RACER_ARG(p && x && a && d3 && d2 && d1 && grad, "racer_policy_backward: null argument");
  return policy_backward(p, x, a->cols, a->h1, a->h2, d3, d2, d1, grad, policy_stream(p));
}

// .npy v1.0 float32 vector (racer/ppo.mojo:341-355, racer/device.mojo:137-143).
int racer_policy_save(racer_policy* p, const char* path, int iteration) {
  RACER_ARG(p && path, "racer_policy_save: null argument");
  int count = policy_params(p);
  std::vector<float> values((size_t)count + 1);
  values[0] = (float)iteration;
  RACER_TRY(cudaMemcpyAsync(values.data() + 1, policy_theta(p), count * sizeof(float), cudaMemcpyDeviceToHost,
                            policy_stream(p)));
  RACER_TRY(cudaStreamSynchronize(policy_stream(p)));
  char dict[128];
  snprintf(dict, sizeof dict, "{'descr': '<f4', 'fortran_order': False, 'shape': (%d,), }", count + 1);
  std::string header(dict);
  size_t total = 10 + header.size() + 1;
  header.append((64 - total % 64) % 64, ' ');
  header.push_back('\n');
  FILE* f = fopen(path, "wb");
  RACER_ARG(f, std::string("racer_policy_save: cannot open ") + path);
  unsigned short hl = (unsigned short)header.size();
  unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, (unsigned char)(hl & 0xff), (unsigned char)(hl >> 8)};
  bool ok = fwrite(pre, 1, 10, f) == 10 && fwrite(header.data(), 1, header.size(), f) == header.size() &&
            fwrite(values.data(), sizeof(float), values.size(), f) == values.size();
  ok = (fclose(f) == 0) && ok;
  RACER_ARG(ok, std::string("racer_policy_save: write failed for ") + path);
  return 0;
}

int racer_policy_load(racer_policy* p, const char* path, int* iteration) {
  RACER_ARG(p && path, "racer_policy_load: null argument");
  FILE* f = fopen(path, "rb");
  RACER_ARG(f, std::string("racer_policy_load: cannot open ") + path);
  unsigned char pre[10];
  std::vector<char> header;
  bool ok = fread(pre, 1, 8, f) == 8 && pre[0] == 0x93 && memcmp(pre + 1, "NUMPY", 5) == 0;
  size_t hl = 0;
  if (ok && pre[6] == 1) {
    ok = fread(pre + 8, 1, 2, f) == 2;
    hl = pre[8] | (pre[9] << 8);
  } else if (ok && (pre[6] == 2 || pre[6] == 3)) {
    unsigned char b[4];
    ok = fread(b, 1, 4, f) == 4;
    hl = b[0] | (b[1] << 8) | (b[2] << 16) | ((size_t)b[3] << 24);
  } else {
    ok = false;
  }
  if (ok) {
    header.resize(hl + 1, 0);
    ok = fread(header.data(), 1, hl, f) == hl;
  }
  std::string h(header.begin(), header.end());
  bool f4 = h.find("'<f4'") != std::string::npos, f8 = h.find("'<f8'") != std::string::npos;
  ok = ok && (f4 || f8) && h.find("'fortran_order': False") != std::string::npos;
  size_t lp = h.find("'shape': ("), count = 0;
  if (ok && lp != std::string::npos) count = strtoul(h.c_str() + lp + 10, nullptr, 10);
  int want = policy_params(p) + 1;
  std::vector<float> values(want);
  if (ok && count == (size_t)want) {
    if (f4) {
      ok = fread(values.data(), sizeof(float), want, f) == (size_t)want;
    } else {
      std::vector<double> dv(want);
      ok = fread(dv.data(), sizeof(double), want, f) == (size_t)want;
      for (int k = 0; k < want; ++k) values[k] = (float)dv[k];
    }
  } else if (ok) {
    fclose(f);
    set_error("checkpoint does not match the network size");
    return 1;
  }
  fclose(f);
  RACER_ARG(ok, std::string("racer_policy_load: not a float .npy vector: ") + path);
  RACER_TRY(cudaMemcpyAsync(policy_theta(p), values.data() + 1, (want - 1) * sizeof(float), cudaMemcpyHostToDevice,
                            policy_stream(p)));
  RACER_TRY(cudaStreamSynchronize(policy_stream(p)));
  if (iteration) *iteration = (int)values[0];
  return policy_refresh(p);
}

// ---------------- Trainer ----------------

int racer_trainer_create(int n, int beams, int rollout, void* stream, racer_trainer** out) {
  RACER_ARG(out, "racer_trainer_create: null output");
  RACER_ARG(n >= 1 && beams >= 2 && rollout >= 1, "racer_trainer_create: bad sizes");
  RACER_ARG(((long)n * rollout) % MINIBATCHES == 0, "racer_trainer_create: n * rollout must divide into 4 minibatches");
  racer_trainer* tr = new racer_trainer();
  tr->n = n;
  tr->beams = beams;
  tr->in_rows = beams + 5;
  tr->rollout = rollout;
  tr->batch = (int)((long)n * rollout / MINIBATCHES);
  int rc;
  if ((rc = own_stream(stream, &tr->st, &tr->owned))) { delete tr; return rc; }
  size_t R = rollout, IN = tr->in_rows, B = tr->batch, P = (size_t)H * IN + H * HA + OUT * HA + 2;
  if ((rc = dalloc(&tr->obs, (R + 1) * IN * n)) || (rc = dalloc(&tr->actions, R * 2 * n)) ||
      (rc = dalloc(&tr->logp, R * n)) || (rc = dalloc(&tr->value, R * n)) || (rc = dalloc(&tr->reward, R * n)) ||
      (rc = dalloc(&tr->done, R * n)) || (rc = dalloc(&tr->advantage, R * n)) || (rc = dalloc(&tr->x, MINIBATCHES * IN * B)) ||
      (rc = dalloc(&tr->d3, (OUT + 3) * B)) || (rc = dalloc(&tr->d2, (size_t)HA * B)) ||
      (rc = dalloc(&tr->d1, (size_t)HA * B)) || (rc = dalloc(&tr->grad, P)) || (rc = dalloc(&tr->first, P)) ||
      (rc = dalloc(&tr->second, P)) || (rc = dalloc(&tr->stats, STATS)) || (rc = dalloc(&tr->red, 4096)) ||
      (rc = dalloc(&tr->c12_dev, 2 * EPOCHS * MINIBATCHES))) {
    racer_trainer_destroy(tr);
    return rc;
  }
  tr->xld = (tr->batch + 7) / 8 * 8;
  {
    uint16_t* xb = nullptr;
    if ((rc = dalloc(&xb, (size_t)MINIBATCHES * IN * tr->xld))) {
      racer_trainer_destroy(tr);
      return rc;
    }
    tr->xb = xb;
    for (int m = 0; m < MINIBATCHES; ++m)
      if ((rc = make_tmap_bf16(&tr->xmaps[m], xb + (size_t)m * IN * tr->xld, IN, tr->xld, tr->xld, 128))) {
        racer_trainer_destroy(tr);
        return rc;
      }
  }
  if (cudaMallocHost((void**)&tr->c12_host, 2 * EPOCHS * MINIBATCHES * sizeof(float)) != cudaSuccess) {
    set_error("racer_trainer_create: pinned allocation failed");
    tr->c12_host = nullptr;
    racer_trainer_destroy(tr);
    return 2;
  }
  racer_acts* a = new racer_acts();
  a->cols = tr->batch;
  if ((rc = dalloc(&a->h1, (size_t)HA * B)) || (rc = dalloc(&a->h2, (size_t)HA * B)) ||
      (rc = dalloc(&a->o, (size_t)OUT * B))) {
    racer_acts_destroy(a);
    racer_trainer_destroy(tr);
    return rc;
  }
  long count = (long)HA * B;
  k_fill<<<(unsigned)((count + 255) / 256), 256>>>(a->h1, count, 1.0f);
  k_fill<<<(unsigned)((count + 255) / 256), 256>>>(a->h2, count, 1.0f);
  tr->acts = a;
  RACER_TRY(cudaDeviceSynchronize());
  *out = tr;
  return 0;
}

int racer_trainer_destroy(racer_trainer* tr) {
  if (!tr) return 0;
  if (tr->update_exec) cudaGraphExecDestroy(tr->update_exec);
  for (float* p : {tr->obs, tr->actions, tr->logp, tr->value, tr->reward, tr->done, tr->advantage, tr->x, tr->d3,
                   tr->d2, tr->d1, tr->grad, tr->first, tr->second, tr->stats, tr->red, tr->c12_dev})
    cudaFree(p);
  if (tr->c12_host) cudaFreeHost(tr->c12_host);
  cudaFree(tr->xb);
  racer_acts_destroy(tr->acts);
  if (tr->owned && tr->st) cudaStreamDestroy(tr->st);
  delete tr;
  return 0;
}

int racer_trainer_get_buffers(racer_trainer* tr, racer_trainer_buffers* out) {
  RACER_ARG(tr && out, "racer_trainer_get_buffers: null argument");
  out->obs = tr->obs;
  out->actions = tr->actions;
  out->logp = tr->logp;
  out->value = tr->value;
  out->reward = tr->reward;
  out->done = tr->done;
  out->advantage = tr->advantage;
  out->x = tr->x;
  out->d3 = tr->d3;
  out->d2 = tr->d2;
  out->d1 = tr->d1;
  out->grad = tr->grad;
  out->first = tr->first;
  out->second = tr->second;
  out->stats = tr->stats;
  out->acts = tr->acts;
  out->batch = tr->batch;
  return 0;
}

int racer_trainer_rollout(racer_trainer* tr, racer_sim* s, racer_policy* p, racer_acts* a, int iteration,
                          float* mean_reward) {
  RACER_ARG(tr && s && p && a, "racer_trainer_rollout: null argument");
  RACER_ARG(s->n == tr->n && s->beams == tr->beams && a->cols == tr->n && policy_inputs(p) == tr->in_rows,
            "racer_trainer_rollout: sizes of sim, policy, activations and trainer differ");
  cudaStream_t st = tr->st;
  const size_t n = tr->n, IN = tr->in_rows, R = tr->rollout;
  const float* logstd = policy_theta(p) + policy_params(p) - 2;
  if (tr->sur)
    if (int rc = surrogate_prepare(tr->sur, s)) return rc;
  RACER_TRY(cudaMemcpyAsync(tr->obs, s->obs, IN * n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  // with rollout chains (racer_sim_set_chains), each car range steps on its own stream
  const int chains = !tr->sur && s->chains > 1 && s->seg.count == 1 && policy_is_bf16(p) ? s->chains : 1;
  int audits = 0;
  int bound[MAX_CHAINS + 1];
  for (int c = 0; c <= chains; ++c) bound[c] = c == chains ? (int)n : std::min((int)n, (int)((long)n * c / chains / 128 * 128));
  if (chains > 1) {
    RACER_TRY(cudaEventRecord(s->chain_fork, st));
    for (int c = 1; c < chains; ++c) RACER_TRY(cudaStreamWaitEvent(s->chain_st[c - 1], s->chain_fork, 0));
  }
  for (size_t t = 0; t < R; ++t) {
    SampleArgs sa;
    sa.seed = s->seed;
    sa.log_std = logstd;
    sa.actions = tr->actions + t * 2 * n;
    sa.logp = tr->logp + t * n;
    sa.value = tr->value + t * n;
    sa.step_add = (int64_t)iteration * (int64_t)R + (int64_t)t;
    if (tr->sur) {  // physics, then the learned lidar (audited every audit_every-th step of training)
      int rc = forward_on(p, tr->obs + t * IN * n, a, st, &sa, 0);
      if (rc) return rc;
      float* obs_next = tr->obs + (t + 1) * IN * n;
      launch_advance(s->seg, s->state, tr->actions + t * 2 * n, tr->reward + t * n, tr->done + t * n, obs_next,
                     (int)n, s->beams, s->ray, st);
      RACER_LAUNCHED();
      const int64_t global = (int64_t)iteration * (int64_t)R + (int64_t)t;
      const bool audit = tr->audit_every > 0 && global % tr->audit_every == 0;
      audits += audit;
      if ((rc = surrogate_lidar(tr->sur, s, obs_next, audit, tr->fallback, st, nullptr, global))) return rc;
      continue;
    }
    if (chains == 1) {
      int rc = forward_on(p, tr->obs + t * IN * n, a, st, &sa, 0);
      if (rc) return rc;
      if ((rc = sim_step_on(s, tr->actions + t * 2 * n, tr->reward + t * n, tr->done + t * n,
                            tr->obs + (t + 1) * IN * n, nullptr, st)))
        return rc;
      continue;
    }
    for (int c = 0; c < chains; ++c) {
      cudaStream_t cs = c ? s->chain_st[c - 1] : st;
      if (int rc = forward_on(p, tr->obs + t * IN * n, a, cs, &sa, 0, bound[c], bound[c + 1])) return rc;
      float* obs_next = tr->obs + (t + 1) * IN * n;
      launch_advance(s->seg, s->state, tr->actions + t * 2 * n, tr->reward + t * n, tr->done + t * n, obs_next,
                     (int)n, s->beams, s->ray, cs, nullptr, nullptr, bound[c], bound[c + 1]);
      launch_lidar_cars(s->seg, s->shape, bound[c], bound[c + 1], s->ray, obs_next, (int)n, s->beams, s->beam_dir,
                        nullptr, cs);
      RACER_LAUNCHED();
    }
  }
  if (chains > 1)
    for (int c = 1; c < chains; ++c) {
      RACER_TRY(cudaEventRecord(s->chain_join[c - 1], s->chain_st[c - 1]));
      RACER_TRY(cudaStreamWaitEvent(st, s->chain_join[c - 1], 0));
    }
  RACER_TRY(cudaMemcpyAsync(s->obs, tr->obs + R * IN * n, IN * n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  int rc = forward_on(p, tr->obs + R * IN * n, a, st);
  if (rc) return rc;
  launch_gae((int)n, (int)R, tr->reward, tr->done, tr->value, a->o + 2 * n, tr->advantage, st);
  launch_rowsum(tr->reward, 1, (int)(R * n), (long)(R * n), tr->stats + ST_REWARD, tr->red, 0, st);
  RACER_LAUNCHED();
  float stats[STATS];
  RACER_TRY(cudaMemcpyAsync(stats, tr->stats, sizeof stats, cudaMemcpyDeviceToHost, st));
  RACER_TRY(cudaStreamSynchronize(st));
  if (tr->sur) surrogate_account(tr->sur, s, (int)R, audits);
  if (mean_reward) *mean_reward = stats[ST_REWARD] / (float)(R * n);
  return 0;
}

int racer_trainer_set_surrogate(racer_trainer* tr, racer_surrogate* sur, int audit_every, float fallback_m) {
  RACER_ARG(tr && audit_every >= 0 && fallback_m >= 0.0f, "racer_trainer_set_surrogate: bad argument");
  tr->sur = sur;
  tr->audit_every = audit_every;
  tr->fallback = fallback_m / RANGE;
  return 0;
}

// One minibatch on the inputs x[m] gathered beforehand (launch_gather_all).
// dgrads_f32: also the FP32 data gradients tr->d2, tr->d1 (an update only needs the weight gradients).
static int minibatch_on(racer_trainer* tr, racer_policy* p, int m, int use_moments, float adv_mean,
                        float adv_scale, bool dgrads_f32 = true) {
  cudaStream_t st = tr->st;
  const int B = tr->batch, IN = tr->in_rows, P = policy_params(p);
  const float* logstd = policy_theta(p) + P - 2;
  const float* x = tr->x + (size_t)m * IN * B;
  int rc = forward_on(p, x, tr->acts, st);
  if (rc) return rc;
  launch_loss(tr->n, B, m, tr->actions, tr->logp, tr->value, tr->advantage, tr->acts->o, logstd,
              tr->stats + ST_ADV, use_moments, adv_mean, adv_scale, tr->d3, st);
  if ((rc = policy_backward(p, x, B, tr->acts->h1, tr->acts->h2, tr->d3, tr->d2, tr->d1, tr->grad, st,
                            &tr->xmaps[m], dgrads_f32)))
    return rc;
  launch_rowsum(tr->d3 + (size_t)OUT * B, 2, B, B, tr->grad + P - 2, tr->red, 0, st);
  launch_rowsum(tr->grad, 1, P, P, tr->stats + ST_NORM, tr->red + 2048, 1, st);
  RACER_LAUNCHED();
  return 0;
}

int racer_trainer_minibatch(racer_trainer* tr, racer_policy* p, int m, float adv_mean, float adv_scale) {
  RACER_ARG(tr && p && m >= 0 && m < MINIBATCHES, "racer_trainer_minibatch: bad argument");
  RACER_ARG(policy_inputs(p) == tr->in_rows, "racer_trainer_minibatch: policy and trainer sizes differ");
  launch_gather_all(tr->in_rows, tr->n, tr->rollout, tr->batch, tr->obs, tr->x, tr->st, tr->xb, tr->xld);
  RACER_LAUNCHED();
  return minibatch_on(tr, p, m, 0, adv_mean, adv_scale);
}

// The launches of one update (racer/ppo.mojo:234-257): advantage moments,
// the minibatch gather, 4 epochs x 4 minibatches of loss, backward, Adam and
// weight repacking. Adam's step k reads its bias corrections from c12_dev[2k].
static int update_body(racer_trainer* tr, racer_policy* p) {
  cudaStream_t st = tr->st;
  const int P = policy_params(p);
  RACER_TRY(cudaMemcpyAsync(tr->c12_dev, tr->c12_host, 2 * EPOCHS * MINIBATCHES * sizeof(float),
                            cudaMemcpyHostToDevice, st));
  launch_moments(tr->advantage, (long)tr->rollout * tr->n, tr->stats, tr->red, st);
  // the minibatches' samples are the same in every epoch: gather them once
  launch_gather_all(tr->in_rows, tr->n, tr->rollout, tr->batch, tr->obs, tr->x, st, tr->xb, tr->xld);
  RACER_LAUNCHED();
  for (int epoch = 0; epoch < EPOCHS; ++epoch) {
    for (int m = 0; m < MINIBATCHES; ++m) {
      int rc = minibatch_on(tr, p, (m + epoch) % MINIBATCHES, 1, 0.0f, 1.0f, false);
      if (rc) return rc;
      launch_adam(P, P - 2, tr->c12_dev + 2 * (epoch * MINIBATCHES + m), tr->stats, policy_theta(p), tr->grad,
                  tr->first, tr->second, st);
      RACER_LAUNCHED();
      if ((rc = policy_refresh_on(p, st))) return rc;
    }
  }
  launch_rowsum(tr->d3 + (size_t)(OUT + 2) * tr->batch, 1, tr->batch, tr->batch, tr->stats + ST_KL, tr->red, 0, st);
  RACER_LAUNCHED();
  return 0;
}

int racer_trainer_update(racer_trainer* tr, racer_policy* p, float* kl) {
  RACER_ARG(tr && p, "racer_trainer_update: null argument");
  RACER_ARG(policy_inputs(p) == tr->in_rows, "racer_trainer_update: policy and trainer sizes differ");
  cudaStream_t st = tr->st;
  for (int k = 0; k < EPOCHS * MINIBATCHES; ++k) {  // Adam's bias corrections, as the reference computes them
    const float t = (float)(tr->step + k + 1);
    tr->c12_host[2 * k] = 1.0f - powf(0.9f, t);
    tr->c12_host[2 * k + 1] = 1.0f - powf(0.999f, t);
  }
  const int generation = policy_generation(p);
  if (tr->update_policy != p || tr->update_generation != generation || !tr->graphs) {
    if (tr->update_exec) cudaGraphExecDestroy(tr->update_exec);
    tr->update_exec = nullptr;
    tr->update_policy = p;
    tr->update_generation = generation;
    tr->update_warm = false;
  }
  if (tr->update_exec) {
    RACER_TRY(cudaGraphLaunch(tr->update_exec, st));
  } else if (tr->graphs && tr->update_warm) {
    cudaGraph_t graph = nullptr;
    RACER_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int rc = update_body(tr, p);
    const cudaError_t end = cudaStreamEndCapture(st, &graph);
    cudaError_t inst = cudaErrorUnknown;
    if (!rc && end == cudaSuccess) inst = cudaGraphInstantiate(&tr->update_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (inst == cudaSuccess) {
      RACER_TRY(cudaGraphLaunch(tr->update_exec, st));
    } else {  // nothing ran during the capture: update eagerly, and from now on always
      tr->update_exec = nullptr;
      cudaGetLastError();
      tr->graphs = false;
      if (int rc2 = update_body(tr, p)) return rc2;
    }
  } else {
    if (int rc = update_body(tr, p)) return rc;
    // the first update of a policy generation set up its workspaces; the next one is captured
    tr->update_warm = policy_generation(p) == generation;
    tr->update_generation = policy_generation(p);
  }
  tr->step += EPOCHS * MINIBATCHES;
  float stats[STATS];
  RACER_TRY(cudaMemcpyAsync(stats, tr->stats, sizeof stats, cudaMemcpyDeviceToHost, st));
  RACER_TRY(cudaStreamSynchronize(st));
  if (kl) *kl = stats[ST_KL] / (float)tr->batch;
  return 0;
}

int racer_trainer_set_graphs(racer_trainer* tr, int enable) {
  RACER_ARG(tr, "racer_trainer_set_graphs: null trainer");
  tr->graphs = enable != 0;
  if (!tr->graphs && tr->update_exec) {
    cudaGraphExecDestroy(tr->update_exec);
    tr->update_exec = nullptr;
  }
  return 0;
}

// ---------------- Runner ----------------

// One Runner step (main.mojo:40-48). With a surrogate, the lidar rows come
// from it (audited by, or falling back to, the exact tracer).
// Cars [c0, c1) only (a rollout chain): policy forward and sampling, physics
// and the lidar of those cars; every per-car result is the full step's.
static int runner_step_cars(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int det, const int64_t* base,
                            int64_t add, cudaStream_t st, int c0, int c1) {
  SampleArgs sa;
  sa.seed = s->seed;
  sa.log_std = policy_theta(p) + policy_params(p) - 2;
  sa.actions = s->actions;
  sa.logp = scratch;
  sa.value = scratch + s->n;
  sa.deterministic = det;
  sa.step_base = base;
  sa.step_add = add;
  if (int rc = forward_on(p, s->obs, a, st, &sa, 0, c0, c1)) return rc;
  launch_advance(s->seg, s->state, s->actions, s->reward, s->done, s->obs, s->n, s->beams, s->ray, st, nullptr,
                 nullptr, c0, c1);
  launch_lidar_cars(s->seg, s->shape, c0, c1, s->ray, s->obs, s->n, s->beams, s->beam_dir, nullptr, st);
  RACER_LAUNCHED();
  return 0;
}

static int runner_step_on(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int det,
                          const int64_t* base, int64_t add, cudaStream_t st, racer_surrogate* sur = nullptr,
                          bool audit = false, float fallback = 0.0f, bool eval = false) {
  SampleArgs sa;
  sa.seed = s->seed;
  sa.log_std = policy_theta(p) + policy_params(p) - 2;
  sa.actions = s->actions;
  sa.logp = scratch;
  sa.value = scratch + s->n;
  sa.deterministic = det;
  sa.step_base = base;
  sa.step_add = add;
  int rc = forward_on(p, s->obs, a, st, &sa, 0);
  if (rc) return rc;
  if (!sur) return sim_step_on(s, s->actions, s->reward, s->done, s->obs, nullptr, st, eval);
  launch_advance(s->seg, s->state, s->actions, s->reward, s->done, s->obs, s->n, s->beams, s->ray, st);
  RACER_LAUNCHED();
  return surrogate_lidar(sur, s, s->obs, audit, fallback, st, base, add);
}

int racer_rollout_surrogate(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, racer_surrogate* sur,
                            int steps, int det, int64_t step0, int audit_every, float fallback_m) {
  RACER_ARG(s && p && a && scratch && sur && steps >= 1 && audit_every >= 0, "racer_rollout_surrogate: bad argument");
  RACER_ARG(a->cols == s->n && policy_inputs(p) == s->in_rows, "racer_rollout_surrogate: sizes differ");
  if (int rc = surrogate_prepare(sur, s)) return rc;
  const float fallback = fallback_m / RANGE;
  auto key = std::make_tuple((const void*)p, (const void*)a, (const void*)scratch, steps, det, (const void*)sur,
                             audit_every, fallback);
  auto it = s->surrogate_graphs.find(key);
  int audits = 0;
  for (int k = 0; k < steps; ++k) audits += audit_every > 0 && k % audit_every == 0;
  if (it == s->surrogate_graphs.end()) {
    cudaGraph_t g;
    RACER_TRY(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int k = 0; k < steps && !rc; ++k)
      rc = runner_step_on(s, p, a, scratch, det, s->step_base, k, s->st, sur, audit_every > 0 && k % audit_every == 0,
                          fallback);
    cudaError_t end = cudaStreamEndCapture(s->st, &g);
    if (rc) return rc;
    RACER_TRY(end);
    cudaGraphExec_t exec;
    cudaError_t inst = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    RACER_TRY(inst);
    it = s->surrogate_graphs.emplace(key, exec).first;
  }
  k_set_i64<<<1, 32, 0, s->st>>>(s->step_base, step0);
  RACER_LAUNCHED();
  RACER_TRY(cudaGraphLaunch(it->second, s->st));
  surrogate_account(sur, s, steps, audits);
  return 0;
}

int racer_runner_step(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int det, int64_t t) {
  RACER_ARG(s && p && a && scratch, "racer_runner_step: null argument");
  RACER_ARG(a->cols == s->n && policy_inputs(p) == s->in_rows, "racer_runner_step: sizes differ");
  return runner_step_on(s, p, a, scratch, det, nullptr, t, s->st);
}

int racer_runner_audit_dynamics(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int det, int steps,
                                int64_t step0, double* out) {
  RACER_ARG(s && p && a && scratch && out && steps >= 1, "racer_runner_audit_dynamics: bad argument");
  RACER_ARG(a->cols == s->n && policy_inputs(p) == s->in_rows, "racer_runner_audit_dynamics: sizes differ");
  cudaStream_t st = s->st;
  float* prev = nullptr;
  double* stats = nullptr;
  const size_t state_bytes = (size_t)STATE * s->n * sizeof(float);
  RACER_TRY(cudaMallocAsync((void**)&prev, state_bytes, st));
  RACER_TRY(cudaMallocAsync((void**)&stats, 7 * sizeof(double), st));
  RACER_TRY(cudaMemsetAsync(stats, 0, 7 * sizeof(double), st));
  int rc = 0;
  for (int k = 0; k < steps && !rc; ++k) {
    SampleArgs sa;
    sa.seed = s->seed;
    sa.log_std = policy_theta(p) + policy_params(p) - 2;
    sa.actions = s->actions;
    sa.logp = scratch;
    sa.value = scratch + s->n;
    sa.deterministic = det;
    sa.step_base = nullptr;
    sa.step_add = step0 + k;
    if ((rc = forward_on(p, s->obs, a, st, &sa, 0))) break;
    RACER_TRY(cudaMemcpyAsync(prev, s->state, state_bytes, cudaMemcpyDeviceToDevice, st));
    if ((rc = sim_step_on(s, s->actions, s->reward, s->done, s->obs, nullptr, st))) break;
    launch_rk4_audit(s->seg, prev, s->actions, s->state, s->done, s->n, stats, st);
    RACER_LAUNCHED();
  }
  cudaError_t copy = cudaMemcpyAsync(out, stats, 7 * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(prev, st);
  cudaFreeAsync(stats, st);
  RACER_TRY(cudaStreamSynchronize(st));
  if (rc) return rc;
  RACER_TRY(copy);
  return 0;
}

// Totals of the per-car evaluation sums in a fixed order (one block): the
// result does not depend on scheduling.
__global__ void k_eval_total(const double* reward, const int* crash, int n, double* out) {
  __shared__ double sr[1024];
  __shared__ long long sc[1024];
  double r = 0;
  long long c = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    r += reward[i];
    c += crash[i];
  }
  sr[threadIdx.x] = r;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      sc[threadIdx.x] += sc[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sr[0];
    out[1] = (double)sc[0];
  }
}

int racer_runner_evaluate(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int steps, int64_t step0,
                          double* out) {
  RACER_ARG(s && p && a && scratch && out && steps >= 1, "racer_runner_evaluate: bad argument");
  RACER_ARG(a->cols == s->n && policy_inputs(p) == s->in_rows, "racer_runner_evaluate: sizes differ");
  cudaStream_t st = s->st;
  if (!s->eval_reward) {
    int rc = 0;
    if ((rc = dalloc(&s->eval_reward, s->n)) || (rc = dalloc(&s->eval_crash, s->n)) ||
        (rc = dalloc(&s->eval_total, 2)))
      return rc;
  }
  RACER_TRY(cudaMemsetAsync(s->eval_reward, 0, (size_t)s->n * sizeof(double), st));
  RACER_TRY(cudaMemsetAsync(s->eval_crash, 0, (size_t)s->n * sizeof(int), st));
  auto key = std::make_tuple((const void*)p, (const void*)a, (const void*)scratch, steps);
  auto it = s->eval_graphs.find(key);
  if (it == s->eval_graphs.end()) {
    cudaGraph_t g;
    RACER_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int k = 0; k < steps && !rc; ++k)
      rc = runner_step_on(s, p, a, scratch, 1, s->step_base, k, st, nullptr, false, 0.0f, true);
    cudaError_t end = cudaStreamEndCapture(st, &g);
    if (rc) return rc;
    RACER_TRY(end);
    cudaGraphExec_t exec;
    cudaError_t inst = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    RACER_TRY(inst);
    it = s->eval_graphs.emplace(key, exec).first;
  }
  k_set_i64<<<1, 32, 0, st>>>(s->step_base, step0);
  RACER_LAUNCHED();
  RACER_TRY(cudaGraphLaunch(it->second, st));
  k_eval_total<<<1, 1024, 0, st>>>(s->eval_reward, s->eval_crash, s->n, s->eval_total);
  RACER_LAUNCHED();
  double host[2];
  RACER_TRY(cudaMemcpyAsync(host, s->eval_total, sizeof host, cudaMemcpyDeviceToHost, st));
  RACER_TRY(cudaStreamSynchronize(st));
  out[0] = host[0] / ((double)s->n * steps);
  out[1] = host[1] / (double)s->n;
  return 0;
}

// [state | obs | actions | reward | done] of every car, row after row.
__global__ void k_pack_snapshot(const float* state, const float* obs, const float* actions, const float* reward,
                                const float* done, long n, int in_rows, float* out) {
  const long total = (STATE + in_rows + 4) * n;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
    const long row = q / n, col = q % n;
    float v;
    if (row < STATE)
      v = state[q];
    else if (row < STATE + in_rows)
      v = obs[q - STATE * n];
    else if (row < STATE + in_rows + 2)
      v = actions[q - (STATE + in_rows) * n];
    else if (row == STATE + in_rows + 2)
      v = reward[col];
    else
      v = done[col];
    out[q] = v;
  }
}

int racer_sim_snapshot(racer_sim* s, float* host, int synchronize) {
  RACER_ARG(s && host, "racer_sim_snapshot: null argument");
  const size_t count = (size_t)(STATE + s->in_rows + 4) * s->n;
  if (!s->snapshot)
    if (int rc = dalloc(&s->snapshot, count)) return rc;
  k_pack_snapshot<<<4 * s->sms, 256, 0, s->st>>>(s->state, s->obs, s->actions, s->reward, s->done, s->n,
                                                  s->in_rows, s->snapshot);
  RACER_LAUNCHED();
  RACER_TRY(cudaMemcpyAsync(host, s->snapshot, count * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  if (synchronize) RACER_TRY(cudaStreamSynchronize(s->st));
  return 0;
}

// Captures (once) the graph of `steps` Runner steps for these arguments.
static int rollout_graph(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int steps, int det,
                         cudaGraphExec_t* exec_out, size_t* kernels) {
  auto key = std::make_tuple((const void*)p, (const void*)a, (const void*)scratch, steps, det);
  auto it = s->graphs.find(key);
  if (it == s->graphs.end()) {
    cudaGraph_t g;
    RACER_TRY(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    const int chains = s->chains > 1 && s->seg.count == 1 && policy_is_bf16(p) ? s->chains : 1;
    if (s->fused && s->seg.count == 1 && policy_is_bf16(p)) {
      // the whole rollout as one launch of the fused persistent kernel
      SampleArgs sa;
      sa.seed = s->seed;
      sa.log_std = policy_theta(p) + policy_params(p) - 2;
      sa.actions = s->actions;
      sa.logp = scratch;
      sa.value = scratch + s->n;
      sa.deterministic = det;
      sa.step_base = s->step_base;
      sa.step_add = 0;
      const cudaError_t e = launch_rollout_fused(s->seg, s->state, s->actions, s->reward, s->done, s->obs, s->n,
                                                 s->beams, s->ray, s->beam_dir, steps, policy_pack(p), a->o, sa,
                                                 policy_err(p), s->sms, s->st);
      if (e != cudaSuccess) {
        set_error(std::string("fused rollout: ") + cudaGetErrorString(e));
        rc = 2;
      }
    } else if (chains == 1) {
      for (int k = 0; k < steps && !rc; ++k) rc = runner_step_on(s, p, a, scratch, det, s->step_base, k, s->st);
    } else {
      // independent chains over car ranges (multiples of 128, the forward's tile), forked from and joined
      // into the sim's stream: parallel branches, so one chain's latency-bound kernels run beside
      // another's lidar
      int bound[MAX_CHAINS + 1];
      for (int c = 0; c <= chains; ++c) bound[c] = c == chains ? s->n : std::min(s->n, (int)((long)s->n * c / chains / 128 * 128));
      cudaError_t e = cudaEventRecord(s->chain_fork, s->st);
      for (int c = 1; c < chains && e == cudaSuccess; ++c) e = cudaStreamWaitEvent(s->chain_st[c - 1], s->chain_fork, 0);
      for (int k = 0; k < steps && !rc && e == cudaSuccess; ++k)
        for (int c = 0; c < chains && !rc; ++c)
          rc = runner_step_cars(s, p, a, scratch, det, s->step_base, k, c ? s->chain_st[c - 1] : s->st, bound[c],
                                bound[c + 1]);
      for (int c = 1; c < chains && e == cudaSuccess; ++c) {
        e = cudaEventRecord(s->chain_join[c - 1], s->chain_st[c - 1]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->st, s->chain_join[c - 1], 0);
      }
      if (e != cudaSuccess && !rc) {
        set_error(std::string("rollout chains: ") + cudaGetErrorString(e));
        rc = 2;
      }
    }
    cudaError_t end = cudaStreamEndCapture(s->st, &g);
    if (rc) return rc;
    RACER_TRY(end);
    size_t count = 0;
    RACER_TRY(cudaGraphGetNodes(g, nullptr, &count));
    std::vector<cudaGraphNode_t> nodes(count);
    size_t kcount = 0;
    if (count) RACER_TRY(cudaGraphGetNodes(g, nodes.data(), &count));
    for (auto nd : nodes) {
      cudaGraphNodeType type;
      RACER_TRY(cudaGraphNodeGetType(nd, &type));
      kcount += type == cudaGraphNodeTypeKernel;
    }
    cudaGraphExec_t exec;
    cudaError_t inst = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    RACER_TRY(inst);
    it = s->graphs.emplace(key, exec).first;
    s->graph_kernels[key] = kcount;
  }
  *exec_out = it->second;
  if (kernels) *kernels = s->graph_kernels[key];
  return 0;
}

int racer_rollout(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int steps, int det, int64_t step0) {
  RACER_ARG(s && p && a && scratch && steps >= 1, "racer_rollout: bad argument");
  RACER_ARG(a->cols == s->n && policy_inputs(p) == s->in_rows, "racer_rollout: sizes differ");
  cudaGraphExec_t exec;
  if (int rc = rollout_graph(s, p, a, scratch, steps, det, &exec, nullptr)) return rc;
  k_set_i64<<<1, 32, 0, s->st>>>(s->step_base, step0);
  RACER_LAUNCHED();
  RACER_TRY(cudaGraphLaunch(exec, s->st));
  return 0;
}

int racer_runner_tune_chains(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int steps, int reps,
                             int* best_chains, float* best_rate) {
  RACER_ARG(s && p && a && scratch && steps >= 1 && reps >= 1, "racer_runner_tune_chains: bad argument");
  cudaEvent_t t0, t1;
  RACER_TRY(cudaEventCreate(&t0));
  RACER_TRY(cudaEventCreate(&t1));
  int best = 1;
  float rate = 0.0f;
  const bool eligible = s->seg.count == 1 && policy_is_bf16(p);
  int64_t step0 = 0;
  // candidates: 1 to 16 chains of kernels (one without a BF16 one-track policy), then (eligible
  // sims) the fused persistent kernel, as 0
  std::vector<int> cands = eligible ? std::vector<int>{1, 2, 3, 4, 6, 8, 12, 16, 0} : std::vector<int>{1};
  for (const int chains : cands) {
    if (int rc = racer_sim_set_fused_rollout(s, chains == 0)) return rc;
    if (int rc = racer_sim_set_chains(s, chains == 0 ? 1 : chains)) return rc;
    if (int rc = racer_rollout(s, p, a, scratch, steps, 0, step0)) return rc;  // capture and warm up
    step0 += steps;
    RACER_TRY(cudaEventRecord(t0, s->st));
    for (int r = 0; r < reps; ++r, step0 += steps)
      if (int rc = racer_rollout(s, p, a, scratch, steps, 0, step0)) return rc;
    RACER_TRY(cudaEventRecord(t1, s->st));
    RACER_TRY(cudaEventSynchronize(t1));
    float ms = 0.0f;
    RACER_TRY(cudaEventElapsedTime(&ms, t0, t1));
    const float r = (float)((double)s->n * steps * reps / (ms / 1000.0));
    if (r > rate) rate = r, best = chains;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (int rc = racer_sim_set_fused_rollout(s, best == 0)) return rc;
  if (int rc = racer_sim_set_chains(s, best == 0 ? 1 : best)) return rc;
  if (best_chains) *best_chains = best;
  if (best_rate) *best_rate = rate;
  return 0;
}

int racer_rollout_kernel_count(racer_sim* s, racer_policy* p, racer_acts* a, float* scratch, int steps, int det,
                               int64_t* count) {
  RACER_ARG(s && p && a && scratch && steps >= 1 && count, "racer_rollout_kernel_count: bad argument");
  RACER_ARG(a->cols == s->n && policy_inputs(p) == s->in_rows, "racer_rollout_kernel_count: sizes differ");
  cudaGraphExec_t exec;
  size_t k = 0;
  if (int rc = rollout_graph(s, p, a, scratch, steps, det, &exec, &k)) return rc;
  *count = (int64_t)k + 1;
  return 0;
}

__global__ void k_sum_i32(const int32_t* v, long count, unsigned long long* out) {
  unsigned long long acc = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x)
    acc += (unsigned long long)v[i];
  atomicAdd(out, acc);
}

int racer_sim_profile(racer_sim* s, const float* actions, int reps, float* physics_ms, float* lidar_ms,
                      int64_t* probe_iterations) {
  RACER_ARG(s && actions && reps >= 1, "racer_sim_profile: bad argument");
  cudaStream_t st = s->st;
  std::vector<cudaEvent_t> ev(3 * reps);
  for (auto& e : ev) RACER_TRY(cudaEventCreate(&e));
  for (int r = 0; r < reps; ++r) {
    RACER_TRY(cudaEventRecord(ev[3 * r], st));
    launch_advance(s->seg, s->state, actions, s->reward, s->done, s->obs, s->n, s->beams, s->ray, st);
    RACER_TRY(cudaEventRecord(ev[3 * r + 1], st));
    if (int rc = lidar_on(s, s->shape, s->obs, nullptr, st)) return rc;
    RACER_TRY(cudaEventRecord(ev[3 * r + 2], st));
  }
  RACER_LAUNCHED();
  int32_t* iters = nullptr;
  unsigned long long* total = nullptr;
  RACER_TRY(cudaMalloc((void**)&iters, (size_t)s->beams * s->n * sizeof(int32_t)));
  RACER_TRY(cudaMalloc((void**)&total, sizeof(unsigned long long)));
  RACER_TRY(cudaMemsetAsync(total, 0, sizeof(unsigned long long), st));
  if (int rc = lidar_on(s, s->shape, s->obs, iters, st)) return rc;
  k_sum_i32<<<s->sms, 256, 0, st>>>(iters, (long)s->beams * s->n, total);
  RACER_LAUNCHED();
  unsigned long long host_total = 0;
  RACER_TRY(cudaMemcpyAsync(&host_total, total, sizeof host_total, cudaMemcpyDeviceToHost, st));
  RACER_TRY(cudaStreamSynchronize(st));
  cudaFree(iters);
  cudaFree(total);
  double phys = 0, lid = 0;
  for (int r = 0; r < reps; ++r) {
    float a = 0, b = 0;
    RACER_TRY(cudaEventElapsedTime(&a, ev[3 * r], ev[3 * r + 1]));
    RACER_TRY(cudaEventElapsedTime(&b, ev[3 * r + 1], ev[3 * r + 2]));
    phys += a;
    lid += b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (physics_ms) *physics_ms = (float)(phys / reps);
  if (lidar_ms) *lidar_ms = (float)(lid / reps);
  if (probe_iterations) *probe_iterations = (int64_t)host_total;
  return 0;
}

// Random 16-byte gathers from an L2-resident buffer: every thread walks its
// own linear congruential sequence of float4 indices (8 loads in flight),
// the way the lidar's probes gather its cells, and folds what it read into
// one value so no load is dead code.
__global__ void k_gather_peak(const float4* __restrict__ buf, unsigned mask, int rounds, unsigned seed,
                              float* sink) {
  unsigned h[8];
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
  for (int u = 0; u < 8; ++u) h[u] = (t * 8u + u) * 2654435761u ^ seed;
  float acc = 0.0f;
  for (int k = 0; k < rounds; ++k) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      h[u] = h[u] * 1664525u + 1013904223u;
      const float4 v = __ldg(buf + ((h[u] >> 8) & mask));
      acc += (v.x + v.y) + (v.z + v.w);
    }
  }
  if (acc == -1.0f) sink[t] = acc;  // never true for the nonnegative buffer
}

int racer_gather_peak(size_t bytes, int reps, float* gbs) {
  RACER_ARG(gbs && reps >= 1 && bytes >= 4096 && (bytes & (bytes - 1)) == 0 && bytes <= (1ull << 28),
            "racer_gather_peak: bytes must be a power of two from 4 KB to 256 MB, reps >= 1");
  float4* buf = nullptr;
  float* sink = nullptr;
  cudaStream_t st = nullptr;
  RACER_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  RACER_TRY(cudaMalloc((void**)&buf, bytes));
  RACER_TRY(cudaMalloc((void**)&sink, sizeof(float) * 4));
  RACER_TRY(cudaMemsetAsync(buf, 0, bytes, st));
  const int sms = device_sms(), blocks = sms * 8, threads = 256, rounds = 64;
  const unsigned mask = (unsigned)(bytes / sizeof(float4)) - 1u;
  cudaEvent_t a, b;
  RACER_TRY(cudaEventCreate(&a));
  RACER_TRY(cudaEventCreate(&b));
  for (int w = 0; w < 3; ++w) k_gather_peak<<<blocks, threads, 0, st>>>(buf, mask, rounds, 17u + w, sink);
  RACER_TRY(cudaEventRecord(a, st));
  for (int r = 0; r < reps; ++r) k_gather_peak<<<blocks, threads, 0, st>>>(buf, mask, rounds, 101u + r, sink);
  RACER_TRY(cudaEventRecord(b, st));
  RACER_TRY(cudaEventSynchronize(b));
  RACER_LAUNCHED();
  float ms = 0.0f;
  RACER_TRY(cudaEventElapsedTime(&ms, a, b));
  const double loaded = (double)blocks * threads * rounds * 8 * sizeof(float4) * reps;
  *gbs = (float)(loaded / (ms / 1000.0) / 1e9);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  cudaFree(sink);
  cudaStreamDestroy(st);
  return 0;
}

// Sum of iters[b * n + c] over all beams b and cars c in [c0, c1).
__global__ void k_sum_cols(const int32_t* iters, int n, int beams, int c0, int c1, unsigned long long* out) {
  const long w = c1 - c0, total = w * beams;
  unsigned long long acc = 0;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x)
    acc += (unsigned long long)iters[(q / w) * n + c0 + q % w];
  for (int off = 16; off; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

static void drop_graphs(racer_sim* s) {
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  for (auto& kv : s->surrogate_graphs) cudaGraphExecDestroy(kv.second);
  for (auto& kv : s->eval_graphs) cudaGraphExecDestroy(kv.second);
  s->eval_graphs.clear();
  s->graphs.clear();
  s->graph_kernels.clear();
  s->surrogate_graphs.clear();
}

static LidarShape from_api(const racer_lidar_shape& in) {
  LidarShape shape;
  shape.cars = in.cars_per_block;
  shape.wide = in.wide;
  shape.split = in.split;
  shape.dynamic = in.dynamic;
  shape.flat = in.flat;
  for (int j = 0; j < MAX_SEGMENTS; ++j) shape.order[j] = in.order[j];
  return shape;
}

static void to_api(const racer_sim* s, const LidarShape& shape, racer_lidar_shape* out) {
  out->cars_per_block = shape.cars;
  out->wide = shape.wide;
  out->split = shape.split;
  out->dynamic = shape.dynamic;
  out->flat = shape.flat;
  int order[MAX_SEGMENTS];
  segment_order(s, shape, order);
  for (int j = 0; j < MAX_SEGMENTS; ++j) out->order[j] = j < s->seg.count ? order[j] : -1;
}

static bool same_shape(const racer_sim* s, const LidarShape& a, const LidarShape& b) {
  int oa[MAX_SEGMENTS], ob[MAX_SEGMENTS];
  segment_order(s, a, oa);
  segment_order(s, b, ob);
  return a.cars == b.cars && a.wide == b.wide && a.split == b.split && a.dynamic == b.dynamic && a.flat == b.flat &&
         std::equal(oa, oa + s->seg.count, ob);
}

int racer_sim_set_chains(racer_sim* s, int chains) {
  RACER_ARG(s && chains >= 1 && chains <= MAX_CHAINS, "racer_sim_set_chains: 1 to 16 chains");
  RACER_TRY(cudaStreamSynchronize(s->st));
  if (!s->chain_fork) RACER_TRY(cudaEventCreateWithFlags(&s->chain_fork, cudaEventDisableTiming));
  while ((int)s->chain_st.size() < chains - 1) {
    cudaStream_t c;
    cudaEvent_t e;
    RACER_TRY(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
    s->chain_st.push_back(c);
    RACER_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    s->chain_join.push_back(e);
  }
  if (chains != s->chains) drop_graphs(s);
  s->chains = chains;
  return 0;
}

int racer_sim_set_fused_rollout(racer_sim* s, int enable) {
  RACER_ARG(s, "racer_sim_set_fused_rollout: null sim");
  RACER_TRY(cudaStreamSynchronize(s->st));
  if ((enable != 0) != (s->fused != 0)) drop_graphs(s);
  s->fused = enable != 0;
  return 0;
}

int racer_sim_set_lidar_shape(racer_sim* s, const racer_lidar_shape* in) {
  RACER_ARG(s && in, "racer_sim_set_lidar_shape: null argument");
  LidarShape shape = from_api(*in);
  RACER_ARG(lidar_shape_ok(shape) && (shape.split == 0 || shape.split == 1) &&
                (shape.dynamic == 0 || shape.dynamic == 1),
            "racer_sim_set_lidar_shape: cars per block must be 2, 4 or 8, wide, split, dynamic and flat 0 or 1");
  bool seen[MAX_SEGMENTS] = {};
  for (int j = 0; j < s->seg.count; ++j) {
    RACER_ARG(in->order[j] >= 0 && in->order[j] < s->seg.count && !seen[in->order[j]],
              "racer_sim_set_lidar_shape: order must be a permutation of the segments");
    seen[in->order[j]] = true;
  }
  RACER_TRY(cudaStreamSynchronize(s->st));
  if (!same_shape(s, shape, s->shape)) drop_graphs(s);
  s->shape = shape;
  return 0;
}

int racer_sim_get_lidar_shape(racer_sim* s, racer_lidar_shape* out) {
  RACER_ARG(s && out, "racer_sim_get_lidar_shape: null argument");
  to_api(s, s->shape, out);
  return 0;
}

int racer_sim_autotune(racer_sim* s, int reps, racer_lidar_shape* best_out, float* best_ms) {
  RACER_ARG(s && reps >= 1, "racer_sim_autotune: bad argument");
  cudaStream_t st = s->st;
  const int count = s->seg.count;
  // probe iterations per segment, from one counted pass
  int32_t* iters = nullptr;
  unsigned long long* sums = nullptr;
  RACER_TRY(cudaMalloc((void**)&iters, (size_t)s->beams * s->n * sizeof(int32_t)));
  RACER_TRY(cudaMalloc((void**)&sums, MAX_SEGMENTS * sizeof(unsigned long long)));
  RACER_TRY(cudaMemsetAsync(sums, 0, MAX_SEGMENTS * sizeof(unsigned long long), st));
  if (int rc = lidar_on(s, s->shape, s->obs, iters, st)) return rc;
  for (int k = 0; k < count; ++k)
    k_sum_cols<<<4 * s->sms, 256, 0, st>>>(iters, s->n, s->beams, s->seg.car0[k], s->seg.car0[k + 1], sums + k);
  RACER_LAUNCHED();
  unsigned long long host[MAX_SEGMENTS] = {};
  RACER_TRY(cudaMemcpyAsync(host, sums, sizeof host, cudaMemcpyDeviceToHost, st));
  RACER_TRY(cudaStreamSynchronize(st));
  cudaFree(iters);
  cudaFree(sums);
  int heavy[MAX_SEGMENTS];
  for (int j = 0; j < MAX_SEGMENTS; ++j) heavy[j] = j;
  std::stable_sort(heavy, heavy + count, [&](int a, int b) { return host[a] > host[b]; });
  std::vector<LidarShape> candidates;
  for (int dynamic : {0, 1})
    for (int cars : {2, 4, 8})
      for (int wide : {0, 1})
        for (int split : {0, 1})
          for (int sorted : {0, 1})
            for (int flat : {0, 1}) {
          if (count == 1 && (split || sorted)) continue;
          if (dynamic && (cars != 2 || (count > 1 && !split))) continue;  // per segment; no cars-per-block
          if (flat && (dynamic || (count > 1 && !split))) continue;       // one-track launches only
          LidarShape shape;
          shape.cars = cars;
          shape.wide = wide;
          shape.split = split;
          shape.dynamic = dynamic;
          shape.flat = flat;
          for (int j = 0; j < MAX_SEGMENTS; ++j) shape.order[j] = sorted ? heavy[j] : j;
          candidates.push_back(shape);
        }
  cudaEvent_t a, b;
  RACER_TRY(cudaEventCreate(&a));
  RACER_TRY(cudaEventCreate(&b));
  // two rounds over the candidates, each candidate's best round kept: the
  // first candidates of a round must not pay for clocks still ramping up
  std::vector<float> per(candidates.size(), 1e30f);
  for (int round = 0; round < 2; ++round)
    for (size_t c = 0; c < candidates.size(); ++c) {
      const LidarShape& shape = candidates[c];
      if (int rc = lidar_on(s, shape, s->obs, nullptr, st)) return rc;
      RACER_TRY(cudaEventRecord(a, st));
      for (int r = 0; r < reps; ++r)
        if (int rc = lidar_on(s, shape, s->obs, nullptr, st)) return rc;
      RACER_TRY(cudaEventRecord(b, st));
      RACER_TRY(cudaEventSynchronize(b));
      float ms = 0;
      RACER_TRY(cudaEventElapsedTime(&ms, a, b));
      per[c] = std::min(per[c], ms / reps);
    }
  float best = 1e30f;
  LidarShape chosen = s->shape;
  for (size_t c = 0; c < candidates.size(); ++c)
    if (per[c] < best) best = per[c], chosen = candidates[c];
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!same_shape(s, chosen, s->shape)) drop_graphs(s);
  s->shape = chosen;
  if (best_out) to_api(s, s->shape, best_out);
  if (best_ms) *best_ms = best;
  return 0;
}

}  // extern "C"
