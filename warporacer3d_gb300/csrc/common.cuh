// Shared definitions for the warporacer3d GB300 kernels: simulator and
// policy constants (racer/sim.mojo:15-56, racer/ppo.mojo:17-37), the device
// view of a track, and host-side error plumbing for the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>

namespace racer {

// racer/sim.mojo:15-56
constexpr float WHEELBASE = 0.3302f, HALF_DIAG = 0.3f, GRIP = 1.05f, GRAV = 9.81f;
constexpr float STEER_MAX = 0.4189f, STEER_RATE = 3.2f, ACCEL_MAX = 9.51f, SPEED_MAX = 5.0f;
constexpr int SUBSTEPS = 4;
constexpr float DT = (float)(1.0 / 240);
constexpr int HORIZON = 3000;
constexpr float RANGE = 10.0f, FOV = 4.71238898f;
constexpr float MOUNT_X = 0.27f, MOUNT_Z = 0.23f;
enum { X = 0, Y, Z, HEADING, SPEED, STEER, STEPS, PROGRESS, EPISODE, FRICTION, RETURN, STATE };
constexpr int OUT = 3;
constexpr int CRASH = 1, TIMEOUT = 2;
constexpr int HEADER = 12;
constexpr float PI_F = 3.14159274f;      // Float32(pi)
constexpr float TWO_PI_F = 6.28318548f;  // Float32(2 pi)
constexpr float HALF_LOG_2PI = 0.918938533f;  // Float32(0.5 log(2 pi))

// racer/ppo.mojo:17-31
constexpr int H = 64, HA = H + 1;
constexpr int MINIBATCHES = 4, EPOCHS = 4, ROLLOUT = 32;
constexpr float GAMMA = 0.99f, LAMBDA = 0.95f, CLIP = 0.2f, LR = 3e-4f, MAX_NORM = 0.5f;
enum { ST_REWARD = 0, ST_ADV = 1, ST_ADV2 = 2, ST_NORM = 3, ST_KL = 4, STATS = 5 };

// Device view of one track. `d` is the reference's float32 track array,
// uploaded unchanged (header, per layer clearance/height/nearest, route).
// `cl` is the same clearance and height repacked per cell as
// [ny * nx][layers] float2 (clearance, height), so one probe of every layer is
// a single contiguous 8 * layers byte read (one float4 for two layers).
struct TrackDev {
  const float* d;
  const float2* cl;
  int nx, ny, waypoints, layers;
  float x0, y0, cell, spacing, slope;
  float inv_cell;  // RN(1 / cell), for the division-free cell index
  float cx, cy;    // RN(-x0 * inv_cell), RN(-y0 * inv_cell): the cell is rint(fma(x, inv_cell, cx))
  float band;      // 0.5 - (5.001 max(nx, ny) + 4.001 max(|x0|, |y0|) / cell + 16) 2^-24: no division inside +-band
  float nxf, nyf;
  long route;
  // The lidar's cells for one or two layers (sim.cu, lidar_probe): float2 or
  // float4 per cell, rows of lw = nx + 1 cells over ny + 1 rows, the last
  // column and row off-map cells; null for three or more layers.
  const float* lc;
  int lw;
  float mband;     // band of the march's cell index (sim.cu, lidar_cell)
  int free_march;  // 1: the march provably stops on tt >= RANGE before max_iters probes
};

// Several tracks in one launch: cars [car0[k], car0[k + 1]) drive on track
// t[k] and respawn from seed[k], with car index car - car0[k] in their Philox
// counters, so segment k evolves exactly as a sim of that track alone.
// Passed by value as a kernel parameter (about 0.8 KB).
constexpr int MAX_SEGMENTS = 8;
// Rollout graphs as at most this many independent chains over car ranges (racer_sim_set_chains).
constexpr int MAX_CHAINS = 16;
struct Segments {
  int count;
  int car0[MAX_SEGMENTS + 1];
  int max_iters[MAX_SEGMENTS];
  uint64_t seed[MAX_SEGMENTS];
  TrackDev t[MAX_SEGMENTS];
};

// Launch shape of the lidar: cars per block (one warp each) and the order in
// which the segments' blocks are laid out along the grid (heavier first lets
// the light segments fill the tail).
// With several segments, split = 1 launches each segment's one-track kernel
// on its own stream (parallel branches of a captured graph) instead of one
// segment-table launch; `order` is then the launch order.
// dynamic = 1 runs each segment's lidar as a persistent grid whose warps take
// (car, beam group) units from a per-segment counter (counters, zeroed before
// each launch); it applies to one-track sims and split launches, as does
// flat = 1 (k_lidar_flat: no idle lanes when beams is not a multiple of 32).
struct LidarShape {
  int cars = 2;  // measured fastest on every built-in track and the occupancy map
  int wide = 0;  // 1: compiled for 48 resident warps per SM (40 registers) instead of 64 (32)
  int split = 0;
  int dynamic = 0;
  int flat = 0;  // 1: one-track launches take (car, beam) items 32 at a time across car boundaries
  int order[MAX_SEGMENTS] = {0, 1, 2, 3, 4, 5, 6, 7};
  unsigned* counters = nullptr;  // [MAX_SEGMENTS] device words owned by the sim
  int sms = 152;
};

// The current device's SM count, queried once per device (grid sizes of
// persistent and grid-stride kernels).
inline int device_sms() {
  static int cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!cache[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 148;
    cache[dev] = v;
  }
  return cache[dev];
}

// Per-device one-time set-up (kernel attributes such as the dynamic shared
// memory limit belong to each device's context): runs `setup` unless it has
// already succeeded on the current device, as recorded in `mask`.
template <typename F>
cudaError_t once_per_device(unsigned long long* mask, F setup) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
  if (bit && (*mask & bit)) return cudaSuccess;
  e = setup();
  if (e == cudaSuccess) *mask |= bit;
  return e;
}

}  // namespace racer

// Host-side error state of the C ABI (one message per thread).
namespace racer_host {
void set_error(const std::string& msg);
const char* get_error();
}  // namespace racer_host

#define RACER_TRY(expr)                                                                      \
  do {                                                                                       \
    cudaError_t err_ = (expr);                                                               \
    if (err_ != cudaSuccess) {                                                               \
      racer_host::set_error(std::string(#expr) + ": " + cudaGetErrorString(err_));           \
      return 2;                                                                              \
    }                                                                                        \
  } while (0)
