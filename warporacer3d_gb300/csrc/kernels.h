// Host-side launchers of the CUDA kernels, shared by the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "mlp_tc.h"

namespace racer {

// sim.cu (bit-exact simulator kernels). Every car kernel takes the segment
// table; a one-track sim is a table of one.
Segments single_segment(const TrackDev& t, int n, uint64_t seed);
void launch_spawn(const Segments& g, float* state, float* actions, int n, cudaStream_t st);
// ray [2, n] float4: the per-car lidar frame the physics kernel leaves for the lidar. With
// eval_reward / eval_crash [n] set, each car adds its reward and crash to them.
void launch_advance(const Segments& g, float* state, const float* actions, float* reward, float* done, float* obs,
                    int n, int beams, float4* ray, cudaStream_t st, double* eval_reward = nullptr,
                    int* eval_crash = nullptr, int c0 = 0, int c1 = -1);
// The lidar of cars [c0, c1) of a one-track sim (its one-track kernel, static shapes).
void launch_lidar_cars(const Segments& g, const LidarShape& shape, int c0, int c1, const float4* ray, float* obs,
                       int n, int beams, const float2* beam_dir, int* iters, cudaStream_t st);
void launch_lidar(const Segments& g, const LidarShape& shape, const float4* ray, float* obs, int n, int beams,
                  const float2* beam_dir, int* iters, cudaStream_t st);
// The lidar of segment k alone (its one-track kernel), for per-segment launches on parallel streams.
void launch_lidar_segment(const Segments& g, int k, const LidarShape& shape, const float4* ray, float* obs, int n,
                          int beams, const float2* beam_dir, int* iters, cudaStream_t st);
// One track, default shape (surrogate labels).
void launch_lidar(const TrackDev& t, const float4* ray, float* obs, int n, int beams, const float2* beam_dir,
                  int* iters, cudaStream_t st);
// Only the cars list[0 .. *list_count) (at most list_max; the count is read on the device): a
// persistent grid pulling (car, beam group) units from `counter` (zeroed here). sms = SM count.
void launch_lidar_list(const TrackDev& t, const float4* ray, float* obs, int n, int beams, const float2* beam_dir,
                       const int* list, const int* list_count, int list_max, unsigned* counter, int sms,
                       cudaStream_t st);
bool lidar_shape_ok(const LidarShape& shape);
// Spot check: beams (step % stride) + k stride of every car traced exactly and compared with the
// predicted rows pred [beams, n]; cars off by more than tol (range / RANGE units) get minr = 0.
// step = *step_base (if given, read on the device) + step_add.
void launch_lidar_spot(const TrackDev& t, const float4* ray, const float* pred, int n, int beams,
                       const float2* beam_dir, int stride, const int64_t* step_base, int64_t step_add, float tol,
                       unsigned* minr, cudaStream_t st);
// The fused persistent rollout (sim.cu, k_rollout_fused): `steps` Runner steps of a one-track
// sim in one launch, each CTA owning cars_per_cta cars for all of them; pack = the policy's BF16
// weight images (mlp_tc.cu), og [3, n] its outputs, sa the sampling (step_add = the first step).
int rollout_fused_cars_per_cta(int n, int sms);
cudaError_t launch_rollout_fused(const Segments& g, float* state, float* actions, float* reward, float* done,
                                 float* obs, int n, int beams, float4* ray, const float2* beam_dir, int steps,
                                 const uint8_t* pack, float* og, const SampleArgs& sa, int* err, int sms,
                                 cudaStream_t st);
// Cars whose smallest predicted range (ordered uint bits of a nonnegative float) is below threshold.
void launch_select_cars(const unsigned* minr, int n, float threshold, int* list, int* count, cudaStream_t st);
int lidar_max_iters(const TrackDev& t);
// FP64 re-integration audit of one physics step: prev/next state [11, n] around the FP32 step,
// stats [7] doubles (count, sums and maxima of position, heading and speed errors).
void launch_rk4_audit(const Segments& g, const float* prev, const float* actions, const float* next,
                      const float* done, int n, double* stats, cudaStream_t st);
// poses [count] (x, y, heading, layer) -> ray [2, count]: the frame of a car at rest there.
void launch_pose_frames(const TrackDev& t, const float4* poses, int count, float4* ray, cudaStream_t st);
void launch_sample(int n, uint64_t seed, const float* output, const float* log_std, float* actions, float* logp,
                   float* value, int deterministic, const int64_t* step_base, int64_t step_add, cudaStream_t st);
void launch_add_i64(int64_t* p, int64_t v, cudaStream_t st);
void beam_table(int beams, float2* out);

// ppo.cu (element-wise PPO kernels, bit-exact with the CPU restatement)
void launch_policy_init(int in, uint64_t seed, float* theta, cudaStream_t st);
void launch_gae(int n, int rollout, const float* reward, const float* done, const float* value,
                const float* last_value, float* advantage, cudaStream_t st);
void launch_gather(int in, int n, int batch, int m, const float* obs, float* x, cudaStream_t st);
// x [4][in, batch]: every minibatch's inputs from rollout storage obs [rollout + 1][in, n] in one pass.
void launch_gather_all(int in, int n, int rollout, int batch, const float* obs, float* x, cudaStream_t st,
                       void* xb = nullptr, int ldb = 0);  // xb: also the BF16 copy [4][in][ldb]
void launch_loss(int n, int batch, int m, const float* actions, const float* logp, const float* value,
                 const float* advantage, const float* o, const float* log_std, const float* adv_moments,
                 int use_moments, float adv_mean, float adv_scale, float* d3, cudaStream_t st);
void launch_adam(int p, int logstd, const float* c12, const float* stats, float* theta, const float* grad,
                 float* first, float* second, cudaStream_t st);
// row sums: out[r] = sum_j x[r * ld + j] for r < rows, j < cols (deterministic two-pass)
void launch_rowsum(const float* x, int rows, int cols, long ld, float* out, float* scratch, int squares,
                   cudaStream_t st);
void launch_moments(const float* adv, long count, float* stats, float* scratch, cudaStream_t st);

// mlp.cu (policy GEMMs)
void launch_sgemm(const float* A, int lda, const float* B, int ldb, float* C, int ldc, int M, int N, int K,
                  int squash, cudaStream_t st);
void launch_backward(int in, const float* theta, const float* x, int cols, const float* h1, const float* h2,
                     const float* d3, float* d2, float* d1, float* grad, float* scratch, cudaStream_t st);
// The FP32 weight-gradient GEMMs split K over the batch into at most SPLIT_CTAS / tiles ranges of
// their 64 x 64 tiles. The plan is the same on every device (two CTAs for each of a GB300's 152
// SMs), so the partial sums add in the same order everywhere and the scratch has a fixed bound.
constexpr int SPLIT_CTAS = 2 * 152;
constexpr size_t BACKWARD_SCRATCH_FLOATS = (size_t)SPLIT_CTAS * 64 * 64;
size_t backward_scratch_floats(int in, int cols);  // BACKWARD_SCRATCH_FLOATS
// Scratch floats launch_backward actually touches for these sizes (<= BACKWARD_SCRATCH_FLOATS).
size_t backward_scratch_needed(int in, int cols);

}  // namespace racer
