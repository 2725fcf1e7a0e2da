// Element-wise PPO kernels: policy initialisation, GAE, minibatch gather,
// clipped-loss derivatives, Adam, and deterministic row reductions.
//
// Reference behaviour: racer/ppo.mojo:74-89 (init), :218-230 (GAE),
// :242-250 (advantage moments), :276-304 (gather, loss), :306-315 (norm),
// :317-337 (Adam). Built like sim.cu with --fmad=false and rmath.h, so init,
// GAE and the loss derivatives repeat the CPU restatement's binary32
// operations; sums use a fixed two-pass tree in double.
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"
#include "philox.h"
#include "rmath.h"

namespace racer {
namespace {

__global__ void k_policy_init(int in, uint64_t seed, float* theta) {
  const int obs = in - 1;
  const int w1 = H * in, w2 = w1 + H * HA, logstd = w2 + OUT * HA, p = logstd + 2;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p) return;
  float scale = 0.0f;
  if (i < w1) {
    scale = (i % in < obs) ? sqrtf(2.0f / (float)obs) : 0.0f;
  } else if (i < w2) {
    scale = (i % HA < H) ? sqrtf(1.0f / (float)H) : 0.0f;
  } else if (i < logstd) {
    scale = (i % HA < H) ? ((i - w2) / HA < 2 ? 0.00125f : 0.125f) : 0.0f;
  } else {
    theta[i] = -0.5f;
    return;
  }
  float z[4];
  philox::normal4(seed, (uint64_t)i, 0, z);
  theta[i] = scale * z[0];
}

__global__ void k_gae(int n, int rollout, const float* reward, const float* done, const float* value,
                      const float* last_value, float* advantage) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
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

__global__ void k_gather(int in, int n, int batch, int m, const float* __restrict__ obs, float* __restrict__ x) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  int r = blockIdx.y;
  if (b >= batch) return;
  long s = (long)b * MINIBATCHES + m;
  x[(long)r * batch + b] = obs[((s / n) * in + r) * n + s % n];
}

__global__ void k_loss(int n, int batch, int m, const float* actions, const float* logp, const float* value,
                       const float* advantage, const float* o, const float* log_std, const float* moments,
                       int use_moments, float adv_mean, float adv_scale, float* d3) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  if (use_moments) {  // racer/ppo.mojo:249-250 from the device-side sums
    float samples = (float)((long)batch * MINIBATCHES);
    adv_mean = moments[0] / samples;
    float var = moments[1] / samples - adv_mean * adv_mean;
    adv_scale = 1.0f / sqrtf(fmaxf(var, 1e-8f));
  }
  long s = (long)b * MINIBATCHES + m;
  long t = s / n, i = s % n;
  float new_logp = 0.0f, error[2], invvar[2];
  for (int a = 0; a < 2; ++a) {
    float ls = log_std[a];
    error[a] = actions[(t * 2 + a) * n + i] - o[(long)a * batch + b];
    invvar[a] = rmath::expf_(-2.0f * ls);
    new_logp -= (((0.5f * error[a]) * error[a]) * invvar[a] + ls) + HALF_LOG_2PI;
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
  float e = (o[2L * batch + b] - value[s]) - advantage[s];
  d3[2L * batch + b] = (0.5f * fminf(fmaxf(e, -1.0f), 1.0f)) / (float)batch;
  d3[(long)(OUT + 2) * batch + b] = (ratio - 1.0f) - logratio;
}

// c12 = (1 - 0.9^t, 1 - 0.999^t) for this step t, read from device memory so a
// captured update replays with each step's values.
__global__ void k_adam(int p, int logstd, const float* c12, const float* stats, float* theta, const float* grad,
                       float* first, float* second) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p) return;
  const float c1 = c12[0], c2 = c12[1];
  float scale = fminf(1.0f, MAX_NORM / (sqrtf(stats[ST_NORM]) + 1e-8f));
  float g = grad[i] * scale;
  float m = 0.9f * first[i] + 0.1f * g;
  float v = 0.999f * second[i] + (0.001f * g) * g;
  first[i] = m;
  second[i] = v;
  float m_hat = m / c1, v_hat = v / c2;
  float value = theta[i] - (LR * m_hat) / (sqrtf(v_hat) + 1e-5f);
  theta[i] = i >= logstd ? fminf(fmaxf(value, -2.0f), 0.0f) : value;
}

// Pass 1: block (c, r) sums its chunk of row r in double.
constexpr int RS_THREADS = 256;
__global__ void k_rowsum_partial(const float* x, int cols, long ld, int chunks, int squares, double* part) {
  int r = blockIdx.y, c = blockIdx.x;
  long per = ((long)cols + chunks - 1) / chunks;
  long j0 = c * per, j1 = min((long)cols, j0 + per);
  const float* row = x + (long)r * ld;
  double acc = 0.0;
  for (long j = j0 + threadIdx.x; j < j1; j += RS_THREADS) {
    double v = row[j];
    acc += squares ? v * v : v;
  }
  __shared__ double sh[RS_THREADS];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = RS_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long)r * chunks + c] = sh[0];
}

// Pass 2: one block per row adds the partials in a fixed order.
__global__ void k_rowsum_final(const double* part, int chunks, float* out) {
  int r = blockIdx.x;
  __shared__ double sh[RS_THREADS];
  double acc = 0.0;
  for (int c = threadIdx.x; c < chunks; c += RS_THREADS) acc += part[(long)r * chunks + c];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = RS_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[r] = (float)sh[0];
}

int rowsum_chunks(long cols) { return (int)std::min<long>(256, (cols + 4095) / 4096); }

}  // namespace

void launch_policy_init(int in, uint64_t seed, float* theta, cudaStream_t st) {
  int p = H * in + H * HA + OUT * HA + 2;
  k_policy_init<<<(p + 255) / 256, 256, 0, st>>>(in, seed, theta);
}

void launch_gae(int n, int rollout, const float* reward, const float* done, const float* value,
                const float* last_value, float* advantage, cudaStream_t st) {
  k_gae<<<(n + 127) / 128, 128, 0, st>>>(n, rollout, reward, done, value, last_value, advantage);
}

void launch_gather(int in, int n, int batch, int m, const float* obs, float* x, cudaStream_t st) {
  dim3 grid((batch + 255) / 256, in);
  k_gather<<<grid, 256, 0, st>>>(in, n, batch, m, obs, x);
}

// All four minibatches at once (racer/ppo.mojo:259-268's sample order
// s = b * 4 + m): obs[t][r][i] -> x[m][r][b] with s = t * n + i, m = s % 4,
// b = s / 4, so every rollout row is read once, coalesced.
__global__ void k_gather_all(int in, int n, int batch, const float* __restrict__ obs, float* __restrict__ x,
                             __nv_bfloat16* __restrict__ xb, int ldb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = blockIdx.y, t = blockIdx.z;
  const long s = (long)t * n + i;
  const long row = (s & (MINIBATCHES - 1)) * in + r;
  const float v = obs[((long)t * in + r) * n + i];
  x[row * batch + (s >> 2)] = v;
  if (xb) xb[row * ldb + (s >> 2)] = __float2bfloat16_rn(v);  // the weight-gradient operand of layer 0
}

void launch_gather_all(int in, int n, int rollout, int batch, const float* obs, float* x, cudaStream_t st, void* xb,
                       int ldb) {
  static_assert(MINIBATCHES == 4, "the sample split assumes four minibatches");
  dim3 grid((n + 255) / 256, in, rollout);
  k_gather_all<<<grid, 256, 0, st>>>(in, n, batch, obs, x, static_cast<__nv_bfloat16*>(xb), ldb);
}

void launch_loss(int n, int batch, int m, const float* actions, const float* logp, const float* value,
                 const float* advantage, const float* o, const float* log_std, const float* adv_moments,
                 int use_moments, float adv_mean, float adv_scale, float* d3, cudaStream_t st) {
  k_loss<<<(batch + 127) / 128, 128, 0, st>>>(n, batch, m, actions, logp, value, advantage, o, log_std, adv_moments,
                                              use_moments, adv_mean, adv_scale, d3);
}

void launch_adam(int p, int logstd, const float* c12, const float* stats, float* theta, const float* grad,
                 float* first, float* second, cudaStream_t st) {
  k_adam<<<(p + 255) / 256, 256, 0, st>>>(p, logstd, c12, stats, theta, grad, first, second);
}

// scratch must hold rows * 256 doubles (2 * rows * 256 floats).
void launch_rowsum(const float* x, int rows, int cols, long ld, float* out, float* scratch, int squares,
                   cudaStream_t st) {
  int chunks = rowsum_chunks(cols);
  double* part = reinterpret_cast<double*>(scratch);
  k_rowsum_partial<<<dim3(chunks, rows), RS_THREADS, 0, st>>>(x, cols, ld, chunks, squares, part);
  k_rowsum_final<<<rows, RS_THREADS, 0, st>>>(part, chunks, out);
}

// stats[ST_ADV] = sum(adv), stats[ST_ADV2] = sum(adv^2)
void launch_moments(const float* adv, long count, float* stats, float* scratch, cudaStream_t st) {
  launch_rowsum(adv, 1, (int)count, count, stats + ST_ADV, scratch, 0, st);
  launch_rowsum(adv, 1, (int)count, count, stats + ST_ADV2, scratch + 512, 1, st);
}

}  // namespace racer
