// Policy parameters and the forward/backward dispatch (racer/ppo.mojo:63-138).
#include <string>

#include "common.cuh"
#include "kernels.h"
#include "policy_fwd.h"

using namespace racer;

struct racer_policy {
  int in = 0, p = 0;
  float* theta = nullptr;
  float* scratch = nullptr;  // split-K partials of the weight gradients
  cudaStream_t st = nullptr;
  bool owned = false;
};

int policy_new(int in_rows, void* stream, racer_policy** out) {
  racer_policy* p = new racer_policy();
  p->in = in_rows;
  p->p = H * in_rows + H * HA + OUT * HA + 2;
  if (stream) {
    p->st = (cudaStream_t)stream;
  } else {
    RACER_TRY(cudaStreamCreate(&p->st));
    p->owned = true;
  }
  RACER_TRY(cudaMalloc((void**)&p->theta, (size_t)p->p * sizeof(float)));
  RACER_TRY(cudaMemset(p->theta, 0, (size_t)p->p * sizeof(float)));
  RACER_TRY(cudaMalloc((void**)&p->scratch, backward_scratch_floats(in_rows, 0) * sizeof(float)));
  *out = p;
  return 0;
}

void policy_delete(racer_policy* p) {
  if (!p) return;
  cudaFree(p->theta);
  cudaFree(p->scratch);
  if (p->owned) cudaStreamDestroy(p->st);
  delete p;
}

float* policy_theta(racer_policy* p) { return p->theta; }
int policy_params(racer_policy* p) { return p->p; }
int policy_inputs(racer_policy* p) { return p->in; }
cudaStream_t policy_stream(racer_policy* p) { return p->st; }
int policy_refresh(racer_policy* p) { return policy_refresh_on(p, p->st); }
int policy_refresh_on(racer_policy* p, cudaStream_t st) {
  (void)p;
  (void)st;
  return 0;
}

int policy_forward(racer_policy* p, const float* x, int cols, float* h1, float* h2, float* o, cudaStream_t st) {
  const int in = p->in, w1 = H * in, w2 = w1 + H * HA;
  launch_sgemm(p->theta, in, x, cols, h1, cols, H, cols, in, 1, st);
  launch_sgemm(p->theta + w1, HA, h1, cols, h2, cols, H, cols, HA, 1, st);
  launch_sgemm(p->theta + w2, HA, h2, cols, o, cols, OUT, cols, HA, 0, st);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    racer_host::set_error(std::string("policy forward: ") + cudaGetErrorString(err));
    return 2;
  }
  return 0;
}

int policy_backward(racer_policy* p, const float* x, int cols, const float* h1, const float* h2, const float* d3,
                    float* d2, float* d1, float* grad, cudaStream_t st) {
  launch_backward(p->in, p->theta, x, cols, h1, h2, d3, d2, d1, grad, p->scratch, st);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    racer_host::set_error(std::string("policy backward: ") + cudaGetErrorString(err));
    return 2;
  }
  return 0;
}
