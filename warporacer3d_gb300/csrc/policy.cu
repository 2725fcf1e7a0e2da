// Policy parameters and the forward/backward dispatch (racer/ppo.mojo:63-138).
//
// Two precisions: BF16 (default) runs the forward (mlp_tc.cu) and the
// backward and weight gradients (policy_tc.cu) on the tcgen05 tensor cores
// with FP32 accumulation; FP32 runs the same products on the CUDA cores
// (mlp.cu), for the same-seed comparison run of a BF16 training. Parameters
// and Adam are FP32 in both.
#include <string>

#include "common.cuh"
#include "kernels.h"
#include "policy_fwd.h"
#include "policy_tc.h"

using namespace racer;

struct racer_policy {
  int in = 0, p = 0;
  int bf16 = 1;              // precision of the products
  float* theta = nullptr;
  float* scratch = nullptr;  // split-K partials of the FP32 weight gradients
  uint8_t* pack = nullptr;   // pre-swizzled BF16 operand images of W0, W1, W2
  int* err = nullptr;        // device error word of the tensor-core kernels
  BackwardWork* work = nullptr;  // BF16 backward workspace for the last batch size
  int generation = 0;            // changes whenever precision or workspace change (captured graphs go stale)
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
  RACER_TRY(cudaMalloc((void**)&p->pack, mlp_pack_bytes(in_rows)));
  RACER_TRY(cudaMalloc((void**)&p->err, sizeof(int)));
  RACER_TRY(cudaMemset(p->err, 0, sizeof(int)));
  *out = p;
  return 0;
}

void policy_delete(racer_policy* p) {
  if (!p) return;
  cudaFree(p->theta);
  cudaFree(p->scratch);
  cudaFree(p->pack);
  cudaFree(p->err);
  backward_work_delete(p->work);
  if (p->owned) cudaStreamDestroy(p->st);
  delete p;
}

float* policy_theta(racer_policy* p) { return p->theta; }
int policy_params(racer_policy* p) { return p->p; }
int policy_inputs(racer_policy* p) { return p->in; }
cudaStream_t policy_stream(racer_policy* p) { return p->st; }
int policy_refresh(racer_policy* p) { return policy_refresh_on(p, p->st); }
int policy_refresh_on(racer_policy* p, cudaStream_t st) {
  launch_pack_weights(p->theta, p->in, p->pack, st);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    racer_host::set_error(std::string("policy weight pack: ") + cudaGetErrorString(err));
    return 2;
  }
  if (p->work) return backward_refresh(p->work, p->theta, st);
  return 0;
}

int policy_is_bf16(racer_policy* p) { return p->bf16; }
const uint8_t* policy_pack(racer_policy* p) { return p->pack; }
int* policy_err(racer_policy* p) { return p->err; }

int policy_set_precision(racer_policy* p, int bf16) {
  if (p->bf16 != (bf16 ? 1 : 0)) ++p->generation;
  p->bf16 = bf16 ? 1 : 0;
  return 0;
}

int policy_generation(racer_policy* p) { return p->generation; }

int policy_forward(racer_policy* p, const float* x, int cols, float* h1, float* h2, float* o, int write_hidden,
                   const SampleArgs* sa, cudaStream_t st, int c0, int c1) {
  cudaError_t err;
  if (c1 < 0) c1 = cols;
  if (p->bf16) {
    SampleArgs none;
    err = launch_mlp_fwd(x, p->in, cols, p->pack, h1, h2, o, write_hidden, sa ? *sa : none, p->err, st, c0, c1);
  } else {
    if (c0 != 0 || c1 != cols) {
      racer_host::set_error("policy forward: column ranges need the BF16 path");
      return 1;
    }
    const int in = p->in, w1 = H * in, w2 = w1 + H * HA;
    launch_sgemm(p->theta, in, x, cols, h1, cols, H, cols, in, 1, st);
    launch_sgemm(p->theta + w1, HA, h1, cols, h2, cols, H, cols, HA, 1, st);
    launch_sgemm(p->theta + w2, HA, h2, cols, o, cols, OUT, cols, HA, 0, st);
    if (sa && sa->actions)
      launch_sample(cols, sa->seed, o, sa->log_std, sa->actions, sa->logp, sa->value, sa->deterministic,
                    sa->step_base, sa->step_add, st);
    err = cudaGetLastError();
  }
  if (err != cudaSuccess) {
    racer_host::set_error(std::string("policy forward: ") + cudaGetErrorString(err));
    return 2;
  }
  return 0;
}

int policy_status(racer_policy* p, int* code) {
  RACER_TRY(cudaStreamSynchronize(p->st));
  RACER_TRY(cudaMemcpy(code, p->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (*code) RACER_TRY(cudaMemset(p->err, 0, sizeof(int)));  // read and clear
  return 0;
}

int policy_wait_probe(racer_policy* p, uint32_t polls) {
  cudaError_t err = launch_wait_probe(p->err, polls, p->st);
  if (err != cudaSuccess) {
    racer_host::set_error(std::string("timeout probe: ") + cudaGetErrorString(err));
    return 2;
  }
  return 0;
}

int policy_backward(racer_policy* p, const float* x, int cols, const float* h1, const float* h2, const float* d3,
                    float* d2, float* d1, float* grad, cudaStream_t st, const CUtensorMap* xb_map, bool dgrads_f32) {
  if (p->bf16) {
    if (backward_work_cols(p->work) != cols) {
      ++p->generation;
      backward_work_delete(p->work);
      p->work = nullptr;
      if (int rc = backward_work_new(p->in, cols, &p->work)) return rc;
      if (int rc = backward_refresh(p->work, p->theta, st)) return rc;
    }
    return backward_tc(p->work, p->theta, x, h1, h2, d3, d2, d1, grad, p->err, st, xb_map, dgrads_f32);
  }
  launch_backward(p->in, p->theta, x, cols, h1, h2, d3, d2, d1, grad, p->scratch, st);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    racer_host::set_error(std::string("policy backward: ") + cudaGetErrorString(err));
    return 2;
  }
  return 0;
}
