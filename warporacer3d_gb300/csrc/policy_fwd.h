// The policy object behind the C ABI: parameters, derived weight copies and
// the forward/backward launchers (racer/ppo.mojo:63-138).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/racer.h"
#include "mlp_tc.h"

int policy_new(int in_rows, void* stream, racer_policy** out);
void policy_delete(racer_policy* p);
float* policy_theta(racer_policy* p);
int policy_params(racer_policy* p);
int policy_inputs(racer_policy* p);
cudaStream_t policy_stream(racer_policy* p);
// Rebuild derived weight copies after theta changed (init, Adam, load).
int policy_refresh(racer_policy* p);
int policy_refresh_on(racer_policy* p, cudaStream_t st);
// x [IN, cols] -> h1, h2 [65, cols] (row 64 stays 1; written only if
// write_hidden), o [3, cols]; with sa->actions set, also the sampled actions.
// Columns [c0, c1) only (c1 < 0: all; BF16 path only).
int policy_forward(racer_policy* p, const float* x, int cols, float* h1, float* h2, float* o, int write_hidden,
                   const racer::SampleArgs* sa, cudaStream_t st, int c0 = 0, int c1 = -1);
// 1 if the policy computes in BF16 on the tensor cores.
int policy_is_bf16(racer_policy* p);
// The BF16 weight images of the tensor-core forward and its error word (the fused rollout kernel).
const uint8_t* policy_pack(racer_policy* p);
int* policy_err(racer_policy* p);
// Device-side error word of the tensor-core kernels (0 = none), read and cleared; synchronises.
int policy_status(racer_policy* p, int* code);
// The timeout probe on the policy's stream, reporting into the policy's error word.
int policy_wait_probe(racer_policy* p, uint32_t polls);
// xb_map (BF16 path only): x already in BF16 behind a tensor map; dgrads_f32 = false (BF16 path
// only): d2 and d1 are not needed in FP32, see backward_tc.
int policy_backward(racer_policy* p, const float* x, int cols, const float* h1, const float* h2, const float* d3,
                    float* d2, float* d1, float* grad, cudaStream_t st, const CUtensorMap* xb_map = nullptr,
                    bool dgrads_f32 = true);
// 1: BF16 tensor-core products (default); 0: FP32 CUDA-core products.
int policy_set_precision(racer_policy* p, int bf16);
// A counter that changes whenever the precision or the backward workspace
// changes: a CUDA graph that captured the policy's launches is stale after.
int policy_generation(racer_policy* p);
