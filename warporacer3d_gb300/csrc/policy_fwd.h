// The policy object behind the C ABI: parameters, derived weight copies and
// the forward/backward launchers (racer/ppo.mojo:63-138).
#pragma once
#include <cuda_runtime.h>

#include "../../include/racer.h"

int policy_new(int in_rows, void* stream, racer_policy** out);
void policy_delete(racer_policy* p);
float* policy_theta(racer_policy* p);
int policy_params(racer_policy* p);
int policy_inputs(racer_policy* p);
cudaStream_t policy_stream(racer_policy* p);
// Rebuild derived weight copies after theta changed (init, Adam, load).
int policy_refresh(racer_policy* p);
int policy_refresh_on(racer_policy* p, cudaStream_t st);
// x [IN, cols] -> h1, h2 [65, cols] (row 64 stays 1), o [3, cols].
int policy_forward(racer_policy* p, const float* x, int cols, float* h1, float* h2, float* o, cudaStream_t st);
int policy_backward(racer_policy* p, const float* x, int cols, const float* h1, const float* h2, const float* d3,
                    float* d2, float* d1, float* grad, cudaStream_t st);
