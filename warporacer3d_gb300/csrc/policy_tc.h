// BF16 tensor-core backward of the policy MLP (policy_tc.cu).
#pragma once
#include "tma.h"
#include <cuda_runtime.h>

namespace racer {

struct BackwardWork;  // BF16 operand copies, tensor maps and split-K scratch for one batch size

int backward_work_new(int in, int cols, BackwardWork** out);
void backward_work_delete(BackwardWork* w);
int backward_work_cols(const BackwardWork* w);
// Rebuild the BF16 W1^T image after theta changed.
int backward_refresh(BackwardWork* w, const float* theta, cudaStream_t st);
// x [IN, cols], h1/h2 [65, cols], d3 [3, cols] (FP32, feature-major) -> d2, d1 [65, cols] and the
// W0/W1/W2 entries of grad. xb_map, if given, is a tensor map (make_tmap_bf16(map, base, IN,
// ld, ld, 128) with ld = cols rounded up to 8) of x already in BF16 with zero padding: the
// conversion of x is then skipped. dgrads_f32 = false leaves d2 and d1 unwritten (their BF16 copies,
// which the weight gradients read, are written either way): for callers that only want grad.
int backward_tc(BackwardWork* w, const float* theta, const float* x, const float* h1, const float* h2,
                const float* d3, float* d2, float* d1, float* grad, int* err, cudaStream_t st,
                const CUtensorMap* xb_map = nullptr, bool dgrads_f32 = true);

}  // namespace racer
