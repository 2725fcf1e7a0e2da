"""The generic tcgen05 GEMM (TMA-fed, BF16 in, FP32 accumulate) against numpy.

Inputs are drawn as BF16 values, so the float64 product of the same values is
the exact reference; the only differences are FP32 accumulation order, bounded
here by 1e-4 relative to the sum of |a_k b_k| per output.
"""
import ctypes

import numpy as np
import pytest

import warporacer3d_gb300 as W
from warporacer3d_gb300._lib import call

pytestmark = pytest.mark.gpu


def to_bf16(x):
    """Round-to-nearest-even float32 -> bfloat16 bit patterns (uint16) and their float values."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r, (r.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("M,N,K,splits", [(128, 64, 64, 1), (300, 200, 520, 1), (1000, 512, 512, 1),
                                          (256, 1081, 512, 1), (130, 64, 4096, 8), (8192, 16, 16, 1),
                                          (8192, 1081, 512, 1), (4096, 512, 1024, 3), (20000, 64, 128, 1)])
def test_gemm_bf16(M, N, K, splits):
    rng = np.random.default_rng(M + N + K)
    lda = ldb = (K + 7) // 8 * 8
    a = np.zeros((M, lda), np.float32)
    b = np.zeros((N, ldb), np.float32)
    a[:, :K] = rng.normal(0, 1, (M, K))
    b[:, :K] = rng.normal(0, 1, (N, K))
    abits, af = to_bf16(a)
    bbits, bf = to_bf16(b)
    A = W.DevArray.empty((M, lda), np.uint16)
    B = W.DevArray.empty((N, ldb), np.uint16)
    A.write(abits)
    B.write(bbits)
    C = W.DevArray.empty((M, N))
    scratch = W.DevArray.empty((splits * M * N,)) if splits > 1 else None
    err = W.DevArray.empty((1,), np.int32)
    call("racer_gemm_bf16", A.c, B.c, C.c, M, N, K, lda, ldb, N, splits, scratch.c if scratch else None, err.c,
         None)
    call("racer_synchronize", None)
    got = C.numpy()
    want = af[:, :K].astype(np.float64) @ bf[:, :K].astype(np.float64).T
    scale = np.abs(af[:, :K]).astype(np.float64) @ np.abs(bf[:, :K]).astype(np.float64).T
    assert np.all(np.abs(got - want) <= 1e-4 * scale + 1e-6), np.abs(got - want).max()
    assert int(err.numpy()[0]) == 0
