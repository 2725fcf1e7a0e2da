"""The allocation-free policy backward, for callers that cannot allocate.

racer_policy_backward_noalloc exists for hosts whose device memory belongs to
another allocator (a Mojo/MAX DeviceContext, or a fixed up-front pool): it
takes every buffer from the caller and keeps its split-K scratch in a static
array inside the library. This test calls it through the C ABI twice in a
row and checks both results against racer_policy_backward on the same
inputs. It lives in its own file, collected last, and passes alone in a fresh
process as well as after the other GPU tests.
"""
import ctypes

import numpy as np
import pytest

import warporacer3d_gb300 as W
from warporacer3d_gb300._lib import call

pytestmark = pytest.mark.gpu

# |noalloc - reference| <= ATOL + RTOL * |reference|: both run the same kernels, so the
# results are expected to be identical; the tolerance only guards the comparison.
ATOL, RTOL = 1e-6, 1e-5


@pytest.mark.parametrize("beams,cols", [(108, 4096), (1081, 2048)])
def test_noalloc_backward_matches_backward_twice(beams, cols):
    rng = np.random.default_rng(beams + cols)
    policy = W.Policy(7, beams=beams)
    policy.set_precision("fp32")  # the allocation-free entry is the variant of the FP32 split-K backward
    IN = beams + 5
    x = rng.uniform(-1, 1, (IN, cols)).astype(np.float32)
    x[-1] = 1
    xd = W.DevArray.empty((IN, cols))
    xd.write(x)
    acts = W.Activations(policy, cols)
    policy.forward(xd, acts)
    d3 = W.DevArray.empty((3, cols))
    d3.write(rng.normal(0, 1e-3, (3, cols)).astype(np.float32))
    ref = [W.DevArray.empty((65, cols)), W.DevArray.empty((65, cols)), W.DevArray.empty((policy.P,))]
    policy.backward(xd, acts, d3, *ref)
    want = [a.numpy() for a in ref]
    for attempt in range(2):
        out = [W.DevArray.empty((65, cols)), W.DevArray.empty((65, cols)), W.DevArray.empty((policy.P,))]
        call("racer_policy_backward_noalloc", beams, policy.theta.c, xd.c, cols, acts.h1.c, acts.h2.c, d3.c,
             out[0].c, out[1].c, out[2].c, policy.stream)
        call("racer_synchronize", policy.stream)
        got = [a.numpy() for a in out]
        for name, g, w in zip(("d2", "d1", "grad"), got, want):
            if name == "grad":  # log std entries are the trainer's, not the backward's
                g, w = g[:-2], w[:-2]
            assert np.all(np.abs(g - w) <= ATOL + RTOL * np.abs(w)), (attempt, name, np.abs(g - w).max())
        assert np.abs(want[2][:-2]).max() > 0


def test_noalloc_rejects_bad_arguments():
    with pytest.raises(W.RacerError, match="bad argument"):
        call("racer_policy_backward_noalloc", 1, None, None, 4, None, None, None, None, None, None, None)
