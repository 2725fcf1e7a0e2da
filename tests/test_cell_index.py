"""The lidar's fast nearest-cell index is exactly the reference's.

racer/sim.mojo:110-111 computes ix = floor((x - x0) / cell + 0.5) with a
binary32 division. The CUDA probe multiplies by r = RN(1 / cell) instead and
falls back to the division only when u' = (x - x0) * r + 0.5 lies within
delta = (|u'| + 1) * 2^-20 of an integer. With |q' - q| <= 3 * 2^-24 |q| for
the two quotients and half an ulp per rounding of the + 0.5, the two values
of u differ by less than delta, so outside the guard band both floors agree.
This test replays both formulas in numpy binary32 (IEEE round-to-nearest,
like the GPU built with --fmad=false) on random coordinates and on
adversarial ones a few ulps either side of every cell boundary.
"""
import numpy as np
import pytest

f32 = np.float32
DELTA = f32(2.0 ** -20)


def exact(x, x0, cell):
    return np.floor((x - x0) / cell + f32(0.5))


def fast(x, x0, cell):
    r = f32(1) / cell
    u = (x - x0) * r + f32(0.5)
    fl = np.floor(u)
    g = u - fl
    d = (np.abs(u) + f32(1)) * DELTA
    ok = (g > d) & (g < f32(1) - d)
    return np.where(ok, fl, exact(x, x0, cell)), ok


@pytest.mark.parametrize("cell", [0.025, 0.05, 0.1, 0.03, 0.0123, 0.07])
def test_fast_cell_index_is_exact(cell):
    cell = f32(cell)
    rng = np.random.default_rng(int(cell * 1e4))
    for x0 in (f32(-8.9999361), f32(-7.9985256), f32(-1), f32(3.3), f32(-52.1)):
        ks = np.arange(-40, 2100)
        base = (x0 + (ks.astype(f32) + f32(0.5)) * cell).astype(f32)
        adv = [base]
        up, down = base.copy(), base.copy()
        for _ in range(12):
            up = np.nextafter(up, f32(np.inf))
            down = np.nextafter(down, f32(-np.inf))
            adv += [up, down]
        uniform = rng.uniform(-60, 120, 400000).astype(f32)
        xs = np.concatenate(adv + [uniform]).astype(f32)
        with np.errstate(all="ignore"):
            want = exact(xs, x0, cell)
            got, ok = fast(xs, x0, cell)
        assert np.array_equal(got, want)
        # the guard band is narrow: almost every uniformly placed lookup skips the division
        assert ok[-uniform.size:].mean() > 0.97
