"""The track compiler's oracle against the reference's own arrays (CPU).

warporacer3d_gb300/tracks/{flat,ramp,bank,bridge}.npz are the reference's
racer/track.py output (tests/golden/make_tracks.py), and
tests/golden/occupancy_small.npz its occupancy-image output
(tests/golden/make_occupancy_golden.py). The oracle (oracle/track.cpp plus the
host part in warporacer3d_gb300/tracks/compile.py) must reproduce them bit for
bit; the GPU compiler is then checked against the oracle and the same arrays
in tests/test_gpu_tracks.py.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest
from scipy.ndimage import distance_transform_edt, gaussian_filter

import oracle
from warporacer3d_gb300.tracks import compile as C
from warporacer3d_gb300.tracks import occupancy

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden" / "occupancy_small.npz"
SMALL = dict(seed=3, size=160, cell=0.1, radius=4.5, amplitude=1.2, ramps=2, knots=12)


def bits(a):
    return a.view(np.uint32)


@pytest.mark.parametrize("name", ["flat", "ramp", "bank", "bridge"])
def test_oracle_ribbon_equals_reference_array(name):
    ours = oracle.track_ribbon(*C.builtin_route(name))
    ref = np.load(ROOT / "warporacer3d_gb300" / "tracks" / f"{name}.npz")["track"]
    assert ours.shape == ref.shape
    assert np.array_equal(bits(ours), bits(ref))


def test_oracle_image_equals_reference_array():
    free, loop, ramps, x0, y0 = occupancy.corridor(**SMALL)
    ours = oracle.track_image(free, loop, x0, y0, SMALL["cell"], ramps)
    ref = np.load(GOLDEN)["track"]
    assert ours.shape == ref.shape
    assert np.array_equal(bits(ours), bits(ref))


def test_feature_transform_and_blur_follow_scipy():
    """The restated feature transform and blur, reached through a one-layer image with
    random walls: the height fill equals scipy's on rough random ramps."""
    rng = np.random.default_rng(7)
    free = rng.random((37, 53)) > 0.35
    free[0, :] = False
    loop = np.column_stack([np.full(60, 18.0) + 6 * np.sin(np.linspace(0, 2 * np.pi, 60, endpoint=False)),
                            np.full(60, 26.0) + 8 * np.cos(np.linspace(0, 2 * np.pi, 60, endpoint=False))])
    ramps = [{"center": [2.0, 1.5], "heading": 0.4, "length": 1.6, "width": 1.0, "height": 0.25},
             {"center": [3.0, 2.5], "heading": -1.1, "length": 1.2, "width": 0.8, "height": 0.3, "rise": 0.4}]
    ours = oracle.track_image(free, loop, 0.0, 0.0, 0.1, ramps)
    ny, nx = free.shape
    cells = nx * ny
    # scipy's own fill and blur of the same ramp heights
    inp = C.ImageInput(free, loop, 0.0, 0.0, 0.1, ramps)
    xy = occupancy.centres((ny, nx), 0.0, 0.0, 0.1)
    height = np.zeros((1, ny, nx))
    for ramp in ramps:
        c, s = np.cos(ramp["heading"]), np.sin(ramp["heading"])
        u = (xy[:, 0] - ramp["center"][0]) * c + (xy[:, 1] - ramp["center"][1]) * s + ramp["length"] / 2
        v = -(xy[:, 0] - ramp["center"][0]) * s + (xy[:, 1] - ramp["center"][1]) * c
        rise = ramp.get("rise", ramp["length"] / 2)
        top = ramp["height"] * np.clip(np.minimum(u, ramp["length"] - u) / rise, 0, 1)
        height += np.where(abs(v) < ramp["width"] / 2, top, 0).reshape(ny, nx)
    clearance = (distance_transform_edt(free) - distance_transform_edt(~free) - 0.5) * 0.1
    iy, ix = distance_transform_edt(clearance <= 0, return_indices=True)[1]
    want = gaussian_filter(height[0, iy, ix], 1.5).astype(np.float32)
    assert np.array_equal(bits(ours[12 + cells:12 + 2 * cells]), bits(want.ravel()))
    assert np.array_equal(bits(ours[12:12 + cells]), bits(clearance.astype(np.float32).ravel()))
    assert inp.slope == 0.25 / 0.8 + 0.3 / 0.4


def test_track_arguments_checked_on_host():
    from warporacer3d_gb300 import build
    import warporacer3d_gb300 as W
    build.build()
    lib = W.load_library()
    inp = C.RibbonInput(*C.builtin_route("flat"))
    inp.route = inp.route[:1].copy()  # one waypoint
    rc, _, _ = C.ribbon_grids(inp, lib.racer_track_ribbon)
    assert rc == 1 and b"invalid" in lib.racer_last_error()
    inp = C.RibbonInput(*C.builtin_route("flat"))
    grids = np.empty(10, np.float32)
    layers = ctypes.c_int()
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = lib.racer_track_ribbon(dp(inp.route), dp(inp.cos_h), dp(inp.sin_h), dp(inp.grade), len(inp.route), 1.3, 0.0,
                                inp.x0, inp.y0, 0.025, inp.nx, inp.ny, None, 0,
                                grids.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), grids.size, ctypes.byref(layers))
    assert rc == 1 and b"6 * nx * ny" in lib.racer_last_error()
