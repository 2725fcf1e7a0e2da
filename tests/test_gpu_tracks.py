"""GPU parity of the track compiler (racer_track_ribbon, racer_track_image).

The built-in tracks and the small occupancy map compiled on the GPU must equal
the reference's own arrays bit for bit; other routes (a figure eight at other
heights and widths, a banked wavy loop with ramp boxes, a loop long enough that
a block's candidate list overflows to the full scan) and the 2048 x 2048
occupancy map must equal the oracle bit for bit.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
import warporacer3d_gb300 as W
from warporacer3d_gb300.tracks import compile as C
from warporacer3d_gb300.tracks import occupancy

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
SMALL = dict(seed=3, size=160, cell=0.1, radius=4.5, amplitude=1.2, ramps=2, knots=12)


def assert_bits(ours, ref, what):
    assert ours.shape == ref.shape, f"{what}: shape {ours.shape} vs {ref.shape}"
    bad = np.nonzero(ours.view(np.uint32) != ref.view(np.uint32))[0]
    assert bad.size == 0, f"{what}: {bad.size} floats differ, first at {bad[:5].tolist()}: {ours[bad[0]]} vs {ref[bad[0]]}"


@pytest.mark.parametrize("name", ["flat", "ramp", "bank", "bridge"])
def test_builtin_tracks_equal_reference_arrays(name):
    ref = np.load(ROOT / "warporacer3d_gb300" / "tracks" / f"{name}.npz")["track"]
    assert_bits(C.load(name), ref, name)


def test_occupancy_image_equals_reference_array():
    free, loop, ramps, x0, y0 = occupancy.corridor(**SMALL)
    ref = np.load(ROOT / "tests" / "golden" / "occupancy_small.npz")["track"]
    assert_bits(C.compile_image(free, loop, x0, y0, SMALL["cell"], ramps), ref, "occupancy small")


def figure_eight(lift=1.2, half_width=0.9, cell=0.03):
    t = np.linspace(0, 2 * np.pi, 200, endpoint=False)
    z = lift * np.clip(np.cos((t - np.pi) * 1.4), 0, 1) ** 2
    return np.column_stack([8 * np.sin(t), 4 * np.sin(2 * t), z]), half_width, 0, cell


def wavy_loop():
    t = np.linspace(0, 2 * np.pi, 240, endpoint=False)
    r = 5 + 0.8 * np.sin(3 * t)
    route = np.column_stack([r * np.cos(t), r * np.sin(t), 0.3 * np.sin(2 * t) + 0.3])
    ramps = [{"center": [5.0, 0.3], "heading": 1.4, "length": 1.6, "width": 1.0, "height": 0.25},
             {"center": [-4.6, -1.0], "heading": -0.3, "length": 1.2, "width": 0.9, "height": 0.2, "rise": 0.5}]
    return route, 1.0, 0.15, 0.04, ramps


def big_loop():  # about 2100 waypoints: blocks near the centre see every one of them
    t = np.linspace(0, 2 * np.pi, 400, endpoint=False)
    return np.column_stack([50 * np.cos(t), 50 * np.sin(t), 0 * t]), 1.3, 0, 0.5


@pytest.mark.parametrize("case", ["eight_low", "eight_high_narrow", "wavy_ramps", "big_loop"])
def test_ribbons_equal_oracle(case):
    args = {"eight_low": figure_eight(lift=0.5, half_width=1.2, cell=0.035),
            "eight_high_narrow": figure_eight(lift=1.5, half_width=0.6, cell=0.025),
            "wavy_ramps": wavy_loop(),
            "big_loop": big_loop()}[case]
    ours, ref = C.ribbon(*args), oracle.track_ribbon(*args)
    assert_bits(ours, ref, case)
    if case.startswith("eight"):
        assert ours[7] == 2  # two layers where the route crosses above itself
    if case == "big_loop":
        assert ours[5] > 2048


def test_occupancy_2048_equals_oracle():
    free, loop, ramps, x0, y0 = occupancy.corridor(0)
    ours = C.compile_image(free, loop, x0, y0, 0.05, ramps)
    assert_bits(ours, oracle.track_image(free, loop, x0, y0, 0.05, ramps), "occupancy 2048")


def ring_image(nx, ny=12):
    """A two-cell-wide ring corridor around a long wall, with its centreline loop as (row, col)."""
    free = np.zeros((ny, nx), bool)
    free[2:10, 2:nx - 2] = True
    free[4:8, 6:nx - 6] = False
    cols = np.arange(4.0, nx - 4.0)
    loop = np.concatenate([np.column_stack([np.full(cols.size, 3.0), cols]),
                           np.column_stack([np.arange(3.0, 9.0), np.full(6, nx - 4.0)]),
                           np.column_stack([np.full(cols.size, 8.5), cols[::-1]]),
                           np.column_stack([np.arange(8.0, 3.0, -1.0), np.full(5, 4.0)])])
    return free, loop


@pytest.mark.parametrize("nx", [5000, 18000])
def test_wide_images_equal_oracle(nx):
    """Rows wider than 4096 cells take the row pass's large shared-memory path, wider than
    17066 its global-memory path."""
    free, loop = ring_image(nx)
    ramps = [{"center": [nx * 0.005, 0.03], "heading": 0.0, "length": 1.6, "width": 0.04, "height": 0.1}]
    ours = C.compile_image(free, loop, 0.0, 0.0, 0.01, ramps)
    assert_bits(ours, oracle.track_image(free, loop, 0.0, 0.0, 0.01, ramps), f"ring {nx}")


def test_image_without_walls_is_rejected():
    free, loop, ramps, x0, y0 = occupancy.corridor(**SMALL)
    with pytest.raises(W.RacerError, match="both free and occupied"):
        C.compile_image(np.ones_like(free), loop, x0, y0, SMALL["cell"], ramps)


def test_compiled_track_drives_like_the_fixture():
    """A sim on the GPU-compiled bridge steps exactly like one on the reference's array."""
    sims = [W.Sim(C.load("bridge"), 256, 5, beams=1081), W.Sim(W.track("bridge"), 256, 5, beams=1081)]
    rng = np.random.default_rng(0)
    for sim in sims:
        sim.reset()
    for _ in range(3):
        act = rng.uniform(-1, 1, (2, 256)).astype(np.float32)
        for sim in sims:
            sim.actions.write(act)
            sim.step(sim.actions, sim.reward, sim.done, sim.obs)
    a, b = sims
    assert np.array_equal(a.state.numpy(), b.state.numpy()) and np.array_equal(a.obs.numpy(), b.obs.numpy())
