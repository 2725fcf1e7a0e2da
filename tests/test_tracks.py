"""The occupancy-image track compiler against the reference's own output.

tests/golden/occupancy_small.npz was made by the reference's racer/track.py
(`load` on a YAML/image map, lines 45-58, and `pack`, lines 108-125) from the
seeded corridor below, with only the skeleton-loop extraction replaced by
the corridor's known centreline (tests/golden/make_occupancy_golden.py).
"""
from pathlib import Path

import numpy as np

import numpy_tracks
import oracle
from warporacer3d_gb300.tracks import occupancy

GOLDEN = Path(__file__).resolve().parent / "golden" / "occupancy_small.npz"
SMALL = dict(seed=3, size=160, cell=0.1, radius=4.5, amplitude=1.2, ramps=2, knots=12)


def test_compile_image_matches_reference_bit_for_bit():
    free, loop, ramps, x0, y0 = occupancy.corridor(**SMALL)
    ours = numpy_tracks.compile_image(free, loop, x0, y0, SMALL["cell"], ramps)
    golden = np.load(GOLDEN)["track"]
    assert ours.shape == golden.shape
    assert np.array_equal(ours, golden)


def test_synthetic_map_layout():
    """2048 x 2048 px at 0.05 m, one layer, slope bound 8 x 0.25 / 0.8 from the ramps, about 50.3 MB
    (the seeded corridor compiled by the oracle here; the GPU compiler's array equals the oracle's,
    tests/test_gpu_tracks.py)."""
    free, loop, ramps, x0, y0 = occupancy.corridor(0)
    t = oracle.track_image(free, loop, x0, y0, 0.05, ramps)
    nx, ny, x0, y0, cell, waypoints, spacing, layers, slope = t[:9]
    assert (nx, ny, layers) == (2048, 2048, 1) and abs(cell - 0.05) < 1e-7 and abs(slope - 2.5) < 1e-6
    assert abs(spacing - 0.15) < 0.01 and t.nbytes == 4 * (12 + 3 * 2048 * 2048 + 4 * int(waypoints))
    clearance = t[12:12 + 2048 * 2048].reshape(2048, 2048)
    assert 0.5 <= clearance.max() <= 1.05  # half-width 0.6-1.0 m
    assert 100_000 < (clearance > 0).sum() < 200_000
