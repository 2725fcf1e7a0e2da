"""CPU checks of the C-ABI library: it builds, loads without a GPU, exports
every entry point include/racer.h declares, and rejects malformed inputs on
the host before touching the device (the reference raises on a short track
array, racer/sim.mojo:97-98, and on a wrong checkpoint size,
racer/ppo.mojo:351-352)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import warporacer3d_gb300 as W
from warporacer3d_gb300 import build

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    build.build()
    return W.load_library()


def declared():
    text = (ROOT / "include" / "racer.h").read_text()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(racer_\w+)\(", text, re.M)))


def test_exports_every_declared_symbol(lib):
    names = declared()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name
        assert ctypes.cast(getattr(lib, name), ctypes.c_void_p).value


def test_bindings_cover_header():
    from warporacer3d_gb300._lib import SIGNATURES
    missing = [n for n in declared() if n not in SIGNATURES and n not in ("racer_last_error", "racer_version")]
    assert not missing, missing


def test_track_validation_on_host(lib):
    track = W.track("flat")
    with pytest.raises(W.RacerError, match="length does not match"):
        W.Sim(track[:-1], 4, 0)
    with pytest.raises(W.RacerError, match="not a track array"):
        W.Sim(track[:5], 4, 0)
    bad = track.copy()
    bad[4] = np.nan
    with pytest.raises(W.RacerError, match="non-finite"):
        W.Sim(bad, 4, 0)
    bad = track.copy()
    bad[12 + 2 * 641 * 641 + 5] = 9999  # a nearest-waypoint entry past the route
    with pytest.raises(W.RacerError, match="nearest-waypoint"):
        W.Sim(bad, 4, 0)
    with pytest.raises(W.RacerError, match="beams"):
        W.Sim(track, 4, 0, beams=1)
    for value in (np.nan, np.inf, 2e6):
        bad = track.copy()
        bad[12 + 641 * 641 + 7] = value  # a height
        with pytest.raises(W.RacerError, match="heights"):
            W.Sim(bad, 4, 0)


def test_errors_are_reported_without_gpu(lib):
    p = ctypes.c_void_p()
    rc = lib.racer_alloc(16, ctypes.byref(p))
    if rc == 0:  # a GPU is present: nothing to check here
        lib.racer_free(p)
        pytest.skip("GPU present")
    assert rc == 2 and lib.racer_last_error()


def test_segment_arguments_checked_on_host(lib):
    track = W.track("flat")
    with pytest.raises(W.RacerError, match="1 to 8 segments"):
        W.Sim.segments([track] * 9, [1] * 9, list(range(9)))
    with pytest.raises(W.RacerError, match="1 to 8 segments"):
        W.Sim.segments([], [], [])
    with pytest.raises(W.RacerError, match="at least one car"):
        W.Sim.segments([track, track], [4, 0], [1, 2])
    with pytest.raises(ValueError):
        W.Sim.segments([track, track], [4], [1, 2])


def test_gather_peak_arguments_checked_on_host(lib):
    gbs = ctypes.c_float()
    for size in (1000, 2048, 3 << 20, 1 << 29):
        assert lib.racer_gather_peak(size, 3, ctypes.byref(gbs)) == 1
        assert b"power of two" in lib.racer_last_error()
    assert lib.racer_gather_peak(1 << 20, 0, ctypes.byref(gbs)) == 1


def test_surrogate_arguments_checked_on_host(lib):
    """The learned lidar's constructor rejects a null sim, a bad width or batch and an unknown
    output frame before touching the device; the Python mirror rejects unknown frame names."""
    out = ctypes.c_void_p()
    assert lib.racer_surrogate_create_frame(None, 512, 8192, 1, 1, ctypes.byref(out)) == 1
    assert b"hidden must be" in lib.racer_last_error()
    assert lib.racer_surrogate_create(None, 512, 8192, 1, ctypes.byref(out)) == 1
    assert lib.racer_surrogate_grid(None, None, None, None, None) == 1
    assert b"feature grids" in lib.racer_last_error()
    assert lib.racer_surrogate_batch_inputs(None, None, None) == 1
    with pytest.raises(ValueError, match="frame"):
        W.Surrogate(None, frame="polar")
