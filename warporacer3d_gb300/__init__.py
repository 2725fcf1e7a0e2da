"""warporacer3d rollout hot path on GB300 (sm_103a).

Simulator (RK4 slope bicycle, layered map probes, sphere-traced lidar), the
tanh-MLP policy and PPO's GAE/update kernels in libracer.so, behind a C ABI
(include/racer.h) that mirrors the reference's Sim / Policy / Trainer
structs. The Python classes here are a thin host over that ABI.
"""
from pathlib import Path

import numpy as np

from ._lib import RacerError, load_library  # noqa: F401
from .racer import (CRASH, STATE, TIMEOUT, Activations, DevArray, Policy, Runner, Sim, Surrogate, Trainer,  # noqa: F401
                    gather_peak, load, save)

TRACKS = Path(__file__).resolve().parent / "tracks"


def track(name):
    """A track array: the built-ins flat, ramp, bank and bridge as compiled by the
    reference's racer/track.py, or "occupancy", the seeded 2048 x 2048 px, 0.05 m
    corridor map with eight ramps (built on first use and cached)."""
    if name == "occupancy":
        from .tracks import occupancy
        return occupancy.synthetic(0)
    return np.load(TRACKS / f"{name}.npz")["track"]
