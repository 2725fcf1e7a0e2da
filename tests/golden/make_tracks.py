"""Regenerate the built-in track arrays (flat, ramp, bank, bridge) as .npz files.

The arrays are produced by the reference's own track compiler
(racer/track.py:37-44 `load`, :61-105 `ribbon`, :108-125 `pack`), imported
unchanged from a checkout of the reference. Its module-level imports of yaml,
PIL and scikit-image serve only the YAML/occupancy-image path
(racer/track.py:45-58), so they are replaced by empty stand-in modules here.

Usage: python tests/golden/make_tracks.py <reference checkout>

The arrays are written to warporacer3d_gb300/tracks/<name>.npz.
"""
import sys
import types
from pathlib import Path

import numpy as np


def main(reference):
    for name in ("yaml", "PIL", "PIL.Image", "skimage", "skimage.morphology"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["PIL"].Image = sys.modules["PIL.Image"]
    sys.modules["skimage.morphology"].skeletonize = None
    sys.path.insert(0, str(reference))
    import racer.track as track

    out = Path(__file__).resolve().parents[2] / "warporacer3d_gb300" / "tracks"
    for name in ("flat", "ramp", "bank", "bridge"):
        array = track.load(name)
        assert array.dtype == np.float32
        np.savez_compressed(out / f"{name}.npz", track=array)
        print(name, array.shape, array[:12].tolist())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_tracks.py <reference checkout>")
    main(sys.argv[1])
