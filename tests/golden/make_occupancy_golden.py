"""Golden track array for the occupancy-image compiler.

Runs the reference's own track compiler (racer/track.py `load`, lines 45-58,
and `pack`, lines 108-125) on a small seeded corridor: the YAML metadata,
the image file and the centreline-loop extraction (skimage, absent here) are
supplied by stand-ins, so every other line of that path runs unchanged. The
output is occupancy_small.npz, which the tests compare with
the numpy restatement (tests/numpy_tracks.py), the oracle and the GPU
compiler on the same inputs.

Usage: python tests/golden/make_occupancy_golden.py <reference checkout>
"""
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

# The small corridor of the fixture (160 x 160 px at 0.1 m, two ramps).
SMALL = dict(seed=3, size=160, cell=0.1, radius=4.5, amplitude=1.2, ramps=2, knots=12)


def reference_compile(reference, free, loop, x0, y0, cell, ramps):
    for name in ("yaml", "PIL", "PIL.Image", "skimage", "skimage.morphology"):
        sys.modules.setdefault(name, types.ModuleType(name))
    meta = {"resolution": cell, "origin": [x0, y0, 0.0], "image": "map.pgm", "ramps": ramps}
    image = np.where(np.flipud(free), 255, 0).astype(np.uint8)  # image rows run from the north

    class Picture:
        def convert(self, mode):
            assert mode == "L"
            return image

    sys.modules["yaml"].safe_load = lambda text: meta
    sys.modules["PIL"].Image = sys.modules["PIL.Image"]
    sys.modules["PIL.Image"].open = lambda path: Picture()
    sys.modules["skimage.morphology"].skeletonize = None
    sys.path.insert(0, str(reference))
    import racer.track as track

    track.skeleton = lambda mask: mask
    track.longest_loop = lambda skel, origin: loop
    with tempfile.TemporaryDirectory() as tmp:
        path = Path(tmp) / "map.yaml"
        path.write_text("stand-in\n")
        return track.load(str(path))


def main(reference):
    from warporacer3d_gb300.tracks import occupancy

    free, loop, ramps, x0, y0 = occupancy.corridor(**SMALL)
    array = reference_compile(reference, free, loop, x0, y0, SMALL["cell"], ramps)
    assert array.dtype == np.float32
    np.savez_compressed(Path(__file__).resolve().parent / "occupancy_small.npz", track=array)
    print(array.shape, array[:12].tolist())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_occupancy_golden.py <reference checkout>")
    main(sys.argv[1])
