"""The reference's occupancy-image compiler restated in numpy and scipy (TEST
CHECKER ONLY).

`compile_image` follows racer/track.py:51-58 step for step and `pack` the
packer racer/track.py:108-125, with the centreline loop passed in (the
reference's skeleton-loop search, racer/track.py:150-202, needs skimage, which
is absent). tests/test_tracks.py pins it to the golden array the reference
itself produced (tests/golden/occupancy_small.npz); the product compiles
tracks on the GPU (warporacer3d_gb300/tracks/compile.py).
"""
import numpy as np
from scipy.ndimage import distance_transform_edt, gaussian_filter
from scipy.signal import savgol_filter
from scipy.spatial import KDTree

from warporacer3d_gb300.tracks.occupancy import arc, centres, headings, resample


def pack(clearance, height, waypoint, route, x0, y0, cell, slope, ramps):
    """Ramps onto the heights, off-road height fill and blur, then the flat
    float32 array (racer/track.py:108-125). `slope` grows by height / rise
    per ramp: it bounds the terrain gradient for the lidar march."""
    ny, nx = clearance.shape[1:]
    xy = centres((ny, nx), x0, y0, cell)
    for ramp in ramps:
        c, s = np.cos(ramp["heading"]), np.sin(ramp["heading"])
        rx, ry = xy[:, 0] - ramp["center"][0], xy[:, 1] - ramp["center"][1]
        u = rx * c + ry * s + ramp["length"] / 2
        v = -rx * s + ry * c
        rise = ramp.get("rise", ramp["length"] / 2)
        top = ramp["height"] * np.clip(np.minimum(u, ramp["length"] - u) / rise, 0, 1)
        height += np.where(abs(v) < ramp["width"] / 2, top, 0).reshape(ny, nx)
        slope += ramp["height"] / rise
    for layer in range(len(clearance)):
        iy, ix = distance_transform_edt(clearance[layer] <= 0, return_indices=True)[1]
        height[layer] = gaussian_filter(height[layer, iy, ix], 1.5)
    header = [nx, ny, x0, y0, cell, len(route), arc(route)[-1] / len(route), len(clearance), slope, 0, 0, 0]
    grids = np.stack([clearance, height, waypoint], 1).ravel()
    tail = np.column_stack([route, headings(route)]).ravel()
    return np.concatenate([header, grids, tail]).astype(np.float32)


def compile_image(free, loop, x0, y0, cell, ramps=()):
    """Free-space image (rows south to north) + centreline loop (row, col) ->
    packed one-layer track (racer/track.py:54-58)."""
    xy = savgol_filter(loop[:, ::-1] * cell + (x0, y0), 51, 3, axis=0, mode="wrap")
    route = resample(np.column_stack([xy, 0 * xy[:, 0]]))
    waypoint = KDTree(route[:, :2]).query(centres(free.shape, x0, y0, cell))[1].reshape(free.shape)
    clearance = (distance_transform_edt(free) - distance_transform_edt(~free) - 0.5) * cell
    return pack(clearance[None], np.zeros(free.shape)[None], waypoint[None], route, x0, y0, cell, 0, list(ramps))
