"""Occupancy-map tracks: a seeded synthetic corridor, and the per-waypoint
helpers the track compiler's host part shares with the reference.

The packed format is the reference's (racer/track.py:14-19): header[12] =
nx, ny, x0, y0, cell, waypoints, spacing, layers, slope bound, 0, 0, 0; then
per layer clearance, height and nearest-waypoint grids of ny*nx; then the
route as (x, y, z, heading) per waypoint.

`centres`, `arc`, `resample` and `headings` are the reference's numpy
expressions (racer/track.py:128-147), kept as they are so the compiled arrays
are the reference's bit for bit (tracks/compile.py). The reference extracts
an occupancy image's centreline loop with skimage's skeletonize plus a loop
search (racer/track.py:150-202), which is not available here; the synthetic
corridor knows its centreline analytically, so that loop is passed to the
compiler directly (as (row, col) pixel coordinates, like the skeleton's).

`synthetic` builds the 2048 x 2048 px, 0.05 m map of the batched-launch
workload on the GPU (tracks/compile.py, racer_track_image): a closed
corridor whose centreline radius is a seeded, smoothed, random function of the
polar angle, half-width 0.6-1.0 m, and eight seeded 1.6 x 1.0 x 0.25 m ramp
boxes on the floor.
"""
from pathlib import Path

import numpy as np
from scipy.ndimage import gaussian_filter1d
from scipy.spatial import KDTree

SPACING = 0.15  # metres between waypoints (racer/track.py:32)


def centres(shape, x0, y0, cell):
    """Cell centres (x, y), row-major over (ny, nx) (racer/track.py:128-130)."""
    gx, gy = np.meshgrid(x0 + cell * np.arange(shape[1]), y0 + cell * np.arange(shape[0]))
    return np.column_stack([gx.ravel(), gy.ravel()])


def arc(route):
    """Cumulative length to every point and back to the first (racer/track.py:133-135)."""
    seg = np.linalg.norm(np.roll(route, -1, 0) - route, axis=1)
    return np.concatenate([[0], np.cumsum(seg)])


def resample(route):
    """Evenly spaced points along the closed polyline (racer/track.py:138-142)."""
    s = arc(route)
    even = np.linspace(0, s[-1], max(2, round(s[-1] / SPACING)), endpoint=False)
    closed = np.vstack([route, route[:1]])
    return np.column_stack([np.interp(even, s, closed[:, k]) for k in range(3)])


def headings(route):
    """Direction to the next waypoint (racer/track.py:145-147)."""
    d = np.roll(route, -1, 0) - route
    return np.arctan2(d[:, 1], d[:, 0])


def _smooth_periodic(rng, count, sigma, knots):
    """A smooth periodic random function on `count` angles, scaled to max |f| = 1."""
    g = gaussian_filter1d(rng.standard_normal(knots), sigma, mode="wrap")
    spectrum = np.fft.rfft(g)
    f = np.fft.irfft(spectrum, count) * (count / knots)  # band-limited periodic interpolation
    return f / np.abs(f).max()


def corridor(seed=0, size=2048, cell=0.05, radius=30.0, amplitude=10.0, half_width=(0.6, 1.0), ramps=8, knots=48):
    """A seeded closed corridor centred in a size x size image of `cell` metres.

    Returns (free [size, size] bool, rows south to north; loop [m, 2] (row, col)
    of the centreline at about one point per pixel; ramps; x0; y0)."""
    rng = np.random.default_rng(seed)
    x0 = y0 = -size * cell / 2
    dense = int(np.ceil(2 * np.pi * (radius + amplitude) / (cell / 8)))
    theta = np.linspace(0, 2 * np.pi, dense, endpoint=False)
    r = radius + amplitude * _smooth_periodic(rng, dense, 2.0, knots)
    hw = half_width[0] + (half_width[1] - half_width[0]) * 0.5 * (1 + _smooth_periodic(rng, dense, 2.0, knots))
    line = np.column_stack([r * np.cos(theta), r * np.sin(theta)])
    # radius of curvature must stay well above the half-width (no pinched or overlapping walls)
    d1 = (np.roll(line, -1, 0) - np.roll(line, 1, 0)) / 2
    d2 = np.roll(line, -1, 0) - 2 * line + np.roll(line, 1, 0)
    curvature = np.abs(d1[:, 0] * d2[:, 1] - d1[:, 1] * d2[:, 0]) / np.linalg.norm(d1, axis=1) ** 3
    assert 1 / curvature.max() > 3 * half_width[1], "corridor too tightly curved"
    assert r.max() + half_width[1] + 1 < size * cell / 2, "corridor leaves the image"
    dist, nearest = KDTree(line).query(centres((size, size), x0, y0, cell), distance_upper_bound=half_width[1] + cell)
    free = (dist < hw[np.minimum(nearest, dense - 1)]).reshape(size, size)
    step = max(1, int(round(cell / (2 * np.pi * radius / dense))))  # about one loop point per pixel
    loop = np.column_stack([(line[::step, 1] - y0) / cell, (line[::step, 0] - x0) / cell])
    boxes = []
    if ramps:
        at = (np.arange(ramps) + rng.uniform(0.2, 0.8, ramps)) * (dense // ramps)
        for k in at.astype(int) % dense:
            tangent = line[(k + 1) % dense] - line[k - 1]
            boxes.append({"center": [float(line[k, 0]), float(line[k, 1])],
                          "heading": float(np.arctan2(tangent[1], tangent[0])),
                          "length": 1.6, "width": 1.0, "height": 0.25})
    return free, loop, boxes, x0, y0


def synthetic(seed=0, cache=True):
    """The 2048 x 2048 px, 0.05 m corridor map with 8 ramps as a packed track
    (about 50 MB), compiled on the GPU and cached under the package's build folder."""
    from .compile import compile_image

    path = Path(__file__).resolve().parent.parent / "_build" / f"occupancy_2048_seed{seed}_gpu.npy"
    if cache and path.exists():
        return np.load(path)
    free, loop, ramps, x0, y0 = corridor(seed)
    array = compile_image(free, loop, x0, y0, 0.05, ramps)
    if cache:
        path.parent.mkdir(parents=True, exist_ok=True)
        np.save(path, array)
    return array
