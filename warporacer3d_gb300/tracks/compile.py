"""Track compilation on the GPU: the reference's track compiler
(racer/track.py) with its per-cell work in libracer.so.

The reference spends its time in a Python loop over every cell of the grid
(racer/track.py:73-86: a KDTree ball query, pass splitting and the nearest
waypoint of each pass), then in scipy's feature transform and Gaussian blur
(racer/track.py:119-121). Here those run as CUDA kernels
(`racer_track_ribbon`, `racer_track_image`); the per-waypoint arithmetic
(resampling, headings, their cos/sin, grade, the header) stays in numpy with
the reference's own expressions, so the packed float32 array is the same,
bit for bit, as the reference's.

    load(name)                    racer/track.py:37-44   built-in ribbons
    ribbon(route, hw, bank, cell) racer/track.py:61-105  then pack :108-125
    compile_image(free, loop, …)  racer/track.py:54-58   then pack :108-125
"""
import ctypes

import numpy as np
from scipy.signal import savgol_filter

from .occupancy import arc, headings, resample

RAMP_FIELDS = 8  # (cx, cy, cos, sin, length, width, height, rise), the layout of racer_ramp

_D, _I = ctypes.c_double, ctypes.c_int
_DP, _FP = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)
# argument types of racer_track_ribbon / racer_track_image (include/racer.h)
RIBBON_ARGS = [_DP, _DP, _DP, _DP, _I, _D, _D, _D, _D, _D, _I, _I, _DP, _I, _FP, ctypes.c_int64, ctypes.POINTER(_I)]
IMAGE_ARGS = [ctypes.POINTER(ctypes.c_uint8), _DP, _I, _D, _D, _D, _I, _I, _DP, _I, _FP, ctypes.c_int64]


def ramp_table(ramps):
    """Ramp boxes as racer_ramp rows (racer/track.py:111-116)."""
    rows = []
    for ramp in ramps:
        c, s = np.cos(ramp["heading"]), np.sin(ramp["heading"])
        rise = ramp.get("rise", ramp["length"] / 2)
        rows.append([ramp["center"][0], ramp["center"][1], c, s, ramp["length"], ramp["width"], ramp["height"], rise])
    return np.ascontiguousarray(np.array(rows, dtype=np.float64).reshape(-1, RAMP_FIELDS))


class RibbonInput:
    """Everything the per-cell kernels of a ribbon track need, computed on the host as
    racer/track.py:66-71 and :105 compute it."""

    def __init__(self, route, half_width, bank, cell, ramps=()):
        self.route = np.ascontiguousarray(resample(np.asarray(route, dtype=np.float64)))
        heading = headings(self.route)
        self.cos_h, self.sin_h = np.ascontiguousarray(np.cos(heading)), np.ascontiguousarray(np.sin(heading))
        self.grade = np.ascontiguousarray(np.gradient(self.route[:, 2], arc(self.route)[:-1]))
        lo = self.route[:, :2].min(0) - 2
        self.ny, self.nx = tuple(reversed((np.ceil((self.route[:, :2].max(0) + 2 - lo) / cell).astype(int) + 1).tolist()))
        self.x0, self.y0 = lo
        self.cell, self.half_width, self.bank = cell, half_width, bank
        self.ramps = ramp_table(ramps)
        self.slope = np.hypot(abs(self.grade).max(), bank)
        for ramp in ramps:  # the reference's running sum (racer/track.py:118)
            self.slope += ramp["height"] / ramp.get("rise", ramp["length"] / 2)

    def grids_len(self):
        return 6 * self.nx * self.ny


class ImageInput:
    """The occupancy-image path's host part (racer/track.py:54-55): the smoothed
    centreline loop, resampled into the route."""

    def __init__(self, free, loop, x0, y0, cell, ramps=()):
        xy = savgol_filter(loop[:, ::-1] * cell + (x0, y0), 51, 3, axis=0, mode="wrap")
        self.route = np.ascontiguousarray(resample(np.column_stack([xy, 0 * xy[:, 0]])))
        self.free = np.ascontiguousarray(free, dtype=np.uint8)
        self.ny, self.nx = free.shape
        self.x0, self.y0, self.cell = x0, y0, cell
        self.ramps = ramp_table(ramps)
        self.slope = 0
        for ramp in ramps:
            self.slope += ramp["height"] / ramp.get("rise", ramp["length"] / 2)

    def grids_len(self):
        return 3 * self.nx * self.ny


def assemble(inp, grids, layers):
    """Header, grids and route into the packed float32 array (racer/track.py:122-125)."""
    route = inp.route
    header = [inp.nx, inp.ny, inp.x0, inp.y0, inp.cell, len(route), arc(route)[-1] / len(route), layers, inp.slope,
              0, 0, 0]
    head = np.array(header, dtype=np.float64).astype(np.float32)
    tail = np.column_stack([route, headings(route)]).ravel().astype(np.float32)
    return np.concatenate([head, grids[:layers * 3 * inp.nx * inp.ny], tail])


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def ribbon_grids(inp, fn):
    """Run a ribbon grid compiler `fn` (the C ABI's signature) on `inp`: (grids, layers)."""
    grids = np.empty(inp.grids_len(), dtype=np.float32)
    layers = ctypes.c_int(0)
    ramps = np.ascontiguousarray(inp.ramps)
    rc = fn(_dp(inp.route), _dp(inp.cos_h), _dp(inp.sin_h), _dp(inp.grade), len(inp.route),
            float(inp.half_width), float(inp.bank), float(inp.x0), float(inp.y0), float(inp.cell), inp.nx, inp.ny,
            _dp(ramps), len(ramps), grids.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), grids.size,
            ctypes.byref(layers))
    return rc, grids, layers.value


def image_grids(inp, fn):
    """Run an image grid compiler `fn` on `inp`: (grids, 1)."""
    grids = np.empty(inp.grids_len(), dtype=np.float32)
    ramps = np.ascontiguousarray(inp.ramps)
    rc = fn(inp.free.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _dp(inp.route), len(inp.route),
            float(inp.x0), float(inp.y0), float(inp.cell), inp.nx, inp.ny, _dp(ramps), len(ramps),
            grids.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), grids.size)
    return rc, grids, 1


def _lib():
    from .._lib import load_library
    return load_library()


def _check(rc, what):
    if rc != 0:
        from .._lib import RacerError
        raise RacerError(f"{what}: {_lib().racer_last_error().decode(errors='replace')}")


def ribbon(route, half_width, bank, cell, ramps=()):
    """A road `half_width` either side of `route` rising `bank` per metre outward,
    compiled on the GPU (racer/track.py:61-125)."""
    inp = RibbonInput(route, half_width, bank, cell, ramps)
    rc, grids, layers = ribbon_grids(inp, _lib().racer_track_ribbon)
    _check(rc, "racer_track_ribbon")
    return assemble(inp, grids, layers)


def compile_image(free, loop, x0, y0, cell, ramps=()):
    """Free-space image (rows south to north) + centreline loop (row, col) -> packed
    one-layer track, compiled on the GPU (racer/track.py:54-58, 108-125)."""
    inp = ImageInput(free, loop, x0, y0, cell, ramps)
    rc, grids, layers = image_grids(inp, _lib().racer_track_image)
    _check(rc, "racer_track_image")
    return assemble(inp, grids, layers)


def builtin_route(name):
    """(route, half_width, bank, cell) of a built-in ribbon (racer/track.py:38-44)."""
    t = np.linspace(0, 2 * np.pi, 160, endpoint=False)
    if name == "bridge":  # a figure eight whose second pass crosses 0.9 m above the first
        z = 0.9 * np.clip(np.cos((t - np.pi) * 1.4), 0, 1) ** 2
        return np.column_stack([7 * np.sin(t), 3.5 * np.sin(2 * t), z]), 1.1, 0, 0.025
    if name not in ("flat", "ramp", "bank"):
        raise ValueError(f"no built-in track {name!r}")
    z = 0.7 * (1 - np.cos(2 * t)) if name == "ramp" else 0 * t
    return np.column_stack([6 * np.cos(t), 6 * np.sin(t), z]), 1.3, 0.25 * (name == "bank"), 0.025


def load(name):
    """A built-in track compiled on the GPU."""
    return ribbon(*builtin_route(name))
