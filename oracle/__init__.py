"""CPU oracle for the rollout hot path (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, always as the checker or as the timed CPU
baseline, never as the product. The per-index kernels are a C++ restatement
of racer/sim.mojo and racer/ppo.mojo (``oracle.cpp``); the classes below
restate the reference's Mojo structs around them with the same buffer layout
(feature-major rows, one column per car):

    Sim          racer/sim.mojo:269-348
    Activations  racer/ppo.mojo:47-60
    Policy       racer/ppo.mojo:63-138
    Trainer      racer/ppo.mojo:141-337   (rollout length is a parameter)
    save / load  racer/ppo.mojo:341-355
    track_ribbon, track_image   racer/track.py:54-125 (per-cell work, track.cpp)

Parity pins: the reference's own tests (tests/test_mojo.mojo) run against this
oracle in tests/test_oracle.py with the reference's tolerances. Random streams
use the project's documented Philox mapping (philox.h); the reference's Mojo
Philox streams are not pinned by any reference test.
"""
import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

# racer/sim.mojo:24-50 and racer/ppo.mojo:17-37
STATE = 11
X, Y, Z, HEADING, SPEED, STEER, STEPS, PROGRESS, EPISODE, FRICTION, RETURN = range(11)
OUT = 3
CRASH, TIMEOUT = 1, 2
HORIZON = 3000
RANGE = 10.0
H, HA = 64, 65
ROLLOUT, EPOCHS, MINIBATCHES = 32, 4, 4
GAMMA, LAMBDA = np.float32(0.99), np.float32(0.95)
STEER_MAX, ACCEL_MAX, SPEED_MAX, GRIP, G = 0.4189, 9.51, 5.0, 1.05, 9.81
REWARD, ADV, NORM, KL, STATS = 0, 1, 3, 4, 5


def build(force=False):
    """Compile oracle.cpp and track.cpp into _build/liboracle.so with contraction disabled."""
    src = HERE / "oracle.cpp"
    deps = [src, HERE / "track.cpp", HERE.parent / "warporacer3d_gb300/csrc/rmath.h", HERE.parent / "warporacer3d_gb300/csrc/philox.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / f"liboracle.{os.getpid()}.so"
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), str(src), str(HERE / "track.cpp")]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        c_int, c_float, u64 = ctypes.c_int, ctypes.c_float, ctypes.c_uint64
        sig = {
            "orc_half_log_2pi": (c_float, []),
            "orc_probe": (None, [f32p, c_float, c_float, c_float, ctypes.POINTER(c_int), ctypes.POINTER(c_float),
                                 ctypes.POINTER(c_float)]),
            "orc_surface": (None, [f32p, c_int, c_float, c_float, f32p]),
            "orc_progress": (c_float, [f32p, c_int, c_float, c_float]),
            "orc_at": (c_float, [f32p, c_int, c_int, c_float, c_float]),
            "orc_derivative": (None, [f32p, c_float, c_float, c_float, c_float, c_float, f32p]),
            "orc_sincos": (None, [f32p, c_int, f32p, f32p]),
            "orc_exp": (None, [f32p, c_int, f32p]),
            "orc_log": (None, [f32p, c_int, f32p]),
            "orc_philox": (None, [u64, u64, u64, u32p]),
            "orc_sim_spawn": (None, [f32p, c_int, u64, f32p, f32p, c_int]),
            "orc_sim_physics": (None, [f32p, c_int, c_int, u64, f32p, f32p, f32p, f32p, f32p, c_int]),
            "orc_sim_lidar": (None, [f32p, c_int, c_int, f32p, f32p, ctypes.c_void_p, c_int]),
            "orc_sim_sample": (None, [c_int, u64, f32p, f32p, f32p, f32p, f32p, c_int, ctypes.c_int64]),
            "orc_policy_size": (c_int, [c_int]),
            "orc_policy_init": (None, [c_int, u64, f32p]),
            "orc_policy_forward": (None, [c_int, f32p, f32p, c_int, f32p, f32p, f32p, c_int]),
            "orc_policy_backward": (None, [c_int, f32p, f32p, c_int, f32p, f32p, f32p, f32p, f32p, f32p, c_int]),
            "orc_gae": (None, [c_int, c_int, f32p, f32p, f32p, f32p, f32p]),
            "orc_gather": (None, [c_int, c_int, c_int, c_int, c_int, f32p, f32p]),
            "orc_loss": (None, [c_int, c_int, c_int, c_int, f32p, f32p, f32p, f32p, f32p, f32p, c_float, c_float,
                                f32p]),
            "orc_adam": (None, [c_int, c_int, c_int, c_float, f32p, f32p, f32p, f32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def threads_default():
    return os.cpu_count() or 1


# ---- Map queries (racer/sim.mojo:81-152) ----

class Spot:
    def __init__(self, layer, clearance, height):
        self.layer, self.clearance, self.height = layer, clearance, height


class Map:
    """Header fields of a track array plus the probe/surface/progress queries."""

    def __init__(self, track):
        d = np.ascontiguousarray(track, np.float32)
        if d.size < 12:
            raise ValueError("not a track array")
        self.d = d
        self.nx, self.ny = int(d[0]), int(d[1])
        self.x0, self.y0, self.cell = d[2], d[3], d[4]
        self.waypoints, self.spacing, self.layers, self.slope = int(d[5]), d[6], int(d[7]), d[8]
        self.route = 12 + 3 * self.layers * self.nx * self.ny

    def probe(self, x, y, z):
        layer, clr, h = ctypes.c_int(), ctypes.c_float(), ctypes.c_float()
        lib().orc_probe(self.d, x, y, z, ctypes.byref(layer), ctypes.byref(clr), ctypes.byref(h))
        return Spot(layer.value, clr.value, h.value)

    def surface(self, layer, x, y):
        out = np.zeros(3, np.float32)
        lib().orc_surface(self.d, layer, x, y, out)
        return out  # height, d height/dx, d height/dy

    def progress(self, layer, x, y):
        return lib().orc_progress(self.d, layer, x, y)

    def waypoint(self, w, field):
        return float(self.d[self.route + 4 * w + field])


def derivative(p, steer, accel, grip, along, across):
    out = np.zeros(4, np.float32)
    lib().orc_derivative(np.asarray(p, np.float32), steer, accel, grip, along, across, out)
    return out


# ---- Sim (racer/sim.mojo:269-348) ----

class Sim:
    def __init__(self, track, n, seed, beams=108, threads=None):
        self.map = Map(track)
        self.data = self.map.d
        self.n, self.seed, self.beams = n, seed, beams
        self.IN = beams + 5
        self.threads = threads or threads_default()
        self.state = np.zeros((STATE, n), np.float32)
        self.obs = np.zeros((self.IN, n), np.float32)
        self.actions = np.zeros((2, n), np.float32)
        self.reward = np.zeros(n, np.float32)
        self.done = np.zeros(n, np.float32)

    def reset(self):
        lib().orc_sim_spawn(self.data, self.n, self.seed, self.state, self.actions, self.threads)
        self.step(self.actions, self.reward, self.done, self.obs)

    def physics(self, actions, reward, done, obs):
        lib().orc_sim_physics(self.data, self.n, self.beams, self.seed, self.state, actions, reward, done, obs,
                              self.threads)

    def lidar(self, obs, iters=None):
        ptr = None if iters is None else iters.ctypes.data_as(ctypes.c_void_p)
        lib().orc_sim_lidar(self.data, self.n, self.beams, self.state, obs, ptr, self.threads)

    def step(self, actions, reward, done, obs, iters=None):
        """Physics, rewards and resets for every car, then every lidar beam."""
        self.physics(actions, reward, done, obs)
        self.lidar(obs, iters)

    def sample(self, output, log_std, actions, logp, value, deterministic, step):
        lib().orc_sim_sample(self.n, self.seed, output, np.ascontiguousarray(log_std, np.float32), actions, logp,
                             value, int(deterministic), step)


# ---- Policy (racer/ppo.mojo:47-138) ----

class Activations:
    def __init__(self, cols):
        self.cols = cols
        self.h1 = np.ones((HA, cols), np.float32)
        self.h2 = np.ones((HA, cols), np.float32)
        self.o = np.zeros((OUT, cols), np.float32)


class Policy:
    def __init__(self, seed, beams=108, threads=None):
        self.IN = beams + 5
        self.W0 = 0
        self.W1 = H * self.IN
        self.W2 = self.W1 + H * HA
        self.LOGSTD = self.W2 + OUT * HA
        self.P = self.LOGSTD + 2
        self.threads = threads or threads_default()
        self.theta = np.zeros(self.P, np.float32)
        lib().orc_policy_init(self.IN, seed, self.theta)

    def log_std(self):
        return self.theta[self.LOGSTD:self.LOGSTD + 2]

    def forward(self, x, a):
        lib().orc_policy_forward(self.IN, self.theta, np.ascontiguousarray(x), a.cols, a.h1, a.h2, a.o, self.threads)

    def backward(self, x, a, d3, d2, d1, grad):
        lib().orc_policy_backward(self.IN, self.theta, np.ascontiguousarray(x), a.cols, a.h1, a.h2,
                                  np.ascontiguousarray(d3[:OUT]), d2, d1, grad, self.threads)


# ---- Trainer (racer/ppo.mojo:141-337) ----

class Trainer:
    def __init__(self, n, beams=108, rollout=ROLLOUT, threads=None):
        self.n, self.R, self.IN = n, rollout, beams + 5
        self.batch = n * rollout // MINIBATCHES
        self.step = 0
        self.threads = threads or threads_default()
        R, IN, B = rollout, self.IN, self.batch
        self.obs = np.zeros((R + 1, IN, n), np.float32)
        self.actions = np.zeros((R, 2, n), np.float32)
        self.logp = np.zeros((R, n), np.float32)
        self.value = np.zeros((R, n), np.float32)
        self.reward = np.zeros((R, n), np.float32)
        self.done = np.zeros((R, n), np.float32)
        self.advantage = np.zeros((R, n), np.float32)
        self.x = np.zeros((IN, B), np.float32)
        self.acts = Activations(B)
        self.d3 = np.zeros((OUT + 3, B), np.float32)
        self.d2 = np.zeros((HA, B), np.float32)
        self.d1 = np.zeros((HA, B), np.float32)
        self.grad = None
        self.first = None
        self.second = None
        self.stats = np.zeros(STATS, np.float32)

    def _adam_state(self, policy):
        if self.grad is None:
            self.grad = np.zeros(policy.P, np.float32)
            self.first = np.zeros(policy.P, np.float32)
            self.second = np.zeros(policy.P, np.float32)

    def rollout(self, sim, policy, acts, iteration):
        """R steps of every car, then advantages; returns the mean reward per step (racer/ppo.mojo:187-232)."""
        n, R = self.n, self.R
        self.obs[0] = sim.obs
        for t in range(R):
            policy.forward(self.obs[t], acts)
            sim.sample(acts.o, policy.log_std(), self.actions[t], self.logp[t], self.value[t], False,
                       iteration * R + t)
            sim.step(self.actions[t], self.reward[t], self.done[t], self.obs[t + 1])
        sim.obs[...] = self.obs[R]
        policy.forward(self.obs[R], acts)
        lib().orc_gae(n, R, self.reward, self.done, self.value, np.ascontiguousarray(acts.o[2]), self.advantage)
        self.stats[REWARD] = np.float32(self.reward.astype(np.float64).sum())
        return np.float32(self.stats[REWARD] / np.float32(R * n))

    def update(self, policy):
        """EPOCHS passes of clipped PPO over the minibatches; returns the last minibatch's KL estimate."""
        self._adam_state(policy)
        samples = self.R * self.n
        adv = self.advantage.astype(np.float64)
        self.stats[ADV] = np.float32(adv.sum())
        self.stats[ADV + 1] = np.float32((adv * adv).sum())
        adv_mean = np.float32(self.stats[ADV] / np.float32(samples))
        var = np.float32(self.stats[ADV + 1] / np.float32(samples)) - adv_mean * adv_mean
        adv_scale = np.float32(1) / np.sqrt(np.float32(max(var, np.float32(1e-8))))
        for epoch in range(EPOCHS):
            for m in range(MINIBATCHES):
                self.minibatch(policy, (m + epoch) % MINIBATCHES, adv_mean, adv_scale)
                self.step += 1
                self.adam(policy)
        self.stats[KL] = np.float32(self.d3[OUT + 2].astype(np.float64).sum())
        return np.float32(self.stats[KL] / np.float32(self.batch))

    def minibatch(self, policy, m, adv_mean, adv_scale):
        self._adam_state(policy)
        L = lib()
        L.orc_gather(self.IN, self.n, self.batch, MINIBATCHES, m, self.obs, self.x)
        policy.forward(self.x, self.acts)
        L.orc_loss(self.n, self.batch, MINIBATCHES, m, self.actions, self.logp, self.value, self.advantage,
                   self.acts.o, np.ascontiguousarray(policy.log_std()), float(adv_mean), float(adv_scale), self.d3)
        policy.backward(self.x, self.acts, self.d3, self.d2, self.d1, self.grad)
        self.grad[policy.LOGSTD:policy.LOGSTD + 2] = self.d3[OUT:OUT + 2].astype(np.float64).sum(1)
        self.stats[NORM] = np.float32((self.grad.astype(np.float64) ** 2).sum())

    def adam(self, policy):
        lib().orc_adam(policy.P, policy.LOGSTD, self.step, float(self.stats[NORM]), policy.theta, self.grad,
                       self.first, self.second)


def save(policy, path, iteration):
    """Weights and iteration count as one float32 .npy (racer/ppo.mojo:341-345)."""
    np.save(path, np.concatenate([[np.float32(iteration)], policy.theta]).astype(np.float32))


def load(policy, path):
    values = np.load(path).astype(np.float32)
    if values.size != 1 + policy.P:
        raise ValueError("checkpoint does not match the network size")
    policy.theta[:] = values[1:]
    return int(values[0])


def corridor():
    """The reference's synthetic 12 x 6 m corridor track (tests/test_mojo.mojo:23-40)."""
    CELL, NX, NY, WP = np.float32(0.05), 281, 161, 74
    d = [NX, NY, -1, -4, CELL, WP, 0.15, 1, 0.5, 0, 0, 0]
    ix = np.arange(NX)
    iy = np.arange(NY)
    x = (np.float32(-1) + CELL * ix.astype(np.float32)).astype(np.float32)
    y = (np.float32(-4) + CELL * iy.astype(np.float32)).astype(np.float32)
    X_, Y_ = np.meshgrid(x, y)
    ramp = lambda v: np.maximum(v - np.float32(8), np.float32(0)) * np.float32(0.5)
    clear = np.minimum(X_, np.minimum(np.float32(12) - X_, np.float32(3) - np.abs(Y_)))
    height = ramp(X_)
    near = np.clip(np.floor((X_ - np.float32(0.5)) / np.float32(0.15) + np.float32(0.5)).astype(np.int64), 0, WP - 1)
    route = []
    for w in range(WP):
        xw = np.float32(0.5) + np.float32(0.15) * np.float32(w)
        route += [xw, 0, ramp(xw), 0]
    return np.concatenate([np.array(d, np.float32), clear.ravel().astype(np.float32),
                           height.ravel().astype(np.float32), near.ravel().astype(np.float32),
                           np.array(route, np.float32)]).astype(np.float32)


def _track_fn(name):
    from warporacer3d_gb300.tracks import compile as C
    fn = getattr(lib(), name)
    fn.restype = ctypes.c_int
    fn.argtypes = C.RIBBON_ARGS if name == "orc_track_ribbon" else C.IMAGE_ARGS
    return fn


def track_ribbon(route, half_width, bank, cell, ramps=()):
    """A ribbon track compiled by the oracle (racer/track.py:61-125): same host part as
    the product's compiler, per-cell work in track.cpp."""
    from warporacer3d_gb300.tracks import compile as C
    inp = C.RibbonInput(route, half_width, bank, cell, ramps)
    rc, grids, layers = C.ribbon_grids(inp, _track_fn("orc_track_ribbon"))
    if rc:
        raise RuntimeError(f"orc_track_ribbon failed ({rc})")
    return C.assemble(inp, grids, layers)


def track_image(free, loop, x0, y0, cell, ramps=()):
    """An occupancy-image track compiled by the oracle (racer/track.py:54-58, 108-125)."""
    from warporacer3d_gb300.tracks import compile as C
    inp = C.ImageInput(free, loop, x0, y0, cell, ramps)
    rc, grids, layers = C.image_grids(inp, _track_fn("orc_track_image"))
    if rc:
        raise RuntimeError(f"orc_track_image failed ({rc})")
    return C.assemble(inp, grids, layers)
