"""Host-side mirror of the reference's Mojo structs over the C ABI.

    Sim          racer/sim.mojo:269-348
    Activations  racer/ppo.mojo:47-60
    Policy       racer/ppo.mojo:63-138
    Trainer      racer/ppo.mojo:141-337 (rollout length is a parameter)
    save / load  racer/ppo.mojo:341-355
    Runner       main.mojo:22-124 (step, benchmark, evaluate, train)

Buffers live on the GPU and are exposed as DevArray views (a device pointer
with a shape, like the reference's `mat[rows](buffer, cols, offset)`);
`.numpy()` reads one back and `.write()` uploads into it. All compute is in
libracer.so; nothing here computes on the CPU.
"""
import ctypes
import time

import numpy as np

from ._lib import LidarShape, RacerError, SimBuffers, TrainerBuffers, call, load_library

STATE = 11
X, Y, Z, HEADING, SPEED, STEER, STEPS, PROGRESS, EPISODE, FRICTION, RETURN = range(11)
OUT, H, HA = 3, 64, 65
CRASH, TIMEOUT = 1, 2
ROLLOUT, EPOCHS, MINIBATCHES = 32, 4, 4
RANGE = 10.0


class DevArray:
    """A float32 (or int32) device array view: pointer, shape, owner."""

    def __init__(self, ptr, shape, dtype=np.float32, owner=None, stream=None):
        self.ptr = int(ptr)
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        self.owner = owner
        self.stream = stream

    @classmethod
    def empty(cls, shape, dtype=np.float32):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = ctypes.c_void_p()
        call("racer_alloc", nbytes, ctypes.byref(p))
        arr = cls(p.value, shape, dtype)
        arr._owned = True
        return arr

    def __del__(self):
        if getattr(self, "_owned", False) and self.ptr:
            try:
                load_library().racer_free(ctypes.c_void_p(self.ptr))
            except Exception:
                pass
            self.ptr = 0

    @property
    def nbytes(self):
        return int(np.prod(self.shape)) * self.dtype.itemsize

    def __getitem__(self, i):
        """Leading-index view (rollout storage step t, a row of a matrix)."""
        if i < 0:
            i += self.shape[0]
        inner = self.shape[1:]
        step = int(np.prod(inner)) * self.dtype.itemsize if inner else self.dtype.itemsize
        return DevArray(self.ptr + i * step, inner if inner else (1,), self.dtype, self, self.stream)

    def rows(self, start, stop):
        inner = self.shape[1:]
        step = int(np.prod(inner)) * self.dtype.itemsize
        return DevArray(self.ptr + start * step, (stop - start,) + inner, self.dtype, self, self.stream)

    @property
    def c(self):
        return ctypes.c_void_p(self.ptr)

    def numpy(self):
        out = np.empty(self.shape, self.dtype)
        call("racer_download", out.ctypes.data_as(ctypes.c_void_p), self.c, self.nbytes, self.stream)
        return out

    def write(self, values):
        v = np.ascontiguousarray(np.asarray(values, self.dtype).reshape(self.shape))
        call("racer_upload", self.c, v.ctypes.data_as(ctypes.c_void_p), self.nbytes, self.stream)


def _stream(stream):
    """Accept None, an int handle, or an object with .cuda_stream (torch.cuda.Stream)."""
    if stream is None:
        return None
    if isinstance(stream, ctypes.c_void_p):
        return stream
    return ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))


class Sim:
    """n cars on a track (racer/sim.mojo:269-348)."""

    def __init__(self, track, n, seed, beams=108, stream=None):
        self._create([track], [n], [seed], beams, stream)

    @classmethod
    def segments(cls, tracks, cars, seeds, beams=108, stream=None):
        """Several tracks in one sim: segment k is cars[k] cars on tracks[k] seeded by seeds[k], in columns
        sum(cars[:k]) .. sum(cars[:k+1]) of every buffer; each launch covers all segments."""
        self = cls.__new__(cls)
        self._create(list(tracks), list(cars), list(seeds), beams, stream)
        return self

    def _create(self, tracks, cars, seeds, beams, stream):
        if not (len(tracks) == len(cars) == len(seeds)):
            raise ValueError("tracks, cars and seeds differ in length")
        arrays = [np.ascontiguousarray(t, np.float32) for t in tracks]
        k = len(arrays)
        fp = ctypes.POINTER(ctypes.c_float)
        ptrs = (fp * k)(*[a.ctypes.data_as(fp) for a in arrays])
        lens = (ctypes.c_size_t * k)(*[a.size for a in arrays])
        counts = (ctypes.c_int * k)(*cars)
        seeds_c = (ctypes.c_uint64 * k)(*seeds)
        self.n, self.seed, self.beams, self.IN = int(sum(cars)), (seeds[0] if seeds else 0), beams, beams + 5
        self.cars = list(cars)
        self.car0 = [int(v) for v in np.concatenate([[0], np.cumsum(cars)])]
        self.stream = _stream(stream)
        h = ctypes.c_void_p()
        call("racer_sim_create_segments", k, ptrs, lens, counts, seeds_c, beams, self.stream, ctypes.byref(h))
        self.handle = h
        n = self.n
        b = SimBuffers()
        call("racer_sim_get_buffers", h, ctypes.byref(b))
        s = self.stream
        self.state = DevArray(b.state, (STATE, n), owner=self, stream=s)
        self.obs = DevArray(b.obs, (self.IN, n), owner=self, stream=s)
        self.actions = DevArray(b.actions, (2, n), owner=self, stream=s)
        self.reward = DevArray(b.reward, (n,), owner=self, stream=s)
        self.done = DevArray(b.done, (n,), owner=self, stream=s)

    def __del__(self):
        if getattr(self, "handle", None):
            load_library().racer_sim_destroy(self.handle)
            self.handle = None

    def reset(self):
        call("racer_sim_reset", self.handle)

    def step(self, actions, reward, done, obs, iters=None):
        if iters is None:
            call("racer_sim_step", self.handle, actions.c, reward.c, done.c, obs.c)
        else:
            call("racer_sim_step_counted", self.handle, actions.c, reward.c, done.c, obs.c, iters.c)

    def sample(self, output, log_std, actions, logp, value, deterministic, step):
        call("racer_sim_sample", self.handle, output.c, log_std.c, actions.c, logp.c, value.c, int(deterministic),
             step)

    def snapshot(self, out=None):
        """state, obs, actions, reward, done of every car as one [(11 + IN + 4), n] float32 array
        (main.mojo:94-124's serve snapshot), from one device-to-host copy."""
        rows = STATE + self.IN + 4
        if out is None:
            out = np.empty((rows, self.n), np.float32)
        assert out.dtype == np.float32 and out.size == rows * self.n and out.flags.c_contiguous
        call("racer_sim_snapshot", self.handle, out.ctypes.data_as(ctypes.c_void_p), 1)
        return out

    def set_lidar_shape(self, cars_per_block, wide=0, split=0, order=None, dynamic=0, flat=0):
        """Lidar launch shape: cars per block (2, 4, 8), the 40-register variant (wide), per-segment
        launches on parallel streams (split), the segments' order (default: index order), the
        persistent grid with dynamically assigned (car, beam group) units (dynamic) and warps taking
        (car, beam) pairs across car boundaries (flat)."""
        order = list(range(len(self.cars))) if order is None else list(order)
        shape = LidarShape(cars_per_block, wide, split, dynamic,
                           (ctypes.c_int * 8)(*(order + [-1] * (8 - len(order)))), flat)
        call("racer_sim_set_lidar_shape", self.handle, ctypes.byref(shape))

    @staticmethod
    def _shape(shape):
        return {"cars_per_block": shape.cars_per_block, "wide": shape.wide, "split": shape.split,
                "dynamic": shape.dynamic, "order": [k for k in shape.order if k >= 0], "flat": shape.flat}

    def lidar_shape(self):
        shape = LidarShape()
        call("racer_sim_get_lidar_shape", self.handle, ctypes.byref(shape))
        return self._shape(shape)

    def set_fused_rollout(self, enable=True):
        """Rollout graphs as one launch of the fused persistent kernel (forward, sampling, physics and
        lidar per step inside it; the same results)."""
        call("racer_sim_set_fused_rollout", self.handle, int(bool(enable)))

    def set_chains(self, chains):
        """Rollout graphs as `chains` independent chains over car ranges (the same results)."""
        call("racer_sim_set_chains", self.handle, int(chains))

    def autotune(self, reps=5):
        """Times every lidar launch shape on the current frames; keeps the fastest and returns it
        with its mean time in ms."""
        shape, ms = LidarShape(), ctypes.c_float()
        call("racer_sim_autotune", self.handle, reps, ctypes.byref(shape), ctypes.byref(ms))
        return self._shape(shape), ms.value


class Policy:
    """Tanh MLP IN -> 64 -> 64 -> 3 with log std (racer/ppo.mojo:63-138)."""

    def __init__(self, seed, beams=108, stream=None):
        self.IN = beams + 5
        self.W0, self.W1 = 0, H * self.IN
        self.W2 = self.W1 + H * HA
        self.LOGSTD = self.W2 + OUT * HA
        self.P = self.LOGSTD + 2
        self.stream = _stream(stream)
        h = ctypes.c_void_p()
        call("racer_policy_create", beams, seed, self.stream, ctypes.byref(h))
        self.handle = h
        ptr, count = ctypes.c_void_p(), ctypes.c_int()
        call("racer_policy_theta", h, ctypes.byref(ptr), ctypes.byref(count))
        assert count.value == self.P
        self.theta = DevArray(ptr.value, (self.P,), owner=self, stream=self.stream)

    def __del__(self):
        if getattr(self, "handle", None):
            load_library().racer_policy_destroy(self.handle)
            self.handle = None

    def log_std(self):
        return DevArray(self.theta.ptr + 4 * self.LOGSTD, (2,), owner=self, stream=self.stream)

    def sync(self):
        call("racer_policy_sync", self.handle)

    def set_precision(self, precision):
        """'bf16' (tensor cores, FP32 accumulation; default) or 'fp32' (CUDA cores)."""
        if precision not in ("bf16", "fp32"):
            raise ValueError(precision)
        call("racer_policy_set_precision", self.handle, int(precision == "bf16"))

    def status(self):
        """Error word of the tensor-core kernels (0 = none), read and cleared."""
        code = ctypes.c_int()
        call("racer_policy_status", self.handle, ctypes.byref(code))
        return code.value

    def wait_test(self, polls):
        """Launch the timeout probe: a tensor-core kernel whose bounded wait (`polls` polls) on an
        mbarrier that nothing arrives on runs out; it records the timeout in the error word (status),
        frees its tensor memory and returns."""
        call("racer_policy_wait_test", self.handle, int(polls))

    def forward(self, x, acts):
        call("racer_policy_forward", self.handle, x.c, acts.handle)

    def backward(self, x, acts, d3, d2, d1, grad):
        call("racer_policy_backward", self.handle, x.c, acts.handle, d3.c, d2.c, d1.c, grad.c)


class Activations:
    """h1, h2 [65, cols] (row 64 = 1) and o [3, cols] (racer/ppo.mojo:47-60)."""

    def __init__(self, policy, cols, handle=None):
        self.cols = cols
        if handle is None:
            h = ctypes.c_void_p()
            call("racer_acts_create", policy.handle, cols, ctypes.byref(h))
            self._owned = True
        else:
            h = ctypes.c_void_p(handle)
            self._owned = False
        self.handle = h
        a, b, c = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        call("racer_acts_buffers", h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        self.h1 = DevArray(a.value, (HA, cols), owner=self)
        self.h2 = DevArray(b.value, (HA, cols), owner=self)
        self.o = DevArray(c.value, (OUT, cols), owner=self)

    def __del__(self):
        if getattr(self, "_owned", False) and getattr(self, "handle", None):
            load_library().racer_acts_destroy(self.handle)
            self.handle = None


class Trainer:
    """Rollout storage, minibatch scratch and Adam state (racer/ppo.mojo:141-337)."""

    def __init__(self, n, beams=108, rollout=ROLLOUT, stream=None, policy=None):
        self.n, self.R, self.IN = n, rollout, beams + 5
        self.stream = _stream(stream)
        h = ctypes.c_void_p()
        call("racer_trainer_create", n, beams, rollout, self.stream, ctypes.byref(h))
        self.handle = h
        b = TrainerBuffers()
        call("racer_trainer_get_buffers", h, ctypes.byref(b))
        self.batch = B = b.batch
        R, IN = rollout, self.IN
        P = H * IN + H * HA + OUT * HA + 2
        s = self.stream
        self.obs = DevArray(b.obs, (R + 1, IN, n), owner=self, stream=s)
        self.actions = DevArray(b.actions, (R, 2, n), owner=self, stream=s)
        for name in ("logp", "value", "reward", "done", "advantage"):
            setattr(self, name, DevArray(getattr(b, name), (R, n), owner=self, stream=s))
        self.x = DevArray(b.x, (MINIBATCHES, IN, B), owner=self, stream=s)
        self.d3 = DevArray(b.d3, (OUT + 3, B), owner=self, stream=s)
        self.d2 = DevArray(b.d2, (HA, B), owner=self, stream=s)
        self.d1 = DevArray(b.d1, (HA, B), owner=self, stream=s)
        self.grad = DevArray(b.grad, (P,), owner=self, stream=s)
        self.first = DevArray(b.first, (P,), owner=self, stream=s)
        self.second = DevArray(b.second, (P,), owner=self, stream=s)
        self.stats = DevArray(b.stats, (5,), owner=self, stream=s)
        self.acts = Activations(None, B, handle=b.acts)

    def __del__(self):
        if getattr(self, "handle", None):
            load_library().racer_trainer_destroy(self.handle)
            self.handle = None

    def rollout(self, sim, policy, acts, iteration):
        r = ctypes.c_float()
        call("racer_trainer_rollout", self.handle, sim.handle, policy.handle, acts.handle, iteration, ctypes.byref(r))
        return r.value

    def update(self, policy):
        kl = ctypes.c_float()
        call("racer_trainer_update", self.handle, policy.handle, ctypes.byref(kl))
        return kl.value

    def set_graphs(self, enable=True):
        """Replay each update from one captured CUDA graph (default) or launch it eagerly."""
        call("racer_trainer_set_graphs", self.handle, int(enable))

    def set_surrogate(self, surrogate, audit_every=16, fallback_m=0.5):
        """Rollouts with the learned lidar (audit every `audit_every`-th step of training, exact fallback
        for cars with a predicted range under `fallback_m`); None restores exact tracing."""
        self._surrogate = surrogate  # the trainer uses it until it is replaced
        call("racer_trainer_set_surrogate", self.handle, surrogate.handle if surrogate else None, int(audit_every),
             float(fallback_m))

    def minibatch(self, policy, m, adv_mean, adv_scale):
        call("racer_trainer_minibatch", self.handle, policy.handle, m, float(adv_mean), float(adv_scale))


class Surrogate:
    """Learned lidar for one sim's track: lidar frame -> all beam ranges (BF16 MLP on tcgen05).

    frame="car": one output per beam from fixed Fourier features of the frame. frame="world": the
    range profile at fixed world angles (the beam spacing), read at each car's heading offset, from
    trainable feature grids of the origin (beams - 1 must be a multiple of 12). frame="car_grid": one
    output per beam from the feature grids beside the frame and heading harmonics."""

    GRID_LEVELS, GRID_F = 5, 8
    FRAMES = {"car": 0, "world": 1, "car_grid": 2}

    def __init__(self, sim, hidden=512, batch=8192, seed=0, frame="car"):
        if frame not in self.FRAMES:
            raise ValueError("frame must be 'car', 'world' or 'car_grid'")
        self.sim = sim
        h = ctypes.c_void_p()
        call("racer_surrogate_create_frame", sim.handle, hidden, batch, seed, self.FRAMES[frame], ctypes.byref(h))
        self.handle = h
        self.batch, self.hidden, self.frame = batch, hidden, frame
        self.nout = 4 * (sim.beams - 1) // 3 if frame == "world" else sim.beams
        th, gr, count = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_long()
        call("racer_surrogate_params", h, ctypes.byref(th), ctypes.byref(gr), ctypes.byref(count), None)
        self.theta = DevArray(th.value, (count.value,), owner=self, stream=sim.stream)
        self.grad = DevArray(gr.value, (count.value,), owner=self, stream=sim.stream)

    def __del__(self):
        if getattr(self, "handle", None):
            load_library().racer_surrogate_destroy(self.handle)
            self.handle = None

    def layout(self):
        """{name: (offset, shape)} of the parameter blocks; the world frame adds the grids G0..G4,
        each [layers, gy, gx, 8]."""
        H, K, n = self.hidden, self.nout, 64
        sizes = [("W1", (H, n)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)), ("W4", (K, H)),
                 ("b4", (K,))]
        out, off = {}, 0
        for name, shape in sizes:
            out[name] = (off, shape)
            off += int(np.prod(shape))
        if self.frame != "car":
            gx, gy, sp, offs = self.grid()
            layers = (offs[1] - offs[0]) // (gx[0] * gy[0] * self.GRID_F)
            for l in range(self.GRID_LEVELS):
                out[f"G{l}"] = (int(offs[l]), (layers, int(gy[l]), int(gx[l]), self.GRID_F))
        return out

    def grid(self):
        """World frame: per level the vertex counts gx, gy, the spacing (m) and the parameter offset."""
        L = self.GRID_LEVELS
        gx, gy, sp, off = (ctypes.c_int * L)(), (ctypes.c_int * L)(), (ctypes.c_float * L)(), (ctypes.c_long * L)()
        call("racer_surrogate_grid", self.handle, gx, gy, sp, off)
        return list(gx), list(gy), list(sp), list(off)

    def batch_inputs(self):
        """Encoded inputs [batch, 64] of the last gradient() batch and (world frame) each sample's k0."""
        x = np.zeros((self.batch, 64), np.float32)
        k0 = np.zeros(self.batch, np.int32)
        fp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
        call("racer_surrogate_batch_inputs", self.handle, x.ctypes.data_as(fp),
             k0.ctypes.data_as(ip) if self.frame == "world" else None)
        return x, (k0 if self.frame == "world" else None)

    def batch_predict(self, pred):
        """Predictions [beams, batch] (DevArray) for the last gradient() batch, through the layered
        inference path."""
        call("racer_surrogate_batch_predict", self.handle, pred.c)

    def set_poses(self, count, seed=1):
        call("racer_surrogate_set_poses", self.handle, count, seed)

    def bind(self, sim):
        """Serve another sim on the same track array (same header, length and beam count)."""
        call("racer_surrogate_bind", self.handle, sim.handle)
        self.sim = sim

    def poses(self):
        p, count = ctypes.c_void_p(), ctypes.c_long()
        call("racer_surrogate_poses", self.handle, ctypes.byref(p), ctypes.byref(count))
        return DevArray(p.value, (count.value, 4), owner=self, stream=self.sim.stream)

    def gradient(self, first=0, labels=None):
        mse = ctypes.c_float()
        call("racer_surrogate_gradient", self.handle, first, ctypes.byref(mse), labels.c if labels else None)
        return mse.value

    def set_fused(self, fused=True):
        """Rollout inference in one fused kernel (512-wide) or as four GEMMs; the same bits either way."""
        call("racer_surrogate_set_fused", self.handle, int(bool(fused)))

    def set_label_cache(self, enable=True):
        """Keep the training set's exact labels after their first tracing (the same bits, faster epochs);
        takes effect from the next set_poses."""
        call("racer_surrogate_set_label_cache", self.handle, int(bool(enable)))

    def set_spot_check(self, stride=64, tolerance_m=0.25):
        """Between audits, trace every `stride`-th beam (offset rotating with the step) exactly and send
        cars with a beam off by more than `tolerance_m` to the exact tracer; stride 0 turns it off."""
        call("racer_surrogate_set_spot_check", self.handle, int(stride), float(tolerance_m))

    def set_loss(self, huber_m=0.0):
        """0: squared range error; > 0: Huber loss with that threshold in metres."""
        call("racer_surrogate_set_loss", self.handle, float(huber_m))

    def train(self, steps, lr=1e-3):
        mse, mae = ctypes.c_float(), ctypes.c_float()
        call("racer_surrogate_train", self.handle, steps, lr, ctypes.byref(mse), ctypes.byref(mae))
        return mse.value, mae.value

    def rollout_stats(self, reset=False):
        """(MAE, RMSE, max error in metres, fraction of audited beams off by > 5 cm, fallback fraction)."""
        out = [ctypes.c_float() for _ in range(5)]
        call("racer_surrogate_rollout_stats", self.handle, *[ctypes.byref(o) for o in out], int(reset))
        return tuple(o.value for o in out)

    def evaluate(self, batches=4, seed=12345):
        """Held-out error against the exact tracer: MAE, RMSE, max (metres) and fraction of beams off by > 5 cm."""
        out = [ctypes.c_float() for _ in range(4)]
        call("racer_surrogate_evaluate", self.handle, batches, seed, *[ctypes.byref(o) for o in out])
        return tuple(o.value for o in out)


def gather_peak(bytes_=8 << 20, reps=20):
    """GB/s of random 16-byte gathers from an L2-resident buffer of `bytes_` (racer_gather_peak):
    the roofline of the lidar's probes."""
    gbs = ctypes.c_float()
    call("racer_gather_peak", int(bytes_), int(reps), ctypes.byref(gbs))
    return gbs.value


def save(policy, path, iteration):
    call("racer_policy_save", policy.handle, str(path).encode(), iteration)


def load(policy, path):
    it = ctypes.c_int()
    call("racer_policy_load", policy.handle, str(path).encode(), ctypes.byref(it))
    return it.value


class Runner:
    """A device, n cars on a track and a policy driving them (main.mojo:22-124)."""

    def __init__(self, track, n, beams=108, seed=42, policy_seed=42, stream=None, sim=None):
        self.sim = sim if sim is not None else Sim(track, n, seed, beams=beams, stream=stream)
        n = self.sim.n
        self.policy = Policy(policy_seed, beams=self.sim.beams, stream=self.sim.stream)
        self.acts = Activations(self.policy, n)
        self.scratch = DevArray.empty((2, n))  # log probabilities and values
        self.sim.reset()

    @classmethod
    def segments(cls, tracks, cars, seeds, beams=108, policy_seed=42, stream=None):
        """One policy driving cars on several tracks at once (Sim.segments)."""
        return cls(None, None, policy_seed=policy_seed, sim=Sim.segments(tracks, cars, seeds, beams, stream))

    def step(self, deterministic, t):
        call("racer_runner_step", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c,
             int(deterministic), t)

    def rollout(self, steps, deterministic=False, step0=0):
        """`steps` Runner steps replayed from one CUDA graph."""
        call("racer_rollout", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c, steps,
             int(deterministic), step0)

    def rollout_surrogate(self, surrogate, steps, deterministic=False, step0=0, audit_every=16, fallback_m=0.5):
        """`steps` Runner steps with the learned lidar, audited every `audit_every` steps."""
        call("racer_rollout_surrogate", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c,
             surrogate.handle, steps, int(deterministic), step0, audit_every, fallback_m)

    def audit_dynamics(self, steps, deterministic=False, step0=0):
        """`steps` Runner steps, each physics step re-integrated in FP64 from the same state and actions.

        Returns the cars audited and the mean and max position (m), heading (rad) and speed (m/s)
        differences between the binary32 step and the FP64 one (cars that ended an episode are skipped).
        """
        out = (ctypes.c_double * 7)()
        call("racer_runner_audit_dynamics", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c,
             int(deterministic), steps, step0, out)
        count = max(out[0], 1.0)
        return {"cars": int(out[0]), "position_mean_m": out[1] / count, "heading_mean_rad": out[2] / count,
                "speed_mean_mps": out[3] / count, "position_max_m": out[4], "heading_max_rad": out[5],
                "speed_max_mps": out[6]}

    def tune_chains(self, steps=50, reps=3):
        """Times rollouts with 1 to 4 chains, keeps the fastest; returns (chains, env-steps/s)."""
        best, rate = ctypes.c_int(), ctypes.c_float()
        call("racer_runner_tune_chains", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c, steps,
             reps, ctypes.byref(best), ctypes.byref(rate))
        return best.value, rate.value

    def synchronize(self):
        call("racer_synchronize", self.sim.stream)

    def rollout_kernel_count(self, steps, deterministic=False):
        count = ctypes.c_int64()
        call("racer_rollout_kernel_count", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c,
             steps, int(deterministic), ctypes.byref(count))
        return count.value

    def profile_sim(self, reps):
        """Mean physics and lidar kernel times (ms) and the probe iterations of one lidar pass."""
        phys, lid, iters = ctypes.c_float(), ctypes.c_float(), ctypes.c_int64()
        call("racer_sim_profile", self.sim.handle, self.sim.actions.c, reps, ctypes.byref(phys), ctypes.byref(lid),
             ctypes.byref(iters))
        return phys.value, lid.value, iters.value

    def benchmark(self, steps, warmup=10):
        """main.mojo:82-92: n cars; ms/step; transitions/s."""
        for t in range(warmup):
            self.step(False, t)
        self.synchronize()
        start = time.perf_counter()
        for t in range(steps):
            self.step(False, t)
        self.synchronize()
        ms = (time.perf_counter() - start) * 1000 / steps
        return ms, self.sim.n * 1000 / ms

    def evaluate_graph(self, steps, step0=0):
        """main.mojo:70-80 on the device: reward per car-step and crashes per car over `steps`
        deterministic steps replayed from one CUDA graph, with one read at the end."""
        out = (ctypes.c_double * 2)()
        call("racer_runner_evaluate", self.sim.handle, self.policy.handle, self.acts.handle, self.scratch.c, steps,
             step0, out)
        return out[0], out[1]

    def serve_step(self, steer_pct, throttle_pct, reset, policy, tick):
        """One request of the reference's serve loop (main.mojo:108-124), headless: optional reset,
        then a deterministic policy step or the same manual action for every car, then the snapshot."""
        if reset:
            self.sim.reset()
        if policy:
            self.step(True, tick)
        else:
            act = np.empty((2, self.sim.n), np.float32)
            act[0], act[1] = np.float32(steer_pct) / np.float32(100), np.float32(throttle_pct) / np.float32(100)
            self.sim.actions.write(act)
            self.sim.step(self.sim.actions, self.sim.reward, self.sim.done, self.sim.obs)
        return self.sim.snapshot()

    def evaluate(self, steps):
        """main.mojo:70-80: reward per step and crashes per car, deterministic actions."""
        reward, crashes = 0.0, 0
        for t in range(steps):
            self.step(True, t)
            reward += float(self.sim.reward.numpy().astype(np.float64).sum())
            crashes += int((self.sim.done.numpy() == CRASH).sum())
        n = self.sim.n
        return reward / (n * steps), crashes / n

    def train(self, iterations, path, resume="", rollout=ROLLOUT, log=print):
        """main.mojo:54-68: rollout + update per iteration, checkpoint every 100."""
        trainer = Trainer(self.sim.n, beams=self.sim.beams, rollout=rollout, stream=self.sim.stream)
        first = load(self.policy, resume) if resume else 0
        start = time.perf_counter()
        for iteration in range(first, first + iterations):
            reward = trainer.rollout(self.sim, self.policy, self.acts, iteration)
            kl = trainer.update(self.policy)
            if not np.isfinite(kl):
                raise RacerError("training diverged (nonfinite KL)")
            log(f"iteration {iteration + 1} reward/step {reward} KL {kl}")
            if (iteration + 1) % 100 == 0:
                save(self.policy, path, iteration + 1)
        save(self.policy, path, first + iterations)
        rate = self.sim.n * rollout * iterations / (time.perf_counter() - start)
        log(f"Saved {path} ; {rate} training transitions/s")
        return rate
