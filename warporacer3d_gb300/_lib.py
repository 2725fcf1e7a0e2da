"""ctypes binding of libracer.so (include/racer.h).

The library is built in-tree by warporacer3d_gb300/build.py. There is no CPU
fallback: if the library is missing or fails to load, every entry point
raises.
"""
import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libracer.so"


class RacerError(RuntimeError):
    pass


c_int, c_float, c_int64, c_uint64, c_size_t, c_void_p = (ctypes.c_int, ctypes.c_float, ctypes.c_int64,
                                                        ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p)
P = ctypes.POINTER


class SimBuffers(ctypes.Structure):
    _fields_ = [("state", c_void_p), ("obs", c_void_p), ("actions", c_void_p), ("reward", c_void_p),
                ("done", c_void_p), ("track", c_void_p)]


class LidarShape(ctypes.Structure):
    _fields_ = [("cars_per_block", c_int), ("wide", c_int), ("split", c_int), ("dynamic", c_int),
                ("order", c_int * 8), ("flat", c_int)]


class TrainerBuffers(ctypes.Structure):
    _fields_ = [(name, c_void_p) for name in ("obs", "actions", "logp", "value", "reward", "done", "advantage", "x",
                                              "d3", "d2", "d1", "grad", "first", "second", "stats", "acts")] + \
               [("batch", c_int)]


# name -> argtypes (every function returns int except racer_last_error / racer_version)
SIGNATURES = {
    "racer_alloc": [c_size_t, P(c_void_p)],
    "racer_free": [c_void_p],
    "racer_upload": [c_void_p, c_void_p, c_size_t, c_void_p],
    "racer_download": [c_void_p, c_void_p, c_size_t, c_void_p],
    "racer_synchronize": [c_void_p],
    "racer_sim_create": [P(c_float), c_size_t, c_int, c_uint64, c_int, c_void_p, P(c_void_p)],
    "racer_sim_create_segments": [c_int, P(P(c_float)), P(c_size_t), P(c_int), P(c_uint64), c_int, c_void_p,
                                  P(c_void_p)],
    "racer_sim_set_lidar_shape": [c_void_p, P(LidarShape)],
    "racer_sim_get_lidar_shape": [c_void_p, P(LidarShape)],
    "racer_sim_autotune": [c_void_p, c_int, P(LidarShape), P(c_float)],
    "racer_sim_set_chains": [c_void_p, c_int],
    "racer_sim_set_fused_rollout": [c_void_p, c_int],
    "racer_runner_tune_chains": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, P(c_int), P(c_float)],
    "racer_sim_destroy": [c_void_p],
    "racer_sim_get_buffers": [c_void_p, P(SimBuffers)],
    "racer_sim_reset": [c_void_p],
    "racer_sim_step": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "racer_sim_step_counted": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "racer_sim_sample": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int64],
    "racer_policy_create": [c_int, c_uint64, c_void_p, P(c_void_p)],
    "racer_policy_destroy": [c_void_p],
    "racer_policy_theta": [c_void_p, P(c_void_p), P(c_int)],
    "racer_policy_sync": [c_void_p],
    "racer_policy_set_precision": [c_void_p, c_int],
    "racer_acts_create": [c_void_p, c_int, P(c_void_p)],
    "racer_acts_destroy": [c_void_p],
    "racer_acts_buffers": [c_void_p, P(c_void_p), P(c_void_p), P(c_void_p)],
    "racer_policy_forward": [c_void_p, c_void_p, c_void_p],
    "racer_policy_backward": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "racer_policy_backward_noalloc": [c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p],
    "racer_policy_status": [c_void_p, P(c_int)],
    "racer_policy_wait_test": [c_void_p, c_int],
    "racer_policy_save": [c_void_p, ctypes.c_char_p, c_int],
    "racer_policy_load": [c_void_p, ctypes.c_char_p, P(c_int)],
    "racer_trainer_create": [c_int, c_int, c_int, c_void_p, P(c_void_p)],
    "racer_trainer_destroy": [c_void_p],
    "racer_trainer_get_buffers": [c_void_p, P(TrainerBuffers)],
    "racer_trainer_rollout": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, P(c_float)],
    "racer_trainer_update": [c_void_p, c_void_p, P(c_float)],
    "racer_trainer_minibatch": [c_void_p, c_void_p, c_int, c_float, c_float],
    "racer_runner_step": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int64],
    "racer_rollout": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int64],
    "racer_runner_evaluate": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int64, P(ctypes.c_double)],
    "racer_sim_snapshot": [c_void_p, c_void_p, c_int],
    "racer_runner_audit_dynamics": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int64,
                                    P(ctypes.c_double)],
    "racer_surrogate_create": [c_void_p, c_int, c_int, c_uint64, P(c_void_p)],
    "racer_surrogate_create_frame": [c_void_p, c_int, c_int, c_uint64, c_int, P(c_void_p)],
    "racer_surrogate_grid": [c_void_p, P(c_int), P(c_int), P(c_float), P(ctypes.c_long)],
    "racer_surrogate_batch_inputs": [c_void_p, P(c_float), P(c_int)],
    "racer_surrogate_batch_predict": [c_void_p, c_void_p],
    "racer_surrogate_destroy": [c_void_p],
    "racer_surrogate_set_loss": [c_void_p, c_float],
    "racer_surrogate_set_spot_check": [c_void_p, c_int, c_float],
    "racer_surrogate_set_fused": [c_void_p, c_int],
    "racer_surrogate_set_label_cache": [c_void_p, c_int],
    "racer_surrogate_params": [c_void_p, P(c_void_p), P(c_void_p), P(ctypes.c_long), P(c_int)],
    "racer_surrogate_set_poses": [c_void_p, ctypes.c_long, c_uint64],
    "racer_surrogate_poses": [c_void_p, P(c_void_p), P(ctypes.c_long)],
    "racer_surrogate_gradient": [c_void_p, ctypes.c_long, P(c_float), c_void_p],
    "racer_surrogate_train": [c_void_p, c_int, c_float, P(c_float), P(c_float)],
    "racer_surrogate_evaluate": [c_void_p, c_int, c_uint64, P(c_float), P(c_float), P(c_float), P(c_float)],
    "racer_rollout_surrogate": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int64, c_int,
                                c_float],
    "racer_surrogate_rollout_stats": [c_void_p, P(c_float), P(c_float), P(c_float), P(c_float), P(c_float), c_int],
    "racer_gemm_bf16":[c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p,
                        c_void_p, c_void_p],
    "racer_rollout_kernel_count":[c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, P(c_int64)],
    "racer_sim_profile": [c_void_p, c_void_p, c_int, P(c_float), P(c_float), P(c_int64)],
    "racer_gather_peak": [c_size_t, c_int, P(c_float)],
    "racer_trainer_set_graphs": [c_void_p, c_int],
    "racer_trainer_set_surrogate": [c_void_p, c_void_p, c_int, c_float],
    "racer_surrogate_bind": [c_void_p, c_void_p],
    "racer_track_ribbon": [P(ctypes.c_double)] * 4 + [c_int] + [ctypes.c_double] * 5 + [c_int, c_int,
                                                                                       P(ctypes.c_double), c_int,
                                                                                       P(c_float), c_int64, P(c_int)],
    "racer_track_image": [P(ctypes.c_uint8), P(ctypes.c_double), c_int] + [ctypes.c_double] * 3 +
                         [c_int, c_int, P(ctypes.c_double), c_int, P(c_float), c_int64],
}

_lib = None


def load_library():
    """Load libracer.so; raises if it was not built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RacerError(f"{LIB_PATH} is missing: build it with warporacer3d_gb300.build.build()")
        lib = ctypes.CDLL(str(LIB_PATH))
        lib.racer_last_error.restype = ctypes.c_char_p
        lib.racer_last_error.argtypes = []
        lib.racer_version.restype = c_int
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = c_int
            fn.argtypes = args
        _lib = lib
    return _lib


def call(name, *args):
    lib = load_library()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise RacerError(f"{name}: {lib.racer_last_error().decode(errors='replace')}")
    return rc
