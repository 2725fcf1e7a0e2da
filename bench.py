"""Benchmark of the rollout hot path: env-steps/s at 1081 beams on GB300.

Workload (one bench step): the `bridge` figure-eight (two layers), 4096 cars,
1081 lidar beams, a 1000-env-step rollout replayed from one CUDA graph; every
env step is the reference's Runner.step (main.mojo:40-48): policy forward on
the observations, Gaussian sampling, physics (4 RK4 substeps, crash, reward,
respawn) and the sphere-traced lidar. Simulator arithmetic is FP32.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). `value` is device-timed (CUDA events on the
launching stream, inputs resident in HBM, L2 flushed by a 256 MB write
between timed steps, the flush outside the events); `e2e` is the same metric
through the public API with host buffers (car state uploaded from pinned
host memory before, rewards and done flags read back after every rollout);
`roofline` covers the dominant kernel (the lidar) with its algorithmic bytes
counted from the kernel's own per-beam probe counts; `cpu_baseline` times the
CPU restatement on this host's cores on a bounded sample of the same
workload. `--impl reference` times that CPU restatement alone (the reference's
Mojo/MAX toolchain does not exist on this machine).

Under torchrun (N > 1) every rank runs the headline rollout on its own GPU
(replicas, max-over-ranks timing); the further sections (FP64 audit,
surrogate, the reference's CPU-runnable benchmark, batched, training, track compilation, CPU baseline) are
single-GPU measurements and run at N = 1 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "env-steps/s at 1081 beams, 1 GB300: exact FP32 vs BF16 surrogate (≤2cm MAE)"
TRACK, CARS, BEAMS, HORIZON_STEPS = "bridge", 4096, 1081, 1000
AUDIT_STEPS = 64
WORKLOAD = (f"{TRACK} (2 layers, 721x441 cells), {CARS} cars, {BEAMS} beams, {HORIZON_STEPS}-env-step rollout "
            "per bench step: policy forward + sampling + RK4 physics + sphere-traced lidar, CUDA graph")
L2_FLUSH_BYTES = 256 << 20
GATHER_PEAK_BYTES = 8 << 20
# what the lidar's ncu capture shows limits it (profiles/lidar_bridge_4096cars_1081beams.md)
LIDAR_LIMITER = "instruction issue: ncu shows the SMs issuing on most cycles while L2 and DRAM throughput stay low"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--surrogate-only", action="store_true", help="print only the surrogate section")
    ap.add_argument("--surrogate-frame", default="world", choices=["world", "car", "car_grid"],
                    help="output frame of the surrogate in --surrogate-only runs")
    ap.add_argument("--no-training", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--batched-only", action="store_true", help="print only the batched multi-track section")
    ap.add_argument("--no-track-compile", action="store_true")
    ap.add_argument("--track-compile-only", action="store_true", help="print only the track compilation section")
    ap.add_argument("--training-iterations", type=int, default=300)
    ap.add_argument("--surrogate-train-steps", type=int, default=None,
                    help="surrogate training steps (default 80000; fewer only to profile the rollout)")
    return ap.parse_args()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([f.strip() for f in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dram_traffic_per_launch():
    """Per-launch DRAM bytes of the lidar kernel from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "lidar_traffic.txt"
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):
                return int(line.split(":", 1)[1])
    return None


def cpu_baseline(track, seconds=12.0, max_steps=200, threads=None, cars=CARS, beams=BEAMS, name=TRACK, seed=42):
    """The CPU restatement (oracle) on this host's cores: Runner steps of the same workload until `seconds`."""
    import oracle as O
    threads = threads or os.cpu_count() or 1
    sim = O.Sim(track, cars, seed, beams=beams, threads=threads)
    pol = O.Policy(42, beams=beams, threads=threads)
    acts = O.Activations(cars)
    logp, value = np.zeros(cars, np.float32), np.zeros(cars, np.float32)
    sim.reset()
    start = time.perf_counter()
    steps = 0
    while steps < max_steps and (time.perf_counter() - start) < seconds:
        pol.forward(sim.obs, acts)
        sim.sample(acts.o, pol.log_std(), sim.actions, logp, value, False, steps)
        sim.step(sim.actions, sim.reward, sim.done, sim.obs)
        steps += 1
    dt = time.perf_counter() - start
    return {"value": cars * steps / dt, "unit": "env-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} env steps of {cars} cars on {name} at {beams} beams (Runner.step: policy forward, "
                      f"sampling, physics, lidar) in {dt:.1f} s"}


def config1_section(torch, W, stream):
    """The reference's CPU-runnable benchmark, `racer benchmark ramp cpu 1024 1000` (main.mojo:82-92): ramp,
    1024 cars, 108 beams, sim seed 0, policy seed 42, 10 warm-up policy steps, then 1000 timed ones; on the
    GPU replayed from one CUDA graph (device-timed) and as the reference's host loop of per-step calls,
    and the CPU restatement on all host cores for a bounded sample."""
    track = W.track("ramp")
    run = W.Runner(track, 1024, beams=108, seed=0, policy_seed=42, stream=stream)
    for t in range(10):
        run.step(False, t)
    state, obs = run.sim.state.numpy(), run.sim.obs.numpy()
    chains, _ = run.tune_chains(50, 3)
    run.sim.state.write(state)  # the timed rollouts start from the state after the 10 warm-up steps
    run.sim.obs.write(obs)
    run.rollout(1000, False, 10)  # capture
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a.record(stream)
        run.rollout(1000, False, 1010)
        b.record(stream)
    torch.cuda.synchronize()
    graph_rate = 1024 * 1000 / (a.elapsed_time(b) / 1000.0)
    loop_ms, loop_rate = run.benchmark(1000, warmup=10)
    cpu = cpu_baseline(track, seconds=10.0, max_steps=1000, cars=1024, beams=108, name="ramp", seed=0)
    return {"workload": "ramp, 1024 cars, 108 beams, 1000 policy steps after 10 warm-up (racer benchmark ramp "
                        "cpu 1024 1000)",
            "gpu_graph_env_steps_per_s": graph_rate, "gpu_step_loop_env_steps_per_s": loop_rate,
            "gpu_step_loop_ms_per_step": loop_ms, "cpu_env_steps_per_s": cpu["value"], "cpu_cores": cpu["cores"],
            "cpu_sample": cpu["sample"], "gpu_graph_vs_cpu": graph_rate / cpu["value"], "rollout_chains": chains}


FP32_STEPS, FP32_REPS = 200, 3


def fp32_policy_section(torch, W, track, stream, flush, runner):
    """The headline workload with every product in FP32 (the simulator and the policy all float32): the
    policy forward on the CUDA cores instead of BF16 tensor cores, rollouts of FP32_STEPS env steps
    from one graph (one chain: the chained graph needs the BF16 forward), device-timed like `value`."""
    state, obs = runner.sim.state.numpy(), runner.sim.obs.numpy()
    fp32 = W.Runner(track, CARS, beams=BEAMS, seed=42, policy_seed=42, stream=stream)
    fp32.policy.set_precision("fp32")
    fp32.sim.state.write(state)
    fp32.sim.obs.write(obs)
    fp32.rollout(FP32_STEPS, False, 0)  # capture and warm up
    torch.cuda.synchronize()
    ms = 0.0
    for k in range(FP32_REPS):
        with torch.cuda.stream(stream):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fp32.rollout(FP32_STEPS, False, (k + 1) * FP32_STEPS)
            b.record(stream)
        torch.cuda.synchronize()
        ms += a.elapsed_time(b)
    rate = CARS * FP32_STEPS * FP32_REPS / (ms / 1000.0)
    return {"workload": f"{TRACK}, {CARS} cars, {BEAMS} beams, {FP32_STEPS}-env-step rollouts, policy in FP32",
            "env_steps_per_s": rate, "ms_per_env_step": ms / (FP32_REPS * FP32_STEPS),
            "policy_precision": "f32 (CUDA cores)", "rollout_chains": 1}


def fused_rollout_section(torch, W, track, stream, flush, runner):
    """The headline workload as one launch of the fused persistent kernel per rollout (each CTA owns
    a slice of cars for all 1000 steps: forward + sampling on tcgen05, physics, lidar), device-timed
    like `value`, beside the chained graph the autotuner chose; both give the same bits."""
    state, obs = runner.sim.state.numpy(), runner.sim.obs.numpy()
    fused = W.Runner(track, CARS, beams=BEAMS, seed=42, policy_seed=42, stream=stream)
    fused.sim.set_fused_rollout(True)
    fused.sim.state.write(state)
    fused.sim.obs.write(obs)
    fused.rollout(HORIZON_STEPS, False, 0)  # capture and warm up
    torch.cuda.synchronize()
    ms = 0.0
    reps = 2
    for k in range(reps):
        with torch.cuda.stream(stream):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fused.rollout(HORIZON_STEPS, False, (k + 1) * HORIZON_STEPS)
            b.record(stream)
        torch.cuda.synchronize()
        ms += a.elapsed_time(b)
    return {"workload": f"{TRACK}, {CARS} cars, {BEAMS} beams, {HORIZON_STEPS}-env-step rollouts",
            "env_steps_per_s": CARS * HORIZON_STEPS * reps / (ms / 1000.0),
            "ms_per_env_step": ms / (reps * HORIZON_STEPS), "kernels_per_rollout": fused.rollout_kernel_count(HORIZON_STEPS),
            "cars_per_cta": -(-CARS // (2 * 152)), "status": fused.policy.status()}


SURR_CARS, SURR_STEPS, SURR_REPS, SURR_TRAIN_STEPS = 65536, 32, 3, 80000
SURR_LR = {"world": 2e-3, "car": 8e-3, "car_grid": 3e-3}
SURR_HUBER_M = 0.02
SPOT_STRIDE, SPOT_TOL_M = 64, 1.0
SURR_NETWORK = {
    "world": "64 inputs (feature grids of the origin: 5 resolutions x 8 features; 22 fixed Fourier features; "
             "heading phase) -> 3 x 512 tanh -> 1440 world samples, each beam read at its heading's offset; "
             "BF16 tcgen05, FP32 Adam",
    "car": "64 encoded inputs (fixed Fourier features of the frame) -> 3 x 512 tanh -> 1081 beams, BF16 "
           "tcgen05, FP32 Adam",
    "car_grid": "64 inputs (feature grids of the origin: 5 resolutions x 8 features; the frame; heading "
                "harmonics; 8 fixed Fourier features) -> 3 x 512 tanh -> 1081 beams, BF16 tcgen05, FP32 Adam"}


def surrogate_section(torch, W, track, stream, flush, train_steps=SURR_TRAIN_STEPS, keep=None, frame="world",
                      spot=True):
    """Learned lidar on bridge at 65536 cars: exact FP32 rollout vs BF16 surrogate rollout
    (audit every 16th step, exact fallback under 0.5 m), both device-timed like `value`. frame: the
    surrogate's output frame (world: world-angle profile read at the heading; car: one output per
    beam)."""
    keep = {} if keep is None else keep
    learned = W.Runner(track, SURR_CARS, beams=BEAMS, seed=7, stream=stream)
    sur = W.Surrogate(learned.sim, hidden=512, batch=8192, seed=1, frame=frame)
    sur.set_poses(1 << 22, seed=2)
    sur.set_loss(SURR_HUBER_M)
    t0 = time.perf_counter()
    sur.train(train_steps, lr=SURR_LR[frame])
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    heldout = sur.evaluate(8, 99)

    def timed(run):
        run(0)
        torch.cuda.synchronize()
        ms = 0.0
        for k in range(SURR_REPS):
            with torch.cuda.stream(stream):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                run((k + 1) * SURR_STEPS)
                b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        return SURR_CARS * SURR_STEPS * SURR_REPS / (ms / 1000.0)

    if "exact" not in keep:  # the exact baseline in its fastest rollout form, timed once
        exact = W.Runner(track, SURR_CARS, beams=BEAMS, seed=7, stream=stream)
        exact_chains, _ = exact.tune_chains(SURR_STEPS, 2)
        keep["exact"] = (timed(lambda t0: exact.rollout(SURR_STEPS, False, t0)), exact_chains)
        del exact
    exact_rate, exact_chains = keep["exact"]
    learned_rate = timed(lambda t0: learned.rollout_surrogate(sur, SURR_STEPS, False, t0, 16, 0.5))
    mae, rmse, mx, over, fallback = sur.rollout_stats(reset=True)
    out = {"workload": f"{TRACK}, {SURR_CARS} cars, {BEAMS} beams, {SURR_STEPS}-step rollouts", "frame": frame,
           "exact_fp32_env_steps_per_s": exact_rate, "exact_rollout_chains": exact_chains,
           "surrogate_bf16_env_steps_per_s": learned_rate,
           "speedup": learned_rate / exact_rate, "audit_every": 16, "fallback_m": 0.5,
           "audited_mae_m": mae, "audited_rmse_m": rmse, "audited_max_m": mx, "audited_frac_over_5cm": over,
           "fallback_frac": fallback,
           "heldout_mae_m": heldout[0], "heldout_rmse_m": heldout[1], "heldout_max_m": heldout[2],
           "heldout_frac_over_5cm": heldout[3], "surrogate": SURR_NETWORK[frame],
           "training": f"{train_steps} Adam steps x 8192 poses from 2^22 drawn over drivable cells, exact-tracer "
                       f"labels, Huber loss ({SURR_HUBER_M} m), lr {SURR_LR[frame]} cosine-decayed, {train_s:.1f} s",
           "target_mae_m": 0.02}
    if spot:  # the same rules plus the spot check between audits (every 64th beam, rotating, 1 m)
        sur.set_spot_check(SPOT_STRIDE, SPOT_TOL_M)
        spot_rate = timed(lambda t0: learned.rollout_surrogate(sur, SURR_STEPS, False, t0, 16, 0.5))
        spot_stats = sur.rollout_stats(reset=True)
        sur.set_spot_check(0, SPOT_TOL_M)
        out["spot_check"] = {"stride": SPOT_STRIDE, "tolerance_m": SPOT_TOL_M, "env_steps_per_s": spot_rate,
                             "speedup": spot_rate / exact_rate, "audited_mae_m": spot_stats[0],
                             "audited_max_m": spot_stats[2], "fallback_frac": spot_stats[4],
                             "rule": "between audits every 64th beam of every car (offset rotating with the step) "
                                     "is traced exactly; a car with one off by more than the tolerance, too long "
                                     "or too short, takes the exact tracer"}
    keep["surrogate"] = sur  # trained once, reused by the training section
    return out


SURR_TRAIN_SEEDS, SURR_TRAIN_ROLLOUT = (42, 43, 44), 32


def surrogate_training_section(W, track, sur, iterations):
    """PPO with the learned lidar driving 65536-car PPO rollouts: bridge, 65536 cars x
    32-step rollouts at 1081 beams, `iterations` iterations of rollout + GAE + update per run, three
    seeds with exact observations and the same three with the surrogate's (audit every 16th step of
    training, exact fallback under 0.5 m; racer/ppo.mojo:187-337 per iteration, main.mojo:54-68 loop).
    The reward comes from the exact physics either way, so the mean reward per step of the last
    iterations compares the policies the two kinds of observation trained."""
    out = {"workload": f"{TRACK}, {SURR_CARS} cars x {SURR_TRAIN_ROLLOUT}-step rollouts, {BEAMS} beams, "
                       f"{iterations} iterations, seeds {list(SURR_TRAIN_SEEDS)}; surrogate: audit every 16th "
                       "step, fallback under 0.5 m"}
    for mode in ("exact", "surrogate"):
        runs = []
        if mode == "surrogate":
            sur.rollout_stats(reset=True)
        for seed in SURR_TRAIN_SEEDS:
            runner = W.Runner(track, SURR_CARS, beams=BEAMS, seed=seed, policy_seed=seed)
            trainer = W.Trainer(SURR_CARS, beams=BEAMS, rollout=SURR_TRAIN_ROLLOUT, stream=runner.sim.stream)
            if mode == "surrogate":
                sur.bind(runner.sim)
                trainer.set_surrogate(sur, audit_every=16, fallback_m=0.5)
            rewards, kls = [], []
            t0 = time.perf_counter()
            for it in range(iterations):
                rewards.append(trainer.rollout(runner.sim, runner.policy, runner.acts, it))
                kls.append(trainer.update(runner.policy))
            dt = time.perf_counter() - t0
            k = max(1, min(20, iterations // 5))
            runs.append({"seed": seed, "training_transitions_per_s": SURR_CARS * SURR_TRAIN_ROLLOUT * iterations / dt,
                         "reward_per_step_first": float(np.mean(rewards[:k])),
                         "reward_per_step_last": float(np.mean(rewards[-k:])), "kl_last": float(kls[-1]),
                         "finite": bool(np.isfinite(rewards).all() and np.isfinite(kls).all()), "seconds": dt})
            trainer.set_surrogate(None)
            del trainer, runner
        out[mode] = {"training_transitions_per_s": float(np.mean([r["training_transitions_per_s"] for r in runs])),
                     "reward_per_step_last_mean": float(np.mean([r["reward_per_step_last"] for r in runs])),
                     "reward_per_step_last_spread": float(np.ptp([r["reward_per_step_last"] for r in runs])),
                     "runs": runs}
        if mode == "surrogate":
            mae, rmse, mx, over, fallback = sur.rollout_stats()
            out[mode].update({"audited_mae_m": mae, "audited_frac_over_5cm": over, "fallback_frac": fallback})
    last_s, last_e = out["surrogate"]["reward_per_step_last_mean"], out["exact"]["reward_per_step_last_mean"]
    out["return_ratio_surrogate_vs_exact"] = last_s / last_e if last_e else None
    out["speedup"] = out["surrogate"]["training_transitions_per_s"] / out["exact"]["training_transitions_per_s"]
    return out


BATCH_TRACKS = ("flat", "ramp", "bank", "bridge", "occupancy")
BATCH_CARS = (1024, 4096, 16384, 32768, 65536)
BATCH_STEPS, BATCH_REPS = 16, 3


def batched_section(torch, W, stream, flush):
    """Five tracks with uneven car counts in one sim (one launch per kernel covers every segment), rollouts
    of BATCH_STEPS env steps from one CUDA graph, after the autotuner picked the lidar launch shape; against
    the same cars as five one-track sims whose rollout graphs run back to back."""
    tracks = [W.track(name) for name in BATCH_TRACKS]
    seeds = [100 + k for k in range(len(tracks))]
    total = sum(BATCH_CARS)
    batch = W.Runner.segments(tracks, BATCH_CARS, seeds, beams=BEAMS, policy_seed=42, stream=stream)
    batch.rollout(BATCH_STEPS, False, 0)  # cars leave the spawn poses
    torch.cuda.synchronize()
    default_shape = batch.sim.lidar_shape()
    default_ms = batch.profile_sim(5)[1]
    tuned, tuned_ms = batch.sim.autotune(5)

    def timed(run):
        run(0)
        torch.cuda.synchronize()
        ms = 0.0
        for k in range(BATCH_REPS):
            with torch.cuda.stream(stream):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                run((k + 1) * BATCH_STEPS)
                b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        return total * BATCH_STEPS * BATCH_REPS / (ms / 1000.0), ms / (BATCH_REPS * BATCH_STEPS)

    batched_rate, batched_ms = timed(lambda t0: batch.rollout(BATCH_STEPS, False, t0))
    phys_ms, lidar_ms, probes = batch.profile_sim(5)
    launches = batch.rollout_kernel_count(BATCH_STEPS)
    del batch
    separate = [W.Runner(t, c, beams=BEAMS, seed=s, policy_seed=42, stream=stream)
                for t, c, s in zip(tracks, BATCH_CARS, seeds)]
    for r in separate:
        r.rollout(BATCH_STEPS, False, 0)
    separate_rate, separate_ms = timed(lambda t0: [r.rollout(BATCH_STEPS, False, t0) for r in separate])
    per_track_lidar, per_track_probes = {}, {}
    for name, r, cars in zip(BATCH_TRACKS, separate, BATCH_CARS):
        _, lid_ms, probes_k = r.profile_sim(3)
        per_track_lidar[name] = lid_ms
        per_track_probes[name] = probes_k / (cars * BEAMS)
    return {"workload": ", ".join(f"{n} {c}" for n, c in zip(BATCH_TRACKS, BATCH_CARS)) +
                        f" cars ({total} in all), {BEAMS} beams, {BATCH_STEPS}-step rollouts from one CUDA graph",
            "batched_env_steps_per_s": batched_rate, "batched_ms_per_env_step": batched_ms,
            "separate_env_steps_per_s": separate_rate, "separate_ms_per_env_step": separate_ms,
            "speedup": batched_rate / separate_rate,
            "lidar_shape_default": dict(default_shape, order=[BATCH_TRACKS[k] for k in default_shape["order"]],
                                        ms=default_ms),
            "lidar_shape_autotuned": dict(tuned, order=[BATCH_TRACKS[k] for k in tuned["order"]], ms=tuned_ms),
            "batched_physics_ms": phys_ms, "batched_lidar_ms": lidar_ms,
            "probes_per_beam": probes / (total * BEAMS), "kernels_per_rollout": launches,
            "separate_lidar_ms": per_track_lidar, "separate_probes_per_beam": per_track_probes,
            "dominant_segment": max(per_track_lidar, key=per_track_lidar.get),
            "dominant_share": max(per_track_lidar.values()) / sum(per_track_lidar.values())}


TRAIN_TRACK, TRAIN_CARS, TRAIN_ROLLOUT, TRAIN_BEAMS = "bank", 16384, 64, 108


TRAIN_SEEDS = (42, 43, 44)


def training_section(W, iterations):
    """PPO on bank, 16384 cars x 64-step rollouts (batch 262144): BF16 tensor-core products vs FP32 from the
    same seeds (racer/ppo.mojo:187-337 per iteration; main.mojo:54-68 loop). Runs differ in accumulation
    order, so single trajectories diverge chaotically; three seeds per precision are reported."""
    out = {"workload": f"{TRAIN_TRACK}, {TRAIN_CARS} cars x {TRAIN_ROLLOUT}-step rollouts, {TRAIN_BEAMS} beams, "
                       f"{iterations} iterations of rollout + GAE + 4 epochs x 4 minibatches of clipped PPO + Adam, "
                       f"seeds {list(TRAIN_SEEDS)}"}
    track = W.track(TRAIN_TRACK)
    for precision in ("bf16", "fp32"):
        runs = []
        for seed in TRAIN_SEEDS:
            runner = W.Runner(track, TRAIN_CARS, beams=TRAIN_BEAMS, seed=seed, policy_seed=seed)
            runner.policy.set_precision(precision)
            state, obs = runner.sim.state.numpy(), runner.sim.obs.numpy()
            shape, _ = runner.sim.autotune(5)  # lidar launch shape (rewrites obs from the same frames)
            chains, _ = runner.tune_chains(64, 3)  # rollout chains (BF16 only), then back to the start state
            runner.sim.state.write(state)
            runner.sim.obs.write(obs)
            trainer = W.Trainer(TRAIN_CARS, beams=TRAIN_BEAMS, rollout=TRAIN_ROLLOUT, stream=runner.sim.stream)
            rewards, kls = [], []
            t0 = time.perf_counter()
            for it in range(iterations):
                rewards.append(trainer.rollout(runner.sim, runner.policy, runner.acts, it))
                kls.append(trainer.update(runner.policy))
            dt = time.perf_counter() - t0
            k = max(1, min(20, iterations // 5))
            runs.append({"seed": seed, "rollout_chains": chains, "lidar_shape": shape,
                         "training_transitions_per_s": TRAIN_CARS * TRAIN_ROLLOUT * iterations / dt,
                         "reward_per_step_first": float(np.mean(rewards[:k])),
                         "reward_per_step_last": float(np.mean(rewards[-k:])), "kl_last": float(kls[-1]),
                         "finite": bool(np.isfinite(rewards).all() and np.isfinite(kls).all()), "seconds": dt})
            del trainer, runner
        out[precision] = {"training_transitions_per_s": float(np.mean([r["training_transitions_per_s"] for r in runs])),
                          "reward_per_step_last_mean": float(np.mean([r["reward_per_step_last"] for r in runs])),
                          "reward_per_step_first_mean": float(np.mean([r["reward_per_step_first"] for r in runs])),
                          "runs": runs}
    last16, last32 = out["bf16"]["reward_per_step_last_mean"], out["fp32"]["reward_per_step_last_mean"]
    out["return_ratio_bf16_vs_fp32"] = last16 / last32 if last32 else None
    return out


def track_compile_section():
    """Track compilation (racer/track.py) on the GPU, timed end to end through the Python
    API (numpy host part, racer_track_ribbon / racer_track_image, assembly) and as the
    bare C-ABI call on prepared inputs, against the oracle's C++ restatement on the host
    cores; both must equal each other bit for bit."""
    import oracle
    from warporacer3d_gb300.tracks import compile as TC
    from warporacer3d_gb300.tracks import occupancy
    lib = __import__("warporacer3d_gb300").load_library()
    free, loop, ramps, x0, y0 = occupancy.corridor(0)
    cases = [(n, TC.builtin_route(n), None) for n in ("flat", "ramp", "bank", "bridge")]
    cases.append(("occupancy_2048", None, (free, loop, x0, y0, 0.05, ramps)))
    out = {}
    for name, rib, img in cases:
        if rib is not None:
            full, ref = (lambda: TC.ribbon(*rib)), (lambda: oracle.track_ribbon(*rib))
            inp = TC.RibbonInput(*rib)
            abi = lambda: TC.ribbon_grids(inp, lib.racer_track_ribbon)
        else:
            full, ref = (lambda: TC.compile_image(*img)), (lambda: oracle.track_image(*img))
            inp = TC.ImageInput(*img)
            abi = lambda: TC.image_grids(inp, lib.racer_track_image)
        full()
        ms, abi_ms = [], []
        for _ in range(5):
            t0 = time.perf_counter()
            a = full()
            ms.append((time.perf_counter() - t0) * 1e3)
            t0 = time.perf_counter()
            abi()
            abi_ms.append((time.perf_counter() - t0) * 1e3)
        t0 = time.perf_counter()
        b = ref()
        cpu_ms = (time.perf_counter() - t0) * 1e3
        out[name] = {"gpu_ms": round(statistics.median(ms), 2), "abi_ms": round(statistics.median(abi_ms), 2),
                     "oracle_ms": round(cpu_ms, 1), "cells": int(a[0]) * int(a[1]), "layers": int(a[7]),
                     "identical_to_oracle": bool(np.array_equal(a.view(np.uint32), b.view(np.uint32)))}
    out["oracle_threads"] = os.cpu_count()
    out["method"] = ("median of 5 compilations after one warm-up; gpu_ms from the route to the packed float32 "
                     "array, abi_ms the library call alone; the oracle once, OpenMP over cells")
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return
    import warporacer3d_gb300 as W
    track = W.track(TRACK)
    import oracle
    oracle.build()
    per_step = []
    for k in range(args.warmup + args.steps):
        res = cpu_baseline(track, seconds=4.0, max_steps=20)
        if k >= args.warmup:
            per_step.append(res)
    value = statistics.mean(r["value"] for r in per_step)
    line = {"metric": METRIC, "value": value, "unit": "env-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * CARS / value if value else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (built-in bridge track, seeded spawns)", "impl": "reference",
            "config": {"workload": WORKLOAD.replace(f"{HORIZON_STEPS}-env-step rollout per bench step",
                                                    "bounded sample of env steps per bench step"),
                       "track": TRACK, "cars": CARS, "beams": BEAMS,
                       "implementation": "CPU restatement of racer/sim.mojo + racer/ppo.mojo (the reference's "
                                         "Mojo/MAX toolchain is not installable here), OpenMP over cars"},
            "cpu_baseline": {k: per_step[-1][k] for k in ("cores", "kind", "sample")} | {"value": value,
                                                                                         "unit": "env-steps/s"},
            "e2e": {"value": value, "unit": "env-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    from warporacer3d_gb300.replicas import max_over_ranks, replica_seed, topology, whole_job_rate
    rank, world, local = topology()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__
    if rank == 0:
        __graft_entry__.build()  # one rank compiles; the others wait, then load the same files
    if dist:
        dist.barrier()
    if rank != 0:
        __graft_entry__.build()  # up to date by now: checks timestamps only
    import warporacer3d_gb300 as W

    track = W.track(TRACK)
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    if args.batched_only:
        print(json.dumps({"batched": batched_section(torch, W, stream, flush)}), flush=True)
        return
    if args.track_compile_only:
        print(json.dumps({"track_compile": track_compile_section()}), flush=True)
        return
    if args.surrogate_only:
        steps = args.surrogate_train_steps if args.surrogate_train_steps is not None else SURR_TRAIN_STEPS
        kept = {}
        out = {"surrogate": surrogate_section(torch, W, track, stream, flush, steps, kept, args.surrogate_frame)}
        if not args.no_training:
            out["surrogate_training"] = surrogate_training_section(W, track, kept["surrogate"],
                                                                   args.training_iterations)
        print(json.dumps(out), flush=True)
        return
    runner = W.Runner(track, CARS, beams=BEAMS, seed=replica_seed(42, rank), policy_seed=42, stream=stream)
    runner.rollout(50, False, 0)  # cars leave their spawn poses
    lidar_shape, _ = runner.sim.autotune(5)  # lidar launch shape (rewrites obs from the same frames)
    chains, _ = runner.tune_chains(50, 3)  # rollout graph: independent chains over car ranges, or the fused kernel
    kernels_per_rollout = runner.rollout_kernel_count(HORIZON_STEPS)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # warm-up
    for k in range(args.warmup):
        runner.rollout(HORIZON_STEPS, False, k * HORIZON_STEPS)
    barrier()

    # device-timed region: K rollouts, L2 flushed between them (outside the events)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with Clocks(local) as clocks:
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                runner.rollout(HORIZON_STEPS, False, (args.warmup + k) * HORIZON_STEPS)
                ends[k].record(stream)
        barrier()
        wall = time.perf_counter() - wall0
    device_ms = max_over_ranks(sum(s.elapsed_time(e) for s, e in zip(starts, ends)), dist, "cuda")
    env_steps = world * CARS * HORIZON_STEPS * args.steps
    value = whole_job_rate(CARS * HORIZON_STEPS * args.steps, world, device_ms / 1000.0)
    ms_per_step = device_ms / args.steps

    # end-to-end through the public API with host buffers
    state_host = torch.empty((11, CARS), dtype=torch.float32).pin_memory()
    state_host.copy_(torch.from_numpy(runner.sim.state.numpy()))
    out_host = torch.empty((2, CARS), dtype=torch.float32).pin_memory()
    barrier()
    e2e0 = time.perf_counter()
    for k in range(args.steps):
        runner.sim.state.write(state_host.numpy())
        runner.rollout(HORIZON_STEPS, False, 10**6 + k * HORIZON_STEPS)
        out_host[0].copy_(torch.from_numpy(runner.sim.reward.numpy()))
        out_host[1].copy_(torch.from_numpy(runner.sim.done.numpy()))
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - e2e0, dist, "cuda")
    e2e = {"value": env_steps / e2e_s, "unit": "env-steps/s", "h2d_bytes_per_step": 11 * CARS * 4,
           "d2h_bytes_per_step": 2 * CARS * 4}

    # roofline of the dominant kernel (lidar): algorithmic bytes from its own probe counts
    phys_ms, lidar_ms, probes = runner.profile_sim(20)
    layers = int(track[7])
    alg_bytes = probes * 8 * layers + CARS * BEAMS * 4 + CARS * 24
    achieved = alg_bytes / (lidar_ms / 1000.0) / 1e9
    peak, peak_kind = peaks()
    traffic = dram_traffic_per_launch()
    gather_gbs = W.gather_peak(GATHER_PEAK_BYTES, 20)
    roofline = {"kernel": "k_lidar_track", "bound": "l2-gather", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "peak_kind": "HBM copy (MEASURED_PEAKS.json)",
                "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": lidar_ms,
                "physics_launch_ms": phys_ms, "probes_per_beam": probes / (CARS * BEAMS),
                "l2_gather_peak": gather_gbs, "l2_frac": achieved / gather_gbs,
                "l2_gather_method": f"random independent 16-byte loads over a {GATHER_PEAK_BYTES >> 20} MB "
                                    "L2-resident buffer, 8 in flight per thread, 8 CTAs of 256 per SM "
                                    "(racer_gather_peak), measured in this run",
                "limiter": LIDAR_LIMITER,
                "note": "the lidar's cells (5.1 MB for bridge) are L2-resident (DRAM traffic in `traffic` is under "
                        "1% of the algorithmic bytes); algorithmic bytes are the 16 B per probe the kernel gathers "
                        "plus its obs writes. frac is against the HBM copy peak, l2_frac against the measured L2 "
                        "random-gather peak; neighbouring beams share cells, so L1 hits can lift l2_frac"}

    line = {"metric": METRIC, "value": value, "unit": "env-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 sim / bf16 policy",
            "data": "synthetic (built-in bridge track, seeded spawns)",
            "config": {"workload": WORKLOAD, "track": TRACK, "cars_per_gpu": CARS, "beams": BEAMS,
                       "sim_precision": "f32 (physics, lidar, sampling: bit-exact with the CPU restatement)",
                       "policy_precision": "bf16 operands, f32 accumulation (tcgen05); f32 master weights",
                       "env_steps_per_bench_step": HORIZON_STEPS, "l2": "flushed between timed steps (256 MB write)",
                       "parallelism": f"replicas x{world} (cars independent, no collective)",
                       "rollout_chains": chains, "lidar_shape": lidar_shape,
                       "rollout_kernel": "fused persistent kernel" if chains == 0 else
                                         f"chained graph of per-step kernels, {chains} chain(s) (autotuned against "
                                         "the fused persistent kernel, timed in `fused_rollout`)",
                       "policy": "tanh MLP 1086-64-64-3"},
            "beam_steps_per_s": value * BEAMS, "wall_s": wall, "gpu_launches": kernels_per_rollout * args.steps,
            "clocks": clocks.summary(), "e2e": e2e, "roofline": roofline}
    # the single-GPU sections: measured at N = 1 only (at N > 1 every GPU would repeat them while
    # all N are held, and only rank 0's line is printed)
    single = world == 1
    if single:
        line["fp32_policy"] = fp32_policy_section(torch, W, track, stream, flush, runner)
        line["fused_rollout"] = fused_rollout_section(torch, W, track, stream, flush, runner)
    if single:
        audit = runner.audit_dynamics(AUDIT_STEPS, False, 10 ** 9)
        audit["workload"] = f"{TRACK}, {CARS} cars, {AUDIT_STEPS} policy steps after the timed rollouts"
        audit["method"] = "each binary32 RK4 step re-integrated in FP64 on the GPU from the same state and actions"
        line["dynamics_fp64_audit"] = audit
    if single and not args.no_surrogate:
        del runner
        steps = args.surrogate_train_steps if args.surrogate_train_steps is not None else SURR_TRAIN_STEPS
        kept = {}
        line["surrogate_car_frame"] = surrogate_section(torch, W, track, stream, flush, steps, kept, "car_grid",
                                                        spot=False)
        line["surrogate"] = surrogate_section(torch, W, track, stream, flush, steps, kept, "world")
        if not args.no_training:
            line["surrogate_training"] = surrogate_training_section(W, track, kept["surrogate"],
                                                                    args.training_iterations)
            line["surrogate_training_return_ratio"] = line["surrogate_training"]["return_ratio_surrogate_vs_exact"]
        del kept
        sur = line["surrogate"]  # the metric's second half, at the top level of the line
        line["surrogate_env_steps_per_s"] = sur["surrogate_bf16_env_steps_per_s"]
        line["surrogate_speedup"] = sur["speedup"]
        line["surrogate_mae_m"] = sur["audited_mae_m"]
        line["surrogate_heldout_mae_m"] = sur["heldout_mae_m"]
    if single and not args.no_config1:
        line["config1"] = config1_section(torch, W, stream)
    if single and not args.no_batched:
        line["batched"] = batched_section(torch, W, stream, flush)
    if single and not args.no_training:
        line["training"] = training_section(W, args.training_iterations)
    if single and not args.no_track_compile:
        line["track_compile"] = track_compile_section()
    if single and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(track)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
