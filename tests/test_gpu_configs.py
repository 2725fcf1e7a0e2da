"""Parity at the benchmark workloads' own sizes.

The other GPU tests check every kernel on small batches; these run the
shapes the benchmark measures, where different launch paths are taken:

- the reference's CPU-runnable benchmark (`racer benchmark ramp cpu 1024
  1000`): ramp, 1024 cars, 108 beams, sim seed 0;
- the headline workload: bridge, 4096 cars, 1081 beams, and its rollout graph
  of independent chains over car ranges;
- the policy forward at 65536 and 119,808 samples (the learned-lidar rollout
  and the uneven five-track batch), where the tiles of 128 samples outnumber
  the SMs and the persistent, TMA-staged forward runs;
- one Runner step of 65536 cars on bridge at 1081 beams (forward with its
  fused sampling, physics, lidar) against the oracle;
- the learned-lidar rollout at 65536 cars with every step audited, which must
  be the exact rollout.

Simulator results are compared bit for bit; the BF16 policy forward within
the forward tolerance of tests/test_gpu_policy.py.
"""
import numpy as np
import pytest

import oracle as O
import warporacer3d_gb300 as W

pytestmark = pytest.mark.gpu

FWD_ATOL, FWD_RTOL = 2e-2, 2e-2  # |gpu - oracle| <= FWD_ATOL + FWD_RTOL * |oracle|, as tests/test_gpu_policy.py


def same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def check_sim(gpu, cpu, what=""):
    for name in ("state", "obs", "reward", "done"):
        g, c = getattr(gpu, name).numpy(), getattr(cpu, name)
        if not same(g, c):
            bad = np.argwhere(~((g == c) | (np.isnan(g) & np.isnan(c))))
            raise AssertionError(f"{what}{name}: {len(bad)} of {g.size} differ, first {bad[:3].tolist()}")


def drive(gpu, cpu, steps, seed):
    """`steps` sim steps with the same random actions on both sides, compared after each."""
    rng = np.random.default_rng(seed)
    n = gpu.n
    for step in range(steps):
        act = rng.uniform(-1.1, 1.1, (2, n)).astype(np.float32)
        act[1] = np.abs(act[1]) * (1 if step % 4 else -1)
        gpu.actions.write(act)
        cpu.actions[:] = act
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step}: ")


def test_ramp_1024_cars_108_beams_seed0_bit_exact():
    """ramp, 1024 cars, 108 beams, sim seed 0: reset and 12 steps."""
    track = W.track("ramp")
    gpu, cpu = W.Sim(track, 1024, 0, beams=108), O.Sim(track, 1024, 0, beams=108)
    gpu.reset()
    cpu.reset()
    check_sim(gpu, cpu, "reset: ")
    drive(gpu, cpu, 12, 1)


def test_bridge_4096_cars_1081_beams_bit_exact():
    """bridge, 4096 cars, 1081 beams: reset and 8 steps."""
    track = W.track("bridge")
    gpu, cpu = W.Sim(track, 4096, 42, beams=1081), O.Sim(track, 4096, 42, beams=1081)
    gpu.reset()
    cpu.reset()
    check_sim(gpu, cpu, "reset: ")
    drive(gpu, cpu, 8, 2)


@pytest.mark.parametrize("chains", [4, 8, 16])
def test_bridge_4096_chained_rollout_graph_equals_step_loop(chains):
    """The benchmark's rollout (one CUDA graph of independent chains over car ranges) gives the bits of
    the reference's host loop of Runner steps, at 4096 cars and 1081 beams."""
    track = W.track("bridge")
    graph = W.Runner(track, 4096, beams=1081, seed=42, policy_seed=42)
    loop = W.Runner(track, 4096, beams=1081, seed=42, policy_seed=42)
    graph.sim.set_chains(chains)
    graph.rollout(10, False, 100)
    for t in range(10):
        loop.step(False, 100 + t)
    for name in ("state", "obs", "reward", "done", "actions"):
        assert same(getattr(graph.sim, name).numpy(), getattr(loop.sim, name).numpy()), name


@pytest.mark.parametrize("cols", [65536, 119808])
def test_persistent_policy_forward_at_config_sizes(cols):
    """1081 beams (1086 inputs), 512 or 936 tiles of 128 samples on the GPU's SMs: the persistent,
    TMA-staged forward against the oracle, and its first 1000 samples bit-equal to the
    one-tile-per-CTA forward of a 1000-sample batch."""
    beams = 1081
    g, c = W.Policy(11, beams=beams), O.Policy(11, beams=beams)
    rng = np.random.default_rng(cols)
    x = np.empty((beams + 5, cols), np.float32)
    x[:4] = rng.uniform(-1, 1, (4, cols))
    x[4:4 + beams] = rng.uniform(0, 1, (beams, cols))  # lidar rows: ranges / 10 m
    x[-1] = 1
    xd = W.DevArray.empty(x.shape)
    xd.write(x)
    ga, ca = W.Activations(g, cols), O.Activations(cols)
    g.forward(xd, ga)
    c.forward(x, ca)
    for name in ("h1", "h2", "o"):
        a, b = getattr(ga, name).numpy(), getattr(ca, name)
        err = np.abs(a - b)
        assert np.all(err <= FWD_ATOL + FWD_RTOL * np.abs(b)), (name, err.max())
    small = W.DevArray.empty((beams + 5, 1000))
    small.write(np.ascontiguousarray(x[:, :1000]))
    sa = W.Activations(g, 1000)
    g.forward(small, sa)
    for name in ("h1", "h2", "o"):
        assert same(getattr(sa, name).numpy(), getattr(ga, name).numpy()[:, :1000]), name
    assert g.status() == 0


def test_runner_step_65536_cars_against_oracle():
    """One Runner step (main.mojo:40-48) of 65536 cars on bridge at 1081 beams, the learned-lidar
    workload's size: the policy outputs within the forward tolerance of the oracle's forward on the
    same observations, the fused sampling bit-exact given those outputs, and the sim step bit-exact."""
    n, beams = 65536, 1081
    track = W.track("bridge")
    run = W.Runner(track, n, beams=beams, seed=7, policy_seed=42)
    cpu = O.Sim(track, n, 7, beams=beams)
    cpu.reset()
    check_sim(run.sim, cpu, "reset: ")
    obs = run.sim.obs.numpy()
    run.step(False, 5)
    pol = O.Policy(42, beams=beams)
    acts = O.Activations(n)
    pol.forward(obs, acts)
    o = run.acts.o.numpy()
    err = np.abs(o - acts.o)
    assert np.all(err <= FWD_ATOL + FWD_RTOL * np.abs(acts.o)), err.max()
    actions, logp, value = np.zeros((2, n), np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
    cpu.sample(o, pol.log_std(), actions, logp, value, False, 5)
    scratch = run.scratch.numpy()
    assert same(run.sim.actions.numpy(), actions) and same(scratch[0], logp) and same(scratch[1], value)
    cpu.actions[:] = actions
    cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
    check_sim(run.sim, cpu, "step: ")
    assert run.policy.status() == 0


def test_surrogate_rollout_audited_every_step_is_exact_at_65536_cars():
    """The learned-lidar rollout of the benchmark's size with an audit on every step: the exact
    tracer rewrites every car's ranges, so the rollout is the exact rollout, bit for bit."""
    n, beams = 65536, 1081
    track = W.track("bridge")
    exact = W.Runner(track, n, beams=beams, seed=7)
    learned = W.Runner(track, n, beams=beams, seed=7)
    sur = W.Surrogate(learned.sim, hidden=512, batch=8192, seed=1)
    exact.rollout(4, False, 0)
    learned.rollout_surrogate(sur, 4, False, 0, audit_every=1, fallback_m=0.5)
    learned.synchronize()
    for name in ("state", "obs", "reward", "done", "actions"):
        assert same(getattr(exact.sim, name).numpy(), getattr(learned.sim, name).numpy()), name
    mae, rmse, mx, over, fb = sur.rollout_stats()
    assert mae > 0 and rmse >= mae and mx >= rmse
