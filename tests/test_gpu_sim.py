"""GPU parity of the simulator kernels against the CPU oracle.

The CUDA simulator kernels and the oracle perform the same binary32
operations, so state, observations (lidar ranges included), rewards, done
flags and per-beam probe counts must be identical bit for bit, step after
step, on every built-in track and on the reference's corridor fixture.
"""
import math

import numpy as np
import pytest

import oracle as O
import warporacer3d_gb300 as W

pytestmark = pytest.mark.gpu


def same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def diff_report(name, a, b):
    a, b = np.asarray(a), np.asarray(b)
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
    return f"{name}: {len(bad)} of {a.size} differ; first {bad[:5].tolist()} gpu {a[tuple(bad[0])]} cpu {b[tuple(bad[0])]}"


def check_sim(gpu, cpu, what=""):
    for name in ("state", "obs", "reward", "done"):
        g = getattr(gpu, name).numpy()
        c = getattr(cpu, name)
        assert same(g, c), what + diff_report(name, g, c)


@pytest.mark.parametrize("name,beams,n", [("flat", 108, 96), ("ramp", 108, 96), ("bank", 108, 96),
                                          ("bridge", 108, 96), ("bridge", 1081, 40)])
def test_reset_and_steps_bit_exact(name, beams, n):
    track = W.track(name)
    gpu = W.Sim(track, n, 42, beams=beams)
    cpu = O.Sim(track, n, 42, beams=beams)
    gpu.reset()
    cpu.reset()
    check_sim(gpu, cpu, "reset ")
    rng = np.random.default_rng(7)
    for step in range(25):
        act = rng.uniform(-1.2, 1.2, (2, n)).astype(np.float32)
        act[1] = np.abs(act[1]) * (1 if step % 5 else -1)  # mostly throttle, sometimes brake
        gpu.actions.write(act)
        cpu.actions[:] = act
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step} ")


def test_timeouts_and_crashes_respawn_bit_exact():
    track = W.track("ramp")
    n = 64
    gpu, cpu = W.Sim(track, n, 3, beams=108), O.Sim(track, n, 3, beams=108)
    gpu.reset()
    cpu.reset()
    s = cpu.state.copy()
    s[O.STEPS, 1::2] = np.float32(2995)  # odd cars time out within a few steps
    s[O.HEADING, 0::2] += np.float32(np.pi / 2)  # even cars face the wall, 1.3 m away
    gpu.state.write(s)
    cpu.state[:] = s
    act = np.stack([np.zeros(n), np.ones(n)]).astype(np.float32)  # full throttle
    gpu.actions.write(act)
    cpu.actions[:] = act
    seen = set()
    for step in range(60):
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step} ")
        seen |= set(np.unique(cpu.done).tolist())
    assert {1.0, 2.0} <= seen, "both crashes and timeouts occurred"


def test_lidar_iterations_match_oracle():
    track = W.track("bridge")
    n, beams = 32, 1081
    gpu, cpu = W.Sim(track, n, 11, beams=beams), O.Sim(track, n, 11, beams=beams)
    gpu.reset()
    cpu.reset()
    it_gpu = W.DevArray.empty((beams, n), np.int32)
    it_cpu = np.zeros((beams, n), np.int32)
    gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs, iters=it_gpu)
    cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs, iters=it_cpu)
    check_sim(gpu, cpu)
    assert same(it_gpu.numpy(), it_cpu)
    assert 3 < it_cpu.mean() < 20


def test_corridor_on_gpu():
    """tests/test_mojo.mojo:58-92 run through the CUDA kernels."""
    track = O.corridor()
    n, beams = 4, 108
    sim = W.Sim(track, n, 1, beams=beams)
    ref = O.Sim(track, n, 1, beams=beams)
    s = np.zeros((O.STATE, n), np.float32)
    s[O.X], s[O.FRICTION], s[O.PROGRESS] = 1, 1, np.float32(0.5 / 0.15)
    s[O.HEADING, 1] = np.float32(math.pi)
    sim.state.write(s)
    ref.state[:] = s
    act = np.array([[0, 0, 0, 1], [0, 1, 1, 1]], np.float32)
    sim.actions.write(act)
    ref.actions[:] = act
    sim.step(sim.actions, sim.reward, sim.done, sim.obs)
    ref.step(ref.actions, ref.reward, ref.done, ref.obs)
    o = sim.obs.numpy()
    assert abs(o[4 + beams // 2, 0] * 10 - 7.1) <= 0.1
    assert abs(o[4 + beams // 2, 1] * 10 - 0.73) <= 0.1
    crashed = False
    for _ in range(60):
        sim.step(sim.actions, sim.reward, sim.done, sim.obs)
        ref.step(ref.actions, ref.reward, ref.done, ref.obs)
        check_sim(sim, ref)
        done = sim.done.numpy()
        assert done[0] == 0 and done[2] == 0 and done[3] == 0
        if done[1] == O.CRASH and not crashed:
            st = sim.state.numpy()
            assert st[O.STEPS, 1] == 0 and st[O.EPISODE, 1] == 1
            crashed = True
    assert crashed
    st = sim.state.numpy()
    assert st[O.SPEED, 2] == O.SPEED_MAX and st[O.X, 2] > 3.5 and abs(st[O.Y, 2]) < 1e-4
    assert abs(st[O.RETURN, 2] - 10 * (st[O.X, 2] - 1)) <= 0.01
    assert st[O.Y, 3] > 0.1 and st[O.X, 3] < st[O.X, 2]


def test_drive_parity_flat():
    """tests/test_mojo.mojo:111-123,229-233 (CPU/GPU drive parity, there within 3e-3; here exact)."""
    track = W.track("flat")
    n = 8
    gpu, cpu = W.Sim(track, n, 42), O.Sim(track, n, 42)
    gpu.reset()
    cpu.reset()
    act = np.array([[0.2] * 8, [1] * 8], np.float32)
    gpu.actions.write(act)
    cpu.actions[:] = act
    for _ in range(10):
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
    a = np.concatenate([cpu.state[:O.STEER + 1].ravel(), cpu.obs.ravel()])
    b = np.concatenate([gpu.state.numpy()[:O.STEER + 1].ravel(), gpu.obs.numpy().ravel()])
    assert np.allclose(a, b, atol=3e-3, rtol=0)
    assert same(a, b)


def test_sample_bit_exact():
    n = 300
    gpu = W.Sim(W.track("flat"), n, 5)
    cpu = O.Sim(W.track("flat"), n, 5)
    rng = np.random.default_rng(1)
    out = rng.normal(0, 0.3, (3, n)).astype(np.float32)
    ls = np.array([-0.5, -1.25], np.float32)
    o_dev, ls_dev = W.DevArray.empty((3, n)), W.DevArray.empty((2,))
    o_dev.write(out)
    ls_dev.write(ls)
    a_dev, lp_dev, v_dev = W.DevArray.empty((2, n)), W.DevArray.empty((n,)), W.DevArray.empty((n,))
    for det, step in ((0, 0), (0, 12345), (1, 7)):
        gpu.sample(o_dev, ls_dev, a_dev, lp_dev, v_dev, det, step)
        a, lp, v = np.zeros((2, n), np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
        cpu.sample(out, ls, a, lp, v, det, step)
        assert same(a_dev.numpy(), a) and same(lp_dev.numpy(), lp) and same(v_dev.numpy(), v)


def _rk4_f64_flat(prev, act):
    """FP64 RK4 of racer/sim.mojo:155-167,189-213 on a level surface (no slope terms)."""
    G, WB, dt = 9.81, 0.3302, 1.0 / 240.0
    x, y, h, s = (prev[k].astype(np.float64) for k in (O.X, O.Y, O.HEADING, O.SPEED))
    steer = prev[O.STEER].astype(np.float64)
    rate = np.float64(np.clip(act[0], -1, 1).astype(np.float32) * np.float32(3.2))
    accel = np.float64(np.clip(act[1], -1, 1).astype(np.float32) * np.float32(9.51))
    load = np.float64(np.float32(1.05) * prev[O.FRICTION]) * G

    def deriv(x, y, h, s, st):
        v = np.maximum(np.abs(s), 0.5) * np.where(s >= 0, 1.0, -1.0)
        lateral = np.clip(v * s * np.sin(st) / np.cos(st) / WB, -load, load)
        lon = np.sqrt(np.maximum(load * load - lateral * lateral, 0))
        return s * np.cos(h), s * np.sin(h), lateral / v, np.clip(accel, -lon, lon)

    for _ in range(4):
        k1 = deriv(x, y, h, s, steer)
        k2 = deriv(x + k1[0] * dt / 2, y + k1[1] * dt / 2, h + k1[2] * dt / 2, s + k1[3] * dt / 2, steer + rate * dt / 2)
        k3 = deriv(x + k2[0] * dt / 2, y + k2[1] * dt / 2, h + k2[2] * dt / 2, s + k2[3] * dt / 2, steer + rate * dt / 2)
        k4 = deriv(x + k3[0] * dt, y + k3[1] * dt, h + k3[2] * dt, s + k3[3] * dt, steer + rate * dt)
        x, y, h, s = ((p + (a + 2 * (b + c) + d) * dt / 6) for p, a, b, c, d in zip((x, y, h, s), k1, k2, k3, k4))
        s = np.clip(s, -5.0, 5.0)
        steer = np.clip(steer + rate * dt, -0.4189, 0.4189)
    return x, y, h, s


def test_rk4_audit_matches_numpy_fp64_on_flat():
    """The FP64 audit kernel's statistics equal a numpy FP64 re-integration of the same step."""
    n = 512
    run = W.Runner(W.track("flat"), n, beams=108, seed=9)
    for t in range(30):
        run.step(False, t)
    prev = run.sim.state.numpy()
    stats = run.audit_dynamics(1, step0=30)
    nxt, done, act = run.sim.state.numpy(), run.sim.done.numpy(), run.sim.actions.numpy()
    x, y, h, s = _rk4_f64_flat(prev, act)
    keep = done == 0
    dh = nxt[O.HEADING].astype(np.float64) - h
    dh -= 2 * np.pi * np.rint(dh / (2 * np.pi))
    pos = np.hypot(nxt[O.X] - x, nxt[O.Y] - y)[keep]
    head, spd = np.abs(dh)[keep], np.abs(nxt[O.SPEED] - s)[keep]
    assert stats["cars"] == keep.sum() > n // 2
    for key, ref in (("position", pos), ("heading", head), ("speed", spd)):
        assert stats[key + "_max_" + ("m" if key == "position" else "rad" if key == "heading" else "mps")] == \
            pytest.approx(ref.max(), rel=1e-3, abs=1e-12), key
        mean = stats[key + "_mean_" + ("m" if key == "position" else "rad" if key == "heading" else "mps")]
        assert mean == pytest.approx(ref.mean(), rel=1e-3, abs=1e-12), key
    assert 0 < stats["position_max_m"] < 1e-4


def test_rk4_audit_error_bounded_on_bank():
    """Binary32 RK4 stays within a micrometre-scale distance of FP64 per step on a sloped track."""
    run = W.Runner(W.track("bank"), 2048, beams=108, seed=4)
    stats = run.audit_dynamics(40)
    assert stats["cars"] > 40 * 2048 * 0.9
    assert stats["position_mean_m"] < 1e-5 and stats["position_max_m"] < 1e-3
    assert stats["speed_mean_mps"] < 1e-5 and stats["heading_mean_rad"] < 1e-5


GOLDEN_OCCUPANCY = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "occupancy_small.npz"


def check_segments(gpu, cpus, what=""):
    for name in ("state", "obs", "reward", "done"):
        g = getattr(gpu, name).numpy()
        for k, cpu in enumerate(cpus):
            lo, hi = gpu.car0[k], gpu.car0[k + 1]
            c = getattr(cpu, name)
            assert same(g[..., lo:hi], c), what + f"segment {k} " + diff_report(name, g[..., lo:hi], c)


def segment_tracks():
    return [W.track("flat"), W.track("bridge"), np.load(GOLDEN_OCCUPANCY)["track"], W.track("ramp")]


def test_segments_match_separate_oracle_sims():
    """A batch of four tracks (one an occupancy-image map with ramps) in one sim: every segment
    evolves bit for bit like the oracle's sim of that track alone; car counts straddle warps and blocks."""
    tracks, cars, seeds = segment_tracks(), [96, 70, 45, 33], [5, 6, 7, 8]
    gpu = W.Sim.segments(tracks, cars, seeds, beams=108)
    cpus = [O.Sim(t, c, s, beams=108) for t, c, s in zip(tracks, cars, seeds)]
    gpu.reset()
    for c in cpus:
        c.reset()
    check_segments(gpu, cpus, "reset ")
    rng = np.random.default_rng(3)
    for step in range(30):
        act = rng.uniform(-1.2, 1.2, (2, gpu.n)).astype(np.float32)
        act[1] = np.abs(act[1]) * (1 if step % 4 else -1)
        gpu.actions.write(act)
        for k, c in enumerate(cpus):
            c.actions[:] = act[:, gpu.car0[k]:gpu.car0[k + 1]]
            c.step(c.actions, c.reward, c.done, c.obs)
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        check_segments(gpu, cpus, f"step {step} ")


def test_lidar_shapes_and_autotune_keep_results():
    tracks, cars, seeds = segment_tracks(), [64, 40, 72, 20], [1, 2, 3, 4]
    a = W.Sim.segments(tracks, cars, seeds, beams=108)
    b = W.Sim.segments(tracks, cars, seeds, beams=108)
    a.reset()
    b.reset()
    rng = np.random.default_rng(5)
    shapes = [(2, 0, 0, [3, 1, 0, 2]), (8, 1, 0, None), (4, 1, 1, [2, 3, 1, 0]), (2, 0, 1, None),
              (2, 0, 1, [1, 0, 2, 3], 1), (2, 1, 1, None, 1), (4, 0, 1, [3, 2, 1, 0], 0, 1), "auto"]
    for shape in shapes:
        if shape == "auto":
            best, ms = b.autotune(3)
            assert best["cars_per_block"] in (2, 4, 8) and best["wide"] in (0, 1) and best["split"] in (0, 1)
            assert sorted(best["order"]) == [0, 1, 2, 3] and ms > 0 and b.lidar_shape() == best
        else:
            b.set_lidar_shape(*shape)
            assert b.lidar_shape()["order"] == (shape[3] or [0, 1, 2, 3])
        for _ in range(4):
            act = rng.uniform(-1, 1, (2, a.n)).astype(np.float32)
            a.actions.write(act)
            b.actions.write(act)
            a.step(a.actions, a.reward, a.done, a.obs)
            b.step(b.actions, b.reward, b.done, b.obs)
            assert same(a.obs.numpy(), b.obs.numpy()) and same(a.state.numpy(), b.state.numpy())
    with pytest.raises(W.RacerError):
        b.set_lidar_shape(3)
    with pytest.raises(W.RacerError):
        b.set_lidar_shape(4, 0, 0, [0, 0, 1, 2])
    with pytest.raises(W.RacerError):
        b.set_lidar_shape(4, 2)


def test_split_lidar_in_captured_rollouts():
    """Rollout graphs captured with per-segment lidar branches give the segment-table launch's results."""
    tracks, cars, seeds = segment_tracks(), [64, 40, 72, 20], [1, 2, 3, 4]
    runs = [W.Runner.segments(tracks, cars, seeds, beams=108) for _ in range(2)]
    runs[1].sim.set_lidar_shape(2, 0, 1, [2, 0, 3, 1], 1)
    for r in runs:
        r.rollout(12, False, 0)
        r.rollout(12, False, 12)
    assert same(runs[0].sim.obs.numpy(), runs[1].sim.obs.numpy())
    assert same(runs[0].sim.state.numpy(), runs[1].sim.state.numpy())


@pytest.mark.parametrize("beams", [1081, 108])
def test_one_track_lidar_shapes_bit_exact(beams):
    """Every launch shape of the one-track lidar kernel gives the oracle's ranges, including warps
    that take (car, beam) pairs across car boundaries (flat; 108 beams = 3.375 warps a car)."""
    track = W.track("bridge")
    n = 50 if beams == 1081 else 77
    cpu = O.Sim(track, n, 9, beams=beams)
    cpu.reset()
    for cars_per_block, dynamic, flat in ((2, 0, 0), (4, 0, 0), (8, 0, 0), (2, 1, 0), (2, 0, 1), (8, 0, 1)):
        for wide in (0, 1):
            gpu = W.Sim(track, n, 9, beams=beams)
            gpu.set_lidar_shape(cars_per_block, wide, 0, None, dynamic, flat)
            gpu.reset()
            check_sim(gpu, cpu, f"shape {cars_per_block}/{wide}/{dynamic}/{flat} ")


def test_synthetic_occupancy_map_bit_exact():
    """The 2048 x 2048 px corridor map (8 ramps, slope bound 2.5: long marches) at 1081 beams."""
    track = W.track("occupancy")
    n = 24
    gpu, cpu = W.Sim(track, n, 11, beams=1081), O.Sim(track, n, 11, beams=1081)
    gpu.reset()
    cpu.reset()
    check_sim(gpu, cpu, "reset ")
    act = np.tile(np.array([[0.1], [1.0]], np.float32), (1, n))
    for step in range(3):
        gpu.actions.write(act)
        cpu.actions[:] = act
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step} ")


def test_segment_runner_rollout_and_audit():
    tracks = [W.track("bank"), W.track("bridge")]
    run = W.Runner.segments(tracks, [300, 212], [1, 2], beams=108)
    run.rollout(8)
    run.synchronize()
    stats = run.audit_dynamics(4, step0=8)
    assert stats["cars"] > 0.9 * 4 * 512 and stats["position_max_m"] < 1e-4
    with pytest.raises(W.RacerError):
        W.Surrogate(run.sim)


def test_device_evaluate_matches_host_loop():
    """main.mojo:70-80's evaluation: graph-captured with device-side sums equals the host loop
    that reads reward and done after every step."""
    a = W.Runner(W.track("ramp"), 300, beams=108, seed=5, policy_seed=8)
    b = W.Runner(W.track("ramp"), 300, beams=108, seed=5, policy_seed=8)
    host_reward, host_crashes = a.evaluate(60)
    dev_reward, dev_crashes = b.evaluate_graph(60)
    assert dev_reward == pytest.approx(host_reward, rel=1e-12, abs=1e-15)
    assert dev_crashes == host_crashes
    assert same(a.sim.state.numpy(), b.sim.state.numpy())
    # a second call replays the captured graph from the state reached (offsets 60..119)
    r2, c2 = b.evaluate_graph(60, step0=60)
    reward, crashes = 0.0, 0  # the host loop over offsets 60..119
    for t in range(60, 120):
        a.step(True, t)
        reward += float(a.sim.reward.numpy().astype(np.float64).sum())
        crashes += int((a.sim.done.numpy() == W.CRASH).sum())
    assert r2 == pytest.approx(reward / (300 * 60), rel=1e-12, abs=1e-15) and c2 == crashes / 300


def test_snapshot_rows_and_serve_step():
    run = W.Runner(W.track("bridge"), 70, beams=108, seed=2)
    snap = run.serve_step(25, 80, reset=False, policy=False, tick=1)
    sim = run.sim
    rows = [sim.state.numpy(), sim.obs.numpy(), sim.actions.numpy(), sim.reward.numpy()[None], sim.done.numpy()[None]]
    assert snap.shape == (11 + 113 + 4, 70) and same(snap, np.concatenate(rows))
    assert np.all(snap[11 + 113] == np.float32(0.25)) and np.all(snap[11 + 113 + 1] == np.float32(0.8))
    snap2 = run.serve_step(0, 0, reset=True, policy=True, tick=2)
    assert same(snap2[:11], sim.state.numpy()) and same(snap2[-1], sim.done.numpy())


@pytest.mark.parametrize("n,beams,name", [(1, 2, "bridge"), (1, 1081, "ramp"), (33, 2, "bank"), (33, 1081, "bridge")])
def test_edge_sizes_bit_exact(n, beams, name):
    """One car, a warp and one, the minimum beam count (2) and the full 1081."""
    track = W.track(name)
    gpu, cpu = W.Sim(track, n, 4, beams=beams), O.Sim(track, n, 4, beams=beams)
    gpu.reset()
    cpu.reset()
    rng = np.random.default_rng(n + beams)
    for step in range(8):
        act = rng.uniform(-1, 1, (2, n)).astype(np.float32)
        gpu.actions.write(act)
        cpu.actions[:] = act
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step} ")


@pytest.mark.parametrize("name", ["bank", "bridge"])
def test_lidar_on_random_drivable_cells_bit_exact(name):
    """The lidar's per-cell layer choice for one and two layers, on clearance grids with 30% of
    cells undrivable (-1, 0, -0.5 or NaN) and the rest drawn up to 3 m, so that every combination
    of drivable layers occurs and long steps carry rays off the map; cars start anywhere on the
    map and up to 2 m beyond its edges."""
    base = W.track(name)
    nx, ny, L = int(base[0]), int(base[1]), int(base[7])
    x0, y0, cell = float(base[2]), float(base[3]), float(base[4])
    rng = np.random.default_rng(17 + L)
    track = base.copy()
    cells = nx * ny
    for l in range(L):
        c = track[12 + 3 * l * cells:12 + (3 * l + 1) * cells]
        c[:] = rng.uniform(0.02, 3.0, cells).astype(np.float32)
        bad = rng.random(cells) < 0.3
        c[bad] = rng.choice(np.array([-1.0, 0.0, -0.5, np.nan], np.float32), int(bad.sum()))
    n, beams = 512, 1081
    gpu, cpu = W.Sim(track, n, 3, beams=beams), O.Sim(track, n, 3, beams=beams)
    gpu.reset()
    cpu.reset()
    check_sim(gpu, cpu, "reset ")
    s = gpu.state.numpy()
    s[O.X] = rng.uniform(x0 - 2, x0 + nx * cell + 2, n).astype(np.float32)
    s[O.Y] = rng.uniform(y0 - 2, y0 + ny * cell + 2, n).astype(np.float32)
    ix = np.clip(np.round((s[O.X] - x0) / cell), 0, nx - 1).astype(np.int64)
    iy = np.clip(np.round((s[O.Y] - y0) / cell), 0, ny - 1).astype(np.int64)
    layer = rng.integers(0, L, n)
    s[O.Z] = track[12 + (3 * layer + 1) * cells + iy * nx + ix] + rng.uniform(-0.2, 1.0, n).astype(np.float32)
    s[O.HEADING] = rng.uniform(-math.pi, math.pi, n).astype(np.float32)
    s[O.SPEED] = rng.uniform(0, 2, n).astype(np.float32)
    gpu.state.write(s)
    cpu.state[:] = s
    for step in range(3):
        act = rng.uniform(-1, 1, (2, n)).astype(np.float32)
        gpu.actions.write(act)
        cpu.actions[:] = act
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step} ")
    ranges = gpu.obs.numpy()[4:]
    assert (ranges == 1.0).any() and (ranges < 0.1).any()


def three_layer_track():
    """bridge's two layers plus a third: layer 0 raised 2.5 m with 40% of its cells undrivable."""
    base = W.track("bridge")
    nx, ny = int(base[0]), int(base[1])
    cells = nx * ny
    grids = base[12:12 + 6 * cells]
    third = grids[:3 * cells].copy()
    third[cells:2 * cells] += np.float32(2.5)
    rng = np.random.default_rng(23)
    third[:cells][rng.random(cells) < 0.4] = np.float32(-1)
    head = base[:12].copy()
    head[7] = 3
    return np.concatenate([head, grids, third, base[12 + 6 * cells:]]).astype(np.float32)


def test_three_layer_track_bit_exact():
    """The probe of three or more layers (the layer count read from the track), alone and as a
    segment beside a one-layer track."""
    track = three_layer_track()
    n, beams = 96, 1081
    gpu, cpu = W.Sim(track, n, 6, beams=beams), O.Sim(track, n, 6, beams=beams)
    gpu.reset()
    cpu.reset()
    check_sim(gpu, cpu, "reset ")
    rng = np.random.default_rng(6)
    for step in range(5):
        act = rng.uniform(-1, 1, (2, n)).astype(np.float32)
        gpu.actions.write(act)
        cpu.actions[:] = act
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        check_sim(gpu, cpu, f"step {step} ")
    tracks, cars, seeds = [W.track("bank"), track], [40, 70], [3, 4]
    seg = W.Sim.segments(tracks, cars, seeds, beams=108)
    cpus = [O.Sim(t, c, s, beams=108) for t, c, s in zip(tracks, cars, seeds)]
    seg.reset()
    for c in cpus:
        c.reset()
    for step in range(4):
        act = rng.uniform(-1, 1, (2, seg.n)).astype(np.float32)
        seg.actions.write(act)
        for k, c in enumerate(cpus):
            c.actions[:] = act[:, seg.car0[k]:seg.car0[k + 1]]
            c.step(c.actions, c.reward, c.done, c.obs)
        seg.step(seg.actions, seg.reward, seg.done, seg.obs)
        check_segments(seg, cpus, f"step {step} ")


def test_car_trajectory_independent_of_batch_size():
    """Size-independent property at 262144 cars: car i's state depends only on its seed, index and
    actions, so the first 1000 cars of a 262144-car sim equal a 1000-car sim bit for bit."""
    track = W.track("ramp")
    big, small = W.Sim(track, 262144, 8, beams=108), W.Sim(track, 1000, 8, beams=108)
    big.reset()
    small.reset()
    rng = np.random.default_rng(2)
    for _ in range(6):
        act = rng.uniform(-1, 1, (2, 262144)).astype(np.float32)
        big.actions.write(act)
        small.actions.write(np.ascontiguousarray(act[:, :1000]))
        big.step(big.actions, big.reward, big.done, big.obs)
        small.step(small.actions, small.reward, small.done, small.obs)
    assert same(big.state.numpy()[:, :1000], small.state.numpy())
    assert same(big.obs.numpy()[:, :1000], small.obs.numpy())


def test_eight_segments_bit_exact():
    """The segment table at its maximum of eight tracks."""
    names = ["flat", "ramp", "bank", "bridge", "flat", "bridge", "ramp", "bank"]
    tracks = [W.track(t) for t in names[:7]] + [np.load(GOLDEN_OCCUPANCY)["track"]]
    cars, seeds = [5, 40, 1, 64, 31, 2, 17, 9], list(range(10, 18))
    gpu = W.Sim.segments(tracks, cars, seeds, beams=108)
    cpus = [O.Sim(t, c, s, beams=108) for t, c, s in zip(tracks, cars, seeds)]
    gpu.reset()
    for c in cpus:
        c.reset()
    rng = np.random.default_rng(9)
    for step in range(6):
        act = rng.uniform(-1, 1, (2, gpu.n)).astype(np.float32)
        gpu.actions.write(act)
        for k, c in enumerate(cpus):
            c.actions[:] = act[:, gpu.car0[k]:gpu.car0[k + 1]]
            c.step(c.actions, c.reward, c.done, c.obs)
        gpu.step(gpu.actions, gpu.reward, gpu.done, gpu.obs)
        check_segments(gpu, cpus, f"step {step} ")


def test_gather_peak_is_plausible():
    """The L2 random-gather roofline: far above zero, and an L2-resident buffer gathers faster than
    one eight times the L2's size, whose loads must come from HBM."""
    l2 = W.gather_peak(8 << 20, 10)
    hbm = W.gather_peak(256 << 20, 5)
    assert 500 < hbm < l2 < 100000, (l2, hbm)


@pytest.mark.parametrize("name,n,beams", [("bridge", 40, 1081), ("bridge", 4096, 1081), ("ramp", 1024, 108),
                                          ("flat", 700, 108), ("bank", 333, 2), ("bridge", 65536, 1081)])
def test_fused_rollout_equals_chained_graph(name, n, beams):
    """The fused persistent rollout kernel (forward + sampling, physics and lidar of a slice of cars
    per CTA, all steps in one launch) gives the chained graph's bits: state, observations, actions,
    rewards, done flags and the policy outputs, over 12 steps; car counts that fill a CTA's slice
    unevenly, one car per CTA, the minimum beam count, and more CTAs than fit on the GPU at once
    (65536 cars: 512 CTAs of 128)."""
    track = W.track(name)
    chained = W.Runner(track, n, beams=beams, seed=13, policy_seed=5)
    fused = W.Runner(track, n, beams=beams, seed=13, policy_seed=5)
    fused.sim.set_fused_rollout(True)
    assert fused.rollout_kernel_count(12) == 2  # one launch of the fused kernel, plus the step offset
    for runner in (chained, fused):
        runner.rollout(12, False, 40)
        runner.rollout(12, False, 52)  # a replay of the captured graph from the state reached
        runner.synchronize()
    for arr in ("state", "obs", "actions", "reward", "done"):
        assert same(getattr(chained.sim, arr).numpy(), getattr(fused.sim, arr).numpy()), arr
    assert same(chained.acts.o.numpy(), fused.acts.o.numpy())
    assert same(chained.scratch.numpy(), fused.scratch.numpy())
    assert fused.policy.status() == 0


def test_fused_rollout_on_three_layers_and_deterministic():
    """Three layers (the probe reads the layer count from the track) and deterministic actions."""
    track = three_layer_track()
    chained = W.Runner(track, 200, beams=1081, seed=2, policy_seed=3)
    fused = W.Runner(track, 200, beams=1081, seed=2, policy_seed=3)
    fused.sim.set_fused_rollout(True)
    for runner in (chained, fused):
        runner.rollout(6, True, 0)
        runner.synchronize()
    for arr in ("state", "obs", "actions"):
        assert same(getattr(chained.sim, arr).numpy(), getattr(fused.sim, arr).numpy()), arr
