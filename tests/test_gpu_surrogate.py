"""The learned lidar surrogate: its labels, its gradient, and its training.

- Labels: the exact tracer's ranges for a car at rest at each training pose
  are bit-identical to the CPU oracle's scan of the same car.
- Gradient: the GPU backward (tcgen05 GEMMs, BF16 operands, FP32
  accumulation) matches a float64 numpy backprop of the same network with the
  same BF16 roundings, within 2e-2 relative (Frobenius) per parameter block,
  in the car frame and in the world frame (its feature grids included).
- World frame: the inputs and the heading offsets match a float64
  recomputation, and inference reads each beam from the world profile at the
  heading's offset.
- Training: a few hundred Adam steps cut the held-out error against the exact
  tracer substantially.
- Gain: a briefly trained surrogate, with its audits and per-car fallback to
  the exact tracer, rolls out faster than the exact tracer alone.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
import warporacer3d_gb300 as W

pytestmark = pytest.mark.gpu


def bf16(x):
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return r.view(np.float32).astype(np.float64)


def rest_frames(track, poses):
    """Per pose (x, y, heading, layer): height, slopes along/across and the lidar origin, in binary32."""
    L = O.lib()
    d = np.ascontiguousarray(track, np.float32)
    out = []
    for x, y, h, layer in poses:
        g = np.zeros(3, np.float32)
        L.orc_surface(d, int(layer), float(x), float(y), g)
        s, c = np.zeros(1, np.float32), np.zeros(1, np.float32)
        L.orc_sincos(np.array([h], np.float32), 1, s, c)
        s, c = s[0], c[0]
        along = g[1] * c + g[2] * s
        across = -g[1] * s + g[2] * c
        f32 = np.float32
        ox = (f32(x) + f32(0.27) * c) + f32(0)
        oy = (f32(y) + f32(0.27) * s) + f32(0)
        oz = (g[0] + f32(0.27) * along) + f32(0.23)
        out.append((g[0], along, across, ox, oy, oz, s, c))
    return np.array(out, np.float32)


def test_labels_match_oracle_scan():
    track = W.track("bridge")
    beams, B = 1081, 256
    sim = W.Sim(track, 8, 0, beams=beams)
    sur = W.Surrogate(sim, hidden=128, batch=B, seed=3)
    sur.set_poses(B, seed=5)
    labels = W.DevArray.empty((beams, B))
    sur.gradient(0, labels)
    poses = sur.poses().numpy()
    fr = rest_frames(track, poses)
    cpu = O.Sim(track, B, 0, beams=beams)
    cpu.state[O.X], cpu.state[O.Y], cpu.state[O.Z] = poses[:, 0], poses[:, 1], fr[:, 0]
    cpu.state[O.HEADING] = poses[:, 2]
    cpu.obs[2], cpu.obs[3] = fr[:, 1], fr[:, 2]
    cpu.lidar(cpu.obs)
    assert np.array_equal(labels.numpy(), cpu.obs[4:4 + beams])
    assert set(np.unique(poses[:, 3]).tolist()) <= {0.0, 1.0}


def test_gradient_matches_float64_backprop():
    track = W.track("bridge")
    beams, B, H = 1081, 256, 128
    sim = W.Sim(track, 8, 0, beams=beams)
    sur = W.Surrogate(sim, hidden=H, batch=B, seed=3)
    sur.set_poses(B, seed=9)
    labels = W.DevArray.empty((beams, B))
    sur.gradient(0, labels)
    T = labels.numpy().T.astype(np.float64)  # [B, beams]
    theta = sur.theta.numpy()
    grad = sur.grad.numpy()
    lay = sur.layout()
    P = {k: theta[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in lay.items()}
    poses = sur.poses().numpy()
    fr = rest_frames(track, poses)
    nx, ny, x0, y0, cell = track[0], track[1], track[2], track[3], track[4]
    hx, hy = np.float32(0.5) * np.float32(nx - 1) * cell, np.float32(0.5) * np.float32(ny - 1) * cell
    xn = (fr[:, 3] - (x0 + hx)) * (np.float32(1) / hx)
    yn = (fr[:, 4] - (y0 + hy)) * (np.float32(1) / hy)
    z, sh, ch = fr[:, 5], fr[:, 6], fr[:, 7]
    cols = [xn, yn, z, sh, ch, poses[:, 3] == 0, poses[:, 3] == 1, np.ones(B)]
    for k in range(10):
        a, b = np.pi * 2.0 ** k * xn.astype(np.float64), np.pi * 2.0 ** k * yn.astype(np.float64)
        cols += [np.sin(a), np.cos(a), np.sin(b), np.cos(b)]
    h = np.arctan2(sh.astype(np.float64), ch.astype(np.float64))
    for j in range(2, 6):
        cols += [np.sin(j * h), np.cos(j * h)]
    cols += [np.sin(np.pi * z), np.cos(np.pi * z), np.sin(2 * np.pi * z), np.cos(2 * np.pi * z)]
    cols += [np.zeros(B)] * 4
    X = bf16(np.stack(cols, 1).astype(np.float32))
    Wb = {k: bf16(P[k]) for k in ("W1", "W2", "W3", "W4")}
    h1 = bf16(np.tanh(X @ Wb["W1"].T))
    h2 = bf16(np.tanh(h1 @ Wb["W2"].T + P["b2"]))
    h3 = bf16(np.tanh(h2 @ Wb["W3"].T + P["b3"]))
    y = h3 @ Wb["W4"].T + P["b4"]
    g4 = bf16(2.0 / (B * beams) * (y - T))
    g3 = bf16((g4 @ Wb["W4"]) * (1 - h3 * h3))
    g2 = bf16((g3 @ Wb["W3"]) * (1 - h2 * h2))
    g1 = bf16((g2 @ Wb["W2"]) * (1 - h1 * h1))
    ref = {"W4": g4.T @ h3, "b4": g4.sum(0), "W3": g3.T @ h2, "b3": g3.sum(0), "W2": g2.T @ h1, "b2": g2.sum(0),
           "W1": g1.T @ X}
    for k, r in ref.items():
        o, s = lay[k]
        g = grad[o:o + int(np.prod(s))].reshape(s)
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel < 2e-2, (k, rel)


FOV = 4.71238898


def world_setup(hidden=128, B=256, steps=20, frame="world"):
    """A briefly trained grid surrogate (world frame, or car frame with grids) on bridge at 1081 beams
    and the gradient of its batch 0."""
    track = W.track("bridge")
    beams = 1081
    sim = W.Sim(track, 8, 0, beams=beams)
    sur = W.Surrogate(sim, hidden=hidden, batch=B, seed=3, frame=frame)
    sur.set_poses(4 * B, seed=9)
    sur.train(steps, lr=3e-3)  # grids and weights away from their initial values
    labels = W.DevArray.empty((beams, B))
    sur.gradient(0, labels)
    return track, sim, sur, labels.numpy().T.astype(np.float64)


def grid_corners(sur, track, ox, oy):
    """Per level: cell (iu, iv) and fractions (fu, fv) of the bilinear lookup, in float64."""
    gx, gy, sp, offs = sur.grid()
    x0, y0 = float(track[2]), float(track[3])
    out = []
    for l in range(W.Surrogate.GRID_LEVELS):
        u = np.clip((ox.astype(np.float64) - x0) / sp[l], 0, gx[l] - 2)
        v = np.clip((oy.astype(np.float64) - y0) / sp[l], 0, gy[l] - 2)
        iu = np.minimum(np.floor(u).astype(int), gx[l] - 3)
        iv = np.minimum(np.floor(v).astype(int), gy[l] - 3)
        out.append((iu, iv, u - iu, v - iv))
    return out


def world_forward(sur, P, X):
    Wb = {k: bf16(P[k]) for k in ("W1", "W2", "W3", "W4")}
    h1 = bf16(np.tanh(X @ Wb["W1"].T))
    h2 = bf16(np.tanh(h1 @ Wb["W2"].T + P["b2"]))
    h3 = bf16(np.tanh(h2 @ Wb["W3"].T + P["b3"]))
    return Wb, h1, h2, h3, h3 @ Wb["W4"].T + P["b4"]


def test_world_frame_inputs_and_gradient_match_float64():
    """The world frame's encoded inputs (feature grids at the lidar origin, Fourier features, heading
    phase) match a float64 recomputation within BF16 rounding, its first world samples the heading's
    offset, and the GPU gradient (world loss read through each sample's offset, the GEMM chain, the
    input gradient scattered onto the grids) matches a float64 backprop with the same BF16 roundings
    within 2e-2 relative (Frobenius) per block."""
    track, sim, sur, T = world_setup()
    B, beams, K = sur.batch, sim.beams, sur.nout
    X, k0 = sur.batch_inputs()
    theta, grad = sur.theta.numpy(), sur.grad.numpy()
    lay = sur.layout()
    P = {k: theta[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in lay.items()}
    poses = sur.poses().numpy()[:B]
    fr = rest_frames(track, poses)
    ox, oy, oz, sh, ch = fr[:, 3], fr[:, 4], fr[:, 5], fr[:, 6], fr[:, 7]
    layer = poses[:, 3].astype(int)
    # first world sample and phase
    u = np.mod((np.arctan2(sh.astype(np.float64), ch.astype(np.float64)) - FOV / 2) * K / (2 * np.pi), K)
    clear = np.abs(u - np.round(u)) > 1e-3
    assert clear.sum() > 0.9 * B
    assert np.array_equal(k0[clear], np.floor(u[clear]).astype(int) % K)
    # inputs
    corners = grid_corners(sur, track, ox, oy)
    ref = np.zeros((B, 64))
    for l, (iu, iv, fu, fv) in enumerate(corners):
        G = P[f"G{l}"]
        ref[:, 8 * l:8 * l + 8] = (G[layer, iv, iu] * ((1 - fu) * (1 - fv))[:, None] +
                                   G[layer, iv, iu + 1] * (fu * (1 - fv))[:, None] +
                                   G[layer, iv + 1, iu] * ((1 - fu) * fv)[:, None] +
                                   G[layer, iv + 1, iu + 1] * (fu * fv)[:, None])
    nx, ny, x0, y0, cell = track[0], track[1], track[2], track[3], track[4]
    hx, hy = np.float32(0.5) * np.float32(nx - 1) * cell, np.float32(0.5) * np.float32(ny - 1) * cell
    xn = ((ox - (x0 + hx)) * (np.float32(1) / hx)).astype(np.float64)
    yn = ((oy - (y0 + hy)) * (np.float32(1) / hy)).astype(np.float64)
    ref[:, 40:46] = np.stack([xn, yn, oz, layer == 0, layer == 1, np.ones(B)], 1)
    for k in range(4):
        a, b = np.pi * 2.0 ** k * xn, np.pi * 2.0 ** k * yn
        ref[:, 46 + 4 * k:50 + 4 * k] = np.stack([np.sin(a), np.cos(a), np.sin(b), np.cos(b)], 1)
    ref[:, 62], ref[:, 63] = np.sin(2 * np.pi * (u - np.floor(u))), np.cos(2 * np.pi * (u - np.floor(u)))
    err = np.abs(X - ref)
    assert np.all(err[clear] <= 2e-3 + 8e-3 * np.abs(ref[clear])), err[clear].max()
    # backprop
    Wb, h1, h2, h3, y = world_forward(sur, P, X.astype(np.float64))
    idx = (k0[:, None] + np.arange(beams)) % K
    G4 = np.zeros((B, K))
    np.put_along_axis(G4, idx, 2.0 / (B * beams) * (np.take_along_axis(y, idx, 1) - T), 1)
    g4 = bf16(G4)
    g3 = bf16((g4 @ Wb["W4"]) * (1 - h3 * h3))
    g2 = bf16((g3 @ Wb["W3"]) * (1 - h2 * h2))
    g1 = bf16((g2 @ Wb["W2"]) * (1 - h1 * h1))
    refg = {"W4": g4.T @ h3, "b4": G4.sum(0), "W3": g3.T @ h2, "b3": g3.sum(0), "W2": g2.T @ h1, "b2": g2.sum(0),
            "W1": g1.T @ X.astype(np.float64)}
    dX = g1 @ Wb["W1"]
    for l, (iu, iv, fu, fv) in enumerate(corners):
        Gg = np.zeros(P[f"G{l}"].shape)
        d = dX[:, 8 * l:8 * l + 8]
        for di, dj, w in ((0, 0, (1 - fu) * (1 - fv)), (1, 0, fu * (1 - fv)), (0, 1, (1 - fu) * fv), (1, 1, fu * fv)):
            np.add.at(Gg, (layer, iv + dj, iu + di), w[:, None] * d)
        refg[f"G{l}"] = Gg
    for k, r in refg.items():
        o, s = lay[k]
        g = grad[o:o + int(np.prod(s))].reshape(s)
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel < 2e-2, (k, rel)


def grid_inputs(sur, track, P, fr, layer):
    """float64 feature-grid inputs [B, 40] at the lidar origins."""
    ref = np.zeros((len(layer), 40))
    for l, (iu, iv, fu, fv) in enumerate(grid_corners(sur, track, fr[:, 3], fr[:, 4])):
        G = P[f"G{l}"]
        ref[:, 8 * l:8 * l + 8] = (G[layer, iv, iu] * ((1 - fu) * (1 - fv))[:, None] +
                                   G[layer, iv, iu + 1] * (fu * (1 - fv))[:, None] +
                                   G[layer, iv + 1, iu] * ((1 - fu) * fv)[:, None] +
                                   G[layer, iv + 1, iu + 1] * (fu * fv)[:, None])
    return ref


def grid_gradient(sur, track, P, fr, layer, dX):
    out = {}
    for l, (iu, iv, fu, fv) in enumerate(grid_corners(sur, track, fr[:, 3], fr[:, 4])):
        Gg = np.zeros(P[f"G{l}"].shape)
        d = dX[:, 8 * l:8 * l + 8]
        for di, dj, w in ((0, 0, (1 - fu) * (1 - fv)), (1, 0, fu * (1 - fv)), (0, 1, (1 - fu) * fv), (1, 1, fu * fv)):
            np.add.at(Gg, (layer, iv + dj, iu + di), w[:, None] * d)
        out[f"G{l}"] = Gg
    return out


def test_car_frame_with_grids_inputs_and_gradient_match_float64():
    """Frame 2 (car-frame outputs, feature-grid inputs): the inputs against a float64 recomputation
    within BF16 rounding, and the gradient, grids included, against a float64 backprop with the same
    BF16 roundings within 2e-2 relative (Frobenius) per block."""
    track, sim, sur, T = world_setup(frame="car_grid")
    B, beams = sur.batch, sim.beams
    X, _ = sur.batch_inputs()
    theta, grad = sur.theta.numpy(), sur.grad.numpy()
    lay = sur.layout()
    P = {k: theta[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in lay.items()}
    poses = sur.poses().numpy()[:B]
    fr = rest_frames(track, poses)
    layer = poses[:, 3].astype(int)
    ref = np.zeros((B, 64))
    ref[:, :40] = grid_inputs(sur, track, P, fr, layer)
    nx, ny, x0, y0, cell = track[0], track[1], track[2], track[3], track[4]
    hx, hy = np.float32(0.5) * np.float32(nx - 1) * cell, np.float32(0.5) * np.float32(ny - 1) * cell
    xn = ((fr[:, 3] - (x0 + hx)) * (np.float32(1) / hx)).astype(np.float64)
    yn = ((fr[:, 4] - (y0 + hy)) * (np.float32(1) / hy)).astype(np.float64)
    sh, ch = fr[:, 6].astype(np.float64), fr[:, 7].astype(np.float64)
    ref[:, 40:48] = np.stack([xn, yn, fr[:, 5], sh, ch, layer == 0, layer == 1, np.ones(B)], 1)
    h = np.arctan2(sh, ch)
    for j in range(2, 6):
        ref[:, 48 + 2 * (j - 2)], ref[:, 49 + 2 * (j - 2)] = np.sin(j * h), np.cos(j * h)
    for k, sc in enumerate((np.pi, 2 * np.pi)):
        ref[:, 56 + 4 * k:60 + 4 * k] = np.stack([np.sin(sc * xn), np.cos(sc * xn), np.sin(sc * yn),
                                                  np.cos(sc * yn)], 1)
    err = np.abs(X - ref)
    assert np.all(err <= 2e-3 + 8e-3 * np.abs(ref)), err.max()
    Wb, h1, h2, h3, y = world_forward(sur, P, X.astype(np.float64))
    G4 = 2.0 / (B * beams) * (y - T)
    g4 = bf16(G4)
    g3 = bf16((g4 @ Wb["W4"]) * (1 - h3 * h3))
    g2 = bf16((g3 @ Wb["W3"]) * (1 - h2 * h2))
    g1 = bf16((g2 @ Wb["W2"]) * (1 - h1 * h1))
    refg = {"W4": g4.T @ h3, "b4": G4.sum(0), "W3": g3.T @ h2, "b3": g3.sum(0), "W2": g2.T @ h1, "b2": g2.sum(0),
            "W1": g1.T @ X.astype(np.float64)}
    refg.update(grid_gradient(sur, track, P, fr, layer, g1 @ Wb["W1"]))
    for k, r in refg.items():
        o, s = lay[k]
        g = grad[o:o + int(np.prod(s))].reshape(s)
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel < 2e-2, (k, rel)


def test_world_frame_prediction_is_the_profile_read_at_the_heading():
    """Inference in the world frame (FP16 world profiles, then the gather by heading): beam b of a
    sample is its clamped world sample (k0 + b) mod K, against a float64 forward of the same inputs."""
    track, sim, sur, T = world_setup()
    B, beams, K = sur.batch, sim.beams, sur.nout
    X, k0 = sur.batch_inputs()
    pred = W.DevArray.empty((beams, B))
    sur.batch_predict(pred)
    got = pred.numpy().T
    theta = sur.theta.numpy()
    P = {k: theta[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in sur.layout().items()}
    y = world_forward(sur, P, X.astype(np.float64))[-1]
    want = np.clip(y, 0, 1).astype(np.float16).astype(np.float64)
    want = np.take_along_axis(want, (k0[:, None] + np.arange(beams)) % K, 1)
    assert np.all((got >= 0) & (got <= 1))
    assert np.abs(got - want).max() < 2e-3


def test_world_frame_on_a_one_layer_track():
    """bank (one layer): one grid layer, the same training and inference paths; training cuts the
    held-out error and a surrogate rollout with audits on every step is the exact rollout."""
    track = W.track("bank")
    sim = W.Sim(track, 8, 0, beams=1081)
    sur = W.Surrogate(sim, hidden=128, batch=1024, seed=1, frame="world")
    lay = sur.layout()
    assert all(lay[f"G{l}"][1][0] == 1 for l in range(W.Surrogate.GRID_LEVELS))
    sur.set_poses(1 << 14, seed=2)
    before = sur.evaluate(batches=2, seed=77)
    sur.train(300, lr=2e-3)
    after = sur.evaluate(batches=2, seed=77)
    assert after[0] < 0.7 * before[0], (before, after)
    exact = W.Runner(track, 256, beams=1081, seed=4)
    run = W.Runner(track, 256, beams=1081, seed=4)
    sur.bind(run.sim)
    exact.rollout(3, False, 0)
    run.rollout_surrogate(sur, 3, False, 0, audit_every=1, fallback_m=0.5)
    run.synchronize()
    for name in ("state", "obs", "reward", "done", "actions"):
        assert np.array_equal(getattr(exact.sim, name).numpy(), getattr(run.sim, name).numpy()), name


def test_world_frame_needs_the_beam_spacing_to_divide_the_circle():
    sim = W.Sim(W.track("bridge"), 8, 0, beams=108)
    with pytest.raises(W.RacerError, match="multiple of 12"):
        W.Surrogate(sim, hidden=128, batch=256, seed=1, frame="world")
    W.Surrogate(W.Sim(W.track("bridge"), 8, 0, beams=109), hidden=128, batch=256, seed=1, frame="world")


@pytest.mark.parametrize("frame", ["car", "world", "car_grid"])
@pytest.mark.parametrize("audit_every,fallback_m", [(1, 0.5), (0, 100.0)])
def test_fully_exact_surrogate_rollout_equals_exact_rollout(audit_every, fallback_m, frame):
    """Audit on every step, or a fallback threshold every car crosses: the rollout is the exact one."""
    track = W.track("bridge")
    n = 512
    exact = W.Runner(track, n, beams=1081, seed=3)
    sur_run = W.Runner(track, n, beams=1081, seed=3)
    sur = W.Surrogate(sur_run.sim, hidden=128, batch=1024, seed=1, frame=frame)
    exact.rollout(6, False, 40)
    sur_run.rollout_surrogate(sur, 6, False, 40, audit_every=audit_every, fallback_m=fallback_m)
    sur_run.synchronize()
    for name in ("state", "obs", "reward", "done", "actions"):
        assert np.array_equal(getattr(exact.sim, name).numpy(), getattr(sur_run.sim, name).numpy()), name
    mae, rmse, mx, over, fb = sur.rollout_stats()
    if audit_every:
        assert mae > 0 and rmse >= mae and mx >= rmse
    else:
        assert fb == 1.0


def test_surrogate_rollout_stats_and_fallback():
    track = W.track("bridge")
    run = W.Runner(track, 1024, beams=1081, seed=5)
    sur = W.Surrogate(run.sim, hidden=128, batch=1024, seed=1)
    sur.set_poses(1 << 14, seed=2)
    sur.train(50, lr=1e-3)
    run.rollout_surrogate(sur, 8, audit_every=4, fallback_m=0.5)
    mae, rmse, mx, over, fb = sur.rollout_stats(reset=True)
    assert np.isfinite([mae, rmse, mx, over, fb]).all() and mae > 0 and 0 <= fb <= 1
    o = run.sim.obs.numpy()
    assert np.isfinite(o).all() and (o[4:-1] >= 0).all() and (o[4:-1] <= 1).all()
    assert sur.rollout_stats()[0] == 0.0  # reset


@pytest.mark.parametrize("frame", ["car", "world", "car_grid"])
def test_training_reduces_heldout_error(frame):
    track = W.track("bridge")
    sim = W.Sim(track, 8, 0, beams=1081)
    sur = W.Surrogate(sim, hidden=256, batch=1024, seed=1, frame=frame)
    sur.set_poses(1 << 16, seed=2)
    before = sur.evaluate(batches=2, seed=77)
    mse, mae = sur.train(300, lr=1e-3)
    after = sur.evaluate(batches=2, seed=77)
    assert np.isfinite(mse) and np.isfinite(mae)
    assert after[0] < 0.7 * before[0], (before, after)


@pytest.mark.parametrize("frame", ["car", "world", "car_grid"])
@pytest.mark.parametrize("cars", [300, 128 * 160 + 37])
def test_fused_inference_equals_layered_gemms(cars, frame):
    """The fused 512-wide inference kernel (activations kept on chip, output in TMEM chunks) gives the
    same bits as the four GEMM launches: obs, the fallback cars picked from the per-car minimum
    ranges, state. 128 * 160 + 37 cars is more tiles than SMs, so CTAs run several tiles. One
    trained surrogate serves both (training sums bias gradients with atomics), and the sim's state
    and observations are restored between the two rollouts."""
    run = W.Runner(W.track("bridge"), cars, beams=1081, seed=5)
    sur = W.Surrogate(run.sim, hidden=512, batch=1024, seed=2, frame=frame)
    sur.set_poses(1 << 14, seed=4)
    sur.train(30 if frame == "car" else 400, lr=2e-3)  # until some cars' smallest prediction passes 0.5 m
    state0, obs0 = run.sim.state.numpy(), run.sim.obs.numpy()
    out = []
    for fused in (True, False):
        run.sim.state.write(state0)
        run.sim.obs.write(obs0)
        sur.set_fused(fused)
        sur.rollout_stats(reset=True)
        run.rollout_surrogate(sur, 6, False, 0, 0, 0.5)
        run.synchronize()
        out.append((run.sim.obs.numpy(), run.sim.state.numpy(), sur.rollout_stats()[4]))
    (obs_f, state_f, fb_f), (obs_l, state_l, fb_l) = out
    assert np.array_equal(obs_f, obs_l) and np.array_equal(state_f, state_l) and fb_f == fb_l
    assert 0.0 < fb_f < 1.0


@pytest.mark.parametrize("frame", ["car", "world"])
def test_trained_surrogate_rollout_beats_exact_rollout(frame):
    """What the learned part gains over the method without it: after 3000 Adam steps on 2^18
    traced poses, the surrogate rollout (every 16th step traced exactly for all cars, and each car
    whose smallest predicted range is under 0.5 m traced exactly) of 16384 cars at 1081 beams takes
    well under the exact rollout's time, at a bounded audited error."""
    import time
    track = W.track("bridge")
    cars, steps = 16384, 32
    exact = W.Runner(track, cars, beams=1081, seed=7)
    learned = W.Runner(track, cars, beams=1081, seed=7)
    sur = W.Surrogate(learned.sim, hidden=512, batch=8192, seed=1, frame=frame)
    sur.set_poses(1 << 18, seed=2)
    sur.set_loss(0.02)
    sur.train(3000, lr=8e-3 if frame == "car" else 2e-3)

    def wall(runner, roll):
        roll(0)  # capture and warm up the graph
        runner.synchronize()
        t0 = time.perf_counter()
        for k in range(3):
            roll((k + 1) * steps)
        runner.synchronize()
        return time.perf_counter() - t0

    t_exact = wall(exact, lambda t0: exact.rollout(steps, False, t0))
    t_learned = wall(learned, lambda t0: learned.rollout_surrogate(sur, steps, False, t0, 16, 0.5))
    mae, rmse, mx, over, fallback = sur.rollout_stats()
    print(f"exact {t_exact * 1e3:.1f} ms, surrogate {t_learned * 1e3:.1f} ms, audited MAE {mae:.3f} m, "
          f"fallback {fallback:.3f}")
    assert t_learned < t_exact / 1.5, (t_learned, t_exact)
    assert 0.0 < mae < 0.5 and 0.0 <= fallback < 0.5, (mae, fallback)


def test_label_cache_serves_the_traced_labels():
    """Labels copied back from the training set's label cache (every epoch after the first) are the
    tracer's own: each batch's labels equal a fresh tracing with the cache switched off, and the
    held-out evaluation in between neither uses nor replaces the cache."""
    track = W.track("bridge")
    sim = W.Sim(track, 8, 0, beams=1081)
    sur = W.Surrogate(sim, hidden=128, batch=1024, seed=1)
    sur.set_poses(3 * 1024, seed=2)
    first, again = [], []
    for b in range(3):
        lab = W.DevArray.empty((1081, 1024))
        sur.gradient(b * 1024, lab)  # traced, then kept
        first.append(lab.numpy())
    sur.evaluate(batches=1, seed=77)
    for b in range(3):
        lab = W.DevArray.empty((1081, 1024))
        sur.gradient(b * 1024, lab)  # copied from the cache
        again.append(lab.numpy())
    sur.set_label_cache(False)
    sur.set_poses(3 * 1024, seed=2)
    for b in range(3):
        lab = W.DevArray.empty((1081, 1024))
        sur.gradient(b * 1024, lab)  # traced again, no cache
        assert np.array_equal(lab.numpy(), first[b]) and np.array_equal(again[b], first[b])


def test_training_with_surrogate_audited_every_step_equals_exact_training():
    """Trainer.rollout (racer/ppo.mojo:187-232) with the learned lidar audited on every step: the
    exact tracer rewrites every car's ranges in rollout storage, so two iterations of rollout and
    update equal exact training bit for bit (storage, advantages, parameters)."""
    track = W.track("bridge")
    n, beams, R = 512, 1081, 8
    runs = [W.Runner(track, n, beams=beams, seed=3, policy_seed=5) for _ in range(2)]
    trainers = [W.Trainer(n, beams=beams, rollout=R, stream=r.sim.stream) for r in runs]
    sur = W.Surrogate(runs[1].sim, hidden=512, batch=1024, seed=1)
    trainers[1].set_surrogate(sur, audit_every=1, fallback_m=0.5)
    for it in range(2):
        rewards = [t.rollout(r.sim, r.policy, r.acts, it) for t, r in zip(trainers, runs)]
        assert rewards[0] == rewards[1]
        for name in ("obs", "actions", "reward", "done", "value", "advantage"):
            assert np.array_equal(getattr(trainers[0], name).numpy(), getattr(trainers[1], name).numpy()), name
        kls = [t.update(r.policy) for t, r in zip(trainers, runs)]
        assert kls[0] == kls[1]
        assert np.array_equal(runs[0].policy.theta.numpy(), runs[1].policy.theta.numpy())
    mae, rmse, mx, over, fb = sur.rollout_stats()
    assert mae > 0 and rmse >= mae and fb == 0.0  # every step audited: no fallback steps


def test_training_with_surrogate_audits_and_fallback():
    """Surrogate rollouts in training with an audit every 4th step and the 0.5 m fallback: finite
    rewards, the audited error and fallback fraction accumulate, and the audited steps' ranges in
    rollout storage are the exact tracer's."""
    track = W.track("bridge")
    n, beams, R = 1024, 1081, 8
    run = W.Runner(track, n, beams=beams, seed=5)
    ref = W.Runner(track, n, beams=beams, seed=5)
    sur = W.Surrogate(run.sim, hidden=512, batch=1024, seed=2)
    sur.set_poses(1 << 14, seed=3)
    sur.train(200, lr=2e-3)
    trainer = W.Trainer(n, beams=beams, rollout=R, stream=run.sim.stream)
    trainer.set_surrogate(sur, audit_every=4, fallback_m=0.5)
    sur.rollout_stats(reset=True)
    reward = trainer.rollout(run.sim, run.policy, run.acts, 0)
    assert np.isfinite(reward)
    mae, rmse, mx, over, fb = sur.rollout_stats()
    assert 0 < mae < 5 and rmse >= mae and 0 <= fb <= 1
    # steps 0 and 4 were audited: storage rows t + 1 = 1, 5 hold the exact ranges of the frames the
    # physics wrote; retrace those frames with an exact sim stepped on the same actions
    obs = trainer.obs.numpy()
    actions = trainer.actions.numpy()
    ref_obs = []
    for t in range(R):
        ref.sim.actions.write(actions[t])
        ref.sim.step(ref.sim.actions, ref.sim.reward, ref.sim.done, ref.sim.obs)
        ref_obs.append(ref.sim.obs.numpy())
    for t in (0, 4):
        assert np.array_equal(obs[t + 1], ref_obs[t]), t
    assert np.isfinite(trainer.update(run.policy))


def test_surrogate_binds_to_sims_of_the_same_track_only():
    track = W.track("bridge")
    a = W.Runner(track, 256, beams=1081, seed=1)
    b = W.Runner(track, 384, beams=1081, seed=2)
    sur = W.Surrogate(a.sim, hidden=128, batch=1024, seed=1)
    a.rollout_surrogate(sur, 2, audit_every=1)
    sur.bind(b.sim)
    b.rollout_surrogate(sur, 2, audit_every=1)  # inference buffers re-sized for 384 cars
    exact = W.Runner(track, 384, beams=1081, seed=2)
    exact.rollout(2)
    assert np.array_equal(b.sim.obs.numpy(), exact.sim.obs.numpy())
    with pytest.raises(W.RacerError, match="differs"):
        sur.bind(W.Sim(W.track("bank"), 16, 1, beams=1081))
    with pytest.raises(W.RacerError, match="differs"):
        sur.bind(W.Sim(track, 16, 1, beams=108))


def test_spot_check_sends_every_mismatching_car_to_the_exact_tracer():
    """The spot check between audits. With every beam checked at a tolerance of 1 um every car of an
    untrained surrogate mismatches, so the rollout is the exact one; with every beam checked at 0.25 m
    no car keeps a range more than 0.25 m from the exact tracer's, while without the check (and no
    fallback threshold) some cars do, including ranges predicted too long."""
    track = W.track("bridge")
    n, beams = 1024, 1081
    exact = W.Runner(track, n, beams=beams, seed=4)
    exact.rollout(3, False, 0)
    run = W.Runner(track, n, beams=beams, seed=4)
    sur = W.Surrogate(run.sim, hidden=512, batch=1024, seed=1)
    sur.set_spot_check(1, 1e-6)
    run.rollout_surrogate(sur, 3, False, 0, audit_every=0, fallback_m=0.0)
    run.synchronize()
    for name in ("state", "obs", "reward", "done", "actions"):
        assert np.array_equal(getattr(exact.sim, name).numpy(), getattr(run.sim, name).numpy()), name
    assert sur.rollout_stats()[4] == 1.0

    ref = W.Runner(track, n, beams=beams, seed=6)
    ref.rollout(1, False, 0)  # one step: the actions come from the (exact) reset observations
    want = ref.sim.obs.numpy()[4:4 + beams] * 10
    trained = W.Runner(track, n, beams=beams, seed=6)
    sur2 = W.Surrogate(trained.sim, hidden=512, batch=1024, seed=2)
    sur2.set_poses(1 << 14, seed=3)
    sur2.train(300, lr=2e-3)
    state0, obs0 = trained.sim.state.numpy(), trained.sim.obs.numpy()
    errs, long_miss = {}, {}
    for stride in (0, 1):
        sur2.set_spot_check(stride, 0.25)
        trained.sim.state.write(state0)  # both runs start from the same reset
        trained.sim.obs.write(obs0)
        trained.rollout_surrogate(sur2, 1, False, 0, audit_every=0, fallback_m=0.0)
        trained.synchronize()
        got = trained.sim.obs.numpy()[4:4 + beams] * 10
        errs[stride] = np.abs(got - want).max(axis=0)  # per car
        long_miss[stride] = int(((got - want) > 0.25 * 1.0001).sum())  # predicted beyond the exact range
    assert (errs[0] > 0.25 * 1.0001).any() and long_miss[0] > 0 and long_miss[1] == 0
    assert (errs[1] <= 0.25 * 1.0001).all()
    with pytest.raises(W.RacerError, match="stride"):
        sur2.set_spot_check(-1, 0.25)
