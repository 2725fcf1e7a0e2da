"""GPU policy, trainer and runner against the CPU oracle.

Policy initialisation, GAE and sampling are element-wise and bit-exact;
the GEMMs differ from the oracle only in summation order and precision, so
they are compared within tolerances stated per test; the PPO gradient is
checked against float64 central differences with the reference's GPU
tolerance (tests/test_mojo.mojo:208).
"""
import numpy as np
import pytest

import oracle as O
import warporacer3d_gb300 as W
from test_oracle import N, host_loss

pytestmark = pytest.mark.gpu

# Forward tolerance: |gpu - oracle| <= FWD_ATOL + FWD_RTOL * |oracle| per output.
FWD_ATOL, FWD_RTOL = 2e-2, 2e-2


def test_policy_init_bit_exact():
    for beams in (108, 1081):
        g = W.Policy(42, beams=beams)
        c = O.Policy(42, beams=beams)
        assert np.array_equal(g.theta.numpy(), c.theta)


@pytest.mark.parametrize("beams,cols", [(108, 1000), (1081, 384), (2, 1), (2, 129), (1081, 1)])
def test_policy_forward(beams, cols):
    g = W.Policy(3, beams=beams)
    c = O.Policy(3, beams=beams)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (beams + 5, cols)).astype(np.float32)
    x[-1] = 1
    xd = W.DevArray.empty(x.shape)
    xd.write(x)
    ga, ca = W.Activations(g, cols), O.Activations(cols)
    g.forward(xd, ga)
    c.forward(x, ca)
    for name in ("h1", "h2", "o"):
        a, b = getattr(ga, name).numpy(), getattr(ca, name)
        assert np.all(np.abs(a - b) <= FWD_ATOL + FWD_RTOL * np.abs(b)), (name, np.abs(a - b).max())
    assert np.all(ga.h1.numpy()[64] == 1) and np.all(ga.h2.numpy()[64] == 1)
    assert g.status() == 0


def test_policy_forward_staging_paths_agree():
    """The BF16 forward with its inputs staged by TMA (sample columns 16-byte aligned: 1000
    columns) and the register-staged forward (1001 columns) give the same bits for the same
    samples."""
    beams = 1081
    g = W.Policy(5, beams=beams)
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (beams + 5, 1001)).astype(np.float32)
    outs = []
    for cols in (1000, 1001):
        xd = W.DevArray.empty((beams + 5, cols))
        xd.write(np.ascontiguousarray(x[:, :cols]))
        a = W.Activations(g, cols)
        g.forward(xd, a)
        outs.append([getattr(a, name).numpy()[:, :1000] for name in ("h1", "h2", "o")])
    for p, q in zip(*outs):
        assert np.array_equal(p, q)
    assert g.status() == 0


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
def test_gae_bit_exact_and_gradient_and_update(precision):
    """tests/test_mojo.mojo:162-215 on the GPU: GAE, FD gradient (GPU tolerance), KL after one update."""
    flat = W.track("flat")
    sim = W.Sim(flat, N, 42)
    sim.reset()
    s = sim.state.numpy()
    for i in range(N):
        s[O.STEPS, i] = np.float32(O.HORIZON - 5 - 7 * i)
    sim.state.write(s)
    policy = W.Policy(42)
    policy.set_precision(precision)
    acts = W.Activations(policy, N)
    trainer = W.Trainer(N)
    assert np.isfinite(trainer.rollout(sim, policy, acts, 0))
    reward, done = trainer.reward.numpy(), trainer.done.numpy()
    value, adv = trainer.value.numpy(), trainer.advantage.numpy()
    last = acts.o.numpy()
    ref_adv = np.zeros_like(adv)
    O.lib().orc_gae(N, O.ROLLOUT, reward, done, value, np.ascontiguousarray(last[2]), ref_adv)
    assert np.array_equal(adv, ref_adv), "GAE is bit-exact given the same inputs"
    assert int((done != 0).sum()) == N, "every car's episode ended once during the rollout"
    trainer.minibatch(policy, 0, 0.0, 1.0)
    analytic = trainer.grad.numpy()

    class View:  # the host loss reads rollout storage as numpy
        pass
    v = View()
    v.obs, v.actions, v.logp = trainer.obs.numpy(), trainer.actions.numpy(), trainer.logp.numpy()
    v.value, v.advantage, v.batch = value, adv, trainer.batch
    pol = O.Policy(42)  # layout only
    w = policy.theta.numpy().astype(np.float64)
    largest = 0.0
    i = 0
    while i < pol.P:
        w[i] += 1e-4
        plus = host_loss(w, v, pol)
        w[i] -= 2e-4
        numeric = (plus - host_loss(w, v, pol)) / 2e-4
        w[i] += 1e-4
        assert abs(numeric - analytic[i]) <= 3e-2 * abs(numeric) + 1e-3, (i, analytic[i], numeric)
        largest = max(largest, abs(numeric))
        i += 293 if i < pol.LOGSTD - 293 else 1
    assert largest > 1e-3
    kl = trainer.update(policy)
    assert np.isfinite(kl) and 0 <= kl < 0.1


@pytest.mark.parametrize("beams,cols", [(108, 4096), (1081, 1000)])
def test_bf16_backward_matches_fp32_backward(beams, cols):
    """The tensor-core backward (BF16 operands, FP32 accumulation) against the FP32 one on the same
    inputs: relative Frobenius error per block below 2e-2."""
    rng = np.random.default_rng(cols)
    IN = beams + 5
    x = rng.uniform(-1, 1, (IN, cols)).astype(np.float32)
    x[-1] = 1
    xd = W.DevArray.empty((IN, cols))
    xd.write(x)
    d3 = W.DevArray.empty((3, cols))
    d3.write(rng.normal(0, 1e-3, (3, cols)).astype(np.float32))
    out = {}
    for precision in ("fp32", "bf16"):
        p = W.Policy(11, beams=beams)
        p.set_precision("fp32")  # identical activations for both backward passes
        acts = W.Activations(p, cols)
        p.forward(xd, acts)
        p.set_precision(precision)
        bufs = [W.DevArray.empty((65, cols)), W.DevArray.empty((65, cols)), W.DevArray.empty((p.P,))]
        p.backward(xd, acts, d3, *bufs)
        out[precision] = [b.numpy() for b in bufs]
        assert p.status() == 0
        lay = {"W0": (0, p.W1), "W1": (p.W1, p.W2), "W2": (p.W2, p.LOGSTD)}
    for name, (a, b) in zip(("d2", "d1"), zip(out["bf16"][:2], out["fp32"][:2])):
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b), name
    for name, (lo, hi) in lay.items():
        a, b = out["bf16"][2][lo:hi], out["fp32"][2][lo:hi]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b), name


def test_runner_graph_matches_steps():
    track = W.track("bridge")
    n = 256
    a = W.Runner(track, n, beams=108, seed=9)
    b = W.Runner(track, n, beams=108, seed=9)
    for t in range(12):
        a.step(False, 100 + t)
    b.rollout(12, False, 100)
    b.synchronize()
    for name in ("state", "obs", "reward", "done", "actions"):
        assert np.array_equal(getattr(a.sim, name).numpy(), getattr(b.sim, name).numpy()), name


def test_runner_step_matches_oracle_given_actions():
    """A policy-driven step: the sim part is bit-exact when the oracle replays the GPU's actions."""
    track = W.track("ramp")
    n = 128
    r = W.Runner(track, n, beams=108, seed=4)
    cpu = O.Sim(track, n, 4, beams=108)
    cpu.state[:] = r.sim.state.numpy()
    cpu.obs[:] = r.sim.obs.numpy()
    for t in range(8):
        r.step(False, t)
        cpu.actions[:] = r.sim.actions.numpy()
        cpu.step(cpu.actions, cpu.reward, cpu.done, cpu.obs)
        for name in ("state", "obs", "reward", "done"):
            assert np.array_equal(getattr(r.sim, name).numpy(), getattr(cpu, name), equal_nan=True), (t, name)


def test_checkpoint_roundtrip(tmp_path):
    p = W.Policy(1)
    path = tmp_path / "agent.npy"
    W.save(p, path, 17)
    arr = np.load(path)
    assert arr.dtype == np.float32 and arr.shape == (1 + p.P,) and arr[0] == 17
    assert np.array_equal(arr[1:], p.theta.numpy())
    q = W.Policy(2)
    assert W.load(q, path) == 17
    assert np.array_equal(q.theta.numpy(), p.theta.numpy())
    np.save(tmp_path / "short.npy", np.zeros(5, np.float32))
    with pytest.raises(W.RacerError, match="does not match the network size"):
        W.load(q, tmp_path / "short.npy")


@pytest.mark.parametrize("chains", [2, 3])
def test_rollout_chains_match_one_chain(chains):
    """Rollout graphs split into independent chains over car ranges give the one-chain results bit for
    bit (cars never interact; sampling offsets and Philox counters are per car)."""
    runs = [W.Runner(W.track("bridge"), 1000, beams=108, seed=6, policy_seed=7) for _ in range(2)]
    runs[1].sim.set_chains(chains)
    for r in runs:
        r.rollout(12, False, 0)
        r.rollout(12, False, 12)
        r.synchronize()
    a, b = runs
    for name in ("state", "obs", "actions", "reward", "done"):
        assert np.array_equal(getattr(a.sim, name).numpy(), getattr(b.sim, name).numpy()), name
    assert b.rollout_kernel_count(12) > a.rollout_kernel_count(12)


def test_trainer_rollout_with_chains_matches_one_chain():
    """Trainer.rollout with rollout chains fills the rollout storage with the one-chain bits."""
    out = []
    for chains in (1, 3):
        sim = W.Sim(W.track("bank"), 1000, 3, beams=108)
        sim.reset()
        policy = W.Policy(5, beams=108)
        acts = W.Activations(policy, 1000)
        sim.set_chains(chains)
        trainer = W.Trainer(1000, beams=108, rollout=8)
        reward = trainer.rollout(sim, policy, acts, 0)
        out.append((reward, trainer.obs.numpy(), trainer.actions.numpy(), trainer.advantage.numpy(),
                    sim.state.numpy()))
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)
    assert out[0][0] == out[1][0]


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
def test_trainer_update_graph_matches_eager(precision):
    """Updates replayed from the captured graph (from the third on) give the eager updates' bits: theta,
    Adam moments and KL over four rollout + update iterations; a policy that changes precision mid-way
    is re-warmed, not replayed with stale launches."""
    out = []
    for graphs in (True, False):
        sim = W.Sim(W.track("bank"), 1024, 3, beams=108)
        sim.reset()
        policy = W.Policy(5, beams=108)
        policy.set_precision(precision)
        acts = W.Activations(policy, 1024)
        trainer = W.Trainer(1024, beams=108, rollout=8)
        trainer.set_graphs(graphs)
        kls = []
        for it in range(5):
            if it == 3:  # switch precision and back: the captured graph must go stale
                policy.set_precision("fp32" if precision == "bf16" else "bf16")
                policy.set_precision(precision)
            trainer.rollout(sim, policy, acts, it)
            kls.append(trainer.update(policy))
        out.append((kls, policy.theta.numpy(), trainer.first.numpy(), trainer.second.numpy()))
    (ka, ta, fa, sa), (kb, tb, fb, sb) = out
    assert ka == kb
    assert np.array_equal(ta, tb) and np.array_equal(fa, fb) and np.array_equal(sa, sb)


@pytest.mark.parametrize("beams,cols", [(1081, 4096), (108, 1000)])
def test_bounded_wait_timeout_is_reported(beams, cols):
    """A bounded wait that runs out (tests/test_mojo.mojo has no counterpart; main.mojo:61-62 is the
    reference's error surface for a failed step). The probe is a tensor-core kernel holding tensor
    memory whose threads wait on an mbarrier that nothing arrives on; after 2048 polls the wait gives
    up, the kernel records the timeout in the policy's error word, frees its tensor memory and
    returns, so the context stays usable: the status reads nonzero once (it is cleared on read), and
    the next forward on the same stream gives the oracle's outputs with the word at 0."""
    g, c = W.Policy(9, beams=beams), O.Policy(9, beams=beams)
    rng = np.random.default_rng(cols)
    x = rng.uniform(-1, 1, (beams + 5, cols)).astype(np.float32)
    x[-1] = 1
    xd = W.DevArray.empty(x.shape)
    xd.write(x)
    ga, ca = W.Activations(g, cols), O.Activations(cols)
    assert g.status() == 0
    g.wait_test(2048)
    assert g.status() == 2, "the timed-out wait is reported"
    assert g.status() == 0, "the status word is read and cleared"
    g.forward(xd, ga)
    c.forward(x, ca)
    for name in ("h1", "h2", "o"):
        a, b = getattr(ga, name).numpy(), getattr(ca, name)
        assert np.all(np.abs(a - b) <= FWD_ATOL + FWD_RTOL * np.abs(b)), (name, np.abs(a - b).max())
    assert g.status() == 0
    with pytest.raises(W.RacerError, match="poll count"):
        g.wait_test(0)
