"""Pins the CPU oracle to the reference's own known answers.

Every test here is a port of a test in the reference's tests/test_mojo.mojo
(dynamics, corridor, bridge layers, GAE, PPO finite-difference gradient,
KL after one update), run against the oracle with the reference's
tolerances, plus checks of the shared math and random-number primitives
against double-precision libm and the published Philox4x32-10 known-answer
vectors.
"""
import math

import numpy as np
import pytest

import oracle as O
from oracle import (ACCEL_MAX, CRASH, EPISODE, FRICTION, G, GRIP, HEADING, HORIZON, PROGRESS, RETURN, SPEED,
                    STATE, STEER, STEER_MAX, STEPS, SPEED_MAX, X, Y)


# ---- tests/test_mojo.mojo:48-55 ----
def test_dynamics():
    d = O.derivative
    assert (d([0, 0, 0, 0], 0, 0, GRIP, 0, 0) == 0).all(), "a car at rest stays at rest"
    assert d([0, 0, 0, 2], 0, 0, GRIP, 0.3, 0)[3] < 0, "an uphill slope slows the car"
    assert d([0, 0, 0, 2], 0, 0, GRIP, 0, 0)[3] == 0, "coasting on the flat holds speed"
    limit = d([0, 0, 0, 5], STEER_MAX, ACCEL_MAX, GRIP, 0, 0)
    assert abs(limit[2] * 5) <= GRIP * G + 1e-4 and limit[3] <= 1e-4, "the friction circle caps the tyres"
    assert d([0, 0, 0, 2], 0.2, 0, GRIP, 0, 0)[2] > 0.5, "steering yaws the car"


# ---- tests/test_mojo.mojo:58-92 ----
def test_corridor():
    track = O.corridor()
    n, beams = 4, 108
    sim = O.Sim(track, n, 1, beams=beams)
    s = np.zeros((STATE, n), np.float32)
    s[X], s[FRICTION], s[PROGRESS] = 1, 1, np.float32(0.5 / 0.15)
    s[HEADING, 1] = np.float32(math.pi)
    sim.state[:] = s
    sim.actions[:] = np.array([[0, 0, 0, 1], [0, 1, 1, 1]], np.float32)
    sim.step(sim.actions, sim.reward, sim.done, sim.obs)
    o = sim.obs
    assert abs(o[4 + beams // 2, 0] * 10 - 7.1) <= 0.1, "the centre beam stops on the ramp face"
    assert abs(o[4 + beams // 2, 1] * 10 - 0.73) <= 0.1, "the centre beam reads the wall"
    crashed = False
    for _ in range(60):
        sim.step(sim.actions, sim.reward, sim.done, sim.obs)
        done = sim.done
        assert done[0] == 0 and done[2] == 0 and done[3] == 0, "the open road does not crash"
        if done[1] == CRASH and not crashed:
            assert sim.state[STEPS, 1] == 0 and sim.state[EPISODE, 1] == 1, "a crash respawns at once"
            crashed = True
    assert crashed, "driving into the wall crashes"
    s, o = sim.state, sim.obs
    assert s[X, 0] == 1 and s[SPEED, 0] == 0 and s[HEADING, 0] == 0, "a car at rest stays at rest"
    assert s[SPEED, 2] == SPEED_MAX and s[X, 2] > 3.5 and abs(s[Y, 2]) < 1e-4, "full throttle"
    assert abs(s[RETURN, 2] - 10 * (s[X, 2] - 1)) <= 0.01, "continuous progress reward"
    assert s[Y, 3] > 0.1 and s[X, 3] < s[X, 2], "steering turns the car left"
    assert o[1, 2] == 1 and o[beams + 4, 2] == 1, "speed and bias observations"
    assert np.isfinite(o).all(), "observations stay finite"


# ---- tests/test_mojo.mojo:95-108 ----
def test_bridge_layers(bridge):
    m = O.Map(bridge)
    assert m.layers == 2 and m.probe(0, 0, 0).layer == 0 and m.probe(0, 0, 0.5).layer == 1, "layer by height"
    assert m.probe(0, 0, 0).clearance > 1 and m.probe(0, 0, 0.9).clearance > 1, "both roads cross at the origin"
    for w in range(0, m.waypoints, 2):
        x, y, z = m.waypoint(w, 0), m.waypoint(w, 1), m.waypoint(w, 2)
        spot = m.probe(x, y, z)
        assert spot.clearance > 0.9, "the route centre is clear of walls"
        assert abs(m.surface(spot.layer, x, y)[0] - z) <= 0.03, "the surface follows the route"
        assert abs(m.progress(spot.layer, x, y) - w) <= 1e-3, "progress counts waypoints"


# ---- tests/test_mojo.mojo:126-215 ----
N = 4


def host_loss(w, trainer, policy):
    """Minibatch 0's clipped PPO objective in float64 with raw advantages (tests/test_mojo.mojo:137-159)."""
    IN, B = policy.IN, trainer.batch
    s = np.arange(B) * O.MINIBATCHES
    x = trainer.obs[s // N, :, s % N].T.astype(np.float64)  # [IN, B]
    ones = np.ones((1, B))
    h1 = np.vstack([np.tanh(w[:O.H * IN].reshape(O.H, IN) @ x), ones])
    h2 = np.vstack([np.tanh(w[policy.W1:policy.W2].reshape(O.H, O.HA) @ h1), ones])
    o = w[policy.W2:policy.LOGSTD].reshape(O.OUT, O.HA) @ h2
    ls = w[policy.LOGSTD:policy.LOGSTD + 2]
    act = trainer.actions[s // N, :, s % N].T.astype(np.float64)
    err = act - o[:2]
    new_logp = -(0.5 * err * err * np.exp(-2 * ls)[:, None] + ls[:, None] + float(O.lib().orc_half_log_2pi())).sum(0)
    ratio = np.exp(new_logp - trainer.logp.ravel()[s].astype(np.float64))
    adv = trainer.advantage.ravel()[s].astype(np.float64)
    total = -(np.minimum(ratio * adv, np.clip(ratio, 0.8, 1.2) * adv) / B).sum()
    e = np.abs(o[2] - (trainer.value.ravel()[s].astype(np.float64) + adv))
    total += (np.where(e <= 1, 0.25 * e * e, 0.5 * e - 0.25) / B).sum()
    return total


def test_ppo_gae_gradient_update(flat):
    sim = O.Sim(flat, N, 42, beams=108)
    sim.reset()
    for i in range(N):
        sim.state[STEPS, i] = np.float32(HORIZON - 5 - 7 * i)  # episodes end mid-rollout
    policy = O.Policy(42, beams=108)
    acts = O.Activations(N)
    trainer = O.Trainer(N, beams=108)
    assert np.isfinite(trainer.rollout(sim, policy, acts, 0)), "rollout reward"
    last = acts.o  # the policy on the final observations: the bootstrap values
    ended = 0
    for i in range(N):
        running = np.float32(0)
        nxt = last[2, i]
        for t in range(O.ROLLOUT - 1, -1, -1):
            alive = np.float32(1 if trainer.done[t, i] == 0 else 0)
            ended += int(trainer.done[t, i] != 0)
            running = trainer.reward[t, i] + O.GAMMA * alive * nxt - trainer.value[t, i] + \
                O.GAMMA * O.LAMBDA * alive * running
            assert abs(trainer.advantage[t, i] - running) <= 1e-4, "GAE advantage"
            nxt = trainer.value[t, i]
    assert ended == N, "every car's episode ended once during the rollout"
    trainer.minibatch(policy, 0, np.float32(0), np.float32(1))
    analytic = trainer.grad.copy()
    w = policy.theta.astype(np.float64)
    largest = 0.0
    i = 0
    while i < policy.P:
        w[i] += 1e-4
        plus = host_loss(w, trainer, policy)
        w[i] -= 2e-4
        numeric = (plus - host_loss(w, trainer, policy)) / 2e-4
        w[i] += 1e-4
        err = abs(numeric - analytic[i])
        assert err <= 5e-3 * abs(numeric) + 1e-5, f"gradient {i}: analytic {analytic[i]} numeric {numeric}"
        largest = max(largest, abs(numeric))
        i += 293 if i < policy.LOGSTD - 293 else 1
    assert largest > 1e-3, "the rollout produces a nontrivial gradient"
    kl = trainer.update(policy)
    assert np.isfinite(kl) and 0 <= kl < 0.1, "KL after one update"


# ---- shared primitives ----
def _ulps(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float64).astype(np.float32)
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


def test_rmath_accuracy():
    rng = np.random.default_rng(0)
    L = O.lib()
    x = np.concatenate([rng.uniform(-7, 7, 200000), rng.uniform(-1e3, 1e3, 20000),
                        np.linspace(-4, 4, 10001)]).astype(np.float32)
    s, c = np.zeros_like(x), np.zeros_like(x)
    L.orc_sincos(x, x.size, s, c)
    xd = x.astype(np.float64)
    # absolute error against double libm, in units of float eps (results near zero have tiny ulps)
    assert np.max(np.abs(s - np.sin(xd))) < 4e-7 and np.max(np.abs(c - np.cos(xd))) < 4e-7
    big = np.abs(np.sin(xd)) > 0.1
    assert _ulps(s[big], np.sin(xd[big])).max() <= 4
    # up to the guard (|x| <= 6426: the three-part pi/2 split is exact for every quadrant there) the
    # reduction keeps its accuracy; past it sin and cos are NaN rather than silently inexact
    edge = np.concatenate([rng.uniform(-6426, 6426, 50000), np.float32(6426) - np.arange(64) * np.float32(2 ** -11),
                           -np.float32(6426) + np.arange(64) * np.float32(2 ** -11)]).astype(np.float32)
    se, ce = np.zeros_like(edge), np.zeros_like(edge)
    L.orc_sincos(edge, edge.size, se, ce)
    ed = edge.astype(np.float64)
    assert np.max(np.abs(se - np.sin(ed))) < 4e-7 and np.max(np.abs(ce - np.cos(ed))) < 4e-7
    past = np.array([np.nextafter(np.float32(6426), np.float32(1e9)), -6500.0, 1e5, np.inf, np.nan], np.float32)
    sp, cp = np.zeros_like(past), np.zeros_like(past)
    L.orc_sincos(past, past.size, sp, cp)
    assert np.isnan(sp).all() and np.isnan(cp).all()
    e_in = np.concatenate([rng.uniform(-80, 80, 100000), rng.uniform(-3, 3, 100000)]).astype(np.float32)
    e = np.zeros_like(e_in)
    L.orc_exp(e_in, e_in.size, e)
    assert _ulps(e, np.exp(e_in.astype(np.float64))).max() <= 4
    l_in = np.concatenate([rng.uniform(1e-7, 1, 100000), rng.uniform(0.5, 2, 100000),
                           np.exp(rng.uniform(-80, 80, 10000))]).astype(np.float32)
    lg = np.zeros_like(l_in)
    L.orc_log(l_in, l_in.size, lg)
    ld = np.log(l_in.astype(np.float64))
    far = np.abs(ld) > 0.05
    assert _ulps(lg[far], ld[far]).max() <= 4 and np.max(np.abs(lg - ld)) < 1e-6 * np.maximum(1, np.abs(ld)).max()


@pytest.mark.parametrize("seed,subseq,offset,expect", [
    # Random123 kat_vectors for philox4x32-10: counter (c0..c3) = (offset lo, hi, subsequence lo, hi),
    # key (k0, k1) = (seed lo, hi).
    (0, 0, 0, [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    (2**64 - 1, 2**64 - 1, 2**64 - 1, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    (0x299F31D0A4093822, 0x0370734413198A2E, 0x85A308D3243F6A88, [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
])
def test_philox_known_answers(seed, subseq, offset, expect):
    out = np.zeros(4, np.uint32)
    O.lib().orc_philox(seed, subseq, offset, out)
    assert [int(v) for v in out] == expect
