"""Batched replicas (rimu_batch_*): one launch per kernel for many independent runs.
A batched step equals the plain step of each replica bit for bit (same shift, replica id r in
the random key); graph replay equals eager launches; the device shift update follows
DoubleLogUpdate; a batch of problems that differ in u gives each problem's exact energy."""
import math

import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import oracle_model

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def random_start(h, n, rng, integer):
    keys = O.basis(oracle_model(h))
    keys = keys[rng.permutation(len(keys))[:n]]
    if integer:
        vals = rng.integers(1, 8, len(keys)) * rng.choice([-1, 1], len(keys))
    else:
        vals = rng.normal(size=len(keys)) * 4
    addr = h.address
    return {type(addr).from_key(int(k), addr.N, addr.M): v for k, v in zip(keys, vals)}


def plain_steps(h, style, start, shift, dt, r, steps):
    """The same replica stepped alone with rimu_apply_operator (replica id r)."""
    v = R.GPUDVec(start, style=style)
    wm = R.GPUWorkingMemory(SEED)
    wm.replica = r
    out = []
    for s in range(1, steps + 1):
        pv = v.similar()
        R.apply_operator(wm, pv, v, R.FirstOrderTransitionOperator(h, shift, dt), step=s)
        v = pv
        out.append((v.sorted_arrays(), dict(wm.last_stats)))
    return out


@pytest.mark.parametrize("kind", ["dss-realspace", "int-real1d"])
def test_batched_step_equals_plain_step_per_replica(kind):
    rng = np.random.default_rng(3)
    if kind == "dss-realspace":
        geo = R.PeriodicBoundaries(3, 3)
        hs = [R.HubbardRealSpace(R.BoseFS([1] * 9), geo, u=[[u]]) for u in (1.0, 3.0, 6.0, 9.0)]
        style = R.IsDynamicSemistochastic()
    else:
        hs = [R.HubbardReal1D(R.BoseFS([1] * 8), u=u) for u in (2.0, 4.0, 6.0)]
        style = R.IsStochasticInteger()
    integer = style.valtype is int
    starts = [random_start(h, 400, rng, integer) for h in hs]
    shifts = [-5.0 - r for r in range(len(hs))]
    dt = 0.01
    want = [plain_steps(h, style, starts[r], shifts[r], dt, r, 3) for r, h in enumerate(hs)]
    b = R.BatchedReplicas(hs, style, dt, targets=1e6, starts=starts, shifts=shifts, seed=SEED,
                          shift_update=False, use_graph=False, autotune=False)
    for s in range(3):
        res = b.run(1)
        for r in range(len(hs)):
            (wk, wv), wst = want[r][s]
            gk, gv = b.sorted_arrays(r)
            assert np.array_equal(gk, wk)
            assert np.array_equal(gv.view(np.uint64), wv.view(np.uint64))
            assert res["norm"][0, r] == wst["norm"]
            assert res["len"][0, r] == wst["len"]
            assert res["spawns"][0, r] == wst["spawns"]
            assert res["spawn_attempts"][0, r] == wst["spawn_attempts"]
            assert res["shift"][0, r] == shifts[r]


def test_graph_replay_equals_eager_launches():
    rng = np.random.default_rng(5)
    geo = R.PeriodicBoundaries(3, 3)
    hs = [R.HubbardRealSpace(R.BoseFS([1] * 9), geo, u=[[u]]) for u in (2.0, 5.0)]
    style = R.IsDynamicSemistochastic()
    starts = [random_start(h, 300, rng, False) for h in hs]

    def run(graph):
        b = R.BatchedReplicas(hs, style, 0.01, targets=[3000, 5000], starts=starts,
                              shifts=[-6.0, -4.0], seed=SEED, segment_steps=4, use_graph=graph,
                              autotune=False)
        res = b.run(16)
        return b, res

    ba, ra = run(False)
    bb, rb = run(True)
    assert bb.info()["graph_segments"] >= 2
    for f in ra:
        assert np.array_equal(ra[f], rb[f]), f
    for r in range(2):
        ka, va = ba.sorted_arrays(r)
        kb, vb = bb.sorted_arrays(r)
        assert np.array_equal(ka, kb) and np.array_equal(va, vb)


def test_device_shift_update_follows_double_log_update():
    h = R.HubbardReal1D(R.BoseFS([1] * 6), u=6.0)
    style = R.IsStochasticInteger()
    b = R.BatchedReplicas([h, h], style, 1e-3, targets=[200, 400], seed=SEED,
                          starts=[{h.address: 10}, {h.address: 20}], autotune=False,
                          segment_steps=8)
    res = b.run(200)
    ζ, ξ, dt = 0.08, 0.08 ** 2 / 4, 1e-3
    S0 = h.diagonal_element(h.address)
    for r, (tgt, n0) in enumerate(((200, 10), (400, 20))):
        S, pn = S0, float(n0)
        for s in range(200):
            N = res["norm"][s, r]
            if res["len"][s, r]:
                S -= ξ / dt * math.log(N / tgt) + ζ / dt * math.log(N / pn)
                pn = N
            assert abs(res["shift"][s, r] - S) <= 1e-12 * max(1.0, abs(S)), (s, r)
            S = res["shift"][s, r]       # follow the device value (ulp-level log differences)


def test_solve_batched_gives_each_problem_its_exact_energy():
    """Four problems that differ only in u, solved together: each problem's shift agrees with
    its exact ground energy within 2 blocking errors (no absolute floor)."""
    us = (2.0, 4.0, 6.0, 8.0)
    probs = []
    for i, u in enumerate(us):
        H = R.HubbardReal1D(R.BoseFS([1] * 6), u=u)
        probs.append(R.ProjectorMonteCarloProblem(H, style=R.IsDynamicSemistochastic(),
                                                  target_walkers=300 * (i + 1), time_step=1e-2,
                                                  last_step=20000, random_seed=77,
                                                  shift_strategy=R.DoubleLogUpdate(300 * (i + 1), 0.05, 0.05 ** 2 / 4)))
    sims = R.solve_batched(probs, segment_steps=64)
    for u, sim in zip(us, sims):
        E0 = O.ground_energy(O.real1d(6, 6, u))
        r = R.shift_estimator(sim.df, skip=2000)
        assert abs(r.mean - E0) < 2 * r.err, (u, r.mean, r.err, E0)


def test_batch_rejects_models_on_different_lattices():
    h1 = R.HubbardReal1D(R.BoseFS([1] * 6), u=6.0)
    h2 = R.HubbardReal1D(R.BoseFS([1] * 5), u=6.0)
    with pytest.raises(R.RimuError):
        R.BatchedReplicas([h1, h2], R.IsStochasticInteger(), 1e-3, targets=100)
