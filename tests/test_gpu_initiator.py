"""Initiator rules (initiators.jl:132-234, InitiatorDVec initiatordvec.jl:186-196): each
contribution is "safe", "unsafe" or "initiator" by its parent, the classes are summed
separately and combined by the rule.  Trajectories against the oracle bit for bit for every
rule and style, and the reference's initiator-bias test (test/lomc.jl:612-676)."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import assert_same_step, gpu_step, oracle_model, oracle_params

pytestmark = pytest.mark.gpu

SEED = 0x5EED
RULES = [R.Initiator(1.0), R.SimpleInitiator(1.0), R.CoherentInitiator(1.0), R.Initiator(2.5)]


def mixed_start(h, n, rng, integer):
    """A vector with initiators and non-initiators (|values| on both sides of the thresholds)."""
    keys = O.basis(oracle_model(h))
    keys = np.sort(keys[rng.permutation(len(keys))[:n]])
    if integer:
        vals = rng.integers(1, 5, len(keys)) * rng.choice([-1, 1], len(keys))
    else:
        vals = rng.choice([-1, 1], len(keys)) * 10.0 ** rng.uniform(-0.5, 0.8, len(keys))
    return keys, vals


@pytest.mark.parametrize("rule", RULES, ids=[repr(r) for r in RULES])
@pytest.mark.parametrize("kind", ["dss-real1d", "int-real1d", "det-real1d", "dss-mom1d"])
def test_initiator_trajectory_matches_oracle(rule, kind):
    rng = np.random.default_rng(21)
    if kind.endswith("mom1d"):
        h = R.HubbardMom1D(R.BoseFS(8, {4: 6}), u=4.0)
    else:
        h = R.HubbardReal1D(R.BoseFS([1] * 8), u=4.0)
    style = {"dss": R.IsDynamicSemistochastic(), "int": R.IsStochasticInteger(),
             "det": R.IsDeterministic(R.ThresholdCompression(0.5))}[kind.split("-")[0]]
    integer = style.valtype is int
    keys, vals = mixed_start(h, 300, rng, integer)
    m = oracle_model(h)
    dt, S = 0.01, -4.0
    wm = R.GPUWorkingMemory(SEED)
    for step in range(1, 13):
        g = gpu_step(h, style, keys, vals, dt, S, SEED, step, wm=wm, initiator=rule)
        o = O.step(m, oracle_params(style, dt, S, SEED, step, initiator=rule), keys, vals)
        assert_same_step(g, o, style)
        keys, vals = o[0], o[1]
        assert len(keys) > 0


def test_no_rule_is_the_plain_step():
    rng = np.random.default_rng(4)
    h = R.HubbardReal1D(R.BoseFS([1] * 8), u=4.0)
    style = R.IsDynamicSemistochastic()
    keys, vals = mixed_start(h, 200, rng, False)
    a = gpu_step(h, style, keys, vals, 0.01, -4.0, SEED, 1, initiator=R.NonInitiator())
    b = gpu_step(h, style, keys, vals, 0.01, -4.0, SEED, 1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_initiator_energies_below_the_plateau():
    """test/lomc.jl:639-676: HubbardMom1D, 10 bosons in k=0 of 10 modes, u=4,
    E0 = -9.251592973178997, 300 walkers: without initiators the shift falls below E0 (the
    annihilation plateau is not reached); every initiator rule biases it above E0, the simple
    rule most."""
    address = R.BoseFS(10, {5: 10})
    H = R.HubbardMom1D(address, u=4.0)
    E0 = -9.251592973178997
    res = {}
    for name, init in (("no", False), ("i1", R.Initiator(1)), ("i2", R.SimpleInitiator(1)),
                       ("i3", R.CoherentInitiator(1))):
        p = R.ProjectorMonteCarloProblem(H, start_at={address: 1.0}, initiator=init,
                                         style=R.IsDynamicSemistochastic(), time_step=5e-4,
                                         last_step=6000, random_seed=8008,
                                         shift_strategy=R.DoubleLogUpdate(300, 0.05, 0.05 ** 2 / 4))
        sim = R.solve(p)
        assert sim.success, sim.message
        res[name] = R.mean_and_se(sim.df["shift"][1999:])
    (E_no, s_no), (E_i1, s_i1), (E_i2, s_i2), (E_i3, s_i3) = (res[k] for k in ("no", "i1", "i2", "i3"))
    assert E_no < E0
    assert E_i1 > E0 and E_i2 > E0 and E_i3 > E0
    assert E_i2 > E_i1
    assert abs(E_i1 - E_i3) <= max(3 * s_i1, 3 * s_i3)
