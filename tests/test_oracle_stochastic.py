"""The oracle's stochastic primitives against the reference's own statistical tests
(test/StochasticStyles.jl:187-275): sampled spawning averages to exact spawning, and threshold
compression leaves a vector unchanged on average.  CPU only: this pins the checker's random
parts before it is trusted for GPU parity."""
import numpy as np
import pytest

import oracle as O


def _sums(outputs):
    """Sum of several sparse vectors given as (keys, values) pairs, as {key: value}."""
    keys = np.concatenate([k for k, _ in outputs])
    vals = np.concatenate([np.asarray(v, dtype=float) for _, v in outputs])
    uniq, inv = np.unique(keys, return_inverse=True)
    return dict(zip(uniq.tolist(), np.bincount(inv, weights=vals).tolist()))


# the reference's two (Hamiltonian, address) cases, test/StochasticStyles.jl:196-199
SPAWN_CASES = [
    ("mom1d", O.mom1d(5, 6, u=6.0), [0, 0, 0, 3, 1, 1]),
    ("real1d", O.real1d(10, 7, u=1.0), [5, 0, 0, 5, 0, 0, 0]),
]


@pytest.mark.parametrize("style", [O.STYLE_DSS, O.STYLE_INTEGER], ids=["dss", "integer"])
@pytest.mark.parametrize("name,m,onr", SPAWN_CASES, ids=[c[0] for c in SPAWN_CASES])
def test_sampled_spawns_average_to_exact_spawns(name, m, onr, style):
    """10 000 columns of one address with random values in [0, 1.2 n_offdiag): the summed
    sampled steps (WithReplacement attempts, exact columns where DynamicSemistochastic switches
    to them; integer walkers rounded stochastically) agree with the summed exact steps within
    10 % on every address, the reference's bound for these strategies."""
    key = O.bose_key(onr)
    noff = O.num_offdiagonals(m, key)
    rng = np.random.default_rng(11)
    sampled, exact = [], []
    for i in range(10000):
        val = rng.random() * noff * 1.2
        if style == O.STYLE_INTEGER:
            val = float(max(1, round(val)))
            src = np.array([int(val)], dtype=np.int64)
        else:
            src = np.array([val])
        k, v, _ = O.step(m, O.StepParams(style, dt=0.1, seed=77, step=i + 1), [key], src)
        sampled.append((k, v))
        k, v, _ = O.step(m, O.StepParams(O.STYLE_DETERMINISTIC, dt=0.1, step=i + 1), [key],
                         np.array([val]))
        exact.append((k, v))
    s, e = _sums(sampled), _sums(exact)
    assert 1 < len(e) <= noff + 1     # the address and its distinct offdiagonal targets
    for a, want in e.items():
        assert s.get(a, 0.0) == pytest.approx(want, rel=0.1), a


@pytest.mark.parametrize("threshold", [1.0, 2.0])
def test_threshold_compression_preserves_the_vector_on_average(threshold):
    """ThresholdCompression(1) and (2) applied 1 000 times to a normalised vector of
    HubbardMom1D(BoseFS(0,0,0,10,0,0,0)) (test/StochasticStyles.jl:240-275): every compressed
    vector is shorter, the source is unchanged, and the average has the source's walker number
    and unit overlap with it within 10 %.  A step with dt = 0 is the compression alone (the
    transition operator is the identity and every spawn is zero)."""
    import scipy.sparse.linalg as sla
    m = O.mom1d(10, 7)
    start = O.bose_key([0, 0, 0, 10, 0, 0, 0])
    keys = O.connected_basis(m, start)
    _, vecs = sla.eigsh(O.sparse_matrix(m, keys), k=1, which="SA")
    dv = vecs[:, 0] / np.linalg.norm(vecs[:, 0])
    keep = dv != 0.0
    keys, dv = np.ascontiguousarray(keys[keep]), np.ascontiguousarray(dv[keep])
    before = dv.copy()
    outs = []
    for i in range(1000):
        k, v, _ = O.step(m, O.StepParams(O.STYLE_DSS, dt=0.0, seed=5, step=i + 1,
                                         compression=threshold), keys, dv)
        assert len(k) < len(keys)
        outs.append((k, v / 1000))
    assert np.array_equal(dv, before)
    avg = _sums(outs)
    pos = {int(a): i for i, a in enumerate(keys.tolist())}
    overlap = sum(val * dv[pos[a]] for a, val in avg.items())
    assert sum(abs(x) for x in avg.values()) == pytest.approx(np.abs(dv).sum(), rel=0.1)
    assert overlap == pytest.approx(1.0, rel=0.1)


def test_style_comparison_on_the_reference_model():
    """The reference's style comparison (test/lomc.jl:543-605) for the styles of this path:
    HubbardReal1D(BoseFS{5,5}(1,1,1,1,1)), one walker to start, DoubleLogUpdate(zeta=0.05,
    xi=zeta^2/4, target 100), dt = 0.01, 2 500 steps.  Every style's shift (steps 500 on)
    lies within 3 of its errors of E0 = -8.280991746582686, and the stochastic-integer error
    exceeds the dynamic-semistochastic one."""
    import rimugpu as R
    from rimugpu.stats import mean_and_se
    from helpers import oracle_solve
    m = O.real1d(5, 5, 1.0, 1.0)
    E0 = -8.280991746582686
    assert O.ground_energy(m) == pytest.approx(E0, abs=1e-12)
    key = R.BoseFS([1] * 5).key
    est = {}
    for name, style, pop in (("st", R.IsStochasticInteger(), 1),
                             ("dy", R.IsDynamicSemistochastic(), 1.0),
                             ("de", R.IsDeterministic(), 1.0),
                             ("dp", R.IsDeterministic(R.ThresholdCompression()), 1.0)):
        df = oracle_solve(m, style, key, pop, 2500, 0.01, 100, 1234, zeta=0.05)
        E, se = mean_and_se(np.asarray(df["shift"][499:]))
        assert abs(E - E0) <= 3 * se, (name, E, se)
        est[name] = se
    assert est["st"] > est["dy"]


def test_initiator_energies_below_the_plateau():
    """The reference's initiator test (test/lomc.jl:611-673) through the oracle:
    HubbardMom1D(BoseFS{10,10} with all bosons in k = 0; u = 4), IsDynamicSemistochastic, one
    walker to start, DoubleLogUpdate(zeta=0.05, xi=zeta^2/4, target 300), dt = 5e-4, 6 000
    steps, shift averaged from step 2 000.  Below the plateau the run without a rule (and with
    NonInitiator) falls below E0; the initiator rules are biased above E0, SimpleInitiator
    most; Initiator and CoherentInitiator agree within 3 errors."""
    import rimugpu as R
    from rimugpu.stats import mean_and_se
    from helpers import oracle_solve
    m = O.mom1d(10, 10, 4.0, 1.0)
    key = O.bose_key([0] * 4 + [10] + [0] * 5)
    E0 = -9.251592973178997
    E, S = {}, {}
    for name, rule in (("no", None), ("i1", R.Initiator(1)), ("i2", R.SimpleInitiator(1)),
                       ("i3", R.CoherentInitiator(1)), ("ni", R.NonInitiator())):
        df = oracle_solve(m, R.IsDynamicSemistochastic(), key, 1.0, 6000, 5e-4, 300, 8008,
                          zeta=0.05, initiator=rule)
        E[name], S[name] = mean_and_se(np.asarray(df["shift"][1999:]))
    assert E["no"] < E0 and E["ni"] < E0
    assert abs(E["no"] - E["ni"]) <= 3 * S["no"]
    assert E["i1"] > E0 and E["i2"] > E0 and E["i3"] > E0
    assert E["i2"] > E["i1"]
    assert abs(E["i1"] - E["i3"]) <= max(3 * S["i1"], 3 * S["i3"])


def test_initiator_energies_above_the_plateau():
    """The second half of the reference's initiator test (test/lomc.jl:675-702) through the
    oracle: HubbardMom1D(BoseFS{10,10}, all bosons in k = 0; u = 1), IsDynamicSemistochastic,
    target 3 000, dt = 1e-2, 2 500 steps, shift averaged from step 500.  Above the plateau
    every rule, and none, gives E0 = -16.36048582876015 within 3 errors."""
    import rimugpu as R
    from rimugpu.stats import mean_and_se
    from helpers import oracle_solve
    m = O.mom1d(10, 10, 1.0, 1.0)
    key = O.bose_key([0] * 4 + [10] + [0] * 5)
    E0 = -16.36048582876015
    for rule in (None, R.Initiator(1), R.SimpleInitiator(1), R.CoherentInitiator(1)):
        df = oracle_solve(m, R.IsDynamicSemistochastic(), key, 1.0, 2500, 1e-2, 3000, 1337,
                          zeta=0.05, initiator=rule)
        E, se = mean_and_se(np.asarray(df["shift"][499:]))
        assert abs(E - E0) <= 3 * se, (rule, E, se)


def test_ground_state_energy_estimates_of_the_seven_site_model():
    """The reference's ground-state estimates (test/mpi_runtests.jl:157-203) through the
    oracle, E0 = -4.628524493494574 for HubbardReal1D(BoseFS(1,1,1,1,1,1,1); u=6).
    IsDynamicSemistochastic from 3 walkers with the default target 1 000 and dt = 0.01, 5 000
    steps: the 3-error interval of the shift (from step 2 000) and of the projected energy
    contain E0.  Integer walkers under Initiator(1) on the momentum-space form
    HubbardMom1D(BoseFS(0,0,0,7,0,0,0); u=6), target 100: the shift stays above E0 (the
    initiator bias).  The reference's other post-step observables are outside this path."""
    import rimugpu as R
    from rimugpu.stats import mean_and_se
    from helpers import oracle_solve
    E0 = -4.628524493494574
    m = O.real1d(7, 7, 6.0, 1.0)
    df = oracle_solve(m, R.IsDynamicSemistochastic(), O.bose_key([1] * 7), 3.0, 5000, 0.01,
                      1000, 13)
    Es, se = mean_and_se(np.asarray(df["shift"][1999:]))
    assert Es - 3 * se < E0 < Es + 3 * se
    pe, pe_err = R.projected_energy(df, skip=1999)
    assert pe - 3 * pe_err < E0 < pe + 3 * pe_err
    mm = O.mom1d(7, 7, 6.0, 1.0)
    k0 = O.bose_key([0, 0, 0, 7, 0, 0, 0])
    assert O.ground_energy(mm, start=k0) == pytest.approx(E0, abs=1e-9)
    df = oracle_solve(mm, R.IsStochasticInteger(), k0, 3, 5000, 0.01, 100, 13,
                      initiator=R.Initiator(1))
    Es, _ = mean_and_se(np.asarray(df["shift"][1999:]))
    assert E0 <= Es
