"""Device dot products between walker lists and the AllOverlaps replica strategy
(replicastrategy.jl:112-190): dot(v, w) against numpy, dot(w, H, v) against the sparse
matrix of the oracle, and the c{i}_dot_c{j} / c{i}_Op{k}_c{j} report columns."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import oracle_model

pytestmark = pytest.mark.gpu


def vec(h, keys, vals, style, capacity):
    v = R.GPUDVec(style=style, address_type=h.address, capacity=capacity)
    v.upload(keys, vals)
    return v


@pytest.mark.parametrize("integer", [False, True])
def test_device_dot_matches_numpy_across_bucket_counts(integer):
    h = R.HubbardReal1D(R.near_uniform(R.BoseFS, 10, 10), u=2.0)
    keys = O.basis(oracle_model(h))
    rng = np.random.default_rng(8)
    style = R.IsStochasticInteger() if integer else R.IsDeterministic()
    ka = keys[rng.permutation(len(keys))[:40000]]
    kb = keys[rng.permutation(len(keys))[:25000]]
    if integer:
        va, vb = rng.integers(-9, 10, len(ka)), rng.integers(-9, 10, len(kb))
        va[va == 0] = 1
        vb[vb == 0] = 1
    else:
        va, vb = rng.normal(size=len(ka)), rng.normal(size=len(kb))
    da = dict(zip(ka.tolist(), va.astype(float)))
    db = dict(zip(kb.tolist(), vb.astype(float)))
    want = float(sum(da[k] * db[k] for k in set(da) & set(db)))
    for cap_a, cap_b in ((0, 0), (1 << 20, 1000), (500, 1 << 18)):
        a = vec(h, ka, va, style, cap_a)
        b = vec(h, kb, vb, style, cap_b)
        got = a.dot(b)
        assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (cap_a, cap_b, got, want)
        assert got == b.dot(a) or abs(got - b.dot(a)) <= 1e-12 * max(1.0, abs(want))
        assert got == a.dot(b)          # fixed order: repeated calls agree exactly


def test_dot_operator_matches_sparse_matrix():
    h = R.HubbardRealSpace(R.BoseFS([1, 1, 0, 1, 0, 1]), R.PeriodicBoundaries(2, 3), u=[[1.5]])
    m = oracle_model(h)
    keys = O.basis(m)
    rng = np.random.default_rng(9)
    x, y = rng.normal(size=len(keys)), rng.normal(size=len(keys))
    H = O.sparse_matrix(m, keys)
    want = float(y @ (H @ x))
    xv = vec(h, keys, x, R.IsDeterministic(), 0)
    yv = vec(h, keys, y, R.IsDeterministic(), 0)
    got = R.dot_operator(yv, h, xv)
    assert abs(got - want) <= 1e-11 * max(1.0, abs(want)), (got, want)
    # integer vectors are promoted on the device
    xi = rng.integers(-5, 6, len(keys))
    xi[xi == 0] = 2
    xiv = vec(h, keys, xi, R.IsStochasticInteger(), 0)
    got_i = R.dot_operator(yv, h, xiv)
    want_i = float(y @ (H @ xi.astype(float)))
    assert abs(got_i - want_i) <= 1e-11 * max(1.0, abs(want_i))


def test_all_overlaps_reports_dot_and_operator_columns():
    addr = R.BoseFS([1] * 6)
    H = R.HubbardReal1D(addr, u=6.0)
    p = R.ProjectorMonteCarloProblem(H, replica_strategy=R.AllOverlaps(2, operator=H),
                                     style=R.IsDynamicSemistochastic(), target_walkers=500,
                                     time_step=0.01, last_step=60, random_seed=5)
    sim = R.solve(p)
    df = sim.df
    assert {"c1_dot_c2", "c1_Op1_c2", "shift_1", "shift_2"} <= set(df)
    assert len(df["c1_dot_c2"]) == 60
    v1, v2 = sim.states[0].v, sim.states[1].v
    k1, a1 = v1.download()
    k2, a2 = v2.download()
    d2 = dict(zip(k2.tolist(), a2))
    want = float(sum(x * d2.get(k, 0.0) for k, x in zip(k1.tolist(), a1)))
    assert abs(df["c1_dot_c2"][-1] - want) <= 1e-12 * max(1.0, abs(want))
    assert abs(df["c1_Op1_c2"][-1] - R.dot_operator(v1, H, v2)) <= 1e-12 * max(1.0, abs(df["c1_Op1_c2"][-1]))
