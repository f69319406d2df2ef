"""The oracle's multi-threaded step (the PDVec restatement, o_step_mt) gives the results of
its single-threaded step bit for bit: addresses, amplitude bits and every statistic, for the
three styles on the three models, any thread count, and when the contributions are processed
in several passes for lack of memory."""
import numpy as np
import pytest

import oracle as O

SEED = 0x5EED


def _cases():
    rng = np.random.default_rng(4)
    real = O.real1d(12, 12, 2.0, 1.0)
    keys = O.basis(real)[:30000]
    yield "int-real1d", real, O.STYLE_INTEGER, keys, rng.integers(-5, 6, len(keys)), {}
    yield "dss-real1d", real, O.STYLE_DSS, keys, rng.normal(size=len(keys)) * 3, \
        dict(proj_threshold=1.0, compression=1.0)
    yield "det-real1d", real, O.STYLE_DETERMINISTIC, keys, rng.normal(size=len(keys)), {}
    rs = O.realspace(9, (3, 3), u=3.0)
    k2 = O.basis(rs)[::7]
    yield "dss-realspace", rs, O.STYLE_DSS, k2, rng.normal(size=len(k2)) * 5, \
        dict(proj_threshold=1.0, compression=1.0)
    mom = O.mom1d(5, 10, 2.0, 1.0)
    k3 = O.basis(mom)[::3]
    yield "det-mom1d", mom, O.STYLE_DETERMINISTIC, k3, rng.normal(size=len(k3)) * 10.0 ** \
        rng.uniform(-12, 2, len(k3)), {}
    yield "int-mom1d", mom, O.STYLE_INTEGER, k3, rng.integers(-4, 5, len(k3)), {}
    fermi = O.realspace(4, (4, 4), u=0.0, fermion=True)
    k4 = O.basis(fermi)
    yield "dss-fermi", fermi, O.STYLE_DSS, k4, rng.normal(size=len(k4)) * 4, \
        dict(proj_threshold=1.0, compression=1.0)


CASES = list(_cases())


@pytest.mark.parametrize("name,m,style,keys,vals,kw", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("threads,budget", [(1, 8e9), (4, 8e9), (3, 2e5)],
                         ids=["1-thread", "4-threads", "passes"])
def test_threaded_step_equals_single_threaded_step(name, m, style, keys, vals, kw, threads,
                                                   budget):
    nz = vals != 0
    k, v = keys[nz], vals[nz]
    p = O.StepParams(style, dt=0.01, shift=-1.0, seed=SEED, step=3, **kw)
    a = O.step(m, p, k, v)
    b = O.step_mt(m, p, k, v, threads=threads, mem_budget=budget)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(np.asarray(a[1]).view(np.uint64), np.asarray(b[1]).view(np.uint64))
    assert a[2] == b[2]


def test_threaded_step_rejects_what_it_does_not_cover():
    m = O.real1d(6, 6, 6.0, 1.0)
    p = O.StepParams(O.STYLE_DSS, init_rule=O.INIT_INITIATOR)
    with pytest.raises(ValueError):
        O.step_mt(m, p, np.array([O.bose_key([1] * 6)], np.uint64), np.array([10.0]))


def test_threaded_hv_adjoint_is_repeatable_and_sums_correctly():
    """The rows of the oracle's H*v adjoint run in parallel and its two sums in row order:
    repeated calls agree bit for bit, and the sums agree with correctly rounded ones."""
    import math
    m = O.real1d(8, 8, 2.0, 1.0)
    keys = O.basis(m)
    rng = np.random.default_rng(3)
    v, gw = rng.normal(size=len(keys)), rng.normal(size=len(keys))
    a = O.hv_basis_adjoint(m, keys, v, gw)
    b = O.hv_basis_adjoint(m, keys, v, gw)
    assert np.array_equal(a[0], b[0]) and a[1] == b[1] and a[2] == b[2]
    inter = np.array([sum(n * (n - 1) for n in O.bose_onr(int(k), 8)) for k in keys])
    kg = O.hv_basis(O.real1d(8, 8, 0.0, 1.0), keys, gw)        # the hopping part K gw
    for got, terms in ((a[1], gw * (inter / 2 * v)), (a[2], v * kg)):
        assert abs(got - math.fsum(terms)) <= 1e-13 * np.abs(terms).sum()


@pytest.mark.parametrize("N,M", [(3, 3), (6, 6), (5, 9), (7, 4), (2, 30), (12, 12)])
def test_bit_level_real1d_equals_occupation_number_functions(N, M):
    """The threaded step's bit-level HubbardReal1D (hopnextneighbour and
    bose_hubbard_interaction on the chunk) against the oracle's occupation-number functions,
    on every basis state (up to 30 000 of them) and every offdiagonal."""
    m = O.real1d(N, M, 3.0, 0.7)
    keys = O.basis(m)
    if len(keys) > 30000:
        keys = keys[np.random.default_rng(1).choice(len(keys), 30000, replace=False)]
    for k in keys:
        k = int(k)
        assert O.real1d_bits_offdiagonals(m, k) == O.offdiagonals(m, k), k
        assert O.real1d_bits_diagonal(m, k) == O.diagonal(m, k), k


def test_bits_path_of_the_threaded_step_gives_the_same_step():
    m = O.real1d(20, 20, 4.0, 1.0)
    # M = N = 20 addresses: the unit filling and its neighbourhood grown by the oracle
    k0 = O.bose_key([1] * 20)
    k, v = np.array([k0], np.uint64), np.array([300.0])
    for s in range(1, 6):
        k, v, _ = O.step(m, O.StepParams(O.STYLE_DETERMINISTIC, dt=0.05, shift=0.0, step=s), k, v)
    for style, vals, kw in ((O.STYLE_DSS, v * 3, dict(compression=1.0)),
                            (O.STYLE_INTEGER, np.round(v).astype(np.int64) + 1, {}),
                            (O.STYLE_DETERMINISTIC, v, {})):
        nz = vals != 0
        p = O.StepParams(style, dt=1e-3, shift=-1.0, seed=SEED, step=2, **kw)
        a = O.step(m, p, k[nz], vals[nz])
        b = O.step_mt(m, p, k[nz], vals[nz], threads=4, bits=True)
        assert np.array_equal(a[0], b[0])
        assert np.array_equal(np.asarray(a[1]).view(np.uint64), np.asarray(b[1]).view(np.uint64))
        assert a[2] == b[2]


def test_fixed_point_conversion_on_bits_agrees():
    """The threaded step converts contributions to fixed point from their IEEE bits; on
    every kind of double (zero, subnormal, tiny, inexact, exact, at and beyond 2^48, inf,
    nan) it decides and converts as the oracle's arithmetic conversion does."""
    lib = O.lib()
    rng = np.random.default_rng(5)
    special = [0.0, -0.0, 5e-324, 1e-310, 2.0 ** -64, 2.0 ** -65, 3 * 2.0 ** -64, 2.0 ** -12,
               2.0 ** -13 * 3, 1.0, -1.5, 0.1, 2.0 ** 47, 2.0 ** 48, -(2.0 ** 48) + 1, 2.0 ** 60,
               float("inf"), float("nan"), 0.057, 1e-3 * 1.4142135623730951]
    xs = special + list(rng.normal(size=2000) * 10.0 ** rng.uniform(-25, 18, 2000))
    xs += list(np.ldexp(rng.integers(1, 2 ** 53, 2000).astype(float), rng.integers(-120, 0, 2000)))
    for x in xs:
        assert lib.o_to_fixed_agree(float(x)) == 1, x
