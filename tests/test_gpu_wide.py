"""Addresses of 65-128 bits (the reference's two-chunk BitString, bitstring.jl:6-18) on the
GPU against the oracle, bit for bit: HubbardReal1D with BoseFS{50,50} (99 bits) and
BoseFS{40,30} (69 bits), HubbardRealSpace with bosons on an 8x8 lattice (103 bits) and with
fermions on a 10x10 lattice (100 bits), HubbardMom1D with 20 bosons in 50 momentum modes
(69 bits); matrix elements and step trajectories of the three styles, whose random numbers are
keyed on lo ^ mix64(hi) of the address; initiator rules (the flag in bit 63 of the top word)
and dot products of two-word lists."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import assert_same_step, gpu_step, oracle_model, oracle_params, run_trajectory

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def _models():
    b8 = [1, 0] * 32
    b8[:8] = [2] * 8      # 40 bosons on 64 sites
    f10 = [1] * 10 + [0] * 90
    return {
        "real1d-99": R.HubbardReal1D(R.BoseFS([1] * 50), u=4.0),
        "real1d-69": R.HubbardReal1D(R.BoseFS([1] * 30 + [0] * 10 + [2] * 5), u=2.0, t=0.5),
        "realspace-bose-103": R.HubbardRealSpace(R.BoseFS(b8), geometry=R.PeriodicBoundaries(8, 8),
                                                 u=[[3.0]], v=[1.5, 0.5]),
        "realspace-fermi-100": R.HubbardRealSpace(R.FermiFS(f10), geometry=R.HardwallBoundaries(10, 10)),
        "mom1d-69": R.HubbardMom1D(R.BoseFS(50, {25: 20}), u=2.0),
    }


def _neighbourhood(m, key, depth=2, cap=300):
    """Addresses reachable from `key` in `depth` hops (oracle), for element checks."""
    seen, frontier = {key}, [key]
    for _ in range(depth):
        nxt = []
        for k in frontier:
            for nk, v in O.offdiagonals(m, k):
                if v != 0.0 and nk not in seen and len(seen) < cap:
                    seen.add(nk)
                    nxt.append(nk)
        frontier = nxt
    return sorted(seen)


@pytest.mark.parametrize("name", list(_models()))
def test_wide_matrix_elements_match_oracle(name):
    h = _models()[name]
    m = oracle_model(h)
    assert h.address.nbits > 64 and m.nbits == h.address.nbits
    keys = _neighbourhood(m, h.address.key)
    got = h.diagonal_elements(keys)
    want = np.array([O.diagonal(m, k) for k in keys])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    for k in keys[:: max(1, len(keys) // 60)]:
        gk, gv = h.offdiagonal_keys(k)
        ref = O.offdiagonals(m, k)
        assert [int(x) for x in gk] == [r[0] for r in ref]
        assert np.array_equal(np.asarray(gv, dtype=float).view(np.uint64),
                              np.array([r[1] for r in ref]).view(np.uint64))


CASES = [
    ("dss-real1d-99", "real1d-99", R.IsDynamicSemistochastic, 500.0, 25, 0.005),
    ("int-real1d-69", "real1d-69", R.IsStochasticInteger, 400, 25, 0.01),
    ("det-real1d-69", "real1d-69", R.IsDeterministic, 1.0, 5, 0.02),
    ("dss-realspace-bose-103", "realspace-bose-103", R.IsDynamicSemistochastic, 300.0, 20, 0.005),
    ("int-realspace-fermi-100", "realspace-fermi-100", R.IsStochasticInteger, 300, 20, 0.01),
    ("det-mom1d-69", "mom1d-69", R.IsDeterministic, 1.0, 3, 0.01),
    ("int-mom1d-69", "mom1d-69", R.IsStochasticInteger, 300, 15, 0.005),
    ("dss-mom1d-69", "mom1d-69", R.IsDynamicSemistochastic, 300.0, 15, 0.005),
]


@pytest.mark.parametrize("case,model,style,pop,steps,dt", CASES, ids=[c[0] for c in CASES])
def test_wide_step_trajectory_matches_oracle(case, model, style, pop, steps, dt):
    h = _models()[model]
    target = None if style is R.IsDeterministic else pop
    run_trajectory(h, style(), {h.address: pop}, steps, dt, target=target)


def test_wide_vectors_store_and_step_many_buckets():
    """A spread-out wide vector (upload, lookup, download, several buckets and passes)."""
    h = _models()["real1d-99"]
    m = oracle_model(h)
    keys = _neighbourhood(m, h.address.key, depth=3, cap=4000)
    rng = np.random.default_rng(31)
    vals = rng.normal(size=len(keys)) * 3
    v = R.GPUDVec(style=R.IsDynamicSemistochastic(), address_type=h.address)
    v.upload(np.array(keys, dtype=object), vals)
    assert len(v) == len(keys)
    assert np.array_equal(v.lookup_keys(keys[:50]), vals[:50])
    wm = R.GPUWorkingMemory(SEED)
    wm.set_launch_shape(64, 512)
    g = gpu_step(h, R.IsDynamicSemistochastic(), np.array(keys, dtype=object), vals, 0.01, -1.0,
                 SEED, 4, wm=wm)
    o = O.step(m, oracle_params(R.IsDynamicSemistochastic(), 0.01, -1.0, SEED, 4), keys, vals)
    assert_same_step(g, o, R.IsDynamicSemistochastic())


@pytest.mark.parametrize("rule", [R.Initiator(2.0), R.SimpleInitiator(2.0), R.CoherentInitiator(2.0)],
                         ids=["initiator", "simple", "coherent"])
def test_wide_initiator_rules_match_oracle(rule):
    """Initiator rules on 99-bit addresses: the class of a spawn travels in bit 63 of the
    address's top word.  Ten DSS steps from 40 walkers, bit for bit against the oracle."""
    h = _models()["real1d-99"]
    m = oracle_model(h)
    style = R.IsDynamicSemistochastic()
    keys = np.array([h.address.key], dtype=object)
    vals = np.array([40.0])
    S = h.diagonal_element(h.address)
    wm = R.GPUWorkingMemory(SEED)
    for step in range(1, 11):
        g = gpu_step(h, style, keys, vals, 0.01, S, SEED, step, wm=wm, initiator=rule)
        o = O.step(m, oracle_params(style, 0.01, S, SEED, step, initiator=rule), keys, vals)
        assert_same_step(g, o, style)
        keys, vals = o[0], o[1]
    assert len(keys) > 20


def test_wide_dot_products():
    """<v|w> of two-word lists with different bucket counts and value types, against the
    products summed on the host."""
    h = _models()["real1d-99"]
    m = oracle_model(h)
    keys = _neighbourhood(m, h.address.key, depth=3, cap=3000)
    rng = np.random.default_rng(8)
    va = rng.normal(size=len(keys))
    ia = rng.choice(len(keys), len(keys) // 2, replace=False)
    vb = rng.integers(-5, 6, len(ia))
    a = R.GPUDVec(style=R.IsDeterministic(), address_type=h.address)
    a.upload(np.array(keys, dtype=object), va)
    b = R.GPUDVec(style=R.IsStochasticInteger(), address_type=h.address, capacity=64)
    b.upload(np.array([keys[i] for i in ia], dtype=object), vb)
    want = float(np.sum(va[ia] * vb))
    assert a.dot(b) == pytest.approx(want, rel=1e-12, abs=1e-12)
    assert b.dot(a) == pytest.approx(want, rel=1e-12, abs=1e-12)
    assert a.dot(a) == pytest.approx(float(np.sum(va * va)), rel=1e-12)


def test_wide_addresses_reject_one_word_projectors():
    h = _models()["real1d-99"]
    wm = R.GPUWorkingMemory(1)
    wm.set_projector(np.array([1, 2], dtype=np.uint64), np.ones(2), np.ones(2), key_words=1)
    with pytest.raises(R.RimuError):     # a one-word projector with a two-word model
        R.apply_operator(wm, R.GPUDVec(style=R.IsDynamicSemistochastic(), address_type=h.address),
                         R.GPUDVec({h.address: 5.0}, style=R.IsDynamicSemistochastic()),
                         R.FirstOrderTransitionOperator(h, 0.0, 0.01))


@pytest.mark.parametrize("name", ["real1d-99", "realspace-bose-103"])
def test_wide_projector_terms(name):
    """ProjectedEnergy with two-word addresses (rimu_wm_set_projector_w): after every step
    vproj = sum_i P_i v'(k_i) and hproj = sum_i (H'P)_i v'(k_i), summed in projector-key order
    exactly as the library does, from the downloaded vector; the vector itself matches the
    oracle step."""
    h = _models()[name]
    m = oracle_model(h)
    pe = R.ProjectedEnergy(h, {h.address: 1.0})
    assert pe.key_words == 2 and len(pe.keys) > 5
    style = R.IsDynamicSemistochastic()
    keys = np.array([h.address.key], dtype=object)
    vals = np.array([400.0])
    S = h.diagonal_element(h.address)
    wm = R.GPUWorkingMemory(SEED)
    wm.set_projector(pe.keys, pe.pvals, pe.hpvals, key_words=2)
    P = dict(zip((int(k) for k in pe.keys), pe.pvals))
    HP = dict(zip((int(k) for k in pe.keys), pe.hpvals))
    order = sorted(P)
    seen = 0
    for step in range(1, 9):
        g = gpu_step(h, style, keys, vals, 0.005, S, SEED, step, wm=wm)
        o = O.step(m, oracle_params(style, 0.005, S, SEED, step), keys, vals)
        assert_same_step(g, o, style)
        v = dict(zip((int(k) for k in g[0]), g[1]))
        vp = hp = 0.0
        for k in order:
            x = v.get(k, 0.0)
            vp += P[k] * x
            hp += HP[k] * x
        assert g[2]["vproj"] == vp and g[2]["hproj"] == hp
        seen += hp != 0.0
        keys, vals = o[0], o[1]
    assert seen > 0


def test_wide_projected_energy_through_solve():
    """solve() with a ProjectedEnergy on a two-word model reports finite vproj and hproj."""
    h = _models()["real1d-69"]
    p = R.ProjectorMonteCarloProblem(h, style=R.IsDynamicSemistochastic(), time_step=0.005,
                                     target_walkers=300, last_step=60, random_seed=7,
                                     post_step_strategy=R.ProjectedEnergy(h, {h.address: 1.0}))
    sim = R.solve(p)
    df = sim.df
    assert np.all(np.isfinite(df["vproj"])) and np.any(np.asarray(df["vproj"]) != 0)
    assert np.all(np.isfinite(df["hproj"]))


def test_wide_addresses_are_rejected_by_batches():
    """Batched runs take one-word addresses only: a two-word model is refused by the Python
    class and by rimu_batch_set_replica, before anything runs."""
    import ctypes as C
    import rimugpu._lib as L
    h = _models()["real1d-69"]
    with pytest.raises(ValueError):
        R.BatchedReplicas([h], R.IsDynamicSemistochastic(), 0.01, targets=1e3,
                          starts=[{h.address: 10.0}])
    lib = L.load()
    b = C.c_void_p()
    L.check(lib.rimu_batch_create(L.default_context().handle, 1, L.VAL_F64, C.byref(b)))
    try:
        k = np.array([h.address.key & ((1 << 64) - 1), h.address.key >> 64], dtype=np.uint64)
        v = np.array([10.0])
        rc = lib.rimu_batch_set_replica(b, 0, h.handle, k.ctypes.data_as(C.POINTER(C.c_uint64)),
                                        v.ctypes.data_as(C.c_void_p), 1, 0.0, 1e3)
        assert rc == L.RIMU_ERR_BADARG
    finally:
        lib.rimu_batch_destroy(b)


@pytest.mark.parametrize("name,style", [("real1d-99", R.IsDynamicSemistochastic()),
                                        ("realspace-bose-103", R.IsStochasticInteger())])
def test_wide_step_with_many_buckets_per_cta(name, style):
    """A two-word list of ~2e4 addresses at 16 contributions per bucket: a few thousand
    buckets, more than the annihilation CTAs resident on the GPU, so each CTA annihilates
    several buckets in turn (most of them empty for the integer case)."""
    h = _models()[name]
    m = oracle_model(h)
    keys = _neighbourhood(m, h.address.key, depth=3, cap=20000)
    rng = np.random.default_rng(41)
    if style.valtype is int:
        vals = rng.integers(1, 6, len(keys)) * rng.choice([-1, 1], len(keys))
    else:
        vals = rng.normal(size=len(keys)) * 3
    wm = R.GPUWorkingMemory(SEED)
    wm.set_launch_shape(16, 0)
    ka = np.array(keys, dtype=object)
    g = gpu_step(h, style, ka, vals, 0.005, -1.0, SEED, 6, wm=wm)
    o = O.step(m, oracle_params(style, 0.005, -1.0, SEED, 6), keys, vals)
    assert_same_step(g, o, style)
    assert g[2]["nb_bits"] >= 11


# ---- multi-component addresses of 65-128 bits (each component at most one word) -------------
def _wide_composites():
    f36a = [0] * 36
    f36b = [0] * 36
    for i in (0, 7, 14):
        f36a[i] = 1
    for i in (3, 10, 21):
        f36b[i] = 1
    b30 = [0] * 30
    b30[4] = 2
    f30 = [0] * 30
    for i in (1, 2, 17):
        f30[i] = 1
    c30 = [0] * 30
    c30[25] = 1
    ma = [0] * 40
    mb = [0] * 40
    for i in (18, 19, 20):
        ma[i] = 1
    for i in (19, 20, 21):
        mb[i] = 1
    return {
        "realspace-2f-6x6": R.HubbardRealSpace(R.CompositeFS(R.FermiFS(f36a), R.FermiFS(f36b)),
                                               geometry=R.PeriodicBoundaries(6, 6), t=[1.0, 1.5],
                                               u=[[0.0, 4.0], [4.0, 0.0]]),
        "realspace-3c-5x6-trap": R.HubbardRealSpace(
            R.CompositeFS(R.BoseFS(b30), R.FermiFS(f30), R.BoseFS(c30)),
            geometry=R.HardwallBoundaries(5, 6), t=[1.0, 0.5, 2.0],
            u=[[2.0, 1.0, -0.5], [1.0, 0.0, 3.0], [-0.5, 3.0, 1.0]],
            v=[[0.5, 0.25], [0.0, 1.0], [1.0, 0.0]]),
        "mom1d-fermi2c-40": R.HubbardMom1D(R.FermiFS2C(ma, mb), u=3.0, t=0.5),
    }


@pytest.mark.parametrize("name", list(_wide_composites()))
def test_wide_composite_matrix_elements_match_oracle(name):
    h = _wide_composites()[name]
    m = oracle_model(h)
    assert h.address.nbits > 64 and m.nbits == h.address.nbits
    keys = _neighbourhood(m, h.address.key, depth=2, cap=400)
    got = h.diagonal_elements(keys)
    want = np.array([O.diagonal(m, k) for k in keys])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    for k in keys[:: max(1, len(keys) // 60)]:
        gk, gv = h.offdiagonal_keys(k)
        ref = O.offdiagonals(m, k)
        assert [int(x) for x in gk] == [r[0] for r in ref]
        assert np.array_equal(np.asarray(gv).view(np.uint64),
                              np.array([r[1] for r in ref]).view(np.uint64))


WIDE_COMPOSITE_CASES = [
    ("dss-realspace-2f-6x6", "realspace-2f-6x6", R.IsDynamicSemistochastic, 300.0, 20, 0.005),
    ("int-realspace-3c-5x6", "realspace-3c-5x6-trap", R.IsStochasticInteger, 300, 20, 0.005),
    ("det-mom1d-fermi2c-40", "mom1d-fermi2c-40", R.IsDeterministic, 1.0, 3, 0.01),
    ("dss-mom1d-fermi2c-40", "mom1d-fermi2c-40", R.IsDynamicSemistochastic, 300.0, 12, 0.005),
]


@pytest.mark.parametrize("case,model,style,pop,steps,dt", WIDE_COMPOSITE_CASES,
                         ids=[c[0] for c in WIDE_COMPOSITE_CASES])
def test_wide_composite_trajectory_matches_oracle(case, model, style, pop, steps, dt):
    h = _wide_composites()[model]
    target = None if style is R.IsDeterministic else pop
    run_trajectory(h, style(), {h.address: pop}, steps, dt, target=target)
