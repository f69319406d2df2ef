"""Addresses of 65-128 bits (the reference's two-chunk BitString, bitstring.jl:6-18) on the
GPU against the oracle, bit for bit: HubbardReal1D with BoseFS{50,50} (99 bits) and
BoseFS{40,30} (69 bits), HubbardRealSpace with bosons on an 8x8 lattice (103 bits) and with
fermions on a 10x10 lattice (100 bits); matrix elements and step trajectories of the three
styles, whose random numbers are keyed on lo ^ mix64(hi) of the address."""
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


def test_wide_addresses_reject_what_they_cannot_do():
    h = _models()["real1d-99"]
    v = R.GPUDVec({h.address: 1.0}, style=R.IsDeterministic())
    with pytest.raises(R.RimuError):
        v.dot(v)
    with pytest.raises(R.RimuError):     # initiator rules use bit 63 of the address
        R.apply_operator(R.GPUWorkingMemory(1),
                         R.GPUDVec(style=R.IsDynamicSemistochastic(), address_type=h.address,
                                   initiator=R.Initiator(1.0)),
                         R.GPUDVec({h.address: 5.0}, style=R.IsDynamicSemistochastic(),
                                   initiator=R.Initiator(1.0)),
                         R.FirstOrderTransitionOperator(h, 0.0, 0.01))
