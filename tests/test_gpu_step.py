"""apply_operator on the GPU against the oracle, step by step and bit for bit: same
addresses, same amplitudes (identical bits, including Float64), same statistics, for the
three styles on the three models, plus the edge cases the step has (empty vectors, heavy
columns, capacity growth, boost, thresholds)."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import assert_same_step, gpu_step, oracle_model, oracle_params, run_trajectory

pytestmark = pytest.mark.gpu

SEED = 0x5EED


B66 = R.BoseFS(1, 1, 1, 1, 1, 1)
CASES = [
    ("int-real1d", R.HubbardReal1D(B66, u=6.0), R.IsStochasticInteger(), {B66: 200}, 40, 0.01, 200),
    ("int-realspace", R.HubbardRealSpace(R.BoseFS([1, 0] * 8), R.PeriodicBoundaries(4, 4), u=[[2.0]]),
     R.IsStochasticInteger(), {R.BoseFS([1, 0] * 8): 300}, 25, 0.01, 300),
    ("int-mom1d", R.HubbardMom1D(R.BoseFS(8, {4: 6}), u=4.0), R.IsStochasticInteger(),
     {R.BoseFS(8, {4: 6}): 300}, 25, 0.005, 300),
    ("int-heavy", R.HubbardReal1D(B66, u=6.0), R.IsStochasticInteger(), {B66: 7000}, 3, 0.01, None),
    ("det-real1d", R.HubbardReal1D(B66, u=6.0), R.IsDeterministic(), {B66: 1.0}, 20, 0.05, None),
    ("det-fermi", R.HubbardRealSpace(R.FermiFS([1, 1, 1] + [0] * 13), R.PeriodicBoundaries(4, 4), u=[[0.0]]),
     R.IsDeterministic(), {R.FermiFS([1, 1, 1] + [0] * 13): 1.0}, 8, 0.05, None),
    ("det-hardwall", R.HubbardRealSpace(R.BoseFS([2, 0, 1, 0, 0, 1]), R.HardwallBoundaries(2, 3), u=[[1.0]]),
     R.IsDeterministic(), {R.BoseFS([2, 0, 1, 0, 0, 1]): 1.0}, 12, 0.05, None),
    ("det-mom1d", R.HubbardMom1D(R.BoseFS(7, {4: 5}), u=2.0), R.IsDeterministic(),
     {R.BoseFS(7, {4: 5}): 1.0}, 6, 0.02, None),
    ("det-compress", R.HubbardReal1D(B66, u=6.0), R.IsDeterministic(R.ThresholdCompression(0.01)),
     {B66: 10.0}, 15, 0.05, None),
    ("dss-real1d", R.HubbardReal1D(R.near_uniform(R.BoseFS, 8, 8), u=4.0), R.IsDynamicSemistochastic(),
     {R.near_uniform(R.BoseFS, 8, 8): 500.0}, 40, 0.01, 500),
    ("dss-realspace", R.HubbardRealSpace(R.BoseFS([1] * 9), R.PeriodicBoundaries(3, 3), u=[[5.0]]),
     R.IsDynamicSemistochastic(), {R.BoseFS([1] * 9): 800.0}, 30, 0.01, 800),
    ("dss-mom1d", R.HubbardMom1D(R.BoseFS(9, {5: 6}), u=3.0), R.IsDynamicSemistochastic(),
     {R.BoseFS(9, {5: 6}): 400.0}, 20, 0.005, 400),
    ("dss-fermi", R.HubbardRealSpace(R.FermiFS([1, 1, 1, 1] + [0] * 12), R.PeriodicBoundaries(4, 4), u=[[0.0]]),
     R.IsDynamicSemistochastic(), {R.FermiFS([1, 1, 1, 1] + [0] * 12): 300.0}, 20, 0.01, 300),
    ("dss-onthefly", R.HubbardReal1D(B66, u=6.0), R.IsDynamicSemistochastic(late_compression=False),
     {B66: 300.0}, 30, 0.01, 300),
    ("dss-thresholds", R.HubbardReal1D(B66, u=6.0),
     R.IsDynamicSemistochastic(threshold=0.5, rel_spawning_threshold=2.0, abs_spawning_threshold=30.0),
     {B66: 300.0}, 30, 0.01, 300),
]


@pytest.mark.parametrize("name,h,style,start,steps,dt,target", CASES, ids=[c[0] for c in CASES])
def test_step_trajectory_matches_oracle(name, h, style, start, steps, dt, target):
    run_trajectory(h, style, start, steps, dt, target=target)


def test_boost_matches_oracle():
    h = R.HubbardReal1D(B66, u=6.0)
    run_trajectory(h, R.IsStochasticInteger(), {B66: 100}, 10, 0.01, boost=2.5)
    run_trajectory(h, R.IsDynamicSemistochastic(), {B66: 100.0}, 10, 0.01, boost=1.7)


def test_empty_source_gives_empty_target():
    h = R.HubbardReal1D(B66, u=6.0)
    for style in (R.IsStochasticInteger(), R.IsDeterministic(), R.IsDynamicSemistochastic()):
        k, v, st = gpu_step(h, style, [], [], 0.01, 0.0, SEED, 1)
        assert len(k) == 0 and st["len"] == 0 and st["norm"] == 0.0


def test_large_vector_rebuckets_and_matches_oracle():
    """30 000 distinct walkers: several buckets, capacity planning and re-bucketing."""
    h = R.HubbardReal1D(R.near_uniform(R.BoseFS, 12, 12), u=2.0)
    m = oracle_model(h)
    keys = O.basis(m)[:30000]
    rng = np.random.default_rng(4)
    for style, vals in ((R.IsStochasticInteger(), rng.integers(-5, 6, len(keys))),
                        (R.IsDynamicSemistochastic(), rng.normal(size=len(keys)) * 3),
                        (R.IsDeterministic(), rng.normal(size=len(keys)))):
        nz = vals != 0
        k, v = keys[nz], vals[nz]
        g = gpu_step(h, style, k, v, 0.01, -1.0, SEED, 3)
        o = O.step(m, oracle_params(style, 0.01, -1.0, SEED, 3), k, v)
        assert_same_step(g, o, style)
        assert g[2]["nb_bits"] > 0


def test_same_seed_same_result_and_seed_matters():
    h = R.HubbardReal1D(B66, u=6.0)
    style = R.IsDynamicSemistochastic()
    # 5 walkers on 12 offdiagonals: the column is sampled, so the seed matters; dt = 0.1
    # makes each spawn larger than the compression threshold
    a = gpu_step(h, style, [B66.key], [5.0], 0.1, 0.0, 7, 1)
    b = gpu_step(h, style, [B66.key], [5.0], 0.1, 0.0, 7, 1)
    c = gpu_step(h, style, [B66.key], [5.0], 0.1, 0.0, 8, 1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not (np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1]))


def test_mul_plain_hamiltonian_matches_sparse_matrix():
    """mul!(y, H, x) (abstractdvec.jl:275-284) with the OP_HAMILTONIAN operator."""
    h = R.HubbardRealSpace(R.BoseFS([1, 1, 0, 1, 0, 1]), R.PeriodicBoundaries(2, 3), u=[[1.5]], t=[0.8])
    m = oracle_model(h)
    keys = O.basis(m)
    x = np.random.default_rng(9).normal(size=len(keys))
    xv = R.GPUDVec(style=R.IsDeterministic(), address_type=h.address)
    xv.upload(keys, x)
    y = R.mul(xv.similar(), h, xv)
    k, v = y.sorted_arrays()
    want = O.sparse_matrix(m, keys) @ x
    got = np.zeros(len(keys))
    got[np.searchsorted(keys, k)] = v
    assert np.allclose(got, want, rtol=1e-13, atol=1e-13)


SHAPES = [(1024, 0), (16, 0), (4096, 512), (256, 1024), (64, 4096)]


@pytest.mark.parametrize("kpb,slots", SHAPES, ids=[f"k{k}-t{t}" for k, t in SHAPES])
def test_launch_shapes_give_identical_results(kpb, slots):
    """Bucket count and table size change only the launch shape: (4096, 512) puts a few
    thousand contributions into a 512-slot table, so buckets run in many passes and passes
    that still overflow are split."""
    h = R.HubbardReal1D(R.near_uniform(R.BoseFS, 12, 12), u=2.0)
    m = oracle_model(h)
    keys = O.basis(m)[:20000]
    rng = np.random.default_rng(11)
    for style, vals in ((R.IsStochasticInteger(), rng.integers(-5, 6, len(keys))),
                        (R.IsDynamicSemistochastic(), rng.normal(size=len(keys)) * 3),
                        (R.IsDeterministic(), rng.normal(size=len(keys)))):
        nz = vals != 0
        k, v = keys[nz], vals[nz]
        wm = R.GPUWorkingMemory(SEED)
        wm.set_launch_shape(kpb, slots)
        g = gpu_step(h, style, k, v, 0.01, -1.0, SEED, 5, wm=wm)
        o = O.step(m, oracle_params(style, 0.01, -1.0, SEED, 5), k, v)
        assert_same_step(g, o, style)


@pytest.mark.parametrize("slots", [0, 512])
def test_inexact_contributions_follow_canonical_order(slots):
    """Amplitudes from 1e-15 to 1e3 on the whole 462-state basis: most addresses receive a
    contribution that is not a multiple of 2^-64 and more than eight spawns, so their sums
    take the canonical-order path (diagonal first, spawns by increasing value)."""
    h = R.HubbardReal1D(B66, u=6.0)
    m = oracle_model(h)
    keys = O.basis(m)
    rng = np.random.default_rng(12)
    vals = rng.choice([-1.0, 1.0], len(keys)) * 10.0 ** rng.uniform(-15, 3, len(keys))
    style = R.IsDeterministic()
    wm = R.GPUWorkingMemory(SEED)
    wm.set_launch_shape(1024, slots)
    g = gpu_step(h, style, keys, vals, 0.05, 1.0, SEED, 2, wm=wm)
    o = O.step(m, oracle_params(style, 0.05, 1.0, SEED, 2), keys, vals)
    assert_same_step(g, o, style)


def test_launch_shape_rejects_bad_values():
    wm = R.GPUWorkingMemory(SEED)
    for kpb, slots in ((8, 0), (8192, 0), (64, 96), (64, 256), (64, 8192)):
        with pytest.raises(R.RimuError):
            wm.set_launch_shape(kpb, slots)
