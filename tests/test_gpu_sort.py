"""The sorted warp annihilation (rimu_wm_set_annihilation(RIMU_ANN_SORT)): the bucket's spawns
ordered by a bitonic network on (address, value) instead of a hash table.  It must give the
oracle's step bit for bit, exactly as the hashed kernel does: every trajectory case of the
plain step tests, the launch shapes that move buckets between the warp and CTA kernels,
addresses whose sums take the canonical-order path, and batched replicas (explicit mode and
the autotuner, which times both)."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import assert_same_step, gpu_step, oracle_model, oracle_params, run_trajectory
from test_gpu_step import CASES

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def sorted_wm(seed=SEED):
    wm = R.GPUWorkingMemory(seed)
    wm.set_annihilation("sort")
    return wm


@pytest.mark.parametrize("name,h,style,start,steps,dt,target", CASES, ids=[c[0] for c in CASES])
def test_sorted_trajectory_matches_oracle(name, h, style, start, steps, dt, target):
    run_trajectory(h, style, start, steps, dt, target=target, wm=sorted_wm())


@pytest.mark.parametrize("kpb", [448, 256, 64, 16])
def test_sorted_launch_shapes(kpb):
    """From 16 contributions per bucket (spawn runs of one or two, sorts of width 2..32) to
    448 (the default; the fullest buckets go on to the CTA kernel)."""
    h = R.HubbardReal1D(R.near_uniform(R.BoseFS, 12, 12), u=2.0)
    m = oracle_model(h)
    keys = O.basis(m)[:20000]
    rng = np.random.default_rng(11)
    for style, vals in ((R.IsStochasticInteger(), rng.integers(-5, 6, len(keys))),
                        (R.IsDynamicSemistochastic(), rng.normal(size=len(keys)) * 3),
                        (R.IsDeterministic(), rng.normal(size=len(keys)))):
        nz = vals != 0
        k, v = keys[nz], vals[nz]
        wm = sorted_wm()
        wm.set_launch_shape(kpb, 0)
        g = gpu_step(h, style, k, v, 0.01, -1.0, SEED, 5, wm=wm)
        o = O.step(m, oracle_params(style, 0.01, -1.0, SEED, 5), k, v)
        assert_same_step(g, o, style)


def test_sorted_inexact_sums_in_canonical_order():
    """Amplitudes from 1e-15 to 1e3: most addresses get a contribution that is not a multiple
    of 2^-64 and several spawns, so their sums run in the sorted order of the run."""
    h = R.HubbardReal1D(R.BoseFS(1, 1, 1, 1, 1, 1), u=6.0)
    m = oracle_model(h)
    keys = O.basis(m)
    rng = np.random.default_rng(12)
    vals = rng.choice([-1.0, 1.0], len(keys)) * 10.0 ** rng.uniform(-15, 3, len(keys))
    style = R.IsDeterministic()
    for kpb in (448, 64):
        wm = sorted_wm()
        wm.set_launch_shape(kpb, 0)
        g = gpu_step(h, style, keys, vals, 0.05, 1.0, SEED, 2, wm=wm)
        o = O.step(m, oracle_params(style, 0.05, 1.0, SEED, 2), keys, vals)
        assert_same_step(g, o, style)


def test_sorted_and_hashed_give_the_same_step_with_a_projector():
    """ProjectedEnergy terms are summed in the same kernel: equal bits both ways."""
    h = R.HubbardReal1D(R.near_uniform(R.BoseFS, 10, 10), u=4.0)
    m = oracle_model(h)
    keys = O.basis(m)[:30000]
    vals = np.random.default_rng(4).normal(size=len(keys))
    style = R.IsDynamicSemistochastic()
    pk = keys[::97]
    out = []
    for mode in ("hash", "sort"):
        wm = R.GPUWorkingMemory(SEED)
        wm.set_annihilation(mode)
        wm.set_projector(pk, np.ones(len(pk)), np.linspace(-1, 1, len(pk)))
        g = gpu_step(h, style, keys, vals, 0.01, -2.0, SEED, 3, wm=wm)
        out.append((g, dict(wm.last_stats)))
    (g0, s0), (g1, s1) = out
    assert np.array_equal(g0[0], g1[0])
    assert np.array_equal(g0[1].view(np.uint64), g1[1].view(np.uint64))
    for k in ("norm", "vproj", "hproj", "spawns", "len"):
        assert s0[k] == s1[k] or (np.isnan(s0[k]) and np.isnan(s1[k]))


def test_bad_annihilation_mode_is_rejected():
    wm = R.GPUWorkingMemory(SEED)
    with pytest.raises(KeyError):
        wm.set_annihilation("radix")
    import rimugpu._lib as L
    assert L.load().rimu_wm_set_annihilation(wm.handle, 7) == L.RIMU_ERR_BADARG


@pytest.mark.parametrize("mode", ["sort", "hash"])
def test_batched_sorted_step_equals_plain_step(mode):
    from test_gpu_batch import plain_steps, random_start
    rng = np.random.default_rng(3)
    geo = R.PeriodicBoundaries(3, 3)
    hs = [R.HubbardRealSpace(R.BoseFS([1] * 9), geo, u=[[u]]) for u in (1.0, 3.0, 6.0)]
    style = R.IsDynamicSemistochastic()
    starts = [random_start(h, 400, rng, False) for h in hs]
    shifts = [-5.0 - r for r in range(len(hs))]
    want = [plain_steps(h, style, starts[r], shifts[r], 0.01, r, 3) for r, h in enumerate(hs)]
    b = R.BatchedReplicas(hs, style, 0.01, targets=1e6, starts=starts, shifts=shifts, seed=SEED,
                          shift_update=False, use_graph=False, autotune=False, annihilation=mode)
    assert b.info()["annihilation"] == mode
    for s in range(3):
        b.run(1)
        for r in range(len(hs)):
            (wk, wv), _ = want[r][s]
            gk, gv = b.sorted_arrays(r)
            assert np.array_equal(gk, wk)
            assert np.array_equal(gv.view(np.uint64), wv.view(np.uint64))


def test_autotuner_times_the_sorted_shape():
    """Four replicas grown to 2^20 entries together: the autotuner times its five shapes, the
    sorted one among them, and the run stays bit-identical to a run with the autotuner off."""
    geo = R.PeriodicBoundaries(4, 4)
    hs = [R.HubbardRealSpace(R.BoseFS([1] * 16), geo, u=[[u]]) for u in (2.0, 3.0, 4.0, 5.0)]
    style = R.IsDynamicSemistochastic()
    start = {R.BoseFS([1] * 16): 10.0}
    runs = []
    for tune in (True, False):
        b = R.BatchedReplicas(hs, style, 1e-3, targets=1e6, starts=[start] * 4, seed=SEED,
                              use_graph=False, autotune=tune)
        runs.append((b, b.run(1500)))
    (bt, rt), (bf, rf) = runs
    assert np.array_equal(rt["norm"], rf["norm"])
    assert np.array_equal(rt["shift"], rf["shift"])
    assert rt["len"][-1].sum() >= 1 << 20
    assert bt.info()["annihilation"] in ("hash", "sort")
    assert bf.info()["annihilation"] == "hash"
