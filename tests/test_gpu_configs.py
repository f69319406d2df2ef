"""Parity at the sizes of the benchmarked configurations, bit for bit against the oracle.

* HubbardReal1D M=N=20, u=4, IsDynamicSemistochastic(threshold 1), dt=1e-3, seed 0x5EED (the
  large plain FCIQMC configuration): a 250-step trajectory from the unit-filling address at
  target 1e5, and one step of a 1e6-walker list grown on the GPU, under three launch shapes
  (the default; 16 contributions per bucket, i.e. 2^16 buckets as at the 1e8 benchmark;
  a 512-slot table, i.e. buckets annihilated in several passes) and with the warps' spawns
  sorted instead of hashed.
* HubbardReal1D M=N=14 on the full basis (D = 20 058 300, the matrix-free H*v
  configuration): forward and adjoint over every row, and the Hellmann-Feynman gradients
  for u in {1, 2, 4, 8} against central finite differences and the interaction expectation.
* HubbardRealSpace 4x4 periodic, N=16 (the batched configuration): five steps from lists of
  2e4 walkers grown on the GPU, and the batched step of 64 replicas (u_i = 1 + 15 i/63,
  uneven targets) checked replica by replica.
* HubbardMom1D M=20, N=10, all bosons in k=0, dt=5e-4 (the momentum-space configuration):
  IsDeterministic power iteration at full size (the support grows to 1e6 addresses and 7.7e8
  contributions per step).

The oracle follows the large lists with its multi-threaded step (the PDVec restatement),
which gives the single-threaded step's results bit for bit (tests/test_oracle_threaded.py).
"""
import math

import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import (assert_same_step, gpu_step, oracle_mem_budget, oracle_model, oracle_params,
                     popcount64, run_trajectory)

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def cuda(x):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def grow_on_gpu(h, style, dt, target, min_steps, seed=SEED + 1):
    """A walker list of about `target` walkers: `solve`'s loop on the GPU from the default
    start, run until the norm reaches 0.9 target and at least `min_steps` steps."""
    p = R.ProjectorMonteCarloProblem(h, style=style, time_step=dt, target_walkers=target,
                                     last_step=10 ** 9, random_seed=seed,
                                     max_length=int(4 * target + 100))
    sim = R.init(p)
    s = sim.states[0]
    n = 0
    while n < 20 * min_steps:
        sim.step_()
        n += 1
        if n >= min_steps and s.wm.last_stats["norm"] >= 0.9 * target:
            break
    k, v = s.v.download()
    o = np.argsort(k)
    return k[o], v[o], s.shift_parameters.shift


# ---- HubbardReal1D M = N = 20 ------------------------------------------------------------
C2_ADDR = R.near_uniform(R.BoseFS, 20, 20)
C2_H = R.HubbardReal1D(C2_ADDR, u=4.0, t=1.0)
C2_STYLE = R.IsDynamicSemistochastic(threshold=1.0)


def test_c2_trajectory_250_steps_bit_exact():
    """250 steps from 1e5 walkers on the unit-filling address, DoubleLogUpdate towards 1e5:
    the list grows to 9e4 addresses; every step's addresses, amplitude bits and statistics
    equal the oracle's."""
    keys, vals = run_trajectory(C2_H, C2_STYLE, {C2_ADDR: 1e5}, 250, 1e-3, target=1e5,
                                threaded=True)
    assert len(keys) > 80000


@pytest.mark.parametrize("kpb,slots,mode", [(1024, 0, "hash"), (16, 0, "hash"), (4096, 512, "hash"),
                                            (448, 0, "sort"), (16, 0, "sort")],
                         ids=["default", "2^16-buckets", "multipass", "sorted", "sorted-2^16-buckets"])
def test_c2_step_of_a_1e6_walker_list(kpb, slots, mode):
    keys, vals, shift = C2_LIST()
    m = oracle_model(C2_H)
    wm = R.GPUWorkingMemory(SEED)
    wm.set_launch_shape(kpb, slots)
    wm.set_annihilation(mode)
    g = gpu_step(C2_H, C2_STYLE, keys, vals, 1e-3, shift, SEED, 7001, wm=wm)
    o = O.step_mt(m, oracle_params(C2_STYLE, 1e-3, shift, SEED, 7001), keys, vals,
                  mem_budget=oracle_mem_budget())
    assert_same_step(g, o, C2_STYLE)
    if kpb == 16:
        assert g[2]["nb_bits"] >= 16
    assert g[2]["len"] > 5e5


_c2_cache = {}


def C2_LIST():
    if "list" not in _c2_cache:
        _c2_cache["list"] = grow_on_gpu(C2_H, C2_STYLE, 1e-3, 1e6, 400)
    return _c2_cache["list"]


# ---- HubbardReal1D M = N = 14 on the full basis ------------------------------------------
def bose_interaction(keys):
    """sum_i n_i (n_i - 1) of BoseFS keys: each run of n ones gives n(n-1) = 2 C(n,2), and
    C(n,2) counts the pairs of adjacent ones at every distance within the run."""
    acc = np.zeros(len(keys), dtype=np.int64)
    y = keys & (keys >> np.uint64(1))
    while np.any(y):
        acc += popcount64(y)
        y &= y >> np.uint64(1)
    return 2 * acc


def test_c4_full_basis_forward_and_adjoint_bit_exact():
    import torch
    h = R.HubbardReal1D(R.BoseFS([1] * 14), u=4.0, t=1.0)
    m = oracle_model(h)
    op = R.BasisOperator(h)
    keys = O.basis(m)
    assert op.dim == len(keys) == 20058300
    assert np.array_equal(op.basis_keys(), keys)
    rng = np.random.default_rng(14)
    v = rng.normal(size=op.dim)
    v /= np.linalg.norm(v)
    gw = rng.normal(size=op.dim)
    w = op(cuda(v)).cpu().numpy()
    assert np.array_equal(w.view(np.uint64), O.hv_basis(m, keys, v).view(np.uint64))
    gv, gu, gt = op.adjoint(cuda(v), cuda(gw))
    ogv, ogu, ogt = O.hv_basis_adjoint(m, keys, v, gw)
    assert np.array_equal(gv.cpu().numpy().view(np.uint64), ogv.view(np.uint64))
    del w, gv, ogv
    torch.cuda.empty_cache()
    # g_u and g_t are sums over 2e7 rows, reduced in a different order than the oracle's
    # sequential sum: both are held to the error bound of blocked summation, 1e-12 of the
    # sum of magnitudes, around the correctly rounded sum (math.fsum)
    tu = gw * (bose_interaction(keys) / 2 * v)
    kg = O.hv_basis(O.real1d(14, 14, 0.0, 1.0), keys, gw)          # K gw: the hopping part
    tt = v * kg
    for got, want, terms in ((gu, ogu, tu), (gt, ogt, tt)):
        exact = math.fsum(terms)
        bound = 1e-12 * float(np.abs(terms).sum())
        assert abs(got - exact) <= bound, (got, exact, bound)
        assert abs(want - exact) <= bound, (want, exact, bound)


@pytest.mark.parametrize("u", [1.0, 2.0, 4.0, 8.0])
def test_c4_hellmann_feynman_against_finite_differences(u):
    """dE/du and dE/dt of the ground state from the adjoint (<psi|dH|psi>) against central
    differences of Lanczos energies (h = 1e-5, tol 1e-10) to 1e-6 relative, and dE/du
    against the expectation of sum n(n-1)/2 to 1e-10."""
    import torch
    h = R.HubbardReal1D(R.BoseFS([1] * 14), u=u, t=1.0)
    op = R.BasisOperator(h)
    E, vecs, info = R.eigsolve(op, tol=1e-10)
    assert info["converged"]
    psi = vecs[0] / torch.linalg.norm(vecs[0])
    _, gu, gt = op.adjoint(psi, psi)
    step = 1e-5

    def energy(uu, tt):
        return R.eigsolve(R.BasisOperator(h.with_params(u=uu, t=tt)), v0=psi, tol=1e-10)[0][0]
    fd_u = (energy(u + step, 1.0) - energy(u - step, 1.0)) / (2 * step)
    fd_t = (energy(u, 1.0 + step) - energy(u, 1.0 - step)) / (2 * step)
    assert gu == pytest.approx(fd_u, rel=1e-6)
    assert gt == pytest.approx(fd_t, rel=1e-6)
    p = psi.cpu().numpy()
    inter = bose_interaction(op.basis_keys()) / 2
    assert gu == pytest.approx(math.fsum(p * p * inter), rel=1e-10)
    assert E[0] == pytest.approx(u * gu + gt, rel=1e-9)      # E = u dE/du + t dE/dt


# ---- HubbardRealSpace 4x4 periodic, N = 16 -----------------------------------------------
C5_ADDR = R.BoseFS([1] * 16)
C5_GEO = R.PeriodicBoundaries(4, 4)


@pytest.mark.parametrize("u", [1.0, 16.0])
def test_c5_five_steps_from_a_2e4_walker_list(u):
    h = R.HubbardRealSpace(C5_ADDR, C5_GEO, u=[[u]], t=[1.0])
    style = R.IsDynamicSemistochastic()
    keys, vals, shift = grow_on_gpu(h, style, 1e-3, 2e4, 300)
    assert len(keys) > 1e4
    run_trajectory(h, style, (keys, vals), 5, 1e-3, shift=shift, target=2e4, threaded=True)


def test_c5_batched_64_replicas_against_the_oracle():
    """64 replicas, u_i = 1 + 15 i/63, targets log-uniform in [1e4, 1e5], grown together by
    the batched step (CUDA-graph segments); then one more batched step is compared, for
    eight replicas spread over the batch, with the oracle's step of that replica's list,
    shift, step number and random key."""
    nrep = 64
    us = [1.0 + 15.0 * i / 63 for i in range(nrep)]
    hs = [R.HubbardRealSpace(C5_ADDR, C5_GEO, u=[[x]], t=[1.0]) for x in us]
    targets = list(10.0 ** np.random.default_rng(2024).uniform(4.0, 5.0, nrep))
    style = R.IsDynamicSemistochastic()
    b = R.BatchedReplicas(hs, style, 1e-3, targets=targets, starts=[{C5_ADDR: 10.0}] * nrep,
                          shifts=[0.0] * nrep, seed=SEED, segment_steps=64, use_graph=True,
                          autotune=False)
    res = b.run(400)
    check = [0, 9, 18, 27, 36, 45, 54, 63]
    before = {r: b.download(r) for r in check}
    shifts = res["shift"][-1]
    step = b.step + 1
    res1 = b.run(1)
    for r in check:
        k, v = before[r]
        o = np.argsort(k)
        ok, ov, ost = O.step_mt(oracle_model(hs[r]),
                                oracle_params(style, 1e-3, float(shifts[r]), SEED, step, replica=r),
                                k[o], v[o])
        gk, gv = b.sorted_arrays(r)
        assert np.array_equal(gk, ok), r
        assert np.array_equal(gv.view(np.uint64), ov.view(np.uint64)), r
        assert res1["norm"][0, r] == ost["norm"] and res1["len"][0, r] == ost["len"], r
    assert max(len(before[r][0]) for r in check) > 1e4


# ---- HubbardMom1D M = 20, N = 10 ---------------------------------------------------------
def test_c3_deterministic_power_iteration_full_size():
    """IsDeterministic steps of HubbardMom1D(BoseFS(20, 10 => 10); u=6, t=1), dt=5e-4, shift
    the start's diagonal element, every step bit for bit against the oracle: by step 8 the
    support has saturated at 1.0e6 addresses with 7.7e8 contributions per step."""
    h = R.HubbardMom1D(R.BoseFS(20, {10: 10}), u=6.0, t=1.0)
    keys, vals = run_trajectory(h, R.IsDeterministic(), {h.address: 1.0}, C3_STEPS, 5e-4,
                                threaded=True)
    assert len(keys) > 1e6


C3_STEPS = 10
