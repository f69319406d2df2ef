"""The momentum-space configuration: HubbardMom1D with all bosons in k = 0 (mode M/2 for even
M, HubbardMom1D.jl:55-61), dense spawning (up to s(s-1)(M-2)+d(M-1) offdiagonals per address).
IsDeterministic steps against the oracle bit for bit -- the first steps of the M=20, N=10
configuration itself, and 50 steps of an M=10, N=5 instance -- and an IsStochasticInteger run
whose shift brackets the exact ground energy of its momentum block."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import assert_same_step, gpu_step, oracle_model, oracle_params

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def k0_address(M, N):
    return R.BoseFS(M, {M // 2: N})


def deterministic_steps(h, steps, dt, shift):
    m = oracle_model(h)
    style = R.IsDeterministic()
    keys = np.array([h.address.key], dtype=np.uint64)
    vals = np.array([1.0])
    wm = R.GPUWorkingMemory(SEED)
    for step in range(1, steps + 1):
        g = gpu_step(h, style, keys, vals, dt, shift, SEED, step, wm=wm)
        o = O.step(m, oracle_params(style, dt, shift, SEED, step), keys, vals)
        assert_same_step(g, o, style)
        keys, vals = o[0], o[1]
    return len(keys)


def test_c3_hamiltonian_first_deterministic_steps_match_oracle():
    """HubbardMom1D M=20, N=10, u=6, dt=5e-4: five power-iteration steps (the support grows
    from 1 to about 8e4 addresses)."""
    h = R.HubbardMom1D(k0_address(20, 10), u=6.0, t=1.0)
    n = deterministic_steps(h, 5, 5e-4, h.diagonal_element(h.address))
    assert n > 50_000


def test_small_mom1d_fifty_deterministic_steps_match_oracle():
    h = R.HubbardMom1D(k0_address(10, 5), u=6.0, t=1.0)
    deterministic_steps(h, 50, 5e-4, h.diagonal_element(h.address))


def test_mom1d_integer_walkers_shift_brackets_exact_energy():
    """HubbardMom1D M=10, N=5 (all bosons in k = 0), u=6, IsStochasticInteger, 2 000 target
    walkers, dt = 5e-4, 20 000 steps.  The GPU run's shift series equals the oracle's CPU run
    of the same trajectory exactly, and shift and projected energy lie within 2 blocking
    errors of the exact energy of the k = 0 sector."""
    from helpers import oracle_solve
    M, N, u = 10, 5, 6.0
    addr = k0_address(M, N)
    h = R.HubbardMom1D(addr, u=u, t=1.0)
    E0 = O.ground_energy(O.mom1d(N, M, u, 1.0), start=addr.key)
    p = R.ProjectorMonteCarloProblem(h, style=R.IsStochasticInteger(), target_walkers=2000,
                                     time_step=5e-4, last_step=20000, random_seed=2024,
                                     population=100,
                                     shift_strategy=R.DoubleLogUpdate(2000, 0.05, 0.05 ** 2 / 4),
                                     post_step_strategy=R.ProjectedEnergy(h, (addr, 1.0)))
    sim = R.solve(p)
    assert sim.success, sim.message
    cpu = oracle_solve(O.mom1d(N, M, u, 1.0), R.IsStochasticInteger(), addr.key, 100, 20000,
                       5e-4, 2000, 2024, zeta=0.05)
    assert np.array_equal(np.asarray(sim.df["shift"], dtype=float), np.asarray(cpu["shift"]))
    r = R.shift_estimator(sim.df, skip=5000)
    assert abs(r.mean - E0) < 2 * r.err, (r.mean, r.err, E0)
    pe, pe_err = R.projected_energy(sim.df, skip=5000)
    assert abs(pe - E0) < 2 * pe_err, (pe, pe_err, E0)
