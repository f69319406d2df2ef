"""End-to-end FCIQMC through ProjectorMonteCarloProblem / solve on the GPU: statistical
agreement with exact energies (blocking analysis), reproducibility, ProjectedEnergy."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R

pytestmark = pytest.mark.gpu


def test_c1_integer_walkers_shift_brackets_exact_energy():
    """HubbardReal1D M=N=6, u=6, IsStochasticInteger, 1 000 target walkers, dt = 1e-3, 20 000
    steps.  The GPU run's shift series equals the oracle's CPU run of the same trajectory
    exactly, and shift and projected energy lie within 2 blocking errors of E0 = -4.0215
    (test/KrylovKit.jl:15) and of the CPU run's estimates."""
    from helpers import oracle_solve
    addr = R.BoseFS([1] * 6)
    H = R.HubbardReal1D(addr, u=6.0, t=1.0)
    p = R.ProjectorMonteCarloProblem(H, style=R.IsStochasticInteger(), target_walkers=1000,
                                     time_step=1e-3, last_step=20000, random_seed=1234,
                                     post_step_strategy=R.ProjectedEnergy(H, (addr, 1.0)))
    sim = R.solve(p)
    assert sim.success
    df = sim.df
    cpu = oracle_solve(O.real1d(6, 6, 6.0, 1.0), R.IsStochasticInteger(), addr.key, 10, 20000,
                       1e-3, 1000, 1234)
    assert np.array_equal(np.asarray(df["shift"], dtype=float), np.asarray(cpu["shift"]))
    E0 = O.ground_energy(O.real1d(6, 6, 6.0))
    r = R.shift_estimator(df, skip=3000)
    assert abs(r.mean - E0) < 2 * r.err, (r.mean, r.err)
    pe, pe_err = R.projected_energy(df, skip=3000)
    assert abs(pe - E0) < 2 * pe_err, (pe, pe_err)
    pc, _ = R.projected_energy(cpu, skip=3000)
    assert abs(pe - pc) < 2 * pe_err, (pe, pc, pe_err)


def test_dss_shift_brackets_exact_energy():
    """HubbardReal1D(BoseFS{5,5}; u=1), E0 = -8.280991746582686 (test/lomc.jl:543-605):
    the IsDynamicSemistochastic shift within 2 blocking errors, no absolute floor."""
    addr = R.BoseFS([1] * 5)
    H = R.HubbardReal1D(addr, u=1.0)
    p = R.ProjectorMonteCarloProblem(H, style=R.IsDynamicSemistochastic(), target_walkers=1000,
                                     time_step=1e-2, last_step=20000, random_seed=99,
                                     shift_strategy=R.DoubleLogUpdate(1000, 0.05, 0.05 ** 2 / 4))
    sim = R.solve(p)
    r = R.shift_estimator(sim.df, skip=2000)
    assert abs(r.mean - (-8.280991746582686)) < 2 * r.err, (r.mean, r.err)


def test_same_seed_identical_reports():
    """Same random_seed => identical DataFrames (test/projector_monte_carlo_problem.jl:126-167)."""
    H = R.HubbardReal1D(R.BoseFS([1] * 6), u=6.0)
    def run():
        p = R.ProjectorMonteCarloProblem(H, target_walkers=300, time_step=1e-2, last_step=300,
                                         random_seed=42)
        return R.solve(p).df
    a, b = run(), run()
    assert set(a) == set(b)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_deterministic_power_iteration_converges_to_ground_state():
    addr = R.BoseFS([1] * 6)
    H = R.HubbardReal1D(addr, u=6.0)
    # dt below 2 / (E_max - E0) so that 1 + dt (S - H) is a contraction on the excited states
    p = R.ProjectorMonteCarloProblem(H, style=R.IsDeterministic(), start_at={addr: 1.0},
                                     target_walkers=10, time_step=0.01, last_step=6000,
                                     max_length=10_000)
    sim = R.solve(p)
    assert sim.df["shift"][-1] == pytest.approx(O.ground_energy(O.real1d(6, 6, 6.0)), abs=1e-7)


def test_abort_when_max_length_is_exceeded():
    """len > max_length aborts the run (fciqmc.jl:176-179)."""
    addr = R.BoseFS([1] * 6)
    H = R.HubbardReal1D(addr, u=6.0)
    p = R.ProjectorMonteCarloProblem(H, style=R.IsDeterministic(), start_at={addr: 1.0},
                                     target_walkers=10, time_step=0.01, last_step=100)
    sim = R.solve(p)
    assert sim.aborted and "max_length" in sim.message


def test_abort_on_dead_population():
    H = R.HubbardReal1D(R.BoseFS([1] * 4), u=1.0)
    # diagonal factor 1 - dt (H - S) = 0.4: the single walker dies within a few steps
    p = R.ProjectorMonteCarloProblem(H, style=R.IsStochasticInteger(), shift=-60.0,
                                     shift_strategy=R.DontUpdate(10 ** 9), time_step=0.01,
                                     last_step=100, population=1, random_seed=3)
    sim = R.solve(p)
    assert sim.aborted and "dead" in sim.message
