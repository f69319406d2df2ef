"""Multi-component addresses on the GPU against the oracle, bit for bit: matrix elements of
HubbardRealSpace with a CompositeFS of two, three and four components (bosons and fermions,
hard-wall and periodic, trap, interactions of both signs) and of HubbardMom1D with FermiFS2C
over whole bases, and step trajectories of the three styles."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import assert_same_step, gpu_step, oracle_model, oracle_params, run_trajectory

pytestmark = pytest.mark.gpu

SEED = 0x5EED

MODELS = {
    "realspace-bose-fermi-trap": lambda: R.HubbardRealSpace(
        R.CompositeFS(R.BoseFS((1, 0, 2, 0, 0, 0)), R.FermiFS((0, 1, 0, 1, 0, 0))),
        geometry=R.CubicGrid((2, 3), (False, True)), t=[1.0, 0.5], u=[[1.5, 2.0], [2.0, 0.0]],
        v=[[0.5, 0.25], [1.0, 2.0]]),
    "realspace-bose-bose": lambda: R.HubbardRealSpace(
        R.CompositeFS(R.BoseFS((1, 1, 1, 0, 0, 0)), R.BoseFS((1, 0, 0, 0, 0, 0))),
        t=[1.0, 4.0], u=[[2.0, 3.0], [3.0, 0.0]]),
    "realspace-fermi-fermi-2d": lambda: R.HubbardRealSpace(
        R.CompositeFS(R.FermiFS((1, 1, 0, 0, 0, 0, 0, 0, 0)), R.FermiFS((0, 0, 0, 1, 1, 0, 0, 0, 0))),
        geometry=R.PeriodicBoundaries(3, 3), t=[1.0, 2.0], u=[[0.0, 4.0], [4.0, 0.0]]),
    # three and four components (one 64-bit key, the last component lowest)
    "realspace-3c-trap": lambda: R.HubbardRealSpace(
        R.CompositeFS(R.BoseFS((1, 0, 1, 0, 0, 0)), R.FermiFS((0, 1, 0, 1, 0, 0)),
                      R.BoseFS((0, 0, 0, 0, 2, 0))),
        geometry=R.CubicGrid((2, 3), (False, True)), t=[1.0, 0.5, 2.0],
        u=[[1.5, 2.0, 0.5], [2.0, 0.0, -1.0], [0.5, -1.0, 3.0]],
        v=[[0.5, 0.25], [1.0, 2.0], [0.0, 0.5]]),
    "realspace-4c": lambda: R.HubbardRealSpace(
        R.CompositeFS(R.BoseFS((2, 0, 0)), R.FermiFS((1, 0, 1)), R.BoseFS((0, 2, 0)),
                      R.BoseFS((1, 0, 0))),
        t=[1.0, 2.0, 0.5, 1.0],
        u=[[1.0, 2.0, 0.0, -1.0], [2.0, 0.0, 1.5, 0.5], [0.0, 1.5, 2.0, 1.0], [-1.0, 0.5, 1.0, 0.25]]),
    "realspace-3f-2d": lambda: R.HubbardRealSpace(
        R.CompositeFS(R.FermiFS((1, 1, 0, 0, 0, 0, 0, 0, 0)), R.FermiFS((0, 0, 0, 1, 1, 0, 0, 0, 0)),
                      R.FermiFS((0, 0, 0, 0, 0, 0, 0, 0, 1))),
        geometry=R.PeriodicBoundaries(3, 3), t=[1.0, 2.0, 1.5],
        u=[[0.0, 4.0, 1.0], [4.0, 0.0, -2.0], [1.0, -2.0, 0.0]]),
    "mom1d-fermi2c": lambda: R.HubbardMom1D(R.FermiFS2C((0, 1, 1, 1, 0, 0), (0, 0, 1, 1, 0, 0)), u=3.0),
    "mom1d-fermi2c-odd": lambda: R.HubbardMom1D(R.FermiFS2C((0, 0, 1, 1, 0, 0, 0), (0, 1, 1, 1, 0, 0, 0)),
                                                u=-2.0, t=0.5),
}


@pytest.mark.parametrize("name", list(MODELS))
def test_matrix_elements_match_oracle_on_the_whole_basis(name):
    h = MODELS[name]()
    m = oracle_model(h)
    keys = O.basis(m)
    assert h.dimension() == len(keys)
    got = h.diagonal_elements(keys)
    want = np.array([O.diagonal(m, int(k)) for k in keys])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    for k in keys[:: max(1, len(keys) // 150)]:
        gk, gv = h.offdiagonal_keys(int(k))
        ref = O.offdiagonals(m, int(k))
        assert len(gk) == len(ref) == h.num_offdiagonals(h.address.with_key(int(k)))
        assert [int(x) for x in gk] == [r[0] for r in ref]
        assert np.array_equal(np.asarray(gv).view(np.uint64),
                              np.array([r[1] for r in ref]).view(np.uint64))


CASES = [
    ("int-realspace2", "realspace-bose-fermi-trap", R.IsStochasticInteger, 300, 25, 0.01),
    ("dss-realspace2", "realspace-bose-bose", R.IsDynamicSemistochastic, 400.0, 30, 0.01),
    ("det-realspace2", "realspace-fermi-fermi-2d", R.IsDeterministic, 1.0, 8, 0.02),
    ("int-mom2c", "mom1d-fermi2c", R.IsStochasticInteger, 300, 25, 0.01),
    ("dss-mom2c", "mom1d-fermi2c-odd", R.IsDynamicSemistochastic, 300.0, 30, 0.01),
    ("det-mom2c", "mom1d-fermi2c", R.IsDeterministic, 1.0, 6, 0.02),
    ("int-realspace3", "realspace-3c-trap", R.IsStochasticInteger, 300, 25, 0.01),
    ("dss-realspace4", "realspace-4c", R.IsDynamicSemistochastic, 400.0, 30, 0.01),
    ("det-realspace3f", "realspace-3f-2d", R.IsDeterministic, 1.0, 6, 0.02),
]


@pytest.mark.parametrize("case,model,style,pop,steps,dt", CASES, ids=[c[0] for c in CASES])
def test_step_trajectory_matches_oracle(case, model, style, pop, steps, dt):
    h = MODELS[model]()
    target = None if style is R.IsDeterministic else pop
    run_trajectory(h, style(), {h.address: pop}, steps, dt, target=target)


def test_random_vectors_step_like_the_oracle():
    """Spread-out start vectors over the composite basis, several buckets, every style."""
    h = MODELS["realspace-bose-fermi-trap"]()
    m = oracle_model(h)
    keys = O.basis(m)
    rng = np.random.default_rng(21)
    for style, vals in ((R.IsStochasticInteger(), rng.integers(-4, 5, len(keys))),
                        (R.IsDynamicSemistochastic(), rng.normal(size=len(keys)) * 2),
                        (R.IsDeterministic(), rng.normal(size=len(keys)))):
        nz = vals != 0
        k, v = keys[nz], vals[nz]
        wm = R.GPUWorkingMemory(SEED)
        wm.set_launch_shape(64, 0)
        g = gpu_step(h, style, k, v, 0.01, -1.0, SEED, 3, wm=wm)
        o = O.step(m, oracle_params(style, 0.01, -1.0, SEED, 3), k, v)
        assert_same_step(g, o, style)


def test_fermi2c_projector_energy_matches_exact_diagonalisation():
    """IsDeterministic power iteration of T = 1 + dt(S - H) on the device, with S the exact
    energy (so the ground-state component keeps its weight), converges to the ground state of
    the momentum block: the Rayleigh quotient <v|H|v>/<v|v> from device dot products reaches
    the oracle's exact energy."""
    h = MODELS["mom1d-fermi2c"]()
    m = oracle_model(h)
    e0 = O.ground_energy(m, start=h.address.key)
    v = R.GPUDVec({h.address: 1.0}, style=R.IsDeterministic())
    wm = R.GPUWorkingMemory(SEED)
    w = v.similar()
    op = R.FirstOrderTransitionOperator(h, e0, 0.05)
    for step in range(1, 1501):
        R.apply_operator(wm, w, v, op, step=step)
        v, w = w, v
    e = R.dot_operator(v, h, v) / v.dot(v)
    assert e == pytest.approx(e0, abs=1e-8)


def test_composite_models_reject_what_they_cannot_do():
    with pytest.raises(TypeError):
        R.HubbardReal1D(R.CompositeFS(R.BoseFS((1, 1)), R.BoseFS((1, 0))))
    with pytest.raises(TypeError):
        R.HubbardMom1D(R.CompositeFS(R.BoseFS((1, 1, 0)), R.FermiFS((1, 0, 0))))
    with pytest.raises(ValueError):
        R.HubbardRealSpace(R.CompositeFS(R.BoseFS((1, 1)), R.BoseFS((1, 0))), u=[[1, 2], [3, 4]])
    h = MODELS["realspace-bose-bose"]()
    with pytest.raises(TypeError):   # the full-basis H·v enumerates one-component bases
        R.BasisOperator(h)
