"""Two-component addresses in the oracle, pinned against the reference's own known answers,
and the host-side CompositeFS / FermiFS2C address classes.

Known answers (test/Hamiltonians.jl):
  * "1D Fermions" (:365-385): two non-interacting fermion components on 6 sites with t = 1, 2
    have E0 = -3 + -6; a repulsive inter-component u raises it, an attractive one lowers it;
  * "1D Bosons (2-component)" (:327-362): one particle in the second component gives the same
    energy as a boson or a fermion, and with the components swapped;
  * "1D trap" (:397-411): the same with a trap potential per component.
Independent of the reference's numbers: HubbardMom1D with FermiFS2C is the Fourier transform of
the two-component real-space Hubbard model, so on the momentum block of the start address the
two exact ground-state energies coincide.  The two oracle models are written from different
reference files (HubbardMom1D.jl / excitations.jl and HubbardRealSpace.jl)."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R


def test_noninteracting_fermion_components_add_up():
    m = O.realspace2(((True, 4), (True, 2)), (6,), t=(1.0, 2.0), u=((0, 0), (0, 0)))
    assert O.ground_energy(m) == pytest.approx(-3 + -6, rel=1e-12)


def test_inter_component_interaction_raises_and_lowers_the_energy():
    rep = O.realspace2(((True, 4), (True, 2)), (6,), t=(1.0, 2.0), u=((0, 1), (1, 0)))
    att = O.realspace2(((True, 4), (True, 2)), (6,), t=(1.0, 2.0), u=((0, -1), (-1, 0)))
    assert O.ground_energy(rep) > -9
    assert O.ground_energy(att) < -9


@pytest.mark.parametrize("trap", [False, True])
def test_single_particle_component_is_bose_or_fermi_in_either_order(trap):
    v2 = ((0.0,), (0.0,))
    cases = [(((False, 3), (False, 1)), (1, 4), ((2, 3), (3, 0)), ((1.0,), (4.0,))),
             (((False, 3), (True, 1)), (1, 4), ((2, 3), (3, 0)), ((1.0,), (4.0,))),
             (((False, 1), (False, 3)), (4, 1), ((0, 3), (3, 2)), ((4.0,), (1.0,))),
             (((True, 1), (False, 3)), (4, 1), ((0, 3), (3, 2)), ((4.0,), (1.0,)))]
    if trap:   # the reference's trap case keeps t = (1, 1)
        cases = [(c, (1, 1), u, v) for c, _, u, v in cases]
    energies = []
    for comps, t, u, v in cases:
        pot = None
        if trap:
            # HubbardRealSpace.jl:214-226 on 6 periodic sites: x in -3..2, pot = v x^2
            x = np.arange(6) - 3
            pot = np.array([v[0][0] * x ** 2, v[1][0] * x ** 2], dtype=float)
        energies.append(O.ground_energy(O.realspace2(comps, (6,), t=t, u=u, pot=pot)))
    assert np.allclose(energies, energies[0], rtol=1e-12)


@pytest.mark.parametrize("M,up,dn,u", [
    (5, (0, 0, 1, 0, 0), (0, 0, 1, 0, 0), 2.0),
    (6, (0, 1, 1, 1, 0, 0), (0, 1, 1, 1, 0, 0), 3.0),
    (6, (0, 1, 1, 1, 0, 0), (0, 1, 1, 1, 0, 0), -2.0),
    (7, (0, 0, 1, 1, 1, 0, 0), (0, 0, 1, 1, 1, 0, 0), 4.0),
])
def test_fermi2c_momentum_space_equals_real_space(M, up, dn, u):
    n1, n2 = sum(up), sum(dn)
    key = (O.fermi_key(up) << M) | O.fermi_key(dn)
    em = O.ground_energy(O.mom1d_2c(n1, n2, M, u=u, t=1.0), start=key)
    er = O.ground_energy(O.realspace2(((True, n1), (True, n2)), (M,), t=(1.0, 1.0),
                                      u=((0, u), (u, 0))))
    assert em == pytest.approx(er, abs=1e-10)


def test_fermi2c_offdiagonal_count_and_hermiticity():
    m = O.mom1d_2c(2, 3, 6, u=1.5)
    keys = O.basis(m)
    for k in keys[::7]:
        assert O.num_offdiagonals(m, int(k)) == 2 * 3 * 5        # HubbardMom1D.jl:141-144
    H = O.sparse_matrix(m, keys)
    assert abs(H - H.T).max() < 1e-14


def test_composite_realspace_is_hermitian_with_hardwall_and_trap():
    pot = np.array([[0.5, 0.0, 0.5, 1.0, 0.25, 0.0], [0.0, 2.0, 0.0, 1.0, 0.0, 3.0]])
    m = O.realspace2(((False, 2), (True, 2)), (2, 3), t=(1.0, 0.5), u=((1.5, 2.0), (2.0, 0.0)),
                     periodic=(False, True), pot=pot)
    H = O.sparse_matrix(m)
    assert H.shape[0] == 21 * 15
    assert abs(H - H.T).max() < 1e-14


def test_composite_key_order_is_component_tuple_order():
    """isless(a, b) = isless(a.components, b.components) (multicomponent.jl:79)."""
    a = R.CompositeFS(R.FermiFS((1, 1, 0, 0, 0, 0)), R.BoseFS((5, 0, 0, 0, 0, 0)))
    b = R.CompositeFS(R.FermiFS((0, 1, 1, 0, 0, 0)), R.BoseFS((1, 1, 1, 1, 1, 0)))
    c = R.CompositeFS(R.FermiFS((0, 1, 1, 0, 0, 0)), R.BoseFS((0, 0, 0, 0, 0, 5)))
    assert (a < b) == ((a.components[0].key, a.components[1].key) <
                       (b.components[0].key, b.components[1].key))
    assert sorted([b, c, a]) == sorted([b, c, a], key=lambda x: tuple(y.key for y in x.components))
    assert a.with_key(a.key) == a and a.with_key(b.key).components == b.components
    assert a.N == 7 and a.M == 6 and a.onr() == ((1, 1, 0, 0, 0, 0), (5, 0, 0, 0, 0, 0))
    with pytest.raises(ValueError):
        R.CompositeFS(R.BoseFS((1, 1)), R.BoseFS((1, 1, 1)))


def test_fermi2c_constructors_agree():
    """The three forms of the FermiFS2C docstring (multicomponent.jl:87-113)."""
    f1 = R.FermiFS2C(R.FermiFS(1, 0, 0), R.FermiFS(0, 1, 1))
    f2 = R.FermiFS2C((1, 0, 0), (0, 1, 1))
    f3 = R.FermiFS2C(3, [(1, 1), (2, -1), (3, -1)])
    assert f1 == f2 == f3
    assert R.FermiFS2C(3, {1: 1}).N == 1 and R.FermiFS2C(3, {1: -1}).N == 1


# ---- three and four components --------------------------------------------------------------
def test_three_noninteracting_fermion_components_add_up():
    """test/Hamiltonians.jl:365-377 with a third component: FermiFS((1,1,1,0,0,0)) with t = 3.5
    alone has E0 = -14 (:366-369), so the three components without interaction have
    -3 + -6 + -14."""
    m = O.realspace_multi(((True, 4), (True, 2), (True, 3)), (6,), t=(1.0, 2.0, 3.5),
                          u=np.zeros((3, 3)))
    assert len(O.basis(m)) == 15 * 15 * 20
    assert O.ground_energy(m) == pytest.approx(-3 - 6 - 14, rel=1e-10)


def test_four_component_offdiagonals_reach_the_whole_basis():
    """test/ExactDiagonalization.jl:152-163: for HubbardRealSpace(CompositeFS(BoseFS(2,0,0),
    FermiFS(1,0,1), BoseFS(0,2,0), BoseFS(1,0,0))) the basis built by following the
    Hamiltonian's offdiagonals equals the address type's basis (product of the component
    bases, in key order)."""
    addr = R.CompositeFS(R.BoseFS((2, 0, 0)), R.FermiFS((1, 0, 1)), R.BoseFS((0, 2, 0)),
                         R.BoseFS((1, 0, 0)))
    m = O.realspace_multi(((False, 2), (True, 2), (False, 2), (False, 1)), (3,))
    assert m.nbits == addr.nbits == 14
    keys = O.basis(m)
    assert len(keys) == 6 * 3 * 6 * 3 and addr.key in set(int(k) for k in keys)
    assert np.array_equal(O.connected_basis(m, addr.key), keys)


@pytest.mark.parametrize("perm", [(1, 2, 0), (2, 0, 1), (0, 2, 1)])
def test_component_order_does_not_change_the_energy(perm):
    """The pattern of test/Hamiltonians.jl:326-362 for three components (bosons and a
    fermion, hopping and interactions all different): listing the components in another order,
    with t and the rows and columns of u permuted alike, gives the same ground-state energy."""
    comps = ((False, 2), (True, 1), (False, 1))
    t = np.array([1.0, 4.0, 2.0])
    u = np.array([[2.0, 3.0, 1.0], [3.0, 0.0, 0.5], [1.0, 0.5, 4.0]])
    e0 = O.ground_energy(O.realspace_multi(comps, (5,), t=t, u=u))
    p = list(perm)
    e1 = O.ground_energy(O.realspace_multi(tuple(comps[i] for i in p), (5,), t=t[p],
                                           u=u[np.ix_(p, p)]))
    assert e1 == pytest.approx(e0, rel=1e-10)


def test_multi_component_diagonal_follows_the_reference_recursion():
    """The diagonal element of a CompositeFS is local_interaction's recursion over the
    components plus the trap (HubbardRealSpace.jl:18-61, 100-107, 284-287): for integer
    occupations every term is exact, so the value equals the closed form
    sum_s u[s,s]/2 sum_i n_si(n_si - 1) (bosons) + sum_{s<j} u[s,j] sum_i n_si n_ji + trap."""
    comps = ((False, 3), (True, 2), (False, 2), (True, 1))
    u = np.array([[1.5, 2.0, 0.5, -1.0], [2.0, 0.0, 1.0, 0.25], [0.5, 1.0, 3.0, 2.0],
                  [-1.0, 0.25, 2.0, 0.0]])
    x = np.arange(4) - 2
    pot = np.array([[0.5 * xx * xx for xx in x], [0.0] * 4, [0.25 * xx * xx for xx in x],
                    [1.0 * xx * xx for xx in x]])
    m = O.realspace_multi(comps, (4,), t=(1.0, 0.5, 2.0, 1.0), u=u, pot=pot)
    rng = np.random.default_rng(5)
    keys = O.basis(m)
    for k in rng.choice(keys, 60, replace=False):
        addr = R.CompositeFS(R.BoseFS((3, 0, 0, 0)), R.FermiFS((1, 1, 0, 0)),
                             R.BoseFS((2, 0, 0, 0)), R.FermiFS((1, 0, 0, 0))).with_key(int(k))
        occ = [np.array(c.onr()) for c in addr.components]
        want = 0.0
        for s in range(4):
            if not comps[s][0]:
                want += u[s, s] * np.sum(occ[s] * (occ[s] - 1)) / 2
            for j in range(s + 1, 4):
                want += u[s, j] * np.sum(occ[s] * occ[j])
            want += np.sum(occ[s] * pot[s])
        assert O.diagonal(m, int(k)) == pytest.approx(want, abs=1e-12)


def test_composite_key_layout_up_to_128_bits():
    """The host CompositeFS: each component above the bits of the ones after it, keys of up to
    128 bits (each component at most 64), with_key inverting the packing; wider layouts are
    refused."""
    a, b, c = R.BoseFS([0, 0, 0, 0, 2] + [0] * 25), R.FermiFS([1, 1] + [0] * 28), R.BoseFS([1] + [0] * 29)
    comp = R.CompositeFS(a, b, c)
    assert comp.nbits == 31 + 30 + 30 == 91
    assert comp.key == (a.key << 60) | (b.key << 30) | c.key
    back = comp.with_key(comp.key)
    assert back == comp and [x.key for x in back.components] == [a.key, b.key, c.key]
    with pytest.raises(ValueError):
        R.CompositeFS(R.BoseFS([1] * 40), R.BoseFS([1] * 40))          # a 79-bit component
    with pytest.raises(ValueError):
        R.CompositeFS(R.FermiFS([1] + [0] * 63), R.FermiFS([1] + [0] * 63), R.FermiFS([1] + [0] * 63))
