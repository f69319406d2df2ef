"""The CPU oracle against the reference's own known answers (tests/golden/reference_goldens.json).
CPU only: this pins the checker before it is trusted for GPU parity."""
import json
import math
import os

import numpy as np
import pytest

import oracle as O

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def test_hopnextneighbour_docstring():
    for c in G["hopnextneighbour"]:
        onr = c["onr"]
        m = O.real1d(sum(onr), len(onr), u=1.0, t=1.0)
        nk, val = O.offdiagonals(m, O.bose_key(onr))[c["chosen"] - 1]
        assert O.bose_onr(nk, len(onr)) == c["new"]
        assert -val == c["value"]          # get_offdiagonal = -t * hopnextneighbour value


def test_real1d_offdiagonals_docstring():
    c = G["real1d_offdiagonals"]
    m = O.real1d(sum(c["onr"]), len(c["onr"]), c["u"], c["t"])
    got = [(O.bose_onr(k, 3), v) for k, v in O.offdiagonals(m, O.bose_key(c["onr"]))]
    assert got == [(p[0], p[1]) for p in c["pairs"]]


def test_bose_hubbard_interaction():
    for c in G["bose_hubbard_interaction"]:
        m = O.real1d(sum(c["onr"]), len(c["onr"]), u=2.0)
        assert O.diagonal(m, O.bose_key(c["onr"])) == c["value"]   # u/2 * interaction with u=2


def test_mom1d_goldens():
    c = G["mom1d"]
    m = O.mom1d(sum(c["onr"]), len(c["onr"]), c["u"], c["t"])
    k = O.bose_key(c["onr"])
    assert O.diagonal(m, k) == c["diagonal"]
    assert O.num_offdiagonals(m, k) == c["num_offdiagonals"]
    nk, v = O.offdiagonals(m, k)[2]
    assert O.bose_onr(nk, 3) == c["offdiag3"][0] and v == c["offdiag3"][1]
    d = G["momentum_transfer_diagonal"]
    m5 = O.mom1d(6, 5)
    kin = sum(m5.kes[i] * n for i, n in enumerate(d["onr"]) if n)
    assert O.diagonal(m5, O.bose_key(d["onr"])) - kin == pytest.approx(d["value"], abs=1e-14)


def test_realspace_fermion_offdiagonal_counts():
    c = G["realspace_fermi_offdiag_counts"]
    f = O.fermi_key([1] * c["N"] + [0] * (c["M"] - c["N"]))
    for dims, periodic, total, nonzero in c["cases"]:
        m = O.realspace(c["N"], tuple(dims), u=0.0, periodic=(periodic, periodic), fermion=True)
        od = O.offdiagonals(m, f)
        assert len(od) == total and sum(1 for _, v in od if v != 0) == nonzero


@pytest.mark.parametrize("case", G["energies"], ids=lambda c: c["src"] + str(c.get("N", "")))
def test_exact_energies(case):
    if case["model"] == "real1d":
        E = O.ground_energy(O.real1d(case["N"], case["M"], case["u"], case["t"]))
    elif case["model"] == "mom1d":
        onr = case["start"]
        E = O.ground_energy(O.mom1d(sum(onr), len(onr), case["u"], case["t"]), O.bose_key(onr))
    elif case["model"] == "realspace_multi":
        E = O.ground_energy(O.realspace_multi(tuple((bool(f), n) for f, n in case["comps"]),
                                              tuple(case["dims"]), t=case["ct"], u=case["cu"]))
    else:
        E = O.ground_energy(O.realspace(case["N"], tuple(case["dims"]), u=case["u"], t=case["t"],
                                        fermion=True))
    assert E == pytest.approx(case["E0"], abs=case["atol"])


def test_krylov_sector_of_a_4x4_fermion_address():
    """test/Hamiltonians.jl:439-444: exact_energy (:13-17, eigsolve from the starting address)
    of five free fermions on the periodic 4x4 lattice started from
    FermiFS((1,0,1,0,1,0,1,0,1,0,0,...)) is -10, although the closed-shell ground state of the
    whole basis is -4 + 4*(-2) = -12: the start address has no overlap with that state, so a
    Krylov space built from it reaches -10 first.  Restated on the dense matrix: the lowest
    eigenvalue whose eigenspace the start address overlaps.  This pins the fermionic hopping
    signs across the periodic boundaries."""
    c = G["krylov_sector"]
    onr = c["start"]
    m = O.realspace(sum(onr), tuple(c["dims"]), u=0.0, t=c["t"], fermion=True)
    keys = O.basis(m)
    start = sum(1 << i for i, x in enumerate(onr) if x)
    H = O.sparse_matrix(m, keys).toarray()
    w, V = np.linalg.eigh(H)
    assert w[0] == pytest.approx(-12.0, abs=1e-9)
    j = int(np.searchsorted(keys, start))
    # group degenerate levels and take the first the start address overlaps
    e_first, i = None, 0
    while i < len(w):
        k = i
        while k < len(w) and w[k] - w[i] < 1e-8:
            k += 1
        if np.linalg.norm(V[j, i:k]) > 1e-8:
            e_first = w[i]
            break
        i = k
    assert e_first == pytest.approx(c["E0"], abs=c["atol"])


def test_real1d_equals_realspace_1d():
    c = G["real1d_equals_realspace"]
    N, M = sum(c["onr"]), len(c["onr"])
    a = O.ground_energy(O.real1d(N, M, c["u"], c["t"]))
    b = O.ground_energy(O.realspace(N, (M,), u=c["u"], t=c["t"]))
    assert a == pytest.approx(b, abs=1e-12)


def test_hopnextneighbour_equals_excitation_on_random_onrs():
    """HubbardReal1D (hop formula) agrees with HubbardRealSpace 1D (excitation formula) on
    random ONRs, as test/BitStringAddresses.jl:251-297 checks hopnextneighbour."""
    rng = np.random.default_rng(7)
    for N, M in ((16, 16), (3, 32), (20, 20), (5, 40)):
        for _ in range(10):
            onr = np.bincount(rng.integers(0, M, N), minlength=M).tolist()
            k = O.bose_key(onr)
            a = O.offdiagonals(O.real1d(N, M), k)
            b = O.offdiagonals(O.realspace(N, (M,)), k)
            assert a == b
            assert O.bose_onr(k, M) == onr


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of the Random123 distribution (Salmon et al.)."""
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_oracle_step_is_deterministic_and_conserves_structure():
    m = O.real1d(6, 6, u=6.0)
    k0 = O.bose_key([1] * 6)
    p = O.StepParams(O.STYLE_INTEGER, dt=1e-3, shift=0.0, seed=11, step=1)
    a = O.step(m, p, [k0], [10])
    b = O.step(m, p, [k0], [10])
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
    assert a[2]["spawn_attempts"] == 10 and a[2]["len"] == len(a[0])
    assert a[2]["norm"] == float(np.abs(a[1]).sum())


def test_oracle_deterministic_step_matches_dense_transition_matrix():
    """IsDeterministic step == (1 + dt(S - H)) v with the dense matrix (fciqmc.jl:78-112)."""
    m = O.real1d(4, 4, u=3.0, t=1.5)
    keys = O.basis(m)
    H = O.sparse_matrix(m, keys).toarray()
    rng = np.random.default_rng(3)
    v = rng.normal(size=len(keys))
    dt, S = 0.01, -1.25
    ok, ov, st = O.step(m, O.StepParams(O.STYLE_DETERMINISTIC, dt=dt, shift=S), keys, v)
    want = (np.eye(len(keys)) + dt * (S * np.eye(len(keys)) - H)) @ v
    got = np.zeros(len(keys))
    got[np.searchsorted(keys, ok)] = ov
    assert np.allclose(got, want, rtol=1e-13, atol=1e-15)
    assert st["exact_steps"] == len(keys)


def test_oracle_hv_matches_sparse_matrix():
    for m in (O.real1d(6, 6, u=2.0), O.realspace(4, (2, 3), u=1.0, t=0.7),
              O.mom1d(4, 5, u=2.0), O.realspace(3, (3, 3), u=0.0, fermion=True)):
        keys = O.basis(m)
        v = np.random.default_rng(1).normal(size=len(keys))
        assert np.allclose(O.hv_basis(m, keys, v), O.sparse_matrix(m, keys) @ v, rtol=1e-13, atol=1e-13)


def test_oracle_adjoint_matches_finite_differences():
    N, M, u, t = 5, 5, 2.0, 1.0
    m = O.real1d(N, M, u, t)
    keys = O.basis(m)
    rng = np.random.default_rng(5)
    v, gw = rng.normal(size=len(keys)), rng.normal(size=len(keys))
    gv, gu, gt = O.hv_basis_adjoint(m, keys, v, gw)
    H = O.sparse_matrix(m, keys)
    assert np.allclose(gv, H.T @ gw, rtol=1e-13, atol=1e-13)
    h = 1e-5
    fu = (gw @ O.hv_basis(O.real1d(N, M, u + h, t), keys, v) - gw @ O.hv_basis(O.real1d(N, M, u - h, t), keys, v)) / (2 * h)
    ft = (gw @ O.hv_basis(O.real1d(N, M, u, t + h), keys, v) - gw @ O.hv_basis(O.real1d(N, M, u, t - h), keys, v)) / (2 * h)
    assert gu == pytest.approx(fu, rel=1e-7) and gt == pytest.approx(ft, rel=1e-7)


def test_oracle_c1_energies_within_two_blocking_errors():
    """The small plain configuration run through the oracle: HubbardReal1D M=N=6, u=6, t=1,
    IsStochasticInteger, 1 000 target walkers, dt = 1e-3, 20 000 steps, seed 1234.  Shift and
    projected energy (blocking analysis, first 3 000 steps skipped) lie within 2 blocking
    errors of the exact energy, which is the reference's E0 = -4.0215 (test/KrylovKit.jl:6-15)."""
    import rimugpu as R
    from helpers import oracle_solve
    m = O.real1d(6, 6, 6.0, 1.0)
    E0 = O.ground_energy(m)
    assert E0 == pytest.approx(-4.0215, abs=1e-4)
    df = oracle_solve(m, R.IsStochasticInteger(), R.BoseFS([1] * 6).key, 10, 20000, 1e-3, 1000, 1234)
    assert len(df["shift"]) == 20000
    r = R.shift_estimator(df, skip=3000)
    pe, pe_err = R.projected_energy(df, skip=3000)
    assert abs(r.mean - E0) < 2 * r.err, (r.mean, r.err)
    assert abs(pe - E0) < 2 * pe_err, (pe, pe_err)


def test_oracle_mom1d_energies_within_two_blocking_errors():
    """HubbardMom1D M=10, N=5 with all bosons in k = 0 (mode M/2, HubbardMom1D.jl:55-61),
    u=6, IsStochasticInteger, 2 000 target walkers, dt = 5e-4, 20 000 steps through the
    oracle: shift and projected energy within 2 blocking errors of the exact energy of the
    k = 0 sector."""
    import rimugpu as R
    from helpers import oracle_solve
    M, N = 10, 5
    addr = R.BoseFS(M, {M // 2: N})
    m = O.mom1d(N, M, 6.0, 1.0)
    E0 = O.ground_energy(m, start=addr.key)
    df = oracle_solve(m, R.IsStochasticInteger(), addr.key, 100, 20000, 5e-4, 2000, 2024, zeta=0.05)
    r = R.shift_estimator(df, skip=5000)
    pe, pe_err = R.projected_energy(df, skip=5000)
    assert abs(r.mean - E0) < 2 * r.err, (r.mean, r.err)
    assert abs(pe - E0) < 2 * pe_err, (pe, pe_err)


@pytest.mark.parametrize("periodic", [(True, True), (False, False)], ids=["periodic", "hardwall"])
def test_oracle_adjoint_realspace_matches_sparse_matrix_and_finite_differences(periodic):
    """The single-pass adjoint on one-component bosonic HubbardRealSpace (2x3 lattice, N=4):
    gv = H^T gw, and the u and t gradients against central finite differences of <gw, H v>."""
    N, dims, u, t = 4, (2, 3), 1.5, 0.7
    def model(uu, tt):
        return O.realspace(N, dims, u=uu, t=tt, periodic=periodic)
    m = model(u, t)
    keys = O.basis(m)
    rng = np.random.default_rng(7)
    v, gw = rng.normal(size=len(keys)), rng.normal(size=len(keys))
    gv, gu, gt = O.hv_basis_adjoint(m, keys, v, gw)
    assert np.allclose(gv, O.sparse_matrix(m, keys).T @ gw, rtol=1e-13, atol=1e-13)
    h = 1e-5
    def f(uu, tt):
        return gw @ O.hv_basis(model(uu, tt), keys, v)
    assert gu == pytest.approx((f(u + h, t) - f(u - h, t)) / (2 * h), rel=1e-7)
    assert gt == pytest.approx((f(u, t + h) - f(u, t - h)) / (2 * h), rel=1e-7)


def test_oracle_momentum_transfer_excitations():
    """momentum_transfer_excitation with fold=true, the periodic form HubbardMom1D uses
    (test/Hamiltonians.jl:97-152), through the oracle's HubbardMom1D offdiagonals, whose values
    are (u/2M) * onproduct, or (u/M) * onproduct for FermiFS2C (HubbardMom1D.jl:189-205)."""
    u = 2.0
    m = O.mom1d(2, 4, u=u)
    # BoseFS((0,1,1,0)): all four excitations reach (1,0,0,1) with onproduct 1
    offs = O.offdiagonals(m, O.bose_key([0, 1, 1, 0]))
    assert len(offs) == 4
    for k, v in offs:
        assert k == O.bose_key([1, 0, 0, 1]) and v == pytest.approx(u / 8)
    # BoseFS((1,1,0,0)): onproduct 1 for all four
    offs = O.offdiagonals(m, O.bose_key([1, 1, 0, 0]))
    assert len(offs) == 4 and all(v == pytest.approx(u / 8) for _, v in offs)
    # BoseFS((0,3,0)): both excitations reach (1,1,1) with onproduct sqrt(6)
    offs = O.offdiagonals(O.mom1d(3, 3, u=u), O.bose_key([0, 3, 0]))
    assert len(offs) == 2
    for k, v in offs:
        assert k == O.bose_key([1, 1, 1]) and v == pytest.approx(u / 6 * math.sqrt(6))
    # FermiFS2C pairs: onproduct 1 for each of the three excitations
    M = 4
    for a, b in (([0, 0, 1, 0], [0, 1, 0, 0]), ([1, 0, 0, 0], [0, 1, 0, 0])):
        key = (O.fermi_key(a) << M) | O.fermi_key(b)
        offs = O.offdiagonals(O.mom1d_2c(1, 1, M, u=u), key)
        assert len(offs) == 3 and all(v == pytest.approx(u / M) for _, v in offs)


@pytest.mark.parametrize("n", [6, 8])
def test_lanczos_host_loop_against_dense_eigenvalues(n):
    """The host side of the KrylovKit path (eigsolve, ext/KrylovKitExt.jl:36-46) with the
    oracle's sparse HubbardReal1D(n, n; u=6) as the operator, on the CPU: the lowest eigenvalue
    agrees with scipy's to 1e-10, and for n = 6 it is the reference's -4.0215
    (test/KrylovKit.jl:6-15)."""
    import scipy.sparse.linalg as sla
    import torch
    import rimugpu as R
    m = O.real1d(n, n, 6.0, 1.0)
    H = O.sparse_matrix(m).tocsr()

    class Op:
        dim = H.shape[0]

        def __call__(self, v):
            return torch.as_tensor(H @ v.numpy())

    v0 = torch.as_tensor(np.random.default_rng(2).normal(size=Op.dim))
    vals, vecs, info = R.eigsolve(Op(), v0=v0, tol=1e-10)
    assert info["converged"]
    want = sla.eigsh(H, k=1, which="SA")[0][0]
    assert vals[0] == pytest.approx(want, abs=1e-10)
    if n == 6:
        assert vals[0] == pytest.approx(-4.0215, abs=1e-4)
    r = H @ vecs[0].numpy() - vals[0] * vecs[0].numpy()
    assert np.linalg.norm(r) / np.linalg.norm(vecs[0].numpy()) < 1e-8


@pytest.mark.parametrize("name,m", [
    ("real1d", O.real1d(5, 6, u=2.0, t=0.7)),
    ("realspace-periodic", O.realspace(4, (2, 3), u=1.5, t=0.8)),
    ("realspace-hardwall", O.realspace(3, (3, 3), u=2.0, periodic=(False, False))),
    ("realspace-fermion", O.realspace(3, (2, 4), u=0.0, fermion=True)),
    ("mom1d", O.mom1d(4, 6, u=3.0)),
    ("mom1d-fermi2c", O.mom1d_2c(2, 2, 5, u=1.5)),
    ("realspace-2c", O.realspace2(((False, 2), (True, 2)), (2, 2), t=(1.0, 0.5),
                                  u=((1.0, 2.0), (2.0, 0.0)))),
])
def test_oracle_hamiltonians_are_symmetric(name, m):
    """Every model's matrix over its full sorted basis is real symmetric, the LOStructure
    IsHermitian the pull-form H*v relies on (HubbardReal1D.jl:44 and its siblings): row i
    read from the offdiagonals of column i is row i of H."""
    H = O.sparse_matrix(m).tocsr()
    assert H.shape[0] > 1
    assert abs(H - H.T).max() <= 1e-14 * max(abs(H).max(), 1.0)


@pytest.mark.parametrize("name,m,key", [
    ("real1d", O.real1d(5, 6, u=2.0, t=0.7), O.bose_key([2, 0, 1, 0, 2, 0])),
    ("realspace-hardwall", O.realspace(4, (2, 3), u=1.5, periodic=(False, True)),
     O.bose_key([1, 0, 2, 0, 0, 1])),
    ("realspace-fermion", O.realspace(3, (2, 4), fermion=True), O.fermi_key([1, 1, 0, 0, 1, 0, 0, 0])),
    ("mom1d", O.mom1d(4, 6, u=3.0), O.bose_key([0, 1, 2, 0, 1, 0])),
    ("mom1d-fermi2c", O.mom1d_2c(2, 2, 5, u=1.5),
     (O.fermi_key([1, 1, 0, 0, 0]) << 5) | O.fermi_key([0, 0, 1, 1, 0])),
])
def test_oracle_hamiltonian_action_on_one_address(name, m, key):
    """The interface test's Hamiltonian action (InterfaceTests.jl:211-226): H applied to
    2 e_addr by one plain-Hamiltonian step equals 2 (diagonal_element e_addr + the sum of the
    offdiagonals), entry by entry."""
    k, v, _ = O.step(m, O.StepParams(O.STYLE_DETERMINISTIC, op=O.OP_HAMILTONIAN), [key],
                     np.array([2.0]))
    want = {key: 2 * O.diagonal(m, key)}
    for nk, hv in O.offdiagonals(m, key):
        want[nk] = want.get(nk, 0.0) + 2 * hv
    want = {a: x for a, x in want.items() if x != 0.0}
    got = dict(zip((int(a) for a in k), v))
    assert set(got) == set(want)
    for a, x in want.items():
        assert got[a] == pytest.approx(x, rel=1e-14, abs=1e-14), a


def test_hubbard_models_with_t_or_u_zero():
    """test/Hamiltonians.jl:217-250 on the oracle with the host's momentum grid and
    dispersions: with t = 0 or u = 0 the diagonal or the offdiagonals vanish; with u = 0 the
    hubbard dispersion of three bosons in the k = 0 mode gives -2tN and the continuum
    dispersion 0; for BoseFS(3,3,3) the continuum diagonal is 6t(2pi/M)^2 and above the
    shifted hubbard one."""
    import rimugpu as R

    def mom(h):
        m = O.mom1d(h.N, h.M, h.u, h.t)
        m.kes = np.array(h.kes)
        return m

    bs1, bs2, bs3 = R.BoseFS((0, 1, 0)), R.BoseFS((3, 3, 3)), R.BoseFS((0, 3, 0))
    assert O.diagonal(mom(R.HubbardMom1D(bs1, t=0.0)), bs1.key) == 0
    assert O.diagonal(O.real1d(bs2.N, bs2.M, 0.0, 1.0), bs2.key) == 0
    assert all(v == 0 for _, v in O.offdiagonals(mom(R.HubbardMom1D(bs1, u=0.0)), bs1.key))
    assert all(v == 0 for _, v in O.offdiagonals(O.real1d(bs2.N, bs2.M, 1.0, 0.0), bs2.key))
    t = 1.0
    c3 = R.HubbardMom1D(bs3, u=0.0, t=t, dispersion=R.hamiltonians.continuum_dispersion)
    h3 = R.HubbardMom1D(bs3, u=0.0, t=t)
    assert O.diagonal(mom(c3), bs3.key) == 0
    assert 2 * t * bs3.N + O.diagonal(mom(h3), bs3.key) == 0
    c2 = R.HubbardMom1D(bs2, u=0.0, t=t, dispersion=R.hamiltonians.continuum_dispersion)
    h2 = R.HubbardMom1D(bs2, u=0.0, t=t)
    d2 = O.diagonal(mom(c2), bs2.key)
    assert d2 > 2 * t * bs2.N + O.diagonal(mom(h2), bs2.key)
    assert d2 == pytest.approx(6 * t * (2 * np.pi / bs2.M) ** 2)


@pytest.mark.parametrize("fermion,onr", [(False, (1, 1, 1, 0, 0, 0)), (True, (1, 0, 0, 0, 1, 0))],
                         ids=["bose", "fermi"])
def test_hardwall_lattice_orientation(fermion, onr):
    """test/Hamiltonians.jl:472-484: HubbardRealSpace with default u and t on hard-wall 2x3 and
    3x2 lattices has the same ground energy from the same start address (eigsolve from the
    starting address: here the block connected to it)."""
    start = sum(1 << i for i, x in enumerate(onr) if x) if fermion else O.bose_key(list(onr))
    e = []
    for dims in ((2, 3), (3, 2)):
        m = O.realspace(sum(onr), dims, u=1.0, t=1.0, periodic=(False, False), fermion=fermion)
        e.append(O.ground_energy(m, start))
    assert e[0] == pytest.approx(e[1], rel=1e-12)
