"""Matrix-free H*v on the full basis and its adjoint, against the oracle; Lanczos against
exact energies; Hellmann-Feynman gradients against finite differences."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import oracle_model

pytestmark = pytest.mark.gpu


def cuda(x):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


HV_MODELS = [
    R.HubbardReal1D(R.BoseFS([1] * 8), u=2.0, t=1.0),
    R.HubbardReal1D(R.BoseFS([3, 0, 0, 2, 0, 1, 0]), u=1.0, t=0.6),
    R.HubbardRealSpace(R.BoseFS([1, 1, 1, 0, 1, 0, 0, 0, 1]), R.PeriodicBoundaries(3, 3), u=[[3.0]]),
    R.HubbardRealSpace(R.BoseFS([1, 0, 2, 0, 1, 0]), R.HardwallBoundaries(2, 3), u=[[1.0]], t=[1.2]),
    R.HubbardRealSpace(R.FermiFS([1, 1, 1] + [0] * 13), R.PeriodicBoundaries(4, 4), u=[[0.0]]),
    R.HubbardMom1D(R.BoseFS([0, 1, 3, 1, 0, 0]), u=2.0),
    # the widths where the kernels change word size: 32-bit addresses (M=30, N=3) run on
    # 32-bit words, 33-bit addresses (M=31, N=3) on 64-bit words
    R.HubbardReal1D(R.BoseFS([1, 0, 1] + [0] * 26 + [1]), u=1.5, t=0.8),
    R.HubbardReal1D(R.BoseFS([1, 0, 1] + [0] * 27 + [1]), u=1.5, t=0.8),
]
ADJOINT_MODELS = HV_MODELS[:4] + HV_MODELS[6:]


@pytest.mark.parametrize("h", HV_MODELS, ids=repr)
def test_hv_basis_bit_exact(h):
    m = oracle_model(h)
    keys = O.basis(m)
    op = R.BasisOperator(h)
    assert op.dim == len(keys)
    assert np.array_equal(op.basis_keys(), keys)
    v = np.random.default_rng(1).normal(size=len(keys))
    w = op(cuda(v)).cpu().numpy()
    want = O.hv_basis(m, keys, v)
    assert np.array_equal(w.view(np.uint64), want.view(np.uint64))


@pytest.mark.parametrize("h", ADJOINT_MODELS, ids=repr)
def test_adjoint_matches_oracle(h):
    m = oracle_model(h)
    keys = O.basis(m)
    rng = np.random.default_rng(2)
    v, gw = rng.normal(size=len(keys)), rng.normal(size=len(keys))
    gv, gu, gt = R.BasisOperator(h).adjoint(cuda(v), cuda(gw))
    ogv, ogu, ogt = O.hv_basis_adjoint(m, keys, v, gw)
    assert np.array_equal(gv.cpu().numpy().view(np.uint64), ogv.view(np.uint64))
    assert gu == pytest.approx(ogu, rel=1e-12) and gt == pytest.approx(ogt, rel=1e-12)


def test_basis_keys_ranges_and_dimension():
    h = R.HubbardReal1D(R.BoseFS([1] * 10), u=1.0)
    op = R.BasisOperator(h)
    keys = O.basis(oracle_model(h))
    assert op.dim == len(keys) == 92378
    assert np.array_equal(op.basis_keys(1000, 50), keys[1000:1050])


def test_lanczos_c1_energy():
    h = R.HubbardReal1D(R.BoseFS([1] * 6), u=6.0, t=1.0)
    vals, vecs, info = R.eigsolve(R.BasisOperator(h), tol=1e-10)
    assert info["converged"]
    assert vals[0] == pytest.approx(-4.0215, abs=1e-4)          # test/KrylovKit.jl:6-15
    assert vals[0] == pytest.approx(O.ground_energy(O.real1d(6, 6, 6.0)), abs=1e-9)


def test_hellmann_feynman_gradients_vs_finite_differences():
    """dE/du = <psi|dH/du|psi> and dE/dt from the adjoint kernel against central finite
    differences of Lanczos energies (h = 1e-5), and dE/du against the expectation of the
    interaction operator sum n(n-1)/2 = (M/2) G2RealCorrelator(0)."""
    import torch
    N = M = 8
    u, t = 4.0, 1.0
    h = R.HubbardReal1D(R.BoseFS([1] * N), u=u, t=t)
    op = R.BasisOperator(h)
    E, vecs, _ = R.eigsolve(op, tol=1e-12)
    psi = vecs[0] / torch.linalg.norm(vecs[0])
    _, gu, gt = op.adjoint(psi, psi)
    step = 1e-5
    def energy(uu, tt):
        return R.eigsolve(R.BasisOperator(h.with_params(u=uu, t=tt)), v0=psi, tol=1e-13)[0][0]
    fd_u = (energy(u + step, t) - energy(u - step, t)) / (2 * step)
    fd_t = (energy(u, t + step) - energy(u, t - step)) / (2 * step)
    assert gu == pytest.approx(fd_u, rel=1e-6)
    assert gt == pytest.approx(fd_t, rel=1e-6)
    keys = op.basis_keys()
    inter = np.array([sum(n * (n - 1) for n in R.BoseFS.from_key(int(k), N, M).onr()) / 2 for k in keys])
    p = psi.cpu().numpy()
    assert gu == pytest.approx(float(np.dot(p * p, inter)), rel=1e-10)
    # Hellmann-Feynman identity for this model: E = u dE/du + t dE/dt
    assert E[0] == pytest.approx(u * gu + t * gt, rel=1e-9)


def test_autograd_rrule():
    import torch
    h = R.HubbardReal1D(R.BoseFS([1] * 6), u=3.0, t=1.0)
    m = oracle_model(h)
    keys = O.basis(m)
    rng = np.random.default_rng(3)
    v = cuda(rng.normal(size=len(keys))).requires_grad_(True)
    gw = cuda(rng.normal(size=len(keys)))
    u = torch.tensor(3.0, dtype=torch.float64, device="cuda", requires_grad=True)
    t = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
    w = R.hv(h, v, u, t)
    (w * gw).sum().backward()
    ogv, ogu, ogt = O.hv_basis_adjoint(m, keys, v.detach().cpu().numpy(), gw.cpu().numpy())
    assert np.allclose(v.grad.cpu().numpy(), ogv, rtol=1e-13, atol=1e-13)
    assert u.grad.item() == pytest.approx(ogu, rel=1e-12)
    assert t.grad.item() == pytest.approx(ogt, rel=1e-12)
