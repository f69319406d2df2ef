"""Matrix-free H*v on the full sorted basis, a Lanczos eigensolver on it, and the adjoint
of w = H(u, t) v as an autograd function (the rrule of mul!).

Vectors are float64 CUDA tensors (torch supplies device memory and the stream); the products
themselves run in librimu_gpu (rimu_hv_basis / rimu_hv_basis_adjoint).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .addresses import CompositeFS


def _torch():
    import torch
    return torch


class BasisOperator:
    """OperatorMultiplier role of ext/KrylovKitExt.jl:23-46 on the full basis:
    ``op(v)`` returns H v for a float64 CUDA tensor v of length ``op.dim``."""

    def __init__(self, hamiltonian):
        if isinstance(hamiltonian.address, CompositeFS):
            raise TypeError("the full-basis H·v enumerates one-component BoseFS/FermiFS bases")
        self.hamiltonian = hamiltonian
        self.dim = hamiltonian.dimension()

    def basis_keys(self, start=0, n=None) -> np.ndarray:
        n = self.dim - start if n is None else n
        out = np.zeros(max(n, 1), dtype=np.uint64)
        _lib.check(_lib.load().rimu_basis_keys(self.hamiltonian.handle, start, n,
                                                out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out[:n]

    def _check(self, v):
        torch = _torch()
        if not (v.is_cuda and v.dtype == torch.float64 and v.is_contiguous() and v.numel() == self.dim):
            raise ValueError("expected a contiguous float64 CUDA tensor of length dim")

    def apply(self, v, out=None):
        torch = _torch()
        self._check(v)
        w = torch.empty_like(v) if out is None else out
        _lib.check(_lib.load().rimu_hv_basis(self.hamiltonian.handle, C.c_void_p(v.data_ptr()),
                                              C.c_void_p(w.data_ptr()), self.dim))
        return w

    __call__ = apply

    def adjoint(self, v, gw):
        """(gv, gu, gt) for w = H(u, t) v and cotangent gw."""
        torch = _torch()
        self._check(v)
        self._check(gw)
        gv = torch.empty_like(v)
        gu, gt = C.c_double(), C.c_double()
        _lib.check(_lib.load().rimu_hv_basis_adjoint(
            self.hamiltonian.handle, C.c_void_p(v.data_ptr()), C.c_void_p(gw.data_ptr()),
            C.c_void_p(gv.data_ptr()), C.byref(gu), C.byref(gt), self.dim))
        return gv, gu.value, gt.value


def eigsolve(op: BasisOperator, v0=None, howmany=1, which="SR", tol=1e-10, krylovdim=64,
             maxiter=200):
    """Lowest eigenpair(s) by thick-restart-free Lanczos with full reorthogonalisation
    (the KrylovKit.eigsolve(H, v, 1, :SR) call of ext/KrylovKitExt.jl:36-46).
    Returns (values, vectors, info)."""
    torch = _torch()
    if which != "SR":
        raise ValueError("only which=:SR is implemented")
    # the Krylov vectors live where the start vector does (the context's device by default)
    dev = v0.device if v0 is not None else torch.device("cuda", _lib.default_context().device)
    v = v0.clone() if v0 is not None else torch.randn(op.dim, dtype=torch.float64, device=dev,
                                                      generator=torch.Generator(dev).manual_seed(1))
    v /= torch.linalg.norm(v)
    converged = False
    it = 0
    # the Krylov basis in one preallocated block (rows are vectors), filled in place: memory
    # is krylovdim + 1 vectors, which matters for bases of 10^8 and more
    Vm = torch.empty((krylovdim + 1, op.dim), dtype=torch.float64, device=dev)
    for restart in range(maxiter):
        Vm[0] = v
        alphas, betas = [], []
        w = op(Vm[0])
        n = 1
        for j in range(krylovdim):
            a = torch.dot(Vm[j], w)
            alphas.append(a.item())
            w -= a * Vm[j]
            if j > 0:
                w -= betas[-1] * Vm[j - 1]
            # full reorthogonalisation against the basis so far
            w -= Vm[:j + 1].T @ (Vm[:j + 1] @ w)
            b = torch.linalg.norm(w).item()
            it += 1
            T = np.diag(alphas) + np.diag(betas, 1) + np.diag(betas, -1)
            evals, evecs = np.linalg.eigh(T)
            resid = abs(b * evecs[-1, :howmany]).max()
            if resid < tol or b < 1e-300 or j == krylovdim - 1:
                break
            betas.append(b)
            torch.div(w, b, out=Vm[j + 1])
            n = j + 2
            w = op(Vm[j + 1])
        coef = torch.as_tensor(evecs[:, :howmany], dtype=torch.float64, device=dev)
        vecs = (Vm[:n].T @ coef).T
        theta = evals[:howmany]
        if resid < tol:
            converged = True
            break
        v = vecs[0] / torch.linalg.norm(vecs[0])
    info = {"converged": converged, "numops": it, "residual": float(resid)}
    return list(map(float, theta)), [vecs[i] for i in range(howmany)], info


class _HvFunction:
    """Holder for the torch.autograd.Function (built lazily so torch is optional)."""
    fn = None


def hv(hamiltonian, v, u=None, t=None):
    """Differentiable w = H(u, t) v on the full basis.  u and t are scalar tensors (or
    floats); gradients with respect to v, u and t come from the hand-written adjoint kernel
    (gv = H^T gw, gu = <gw, dH/du v>, gt = <gw, dH/dt v>)."""
    torch = _torch()
    if _HvFunction.fn is None:
        class HvFunction(torch.autograd.Function):
            @staticmethod
            def forward(ctx, v, u, t, ham):
                h = ham.with_params(u=float(u), t=float(t))
                op = BasisOperator(h)
                ctx.op = op
                ctx.save_for_backward(v)
                return op(v.contiguous())

            @staticmethod
            def backward(ctx, gw):
                (v,) = ctx.saved_tensors
                gv, gu, gt = ctx.op.adjoint(v.contiguous(), gw.contiguous())
                dev = v.device
                return (gv, torch.tensor(gu, dtype=torch.float64, device=dev),
                        torch.tensor(gt, dtype=torch.float64, device=dev), None)
        _HvFunction.fn = HvFunction
    dev = v.device
    u = torch.as_tensor(hamiltonian.u if u is None else u, dtype=torch.float64, device=dev)
    t = torch.as_tensor(hamiltonian.t if t is None else t, dtype=torch.float64, device=dev)
    return _HvFunction.fn.apply(v, u, t, hamiltonian)
