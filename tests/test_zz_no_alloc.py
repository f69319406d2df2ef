"""The allocation-free adjoint entry point, called through the C ABI.

Some callers cannot let a library allocate device memory: programs whose GPU memory belongs to
their own allocator or budget, where a cudaMalloc fails or takes memory promised elsewhere.
They use rimu_hv_basis_adjoint_noalloc, which keeps its scratch in a fixed static device array
instead of asking for memory.  It runs the same kernels as the handle-based
rimu_hv_basis_adjoint, so on consecutive calls that reuse the array its g_v must be identical
bit for bit and its g_u, g_t (sums reduced in the same fixed order) equal too.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call_noalloc(lib, desc, v, gw, gv):
    gu, gt = C.c_double(), C.c_double()
    rc = lib.rimu_hv_basis_adjoint_noalloc(C.byref(desc), C.c_void_p(v.data_ptr()),
                                           C.c_void_p(gw.data_ptr()), C.c_void_p(gv.data_ptr()),
                                           C.byref(gu), C.byref(gt), v.numel(), None)
    return rc, gu.value, gt.value


@pytest.mark.parametrize("which", ["real1d", "real1d-64bit", "realspace"])
def test_noalloc_adjoint_matches_handle_entry_point_on_two_calls(which):
    import torch
    import rimugpu as R
    from rimugpu import _lib
    lib = _lib.load()
    if which == "real1d":             # 17-bit addresses: the 32-bit-word kernel
        h = R.HubbardReal1D(R.BoseFS([1] * 9), u=3.0, t=0.9)
    elif which == "real1d-64bit":     # N=3, M=31: 33-bit addresses on 64-bit words, dim 5456
        h = R.HubbardReal1D(R.BoseFS([1, 0, 1] + [0] * 27 + [1]), u=1.5, t=0.8)
    else:
        h = R.HubbardRealSpace(R.BoseFS([1, 0, 2, 1, 0, 1, 0, 1, 1]), R.PeriodicBoundaries(3, 3),
                               u=[[2.0]], t=[1.1])
    op = R.BasisOperator(h)
    gen = torch.Generator(device="cuda").manual_seed(5)
    for call in range(2):
        v = torch.randn(op.dim, dtype=torch.float64, device="cuda", generator=gen)
        gw = torch.randn(op.dim, dtype=torch.float64, device="cuda", generator=gen)
        gv_ref, gu_ref, gt_ref = op.adjoint(v, gw)
        gv = torch.full_like(v, float("nan"))
        rc, gu, gt = _call_noalloc(lib, h._desc(), v, gw, gv)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        # same kernels, same block count, same fixed-order reduction: identical bits
        a = gv.cpu().numpy().view(np.uint64)
        b = gv_ref.cpu().numpy().view(np.uint64)
        assert np.array_equal(a, b), call
        assert gu == gu_ref and gt == gt_ref, (call, gu, gu_ref, gt, gt_ref)


def test_noalloc_rejects_models_beyond_the_static_limit():
    import torch
    import rimugpu as R
    from rimugpu import _lib
    lib = _lib.load()
    desc = R.HubbardReal1D(R.BoseFS([1] * 4), u=1.0)._desc()
    desc.n_particles, desc.n_modes = 40, 30          # 69-bit addresses: beyond the tables
    v = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc, _, _ = _call_noalloc(lib, desc, v, v, v.clone())
    assert rc == _lib.RIMU_ERR_BADARG
    assert "63" in _lib.last_error()
    small = R.HubbardReal1D(R.BoseFS([1] * 4), u=1.0)._desc()   # dim 35, not 4
    rc, _, _ = _call_noalloc(lib, small, v, v, v.clone())
    assert rc == _lib.RIMU_ERR_BADARG and "dim" in _lib.last_error()
