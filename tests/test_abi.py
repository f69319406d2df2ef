"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/rimu_gpu.h declares (no compute call: runs without a GPU)."""
import ctypes
import os
import re

import pytest

import rimugpu
from rimugpu import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rimu_gpu.h")).read()
    return sorted(set(re.findall(r"^int\s+(rimu_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_bound_entry_points():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.load().__dict__["_name"])
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version_and_error_string_without_gpu():
    lib = _lib.load()
    assert lib.rimu_version() >= 10000
    buf = ctypes.create_string_buffer(64)
    assert lib.rimu_last_error(buf, 64) == 0


def test_bad_arguments_fail_loudly_without_touching_the_gpu():
    lib = _lib.load()
    # NULL handles are rejected with RIMU_ERR_BADARG before any CUDA call
    assert lib.rimu_apply_operator(None, None, None, None, None, None) == _lib.RIMU_ERR_BADARG
    assert "NULL" in _lib.last_error()
    assert lib.rimu_vec_length(None, None) == _lib.RIMU_ERR_BADARG


def test_address_encoding_matches_reference_layout():
    b = rimugpu.BoseFS(1, 0, 2)        # bits: mode1 '1', sep, mode2 sep, mode3 '11'
    assert b.key == 0b11001 and b.onr() == (1, 0, 2)
    assert rimugpu.BoseFS.from_key(b.key, 3, 3) == b
    f = rimugpu.FermiFS(1, 1, 0, 1)
    assert f.key == 0b1011 and f.onr() == (1, 1, 0, 1)
    assert rimugpu.near_uniform(rimugpu.BoseFS, 7, 5).onr() == (2, 2, 1, 1, 1)
    assert sorted([rimugpu.BoseFS(0, 2), rimugpu.BoseFS(2, 0), rimugpu.BoseFS(1, 1)])[0].onr() == (2, 0)


def test_host_address_encoding_agrees_with_oracle():
    import numpy as np
    import oracle as O
    rng = np.random.default_rng(2)
    for N, M in ((6, 6), (20, 20), (10, 20), (3, 30)):
        for _ in range(20):
            onr = np.bincount(rng.integers(0, M, N), minlength=M).tolist()
            assert rimugpu.BoseFS(onr).key == O.bose_key(onr)


def test_blocking_analysis_on_correlated_series():
    import numpy as np
    rng = np.random.default_rng(0)
    x = np.convolve(rng.normal(size=2 ** 14 + 63), np.ones(64) / 64, mode="valid")
    r = rimugpu.blocking_analysis(x)
    assert r.k > 1 and r.err > np.std(x) / np.sqrt(len(x))


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the ABI structs have the size and field offsets of the C
    declarations in include/rimu_gpu.h (compiled with the host C compiler)."""
    import ctypes as C
    import shutil
    import subprocess
    from rimugpu import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    pairs = [("rimu_model_desc", _lib.ModelDesc), ("rimu_step_params", _lib.StepParams),
             ("rimu_step_stats", _lib.StepStats), ("rimu_batch_params", _lib.BatchParams),
             ("rimu_batch_stats", _lib.BatchStats)]
    lines = ['#include <stdio.h>', '#include "rimu_gpu.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c99", "-I", inc, str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, val = ln.split()
        got[(name, field)] = int(val)
    for cname, py in pairs:
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_noalloc_adjoint_rejects_bad_descriptors_before_any_cuda_call():
    """rimu_hv_basis_adjoint_noalloc repeats rimu_model_create's checks on the plain
    description: every lattice extent at least 2 (an extent of 1 or a negative pair whose
    product is n_modes would let neighbour sites leave the lattice) and no FermiFS flag on a
    bosonic model.  All are rejected before the library touches a GPU."""
    import ctypes as C
    import numpy as np
    lib = _lib.load()
    buf = np.zeros(8)
    p = C.c_void_p(buf.ctypes.data)
    gu, gt = C.c_double(), C.c_double()

    def call(desc, dim):
        return lib.rimu_hv_basis_adjoint_noalloc(C.byref(desc), p, p, p, C.byref(gu),
                                                 C.byref(gt), dim, None)

    h = rimugpu.HubbardRealSpace(rimugpu.BoseFS([1, 0, 1, 0, 1, 0]), rimugpu.PeriodicBoundaries(2, 3))
    for dims in ((1, 6), (-2, -3), (6, 1)):
        d = h._desc()
        d.dims[0], d.dims[1] = dims
        assert call(d, 56) == _lib.RIMU_ERR_BADARG, dims
        assert "at least 2" in _lib.last_error()
    d = rimugpu.HubbardReal1D(rimugpu.BoseFS([1] * 4), u=1.0)._desc()
    d.fermion = 1
    assert call(d, 35) == _lib.RIMU_ERR_BADARG
    assert "bosonic" in _lib.last_error()
