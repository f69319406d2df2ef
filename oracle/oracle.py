"""ctypes front end of the CPU oracle (rimu_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
``bench.py``'s CPU-baseline leg as the checker.  The product package never imports it.

The C restatement follows the Rimu.jl hot path (file:line citations are in the C source).
This module adds exact diagonalisation helpers (scipy) used to pin the oracle against the
reference's published energies.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "librimu_oracle.so")
SRC = os.path.join(HERE, "rimu_oracle.c")

REAL1D, REALSPACE, MOM1D = 1, 2, 3
STYLE_INTEGER, STYLE_DETERMINISTIC, STYLE_DSS = 0, 1, 2
OP_TRANSITION, OP_HAMILTONIAN = 0, 1


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, so float results are portable)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
               "-o", LIB, SRC, "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


MAXC = 4   # O_MAXC: components of a CompositeFS


class _OModel(C.Structure):
    _fields_ = [("kind", C.c_int), ("fermion", C.c_int), ("N", C.c_int), ("M", C.c_int),
                ("u", C.c_double), ("t", C.c_double), ("ndim", C.c_int),
                ("dims", C.c_int * 3), ("periodic", C.c_int * 3),
                ("pot", C.POINTER(C.c_double)), ("kes", C.POINTER(C.c_double)),
                ("ncomp", C.c_int), ("cferm", C.c_int * MAXC), ("cN", C.c_int * MAXC),
                ("ct", C.c_double * MAXC), ("cu", C.c_double * (MAXC * (MAXC + 1) // 2))]


class _OParams(C.Structure):
    _fields_ = [("style", C.c_int), ("op", C.c_int), ("dt", C.c_double), ("shift", C.c_double),
                ("boost", C.c_double), ("proj_threshold", C.c_double),
                ("compression", C.c_double), ("rel_threshold", C.c_double),
                ("abs_threshold", C.c_double), ("seed", C.c_uint64), ("step", C.c_uint32),
                ("replica", C.c_uint32), ("init_rule", C.c_int), ("init_threshold", C.c_double)]


class _OStats(C.Structure):
    _fields_ = [("norm", C.c_double), ("len", C.c_int64), ("len_before", C.c_int64),
                ("exact_steps", C.c_int64), ("inexact_steps", C.c_int64),
                ("spawn_attempts", C.c_int64), ("spawns", C.c_double),
                ("clones", C.c_int64), ("deaths", C.c_int64), ("zombies", C.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.POINTER
        u64p, f64p, i64p = P(C.c_uint64), P(C.c_double), P(C.c_int64)
        _lib.o_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        _lib.o_draw.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64,
                                C.c_uint32, P(C.c_uint32)]
        _lib.o_bose_from_onr.argtypes = [P(C.c_int), C.c_int]
        _lib.o_bose_from_onr.restype = C.c_uint64
        _lib.o_bose_to_onr.argtypes = [C.c_uint64, C.c_int, P(C.c_int)]
        _lib.o_fermi_from_onr.argtypes = [P(C.c_int), C.c_int]
        _lib.o_fermi_from_onr.restype = C.c_uint64
        _lib.o_num_offdiagonals.argtypes = [P(_OModel), C.c_uint64]
        _lib.o_get_offdiagonal.argtypes = [P(_OModel), C.c_uint64, C.c_int, u64p, f64p]
        _lib.o_diagonal.argtypes = [P(_OModel), C.c_uint64]
        _lib.o_diagonal.restype = C.c_double
        _lib.o_step.argtypes = [P(_OModel), P(_OParams), u64p, f64p, i64p, C.c_int64,
                                P(u64p), P(f64p), P(i64p), i64p, P(_OStats)]
        _lib.o_free.argtypes = [C.c_void_p]
        _lib.o_hv_basis.argtypes = [P(_OModel), u64p, C.c_int64, f64p, f64p]
        _lib.o_hv_basis.restype = C.c_int64
        _lib.o_hv_basis_adjoint.argtypes = [P(_OModel), u64p, C.c_int64, f64p, f64p, f64p,
                                            f64p, f64p]
        _lib.o_hv_basis_adjoint.restype = C.c_int64
        _lib.o_count_nnz.argtypes = [P(_OModel), u64p, C.c_int64]
        _lib.o_count_nnz.restype = C.c_int64
        _lib.o_build_coo.argtypes = [P(_OModel), u64p, C.c_int64, i64p, i64p, f64p, i64p]
        _lib.o_enumerate_fixed_weight.argtypes = [C.c_int, C.c_int, u64p, C.c_int64]
        _lib.o_enumerate_fixed_weight.restype = C.c_int64
        _lib.o_connected_basis.argtypes = [P(_OModel), C.c_uint64, u64p, C.c_int64]
        _lib.o_connected_basis.restype = C.c_int64
        # addresses of up to 128 bits as (lo, hi) word pairs
        _lib.o_num_offdiagonals_w.argtypes = [P(_OModel), C.c_uint64, C.c_uint64]
        _lib.o_get_offdiagonal_w.argtypes = [P(_OModel), C.c_uint64, C.c_uint64, C.c_int, u64p, f64p]
        _lib.o_diagonal_w.argtypes = [P(_OModel), C.c_uint64, C.c_uint64]
        _lib.o_diagonal_w.restype = C.c_double
        _lib.o_step_w.argtypes = [P(_OModel), P(_OParams), u64p, f64p, i64p, C.c_int64,
                                  P(u64p), P(f64p), P(i64p), i64p, P(_OStats)]
        _lib.o_step_mt.argtypes = [P(_OModel), P(_OParams), u64p, f64p, i64p, C.c_int64, C.c_int,
                                   C.c_int64, C.c_int, P(u64p), P(f64p), P(i64p), i64p, P(_OStats)]
        _lib.o_real1d_bits_offdiag.argtypes = [P(_OModel), C.c_uint64, C.c_int, u64p, f64p]
        _lib.o_real1d_bits_diagonal.argtypes = [P(_OModel), C.c_uint64]
        _lib.o_real1d_bits_diagonal.restype = C.c_double
        _lib.o_to_fixed_agree.argtypes = [C.c_double]
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


# ----------------------------------------------------------------------------------------
# Models (plain descriptions; the same fields drive the GPU library)
# ----------------------------------------------------------------------------------------
@dataclass
class Model:
    kind: int
    N: int
    M: int
    u: float = 1.0
    t: float = 1.0
    fermion: bool = False
    dims: tuple = ()
    periodic: tuple = ()
    pot: np.ndarray | None = None
    kes: np.ndarray | None = None
    # C >= 2 components (CompositeFS / FermiFS2C): per-component fermion flags, particle
    # numbers, HubbardRealSpace hoppings and the interactions (upper triangle of u, row by row)
    comps: tuple = ()
    ct: tuple = (1.0, 1.0)
    cu: tuple = (0.0, 0.0, 0.0)
    _keep: list = field(default_factory=list, repr=False)

    def struct(self) -> _OModel:
        m = _OModel()
        m.kind, m.fermion, m.N, m.M = self.kind, int(self.fermion), self.N, self.M
        m.u, m.t = float(self.u), float(self.t)
        dims = self.dims or (self.M,)
        per = self.periodic or tuple(True for _ in dims)
        m.ndim = len(dims)
        for i in range(3):
            m.dims[i] = dims[i] if i < len(dims) else 1
            m.periodic[i] = int(per[i]) if i < len(per) else 1
        if self.pot is not None:
            arr = np.ascontiguousarray(self.pot, dtype=np.float64)
            self._keep.append(arr)
            m.pot = _p(arr, C.c_double)
        if self.kes is not None:
            arr = np.ascontiguousarray(self.kes, dtype=np.float64)
            self._keep.append(arr)
            m.kes = _p(arr, C.c_double)
        m.ncomp = len(self.comps) if self.comps else 1
        for c, (ferm, n) in enumerate(self.comps):
            m.cferm[c], m.cN[c] = int(ferm), int(n)
        for c, x in enumerate(self.ct):
            m.ct[c] = float(x)
        for i, x in enumerate(self.cu):
            m.cu[i] = float(x)
        return m

    def comp_bits(self, c: int) -> int:
        ferm, n = self.comps[c]
        return self.M if ferm else n + self.M - 1

    @property
    def nbits(self) -> int:
        if self.comps:
            return sum(self.comp_bits(c) for c in range(len(self.comps)))
        return self.M if self.fermion else self.N + self.M - 1


def mom1d_kes(M: int, t: float) -> np.ndarray:
    """Dispersion -2t cos(k) on the grid of HubbardMom1D.jl:49-65 (Python floats are IEEE
    doubles; range(start; step, length) is start + i*step)."""
    import math
    step = 2 * math.pi / M
    start = (-math.pi * (1 + 1 / M) + step) if M % 2 == 1 else (-math.pi + step)
    return np.array([-2 * t * math.cos(start + i * step) for i in range(M)])


def real1d(N, M, u=1.0, t=1.0):
    return Model(REAL1D, N, M, u, t)


def realspace(N, dims, u=1.0, t=1.0, periodic=None, fermion=False, pot=None):
    M = int(np.prod(dims))
    periodic = periodic if periodic is not None else tuple(True for _ in dims)
    return Model(REALSPACE, N, M, u, t, fermion, tuple(dims), tuple(periodic), pot)


def mom1d(N, M, u=1.0, t=1.0):
    return Model(MOM1D, N, M, u, t, kes=mom1d_kes(M, t))


def realspace_multi(comps, dims, t=None, u=None, periodic=None, pot=None):
    """HubbardRealSpace with a CompositeFS of C = len(comps) components (2..4): `comps` =
    ((fermion, N), ...) in component order; `t` the C hoppings (default ones); `u` the
    symmetric C x C interaction matrix (default ones); `pot` (C, M) or None."""
    Cn = len(comps)
    M = int(np.prod(dims))
    periodic = periodic if periodic is not None else tuple(True for _ in dims)
    u = np.ones((Cn, Cn)) if u is None else np.asarray(u, dtype=float).reshape(Cn, Cn)
    t = tuple(1.0 for _ in range(Cn)) if t is None else tuple(float(x) for x in t)
    p = None if pot is None else np.ascontiguousarray(np.ravel(np.asarray(pot, dtype=float)))
    N = sum(n for _, n in comps)
    return Model(REALSPACE, N, M, 0.0, 0.0, False, tuple(dims), tuple(periodic), p,
                 comps=tuple((bool(f), int(n)) for f, n in comps), ct=t,
                 cu=tuple(u[i, j] for i in range(Cn) for j in range(i, Cn)))


def realspace2(comps, dims, t=(1.0, 1.0), u=((1.0, 1.0), (1.0, 1.0)), periodic=None, pot=None):
    """HubbardRealSpace with a two-component CompositeFS (realspace_multi with C = 2)."""
    return realspace_multi(comps, dims, t=t, u=u, periodic=periodic, pot=pot)


def mom1d_2c(N1, N2, M, u=1.0, t=1.0):
    """HubbardMom1D with a FermiFS2C address of N1 and N2 fermions in M modes."""
    return Model(MOM1D, N1 + N2, M, u, t, kes=mom1d_kes(M, t), comps=((True, N1), (True, N2)))


# ----------------------------------------------------------------------------------------
# Address helpers
# ----------------------------------------------------------------------------------------
def bose_key(onr) -> int:
    if sum(onr) + len(onr) - 1 > 64:     # two chunks: the same encoding on a Python int
        key = 0
        for n in reversed(list(onr)):
            key = (key << (n + 1)) | ((1 << n) - 1)
        return key
    a = np.ascontiguousarray(onr, dtype=np.int32)
    return int(lib().o_bose_from_onr(_p(a, C.c_int), len(a)))


_M64 = (1 << 64) - 1


def _wide(m: "Model") -> bool:
    return m.nbits > 64


def _split(key: int):
    key = int(key)
    return C.c_uint64(key & _M64), C.c_uint64(key >> 64)


def bose_onr(key: int, M: int) -> list:
    a = np.zeros(M, dtype=np.int32)
    lib().o_bose_to_onr(C.c_uint64(key), M, _p(a, C.c_int))
    return a.tolist()


def fermi_key(onr) -> int:
    a = np.ascontiguousarray(onr, dtype=np.int32)
    return int(lib().o_fermi_from_onr(_p(a, C.c_int), len(a)))


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().o_philox4x32_10(c, k, o)
    return list(o)


def draw(seed, purpose, replica, step, addr, j):
    o = (C.c_uint32 * 4)()
    lib().o_draw(seed, purpose, replica, step, addr, j, o)
    return list(o)


# ----------------------------------------------------------------------------------------
# Operator interface
# ----------------------------------------------------------------------------------------
def num_offdiagonals(m: Model, key: int) -> int:
    s = m.struct()
    if _wide(m):
        return lib().o_num_offdiagonals_w(C.byref(s), *_split(key))
    return lib().o_num_offdiagonals(C.byref(s), C.c_uint64(key))


def offdiagonals(m: Model, key: int):
    s = m.struct()
    out = []
    if _wide(m):
        n = lib().o_num_offdiagonals_w(C.byref(s), *_split(key))
        for c in range(1, n + 1):
            nk, hv = (C.c_uint64 * 2)(), C.c_double()
            lib().o_get_offdiagonal_w(C.byref(s), *_split(key), c, nk, C.byref(hv))
            out.append((int(nk[0]) | (int(nk[1]) << 64), float(hv.value)))
        return out
    n = lib().o_num_offdiagonals(C.byref(s), C.c_uint64(key))
    for c in range(1, n + 1):
        nk, hv = C.c_uint64(), C.c_double()
        lib().o_get_offdiagonal(C.byref(s), C.c_uint64(key), c, C.byref(nk), C.byref(hv))
        out.append((int(nk.value), float(hv.value)))
    return out


def diagonal(m: Model, key: int) -> float:
    s = m.struct()
    if _wide(m):
        return float(lib().o_diagonal_w(C.byref(s), *_split(key)))
    return float(lib().o_diagonal(C.byref(s), C.c_uint64(key)))


# ----------------------------------------------------------------------------------------
# FCIQMC step
# ----------------------------------------------------------------------------------------
INIT_NONE, INIT_INITIATOR, INIT_SIMPLE, INIT_COHERENT = 0, 1, 2, 3


@dataclass
class StepParams:
    style: int
    dt: float = 0.01
    shift: float = 0.0
    seed: int = 0
    step: int = 0
    op: int = OP_TRANSITION
    boost: float = 1.0
    proj_threshold: float = 0.0
    compression: float = 0.0
    rel_threshold: float = 1.0
    abs_threshold: float = float("inf")
    replica: int = 0
    init_rule: int = 0           # INIT_*: initiator rule (initiators.jl:132-234)
    init_threshold: float = 1.0

    def struct(self) -> _OParams:
        p = _OParams()
        p.style, p.op, p.dt, p.shift = self.style, self.op, self.dt, self.shift
        p.boost, p.proj_threshold, p.compression = self.boost, self.proj_threshold, self.compression
        p.rel_threshold, p.abs_threshold = self.rel_threshold, self.abs_threshold
        p.seed, p.step, p.replica = self.seed, self.step, self.replica
        p.init_rule, p.init_threshold = self.init_rule, self.init_threshold
        return p


def step(m: Model, prm: StepParams, keys, vals):
    """One projector step; returns (sorted keys, values, stats dict).  Addresses wider than 64
    bits are Python ints in and out (object arrays)."""
    if _wide(m):
        return _step_wide(m, prm, keys, vals)
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    n = len(keys)
    is_int = prm.style == STYLE_INTEGER
    fv = np.ascontiguousarray(vals if not is_int else np.zeros(n), dtype=np.float64)
    iv = np.ascontiguousarray(vals if is_int else np.zeros(n), dtype=np.int64)
    ok, ov, oi = C.POINTER(C.c_uint64)(), C.POINTER(C.c_double)(), C.POINTER(C.c_int64)()
    on = C.c_int64()
    st = _OStats()
    ms, ps = m.struct(), prm.struct()
    rc = lib().o_step(C.byref(ms), C.byref(ps), _p(keys, C.c_uint64), _p(fv, C.c_double),
                      _p(iv, C.c_int64), n, C.byref(ok), C.byref(ov), C.byref(oi),
                      C.byref(on), C.byref(st))
    if rc != 0:
        raise MemoryError("oracle step failed")
    k = np.ctypeslib.as_array(ok, shape=(on.value,)).copy() if on.value else np.zeros(0, np.uint64)
    if is_int:
        v = np.ctypeslib.as_array(oi, shape=(on.value,)).copy() if on.value else np.zeros(0, np.int64)
    else:
        v = np.ctypeslib.as_array(ov, shape=(on.value,)).copy() if on.value else np.zeros(0)
    for p in (ok, ov, oi):
        lib().o_free(C.cast(p, C.c_void_p))
    stats = {f: getattr(st, f) for f, _ in _OStats._fields_}
    return k, v, stats


def step_mt(m: Model, prm: StepParams, keys, vals, threads: int = 0, mem_budget: float = 8e9,
            sort: bool = True, bits: bool = False):
    """One projector step on `threads` host threads (0: all), restating the PDVec step
    (perform_spawns!, collect_local!, move_and_compress!, pdworkingmemory.jl:191-309).  Same
    results as step(); the output is sorted only when `sort`.  Contributions beyond
    `mem_budget` bytes are processed in passes.  With `bits`, HubbardReal1D columns use the
    reference's bit-level algorithms instead of occupation-number arrays (same results,
    faster).  Addresses of at most 64 bits, no initiator rule."""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    n = len(keys)
    is_int = prm.style == STYLE_INTEGER
    fv = np.ascontiguousarray(vals if not is_int else np.zeros(n), dtype=np.float64)
    iv = np.ascontiguousarray(vals if is_int else np.zeros(n), dtype=np.int64)
    ok, ov, oi = C.POINTER(C.c_uint64)(), C.POINTER(C.c_double)(), C.POINTER(C.c_int64)()
    on = C.c_int64()
    st = _OStats()
    ms, ps = m.struct(), prm.struct()
    rc = lib().o_step_mt(C.byref(ms), C.byref(ps), _p(keys, C.c_uint64), _p(fv, C.c_double),
                         _p(iv, C.c_int64), n, int(threads), int(mem_budget), int(bits), C.byref(ok),
                         C.byref(ov), C.byref(oi), C.byref(on), C.byref(st))
    if rc == 2:
        raise ValueError("step_mt: needs addresses of at most 64 bits and no initiator rule")
    if rc != 0:
        raise MemoryError("oracle step failed")
    nn = on.value
    k = np.ctypeslib.as_array(ok, shape=(nn,)).copy() if nn else np.zeros(0, np.uint64)
    if is_int:
        v = np.ctypeslib.as_array(oi, shape=(nn,)).copy() if nn else np.zeros(0, np.int64)
    else:
        v = np.ctypeslib.as_array(ov, shape=(nn,)).copy() if nn else np.zeros(0)
    for p in (ok, ov, oi):
        lib().o_free(C.cast(p, C.c_void_p))
    if sort:
        order = np.argsort(k, kind="stable")
        k, v = k[order], v[order]
    stats = {f: getattr(st, f) for f, _ in _OStats._fields_}
    return k, v, stats


def real1d_bits_offdiagonals(m: Model, key: int):
    """Offdiagonals of a HubbardReal1D column by the bit-level path of the threaded step."""
    s = m.struct()
    out = []
    for c in range(1, num_offdiagonals(m, key) + 1):
        nk, hv = C.c_uint64(), C.c_double()
        lib().o_real1d_bits_offdiag(C.byref(s), C.c_uint64(key), c, C.byref(nk), C.byref(hv))
        out.append((int(nk.value), float(hv.value)))
    return out


def real1d_bits_diagonal(m: Model, key: int) -> float:
    return float(lib().o_real1d_bits_diagonal(C.byref(m.struct()), C.c_uint64(key)))


def _step_wide(m: Model, prm: StepParams, keys, vals):
    n = len(keys)
    k2 = np.zeros(2 * max(n, 1), dtype=np.uint64)
    for i, k in enumerate(keys):
        k2[2 * i], k2[2 * i + 1] = int(k) & _M64, int(k) >> 64
    is_int = prm.style == STYLE_INTEGER
    fv = np.ascontiguousarray(vals if not is_int else np.zeros(n), dtype=np.float64)
    iv = np.ascontiguousarray(vals if is_int else np.zeros(n), dtype=np.int64)
    ok, ov, oi = C.POINTER(C.c_uint64)(), C.POINTER(C.c_double)(), C.POINTER(C.c_int64)()
    on = C.c_int64()
    st = _OStats()
    ms, ps = m.struct(), prm.struct()
    rc = lib().o_step_w(C.byref(ms), C.byref(ps), _p(k2, C.c_uint64), _p(fv, C.c_double),
                        _p(iv, C.c_int64), n, C.byref(ok), C.byref(ov), C.byref(oi),
                        C.byref(on), C.byref(st))
    if rc != 0:
        raise MemoryError("oracle step failed")
    nn = on.value
    w = np.ctypeslib.as_array(ok, shape=(2 * nn,)).copy() if nn else np.zeros(0, np.uint64)
    k = np.array([int(w[2 * i]) | (int(w[2 * i + 1]) << 64) for i in range(nn)], dtype=object)
    if is_int:
        v = np.ctypeslib.as_array(oi, shape=(nn,)).copy() if nn else np.zeros(0, np.int64)
    else:
        v = np.ctypeslib.as_array(ov, shape=(nn,)).copy() if nn else np.zeros(0)
    for p in (ok, ov, oi):
        lib().o_free(C.cast(p, C.c_void_p))
    stats = {f: getattr(st, f) for f, _ in _OStats._fields_}
    return k, v, stats


# ----------------------------------------------------------------------------------------
# Full-basis products and exact diagonalisation
# ----------------------------------------------------------------------------------------
def _fixed_weight(B, w):
    n = lib().o_enumerate_fixed_weight(B, w, None, 0)
    out = np.zeros(n, dtype=np.uint64)
    lib().o_enumerate_fixed_weight(B, w, _p(out, C.c_uint64), n)
    return out


def basis(m: Model) -> np.ndarray:
    """All addresses with the model's particle numbers, in increasing order (build_basis,
    basis_fock.jl:12-36); for two components the product of the component bases."""
    if m.comps:
        out = _fixed_weight(m.comp_bits(0), m.comps[0][1])
        for c in range(1, len(m.comps)):
            bc = _fixed_weight(m.comp_bits(c), m.comps[c][1])
            out = ((out[:, None] << np.uint64(m.comp_bits(c))) | bc[None, :]).ravel()
        return out
    return _fixed_weight(m.nbits, m.N)


def hv_basis(m: Model, keys, v):
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    w = np.zeros_like(v)
    s = m.struct()
    missing = lib().o_hv_basis(C.byref(s), _p(keys, C.c_uint64), len(keys), _p(v, C.c_double),
                               _p(w, C.c_double))
    assert missing == 0
    return w


def hv_basis_adjoint(m: Model, keys, v, gw):
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    gw = np.ascontiguousarray(gw, dtype=np.float64)
    gv = np.zeros_like(v)
    gu, gt = C.c_double(), C.c_double()
    s = m.struct()
    missing = lib().o_hv_basis_adjoint(C.byref(s), _p(keys, C.c_uint64), len(keys),
                                       _p(v, C.c_double), _p(gw, C.c_double),
                                       _p(gv, C.c_double), C.byref(gu), C.byref(gt))
    assert missing == 0
    return gv, gu.value, gt.value


def sparse_matrix(m: Model, keys=None):
    import scipy.sparse as sp
    keys = basis(m) if keys is None else np.ascontiguousarray(keys, dtype=np.uint64)
    s = m.struct()
    nnz = lib().o_count_nnz(C.byref(s), _p(keys, C.c_uint64), len(keys))
    rows = np.zeros(nnz, np.int64)
    cols = np.zeros(nnz, np.int64)
    vals = np.zeros(nnz)
    z = C.c_int64()
    rc = lib().o_build_coo(C.byref(s), _p(keys, C.c_uint64), len(keys), _p(rows, C.c_int64),
                           _p(cols, C.c_int64), _p(vals, C.c_double), C.byref(z))
    assert rc == 0
    n = z.value
    return sp.csr_matrix((vals[:n], (rows[:n], cols[:n])), shape=(len(keys), len(keys)))


def connected_basis(m: Model, start: int, cap: int = 1 << 22) -> np.ndarray:
    """Sorted basis of the block reachable from `start` (the reference's
    build_basis(H, address))."""
    s = m.struct()
    out = np.zeros(cap, dtype=np.uint64)
    n = lib().o_connected_basis(C.byref(s), C.c_uint64(start), _p(out, C.c_uint64), cap)
    if n < 0 or n > cap:
        raise MemoryError("connected basis larger than cap")
    return out[:n].copy()


def ground_energy(m: Model, start: int | None = None) -> float:
    """Exact ground-state energy (dense eigvalsh for small bases, Lanczos otherwise), on the
    full basis or on the block connected to `start`."""
    keys = basis(m) if start is None else connected_basis(m, start)
    H = sparse_matrix(m, keys)
    if H.shape[0] <= 3000:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    import scipy.sparse.linalg as sla
    vals = sla.eigsh(H, k=1, which="SA", tol=1e-12, maxiter=20000)[0]
    return float(vals[0])
