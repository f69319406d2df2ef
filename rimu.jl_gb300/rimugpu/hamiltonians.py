"""Hamiltonians: the AbstractHamiltonian interface on device-side model handles.

HubbardReal1D (src/Hamiltonians/HubbardReal1D.jl), HubbardRealSpace with one component or a
multi-component CompositeFS (HubbardRealSpace.jl, geometry.jl) and HubbardMom1D with BoseFS or
FermiFS2C (HubbardMom1D.jl).  Matrix
elements are evaluated by librimu_gpu; this module only holds parameters and converts.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .dvec import pack_keys, unpack_keys
from .addresses import BoseFS, CompositeFS, FermiFS, is_fermi2c


class CubicGrid:
    """CubicGrid(dims, fold) (geometry.jl:45-54): `fold[i]` True for periodic boundaries."""

    def __init__(self, dims, fold=None):
        dims = tuple(int(d) for d in dims)
        if any(d <= 1 for d in dims):
            raise ValueError("All dimensions must be at least 2 in size")
        if not 1 <= len(dims) <= 3:
            raise ValueError("1 to 3 dimensions are supported")
        self.dims = dims
        self.fold = tuple(bool(f) for f in fold) if fold is not None else tuple(True for _ in dims)

    def __len__(self):
        return int(np.prod(self.dims))

    def __repr__(self):
        return f"CubicGrid({self.dims}, {self.fold})"


def PeriodicBoundaries(*dims):
    dims = dims[0] if len(dims) == 1 and isinstance(dims[0], tuple) else dims
    return CubicGrid(dims, tuple(True for _ in dims))


def HardwallBoundaries(*dims):
    dims = dims[0] if len(dims) == 1 and isinstance(dims[0], tuple) else dims
    return CubicGrid(dims, tuple(False for _ in dims))


def LadderBoundaries(*dims):
    """First dimension hard-wall, the rest periodic (geometry.jl:87-90)."""
    dims = dims[0] if len(dims) == 1 and isinstance(dims[0], tuple) else dims
    return CubicGrid(dims, tuple(i > 0 for i in range(len(dims))))


def hubbard_dispersion(t, k):
    """-2t cos(k) (HubbardMom1D.jl:7)."""
    return -2 * t * math.cos(k)


def continuum_dispersion(t, k):
    """t k^2 (HubbardMom1D.jl:17)."""
    return t * k ** 2


class AbstractHamiltonian:
    kind = 0

    def __init__(self, address):
        self.address = address
        self._handle = None
        self._keep = []

    # ---- device handle -------------------------------------------------------------
    def _desc(self) -> _lib.ModelDesc:
        raise NotImplementedError

    @property
    def handle(self):
        if self._handle is None:
            lib = _lib.load()
            ctx = _lib.default_context()
            h = C.c_void_p()
            _lib.check(lib.rimu_model_create(ctx.handle, C.byref(self._desc()), C.byref(h)))
            self._handle = h
            self._ctx = ctx
        return self._handle

    def __del__(self):
        try:
            if self._handle is not None:
                _lib.load().rimu_model_destroy(self._handle)
        except Exception:
            pass

    # ---- AbstractHamiltonian interface (Interfaces/hamiltonians.jl:201-421) ----------
    def starting_address(self):
        return self.address

    def LOStructure(self):
        return "IsHermitian"

    @property
    def N(self):
        return self.address.N

    @property
    def M(self):
        return self.address.M

    def _addr(self, key):
        return self.address.with_key(key)

    @property
    def key_words(self) -> int:
        """1 for addresses of at most 64 bits, 2 for two-chunk addresses (65-128 bits)."""
        return 2 if self.address.nbits > 64 else 1

    def diagonal_element(self, address) -> float:
        return float(self.diagonal_elements([address.key])[0])

    def diagonal_elements(self, keys) -> np.ndarray:
        words = pack_keys(keys, self.key_words)
        out = np.zeros(len(keys))
        _lib.check(_lib.load().rimu_model_diagonal(
            self.handle, words.ctypes.data_as(C.POINTER(C.c_uint64)), len(keys),
            out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def num_offdiagonals(self, address) -> int:
        n = C.c_int()
        k2 = pack_keys([address.key], 2)
        _lib.check(_lib.load().rimu_model_num_offdiagonals_w(
            self.handle, k2.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(n)))
        return n.value

    def offdiagonal_keys(self, key: int):
        """(keys, values) of all offdiagonals of column `key`, in the reference's order
        (keys as Python ints for addresses wider than 64 bits)."""
        lib = _lib.load()
        n = C.c_int()
        k2 = pack_keys([key], 2)
        kp = k2.ctypes.data_as(C.POINTER(C.c_uint64))
        _lib.check(lib.rimu_model_num_offdiagonals_w(self.handle, kp, C.byref(n)))
        kw = self.key_words
        ks = np.zeros(max(n.value, 1) * kw, dtype=np.uint64)
        vs = np.zeros(max(n.value, 1))
        got = C.c_int()
        _lib.check(lib.rimu_model_offdiagonals_w(
            self.handle, kp, ks.ctypes.data_as(C.POINTER(C.c_uint64)),
            vs.ctypes.data_as(C.POINTER(C.c_double)), max(n.value, 1), C.byref(got)))
        return unpack_keys(ks[:got.value * kw], kw), vs[:got.value]

    def offdiagonals(self, address):
        """offdiagonals(H, address): list of (address, matrix element)."""
        ks, vs = self.offdiagonal_keys(address.key)
        return [(self._addr(int(k)), float(v)) for k, v in zip(ks, vs)]

    def get_offdiagonal(self, address, chosen: int):
        return self.offdiagonals(address)[chosen - 1]

    def dimension(self) -> int:
        d = C.c_int64()
        _lib.check(_lib.load().rimu_basis_dimension(self.handle, C.byref(d)))
        return d.value


class HubbardReal1D(AbstractHamiltonian):
    """HubbardReal1D(address; u=1.0, t=1.0) (HubbardReal1D.jl:26-29)."""
    kind = _lib.MODEL_REAL1D

    def __init__(self, address: BoseFS, u=1.0, t=1.0):
        if not isinstance(address, BoseFS):
            raise TypeError("HubbardReal1D needs a BoseFS address")
        super().__init__(address)
        self.u, self.t = float(u), float(t)

    def _desc(self):
        d = _lib.ModelDesc()
        d.kind, d.fermion, d.n_particles, d.n_modes = self.kind, 0, self.N, self.M
        d.u, d.t, d.ndim = self.u, self.t, 1
        d.dims[0], d.periodic[0] = self.M, 1
        return d

    def with_params(self, u=None, t=None):
        return HubbardReal1D(self.address, self.u if u is None else u, self.t if t is None else t)

    def __repr__(self):
        return f"HubbardReal1D({self.address}; u={self.u}, t={self.t})"


def _trap_potential(dims, vrow):
    """Trap energy per site for one component: sum_d v[d] * x_d^2 with x_d centred on the
    grid (HubbardRealSpace.jl:214-226; sites in linear order, first dimension fastest)."""
    ranges = [[-(Md // 2) + i for i in range(Md)] for Md in dims]
    pot = []
    for lin in range(int(np.prod(dims))):
        rem, acc = lin, None
        for d, Md in enumerate(dims):
            x = ranges[d][rem % Md]
            rem //= Md
            term = vrow[d] * (x ** 2)
            acc = term if acc is None else acc + term
        pot.append(acc)
    return np.array(pot, dtype=np.float64)


class HubbardRealSpace(AbstractHamiltonian):
    """HubbardRealSpace(address; geometry, t, u, v) (HubbardRealSpace.jl:182-231) with a
    BoseFS/FermiFS address or a CompositeFS of C = 2..4 components.  One component: `t` and `u`
    scalars or 1-element sequences.  C components: `t` of length C, `u` a symmetric C x C
    matrix (defaults all ones), `v` a C x D matrix of trap strengths."""
    kind = _lib.MODEL_REALSPACE

    def __init__(self, address, geometry: CubicGrid | None = None, t=None, u=None, v=None):
        if not isinstance(address, (BoseFS, FermiFS, CompositeFS)):
            raise TypeError("HubbardRealSpace needs a BoseFS, FermiFS or CompositeFS address")
        super().__init__(address)
        self.geometry = geometry if geometry is not None else PeriodicBoundaries(address.M)
        if len(self.geometry) != address.M:
            raise ValueError("`geometry` does not have the correct number of sites")
        D = len(self.geometry.dims)
        self.ncomp = len(address.components) if isinstance(address, CompositeFS) else 1
        C_ = self.ncomp
        tv = np.ravel(np.asarray(1.0 if t is None else t, dtype=float))
        um = np.asarray(1.0 if u is None else u, dtype=float)
        if C_ == 1:
            self.t = float(tv[0])
            self.u = float(np.ravel(um)[0])
            self.v = None if v is None or not np.any(v) else np.ravel(np.asarray(v, dtype=float))
            self.potential = None if self.v is None else _trap_potential(self.geometry.dims, self.v)
            return
        if t is not None and tv.size != C_:
            raise ValueError(f"`t` must be a vector of length {C_}")
        self.t = tuple(float(x) for x in (tv if tv.size == C_ else np.ones(C_)))
        if u is not None and um.size != C_ * C_:
            raise ValueError(f"`u` must be a {C_} × {C_} matrix")
        um = um.reshape(C_, C_) if um.size == C_ * C_ else np.ones((C_, C_))
        if not np.array_equal(um, um.T):
            raise ValueError("`u` must be symmetric")
        self.u = um
        vm = None if v is None else np.asarray(v, dtype=float)
        if vm is not None and vm.size != C_ * D:
            raise ValueError(f"`v` must be a {C_} × {D} matrix")
        self.v = None if vm is None or not np.any(vm) else vm.reshape(C_, D)
        self.potential = None
        if self.v is not None:
            self.potential = np.concatenate([_trap_potential(self.geometry.dims, self.v[c])
                                             for c in range(C_)])

    def _desc(self):
        d = _lib.ModelDesc()
        d.kind, d.n_particles, d.n_modes = self.kind, self.N, self.M
        g = self.geometry
        d.ndim = len(g.dims)
        for i in range(3):
            d.dims[i] = g.dims[i] if i < len(g.dims) else 1
            d.periodic[i] = int(g.fold[i]) if i < len(g.dims) else 1
        if self.ncomp == 1:
            d.fermion = 1 if isinstance(self.address, FermiFS) else 0
            d.u, d.t = self.u, self.t
        else:
            d.fermion = 0
            d.n_components = self.ncomp
            d.u, d.t = float(self.u[0, 0]), self.t[0]
            for c, comp in enumerate(self.address.components):
                d.comp_fermion[c] = 1 if isinstance(comp, FermiFS) else 0
                d.comp_particles[c] = comp.N
                d.comp_t[c] = self.t[c]
            # the upper triangle of u, row by row
            upper = [self.u[i, j] for i in range(self.ncomp) for j in range(i, self.ncomp)]
            for i, x in enumerate(upper):
                d.comp_u[i] = float(x)
        if self.potential is not None:
            arr = np.ascontiguousarray(self.potential)
            self._keep.append(arr)
            d.potential = arr.ctypes.data_as(C.POINTER(C.c_double))
        return d

    def dimension(self) -> int:
        if self.ncomp == 1:
            return super().dimension()
        return math.prod(_component_dimension(c) for c in self.address.components)

    def with_params(self, u=None, t=None):
        return HubbardRealSpace(self.address, self.geometry, self.t if t is None else t,
                                self.u if u is None else u, self.v)

    def __repr__(self):
        return f"HubbardRealSpace({self.address}; geometry={self.geometry}, t={self.t}, u={self.u})"


def _component_dimension(c) -> int:
    """number_conserving_dimension of one component: C(N+M-1, N) or C(M, N)."""
    return math.comb(c.M, c.N) if isinstance(c, FermiFS) else math.comb(c.N + c.M - 1, c.N)


class HubbardMom1D(AbstractHamiltonian):
    """HubbardMom1D(address; u=1.0, t=1.0, dispersion=hubbard_dispersion) with a BoseFS or a
    FermiFS2C address (HubbardMom1D.jl:49-65, 141-205)."""
    kind = _lib.MODEL_MOM1D

    def __init__(self, address, u=1.0, t=1.0, dispersion=hubbard_dispersion):
        if not (isinstance(address, BoseFS) or is_fermi2c(address)):
            raise TypeError("HubbardMom1D is supported with BoseFS and FermiFS2C addresses")
        super().__init__(address)
        self.u, self.t = float(u), float(t)
        M = address.M
        step = 2 * math.pi / M
        start = (-math.pi * (1 + 1 / M) + step) if M % 2 == 1 else (-math.pi + step)
        self.ks = np.array([start + i * step for i in range(M)])
        self.kes = np.array([dispersion(self.t, k) for k in self.ks], dtype=np.float64)

    def _desc(self):
        d = _lib.ModelDesc()
        d.kind, d.fermion, d.n_particles, d.n_modes = self.kind, 0, self.N, self.M
        d.u, d.t, d.ndim = self.u, self.t, 1
        d.dims[0], d.periodic[0] = self.M, 1
        if isinstance(self.address, CompositeFS):
            d.n_components = 2
            for c, comp in enumerate(self.address.components):
                d.comp_fermion[c] = 1
                d.comp_particles[c] = comp.N
        arr = np.ascontiguousarray(self.kes)
        self._keep.append(arr)
        d.dispersion = arr.ctypes.data_as(C.POINTER(C.c_double))
        return d

    def dimension(self) -> int:
        if isinstance(self.address, CompositeFS):
            return math.prod(_component_dimension(c) for c in self.address.components)
        return super().dimension()

    def __repr__(self):
        return f"HubbardMom1D({self.address}; u={self.u}, t={self.t})"
