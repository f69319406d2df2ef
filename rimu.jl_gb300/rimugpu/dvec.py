"""Device-resident walker list (the DVec/PDVec replacement) and apply_operator!.

GPUDVec implements the AbstractDVec interface of src/Interfaces/dictvectors.jl:40 over a
librimu_gpu vector handle; GPUWorkingMemory stands behind working_memory (dictvectors.jl:87)
and apply_operator (dictvectors.jl:112-140) performs one projector step on the GPU.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .addresses import BoseFS
from .initiators import initiator_rule
from .styles import IsDeterministic, IsDynamicSemistochastic, StochasticStyle, default_style


_M64 = (1 << 64) - 1


def pack_keys(keys, kw: int) -> np.ndarray:
    """Addresses as the C ABI takes them: uint64 words, (lo, hi) pairs when kw == 2."""
    if kw == 1:
        return np.ascontiguousarray(keys, dtype=np.uint64)
    out = np.zeros(2 * len(keys), dtype=np.uint64)
    for i, k in enumerate(keys):
        k = int(k)
        out[2 * i], out[2 * i + 1] = k & _M64, k >> 64
    return out


def unpack_keys(words: np.ndarray, kw: int) -> np.ndarray:
    """Inverse of pack_keys: uint64 keys, or Python ints (object array) when kw == 2."""
    if kw == 1:
        return words
    return np.array([int(words[2 * i]) | (int(words[2 * i + 1]) << 64)
                     for i in range(len(words) // 2)], dtype=object)


def _u64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


class GPUDVec:
    """Sparse vector of (address => value) pairs living in GPU memory.

    ``GPUDVec({addr: val, ...}, style=...)``, ``GPUDVec(addr => val)`` as a tuple
    ``(addr, val)``, or ``GPUDVec(style=..., address_type=addr)`` for an empty vector."""

    def __init__(self, pairs=None, style: StochasticStyle | None = None, address_type=None,
                 capacity: int = 0, initiator=None):
        if isinstance(pairs, tuple) and len(pairs) == 2 and not isinstance(pairs[0], tuple):
            pairs = {pairs[0]: pairs[1]}
        pairs = dict(pairs or {})
        if style is None:
            vt = type(next(iter(pairs.values()))) if pairs else float
            style = default_style(int if issubclass(vt, (int, np.integer)) else float)
        self.style = style
        self.valtype = style.valtype
        # initiator rule of an InitiatorDVec (initiatordvec.jl): NonInitiator() is a plain DVec
        self.initiator = initiator_rule(initiator)
        proto = address_type if address_type is not None else (next(iter(pairs)) if pairs else None)
        # an address of the vector's type (its key is irrelevant): makes addresses from keys
        self._proto = proto.with_key(0) if proto is not None else BoseFS.from_key(0, 0, 0)
        self.address_type = (type(self._proto), self._proto.N, self._proto.M)
        # addresses wider than 64 bits (two BitString chunks) use two-word walker records
        self.kw = 2 if self._proto.nbits > 64 else 1
        lib = _lib.load()
        self._ctx = _lib.default_context()
        h = C.c_void_p()
        vk = _lib.VAL_I64 if self.valtype is int else _lib.VAL_F64
        _lib.check(lib.rimu_vec_create_kw(self._ctx.handle, vk, self.kw, max(capacity, len(pairs)),
                                          C.byref(h)))
        self.handle = h
        if pairs:
            self.set_pairs(pairs)

    # ---- storage ---------------------------------------------------------------------
    def _np_vals(self, vals):
        return np.ascontiguousarray(vals, dtype=np.int64 if self.valtype is int else np.float64)

    def upload(self, keys, vals):
        n = len(keys)
        words = pack_keys(keys, self.kw)
        vals = self._np_vals(vals)
        _lib.check(_lib.load().rimu_vec_upload(self.handle, _u64p(words), vals.ctypes.data_as(C.c_void_p),
                                                n))

    def set_pairs(self, pairs: dict):
        keys = [a.key for a in pairs]
        vals = list(pairs.values())
        self.upload(keys, vals)

    def download(self):
        """(keys, values) as numpy arrays, in bucket order."""
        lib = _lib.load()
        n = C.c_int64()
        _lib.check(lib.rimu_vec_length(self.handle, C.byref(n)))
        cap = max(n.value, 1)
        words = np.zeros(cap * self.kw, dtype=np.uint64)
        vals = np.zeros(cap, dtype=np.int64 if self.valtype is int else np.float64)
        got = C.c_int64()
        _lib.check(lib.rimu_vec_download(self.handle, _u64p(words), vals.ctypes.data_as(C.c_void_p),
                                          cap, C.byref(got)))
        return unpack_keys(words[:got.value * self.kw], self.kw), vals[:got.value]

    def sorted_arrays(self):
        k, v = self.download()
        o = np.argsort(k, kind="stable")
        return k[o], v[o]

    # ---- AbstractDVec interface --------------------------------------------------------
    def __len__(self):
        n = C.c_int64()
        _lib.check(_lib.load().rimu_vec_length(self.handle, C.byref(n)))
        return n.value

    def _addr(self, key):
        return self._proto.with_key(int(key))

    def pairs(self):
        k, v = self.sorted_arrays()
        return [(self._addr(a), self.valtype(b)) for a, b in zip(k, v)]

    def keys(self):
        return [a for a, _ in self.pairs()]

    def values(self):
        return [b for _, b in self.pairs()]

    def to_dict(self):
        return dict(self.pairs())

    def __getitem__(self, addr):
        return self.valtype(self.lookup_keys([addr.key])[0])

    def lookup_keys(self, keys):
        n = len(keys)
        words = pack_keys(keys, self.kw)
        out = np.zeros(n, dtype=np.int64 if self.valtype is int else np.float64)
        if n:
            _lib.check(_lib.load().rimu_vec_lookup(self.handle, _u64p(words), n,
                                                    out.ctypes.data_as(C.c_void_p)))
        return out

    def walkernumber_and_length(self):
        """walkernumber_and_length (abstractdvec.jl:270): 1-norm and length."""
        norm, n = C.c_double(), C.c_int64()
        _lib.check(_lib.load().rimu_vec_walkernumber_and_length(self.handle, C.byref(norm),
                                                                 C.byref(n)))
        return norm.value, n.value

    def walkernumber(self):
        return self.walkernumber_and_length()[0]

    def StochasticStyle(self):
        return self.style

    def empty(self):
        _lib.check(_lib.load().rimu_vec_empty(self.handle))
        return self

    zerovector_ = empty

    def similar(self):
        return GPUDVec(style=self.style, address_type=self._proto, initiator=self.initiator)

    def copy(self):
        w = self.similar()
        _lib.check(_lib.load().rimu_vec_copy(w.handle, self.handle))
        return w

    def dot(self, other) -> float:
        """dot(self, other) (abstractdvec.jl:214-230): with a dict `other` its addresses are
        looked up; with a GPUDVec the product is computed on the device."""
        if isinstance(other, dict):
            keys = np.array([a.key for a in other], dtype=np.uint64)
            mine = self.lookup_keys(keys)
            return float(sum(float(m) * float(o) for m, o in zip(mine, other.values())))
        out = C.c_double()
        _lib.check(_lib.load().rimu_vec_dot(self.handle, other.handle, C.byref(out)))
        return out.value

    def scale_(self, alpha) -> "GPUDVec":
        """scale!(v, alpha) (abstractdvec.jl:131-140), on the device."""
        _lib.check(_lib.load().rimu_vec_scale(self.handle, float(alpha)))
        return self

    def add_(self, other: "GPUDVec", alpha=1.0, beta=1.0) -> "GPUDVec":
        """add!(self, other, alpha, beta) = beta*self + alpha*other (abstractdvec.jl:180-188),
        on the device."""
        _lib.check(_lib.load().rimu_vec_add(self.handle, other.handle, float(alpha), float(beta)))
        return self

    def norm(self, p=2) -> float:
        """norm(v, p) for p = 1 (the walker number) and 2 (abstractdvec.jl:233-246)."""
        if p == 1:
            return self.walkernumber()
        if p == 2:
            return math.sqrt(self.dot(self))
        raise ValueError(f"{p}-norm is not implemented")

    def as_float(self) -> "GPUDVec":
        """A Float64 copy on the device (IsDeterministic style)."""
        w = GPUDVec(style=IsDeterministic(), address_type=self._addr(0))
        _lib.check(_lib.load().rimu_vec_convert(w.handle, self.handle, _lib.VAL_F64))
        return w

    def __del__(self):
        try:
            if self.handle:
                _lib.load().rimu_vec_destroy(self.handle)
        except Exception:
            pass

    def __repr__(self):
        return f"GPUDVec(len={len(self)}, style={self.style})"


class GPUWorkingMemory:
    """Working memory of one projector step: spawn buffers, statistics and the
    ProjectedEnergy projector.  Holds the random-stream state (seed, counter)."""

    def __init__(self, seed: int = 0):
        lib = _lib.load()
        self._ctx = _lib.default_context()
        h = C.c_void_p()
        _lib.check(lib.rimu_wm_create(self._ctx.handle, C.byref(h)))
        self.handle = h
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.counter = 0
        self.replica = 0
        self.projector_keys = None

    def set_projector(self, keys, pvals, hpvals, key_words=None):
        """ProjectedEnergy projector: addresses with P and H'P values.  key_words 2 for a
        model of 65-128-bit addresses (keys as Python ints); by default 2 when a key needs it."""
        ik = [int(k) for k in keys]
        kw = key_words or (2 if any(k >> 64 for k in ik) else 1)
        o = sorted(range(len(ik)), key=lambda i: ik[i])
        ik = [ik[i] for i in o]
        pv = np.ascontiguousarray(np.asarray(pvals, float)[o] if len(o) else np.zeros(0))
        hv = np.ascontiguousarray(np.asarray(hpvals, float)[o] if len(o) else np.zeros(0))
        words = pack_keys(np.array(ik, dtype=object if kw == 2 else np.uint64), kw)
        fn = _lib.load().rimu_wm_set_projector_w if kw == 2 else _lib.load().rimu_wm_set_projector
        _lib.check(fn(self.handle, _u64p(words), pv.ctypes.data_as(C.POINTER(C.c_double)),
                      hv.ctypes.data_as(C.POINTER(C.c_double)), len(ik)))
        self.projector_keys = (np.array(ik, dtype=object if kw == 2 else np.uint64)
                               if len(ik) else None)

    def set_timing(self, enable=True):
        _lib.check(_lib.load().rimu_wm_set_timing(self.handle, int(enable)))

    def set_launch_shape(self, keys_per_bucket: int = 1024, table_slots: int = 0):
        """Launch shape of the step kernels: expected contributions per bucket (16..4096) and
        annihilation table slots per CTA (0 = automatic, else a power of two 512..4096)."""
        _lib.check(_lib.load().rimu_wm_set_launch_shape(self.handle, int(keys_per_bucket),
                                                        int(table_slots)))

    def set_annihilation(self, mode: str = "hash"):
        """How one warp groups the spawns of its bucket by address: "hash" (a shared-memory
        table, the default) or "sort" (a bitonic sort by address and value).  The results are
        the same bit for bit."""
        m = {"hash": _lib.ANN_HASH, "sort": _lib.ANN_SORT}[mode]
        _lib.check(_lib.load().rimu_wm_set_annihilation(self.handle, m))

    def timing(self) -> dict:
        """Per-kernel milliseconds and algorithmic bytes accumulated since set_timing."""
        out = np.zeros(7)
        _lib.check(_lib.load().rimu_wm_timing(self.handle, out.ctypes.data_as(C.POINTER(C.c_double))))
        return dict(spawn_ms=out[0], heavy_ms=out[1], annihilate_ms=out[2], steps=int(out[3]),
                    spawn_bytes=out[4], annihilate_bytes=out[5])

    def __del__(self):
        try:
            if self.handle:
                _lib.load().rimu_wm_destroy(self.handle)
        except Exception:
            pass


def working_memory(v: GPUDVec, seed: int = 0) -> GPUWorkingMemory:
    return GPUWorkingMemory(seed)


class FirstOrderTransitionOperator:
    """T = 1 + dt (S - H) (src/fciqmc.jl:78-112)."""

    def __init__(self, hamiltonian, shift: float, time_step: float):
        self.hamiltonian = hamiltonian
        self.shift = float(shift)
        self.time_step = float(time_step)


def apply_operator(wm: GPUWorkingMemory, target: GPUDVec, source: GPUDVec, op, boost=1.0,
                   step: int | None = None):
    """apply_operator!(wm, target, source, op, boost) -> (stat_names, stats, wm, target)
    (dictvectors.jl:112-140).  `op` is a FirstOrderTransitionOperator or a Hamiltonian
    (plain multiplication, used by mul!).  `step` fixes the random counter; by default the
    working memory's counter is used and advanced."""
    if target is source:
        raise ValueError("`target` and `source` must not have the same local storage")
    style = source.style
    p = _lib.StepParams()
    sp = style.params()
    p.style = sp["style"]
    if isinstance(op, FirstOrderTransitionOperator):
        ham = op.hamiltonian
        p.op, p.dt, p.shift = _lib.OP_TRANSITION, op.time_step, op.shift
    else:
        ham = op
        p.op, p.dt, p.shift = _lib.OP_HAMILTONIAN, 0.0, 0.0
        if not isinstance(style, IsDeterministic):
            raise ValueError("plain multiplication needs IsDeterministic")
    p.boost = float(boost)
    p.proj_threshold = sp["proj_threshold"]
    p.compression = sp["compression"]
    p.rel_spawning_threshold = sp["rel_spawning_threshold"]
    p.abs_spawning_threshold = sp["abs_spawning_threshold"]
    p.seed = wm.seed
    if step is None:
        step = wm.counter
        wm.counter += 1
    p.step = int(step) & 0xFFFFFFFF
    p.replica = wm.replica
    p.initiator = source.initiator.code
    p.initiator_threshold = source.initiator.threshold
    target.style, target.valtype, target.address_type = source.style, source.valtype, source.address_type
    target._proto, target.kw = source._proto, source.kw
    target.initiator = source.initiator
    st = _lib.StepStats()
    _lib.check(_lib.load().rimu_apply_operator(ham.handle, wm.handle, target.handle, source.handle,
                                                C.byref(p), C.byref(st)))
    names = style.step_stat_names() + style.compression_names()
    full = {f: getattr(st, f) for f, _ in _lib.StepStats._fields_}
    stats = tuple(full[n] for n in names)
    wm.last_stats = full
    return names, stats, wm, target


def scale_(v: GPUDVec, alpha) -> GPUDVec:
    """scale!(v, alpha) (VectorInterface, abstractdvec.jl:131-140)."""
    return v.scale_(alpha)


def add_(w: GPUDVec, v: GPUDVec, alpha=1.0, beta=1.0) -> GPUDVec:
    """add!(w, v, alpha, beta) = axpby!(alpha, v, beta, w) (abstractdvec.jl:180-208)."""
    return w.add_(v, alpha, beta)


def mul(y: GPUDVec, H, x: GPUDVec, wm: GPUWorkingMemory | None = None) -> GPUDVec:
    """mul!(y, H, x) for sparse vectors (abstractdvec.jl:275-284, pdvec.jl:810-822)."""
    if not isinstance(x.style, IsDeterministic):
        raise ValueError("mul! needs IsDeterministic vectors")
    wm = wm or GPUWorkingMemory()
    apply_operator(wm, y, x, H)
    return y


def dot_operator(w: GPUDVec, H, v: GPUDVec) -> float:
    """dot(w, H, v) (abstractdvec.jl:298-324) = <w | H v>: H v by the deterministic step on
    a Float64 copy of v, then the device dot product; nothing leaves the GPU."""
    tmp = GPUDVec(style=IsDeterministic(), address_type=v._addr(0))
    src = v if isinstance(v.style, IsDeterministic) else v.as_float()
    mul(tmp, H, src)
    return tmp.dot(w)
