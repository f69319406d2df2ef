"""Fock-state addresses as single-chunk bit strings (host side).

The encodings are the ones of Rimu.jl's BitString-backed addresses, so keys produced here
are the raw chunk values the device kernels operate on:
  BoseFS{N,M}: N + M - 1 bits, mode 1 at the least significant end, each mode written as
  n_i ones followed by a zero separator (src/BitStringAddresses/bitstring.jl:464-472,
  511-520); FermiFS{N,M}: mode k <-> bit k-1 (bitstring.jl:713-723).
Ordering of addresses is the unsigned integer order of the key (bitstring.jl:317-324).
CompositeFS of two components (multicomponent.jl:10-30; FermiFS2C, :87-103) puts component 1
in the high bits and component 2 in the low bits of one key, so key order is the order of the
component tuple (multicomponent.jl:79).
"""
from __future__ import annotations

from functools import total_ordering


def _bose_key(onr) -> int:
    key = 0
    for n in reversed(onr):
        key = (key << (n + 1)) | ((1 << n) - 1)
    return key


def _bose_onr(key: int, M: int) -> tuple:
    onr = []
    for _ in range(M):
        n = 0
        while key & 1:
            n += 1
            key >>= 1
        onr.append(n)
        key >>= 1
    return tuple(onr)


@total_ordering
class BoseFS:
    """BoseFS{N,M} (src/BitStringAddresses/bosefs.jl:54-112).

    ``BoseFS(1, 1, 2)``, ``BoseFS((1, 1, 2))``, ``BoseFS(M, {mode: occupation})`` (sparse,
    1-based modes) or ``BoseFS.from_key(key, N, M)``."""

    __slots__ = ("N", "M", "key")
    fermion = False

    def __init__(self, *args):
        if len(args) == 2 and isinstance(args[1], dict):
            M, pairs = args
            onr = [0] * M
            for mode, occ in pairs.items():
                onr[mode - 1] = occ
        elif len(args) == 1 and not isinstance(args[0], int):
            onr = list(args[0])
        else:
            onr = list(args)
        if any(n < 0 for n in onr):
            raise ValueError("invalid ONR: negative occupation")
        self.N = int(sum(onr))
        self.M = len(onr)
        if self.N + self.M - 1 > 128:
            raise ValueError("BoseFS wider than 128 bits is not supported")
        self.key = _bose_key(onr)

    @classmethod
    def from_key(cls, key: int, N: int, M: int) -> "BoseFS":
        b = cls.__new__(cls)
        b.N, b.M, b.key = N, M, int(key)
        return b

    @property
    def nbits(self) -> int:
        return self.N + self.M - 1

    def with_key(self, key: int) -> "BoseFS":
        """The address of this type (same N, M) with chunk `key`."""
        return BoseFS.from_key(key, self.N, self.M)

    def onr(self) -> tuple:
        return _bose_onr(self.key, self.M)

    def num_occupied_modes(self) -> int:
        return sum(1 for n in self.onr() if n)

    def __eq__(self, o):
        return isinstance(o, BoseFS) and (self.N, self.M, self.key) == (o.N, o.M, o.key)

    def __lt__(self, o):
        return self.key < o.key

    def __hash__(self):
        return hash(("B", self.N, self.M, self.key))

    def __repr__(self):
        return f"BoseFS{{{self.N},{self.M}}}{self.onr()}"


@total_ordering
class FermiFS:
    """FermiFS{N,M} (src/BitStringAddresses/fermifs.jl:54-161)."""

    __slots__ = ("N", "M", "key")
    fermion = True

    def __init__(self, *args):
        if len(args) == 2 and isinstance(args[1], dict):
            M, pairs = args
            onr = [0] * M
            for mode, occ in pairs.items():
                onr[mode - 1] = occ
        elif len(args) == 1 and not isinstance(args[0], int):
            onr = list(args[0])
        else:
            onr = list(args)
        if any(n not in (0, 1) for n in onr):
            raise ValueError("invalid fermionic ONR")
        self.N = int(sum(onr))
        self.M = len(onr)
        if self.M > 128:
            raise ValueError("FermiFS wider than 128 bits is not supported")
        self.key = sum(1 << k for k, n in enumerate(onr) if n)

    @classmethod
    def from_key(cls, key: int, N: int, M: int) -> "FermiFS":
        f = cls.__new__(cls)
        f.N, f.M, f.key = N, M, int(key)
        return f

    @property
    def nbits(self) -> int:
        return self.M

    def with_key(self, key: int) -> "FermiFS":
        return FermiFS.from_key(key, self.N, self.M)

    def onr(self) -> tuple:
        return tuple((self.key >> k) & 1 for k in range(self.M))

    def num_occupied_modes(self) -> int:
        return self.N

    def __eq__(self, o):
        return isinstance(o, FermiFS) and (self.N, self.M, self.key) == (o.N, o.M, o.key)

    def __lt__(self, o):
        return self.key < o.key

    def __hash__(self):
        return hash(("F", self.N, self.M, self.key))

    def __repr__(self):
        return f"FermiFS{{{self.N},{self.M}}}{self.onr()}"


def near_uniform_onr(N: int, M: int) -> tuple:
    """near_uniform_onr (bosefs.jl:139-148)."""
    f, extras = divmod(N, M)
    return tuple(f + (1 if i < extras else 0) for i in range(M))


def near_uniform(kind, N: int, M: int):
    """near_uniform(BoseFS{N,M}) / near_uniform(FermiFS{N,M})."""
    if kind is FermiFS:
        return FermiFS([1] * N + [0] * (M - N))
    return BoseFS(near_uniform_onr(N, M))


@total_ordering
class CompositeFS:
    """CompositeFS(a, b, ...) of two to four single-component addresses with the same number
    of modes (multicomponent.jl:10-30).  One key of up to 128 bits (each component at most 64):
    the last component in the low bits, the one before it above them, and so on, so that key
    order is the order of the component tuple."""

    __slots__ = ("components", "N", "M", "key")
    fermion = False

    def __init__(self, *components):
        if not 2 <= len(components) <= 4:
            raise ValueError("CompositeFS with two to four components is supported")
        if not all(isinstance(c, (BoseFS, FermiFS)) for c in components):
            raise TypeError("CompositeFS components must be BoseFS or FermiFS")
        if any(c.M != components[0].M for c in components):
            raise ValueError("all addresses must have the same number of modes")
        if sum(c.nbits for c in components) > 128 or any(c.nbits > 64 for c in components):
            raise ValueError("CompositeFS wider than 128 bits, or with a component wider than "
                             "64 bits, is not supported")
        self.components = tuple(components)
        self.N, self.M = sum(c.N for c in components), components[0].M
        key = 0
        for c in components:
            key = (key << c.nbits) | c.key
        self.key = key

    @property
    def nbits(self) -> int:
        return sum(c.nbits for c in self.components)

    def with_key(self, key: int) -> "CompositeFS":
        key = int(key)
        parts = []
        rest = key
        for comp in reversed(self.components):
            parts.append(comp.with_key(rest & ((1 << comp.nbits) - 1)))
            rest >>= comp.nbits
        c = CompositeFS.__new__(CompositeFS)
        c.components = tuple(reversed(parts))
        c.N, c.M, c.key = self.N, self.M, key
        return c

    def onr(self) -> tuple:
        return tuple(c.onr() for c in self.components)

    def num_occupied_modes(self) -> int:
        return sum(c.num_occupied_modes() for c in self.components)

    def __eq__(self, o):
        return (isinstance(o, CompositeFS) and self.key == o.key and
                len(self.components) == len(o.components) and
                all(type(x) is type(y) and x.N == y.N and x.M == y.M
                    for x, y in zip(self.components, o.components)))

    def __lt__(self, o):
        return self.key < o.key

    def __hash__(self):
        return hash(("C",) + tuple((type(c).__name__, c.N, c.M) for c in self.components) +
                    (self.key,))

    def __repr__(self):
        return "CompositeFS(" + ", ".join(repr(c) for c in self.components) + ")"


def FermiFS2C(*args):
    """FermiFS2C(f1, f2), FermiFS2C(onr_a, onr_b) or FermiFS2C(M, pairs) with pairs
    `mode => 1` (first component) or `mode => -1` (second), as a dict or a list of
    (mode, +-1) (multicomponent.jl:87-103)."""
    if len(args) == 2 and isinstance(args[0], FermiFS) and isinstance(args[1], FermiFS):
        return CompositeFS(args[0], args[1])
    if len(args) == 2 and isinstance(args[0], int):
        M, pairs = args
        items = list(pairs.items()) if isinstance(pairs, dict) else list(pairs)
        up, dn = [0] * M, [0] * M
        for mode, occ in items:
            if occ > 0:
                up[mode - 1] = occ
            elif occ < 0:
                dn[mode - 1] = -occ
        return CompositeFS(FermiFS(up), FermiFS(dn))
    if len(args) == 2:
        return CompositeFS(FermiFS(args[0]), FermiFS(args[1]))
    raise TypeError("FermiFS2C(f1, f2), FermiFS2C(onr_a, onr_b) or FermiFS2C(M, pairs)")


def is_fermi2c(address) -> bool:
    return (isinstance(address, CompositeFS) and len(address.components) == 2 and
            all(isinstance(c, FermiFS) for c in address.components))
