"""Checkpoint files in the reference's format: RimuIO.save_state / load_state
(src/RimuIO/RimuIO.jl:92-195), so that a GPU run can resume from, or hand off to, a CPU run.

An Arrow IPC file (zstd-compressed) with two columns, `key` and `value`, and the keyword
arguments of save_state as string metadata.  A BoseFS/FermiFS address is the Arrow extension
type "JuliaLang.Rimu.BoseFS.BitString" (or "...FermiFS.BitString") with metadata "N.M.B" over
a fixed-size list of its BitString chunks (RimuIO/arrowtypes.jl): one UInt8/16/32/64 chunk for
B <= 64 bits, two UInt64 chunks for 65-128 bits, the most significant chunk first (num_chunks,
bitstring.jl:6-18; chunk order, :250-252).  Values are Float64 or Int64.  pyarrow is imported
only when a file is read or written.
"""
from __future__ import annotations

import numpy as np

from .addresses import BoseFS, FermiFS

PACKAGE_VERSION = "0.14.0"      # Rimu version whose file format is written
_EXT_NAME = "ARROW:extension:name"
_EXT_META = "ARROW:extension:metadata"


def _chunk_dtype(bits: int):
    """Chunk type of a single-chunk BitString with `bits` bits (num_chunks, bitstring.jl:6-18)."""
    if bits <= 0:
        raise ValueError("addresses need at least one bit")
    if bits <= 8:
        return np.uint8
    if bits <= 16:
        return np.uint16
    if bits <= 32:
        return np.uint32
    if bits <= 128:
        return np.uint64
    raise ValueError("addresses of more than 128 bits are not supported")


def _address_info(proto):
    if isinstance(proto, BoseFS):
        return "BoseFS", proto.N, proto.M, proto.N + proto.M - 1
    if isinstance(proto, FermiFS):
        return "FermiFS", proto.N, proto.M, proto.M
    raise TypeError("save_state supports BoseFS and FermiFS addresses")


def _to_string(v) -> str:
    """Metadata values as Julia's `string` writes them."""
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, complex):
        im = v.imag
        sign = "-" if im < 0 or (im == 0 and str(im).startswith("-")) else "+"
        return f"{float(v.real)!r} {sign} {abs(float(im))!r}im"
    return str(v)


def _parse(v: str):
    """Metadata values parsed as load_state does: Int, Float64, ComplexF64, Bool, or string."""
    try:
        return int(v)
    except ValueError:
        pass
    try:
        return float(v)
    except ValueError:
        pass
    if v.endswith("im"):
        try:
            return complex(v[:-2].replace(" ", "") + "j")
        except ValueError:
            pass
    if v in ("true", "false"):
        return v == "true"
    return v


def save_pairs(filename, keys, vals, proto, **metadata):
    """Write (address key, value) pairs of addresses like `proto` in the save_state format."""
    import pyarrow as pa
    kind, N, M, B = _address_info(proto)
    vals = np.asarray(vals)
    if vals.dtype.kind in "iu":
        vals = vals.astype(np.int64)
    else:
        vals = vals.astype(np.float64)
    dt = _chunk_dtype(B)
    if B > 64:                          # two chunks per address, (hi, lo)
        ik = [int(k) for k in keys]
        words = np.zeros(2 * len(ik), dtype=np.uint64)
        for i, k in enumerate(ik):
            words[2 * i], words[2 * i + 1] = k >> 64, k & ((1 << 64) - 1)
        key_arr = pa.FixedSizeListArray.from_arrays(pa.array(words), 2)
    else:
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        key_arr = pa.FixedSizeListArray.from_arrays(pa.array(keys.astype(dt)), 1)
    key_field = pa.field("key", key_arr.type, nullable=False,
                         metadata={_EXT_NAME: f"JuliaLang.Rimu.{kind}.BitString",
                                   _EXT_META: f"{N}.{M}.{B}"})
    val_field = pa.field("value", pa.from_numpy_dtype(vals.dtype), nullable=False)
    meta = {"RIMU_PACKAGE_VERSION": PACKAGE_VERSION}
    meta.update({str(k): _to_string(v) for k, v in metadata.items()})
    schema = pa.schema([key_field, val_field], metadata=meta)
    table = pa.Table.from_arrays([key_arr, pa.array(vals)], schema=schema)
    with pa.ipc.new_file(str(filename), schema,
                         options=pa.ipc.IpcWriteOptions(compression="zstd")) as w:
        w.write_table(table)


def load_pairs(filename):
    """(keys, values, address prototype, metadata) of a save_state file."""
    import pyarrow as pa
    with pa.memory_map(str(filename)) as src:
        table = pa.ipc.open_file(src).read_all()
    if table.schema.names != ["key", "value"]:
        raise ValueError(f"`{filename}` is not a valid Rimu state file")
    kf = table.schema.field("key")
    fmeta = {k.decode(): v.decode() for k, v in (kf.metadata or {}).items()}
    name, meta = fmeta.get(_EXT_NAME, ""), fmeta.get(_EXT_META, "")
    if name not in ("JuliaLang.Rimu.BoseFS.BitString", "JuliaLang.Rimu.FermiFS.BitString"):
        raise ValueError(f"`{filename}`: unsupported address type {name!r}")
    N, M, B = (int(x) for x in meta.split("."))
    col = table.column("key").combine_chunks()
    nchunks = 1 if B <= 64 else (B - 1) // 64 + 1
    if col.type.list_size != nchunks or nchunks > 2:
        raise ValueError(f"`{filename}`: {col.type.list_size} chunks for {B}-bit addresses")
    flat = np.asarray(col.flatten().to_numpy(zero_copy_only=False), dtype=np.uint64)
    if nchunks == 1:
        keys = flat
    else:                               # (hi, lo) chunks: Python ints
        keys = np.array([(int(flat[2 * i]) << 64) | int(flat[2 * i + 1])
                         for i in range(len(flat) // 2)], dtype=object)
    vals = table.column("value").to_numpy()
    proto = (BoseFS if "BoseFS" in name else FermiFS).from_key(0, N, M)
    smeta = {k.decode(): _parse(v.decode()) for k, v in (table.schema.metadata or {}).items()}
    if "RIMU_PACKAGE_VERSION" in smeta:
        smeta["RIMU_PACKAGE_VERSION"] = str(smeta["RIMU_PACKAGE_VERSION"])
    return keys, vals, proto, smeta


def save_state(filename, vector, **metadata):
    """save_state(filename, vector; kwargs...) (RimuIO.jl:92-110): the walker list of a
    GPUDVec with the keyword arguments as metadata."""
    keys, vals = vector.sorted_arrays()
    save_pairs(filename, keys, vals, vector._addr(0), **metadata)


def load_state(filename, style=None, **kwargs):
    """load_state(filename; style) -> (GPUDVec, metadata) (RimuIO.jl:150-188): the default
    style is IsDynamicSemistochastic for Float64 values and IsStochasticInteger for Int64."""
    from .dvec import GPUDVec
    from .styles import IsDynamicSemistochastic, IsStochasticInteger
    keys, vals, proto, meta = load_pairs(filename)
    if style is None:
        style = IsDynamicSemistochastic() if vals.dtype.kind == "f" else IsStochasticInteger()
    v = GPUDVec(style=style, address_type=proto, capacity=len(keys), **kwargs)
    v.upload(keys, vals.astype(np.int64 if style.valtype is int else np.float64))
    return v, meta
