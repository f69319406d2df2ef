"""Checkpoint files in the reference's save_state/load_state format (RimuIO.jl:92-195,
arrowtypes.jl; the reference's own tests test/RimuIO.jl:98-175): round trips of keys, values
and metadata, the Arrow schema the reference's reader expects, and the errors for files that
are not state files.  Host-side only (the files are written from downloaded lists)."""
import numpy as np
import pytest

pa = pytest.importorskip("pyarrow")

import rimugpu as R                      # noqa: E402
from rimugpu import rimuio               # noqa: E402


@pytest.mark.parametrize("proto,dtype", [
    (R.BoseFS([1] * 6), np.uint16),                # 11 bits
    (R.BoseFS(4, {2: 2}), np.uint8),               # 5 bits
    (R.BoseFS(20, {10: 10}), np.uint32),           # 29 bits
    (R.near_uniform(R.BoseFS, 20, 20), np.uint64),  # 39 bits
    (R.FermiFS([1, 1, 1] + [0] * 13), np.uint16),  # 16 bits
])
def test_round_trip_and_schema(tmp_path, proto, dtype):
    rng = np.random.default_rng(1)
    B = proto.N + proto.M - 1 if isinstance(proto, R.BoseFS) else proto.M
    keys = np.unique(rng.integers(0, 2 ** min(B, 62), 500, dtype=np.uint64))
    for vals in (rng.normal(size=len(keys)), rng.integers(-9, 10, len(keys))):
        f = tmp_path / "state.arrow"
        rimuio.save_pairs(f, keys, vals, proto, int=1, float=2.3, complex=1.2 + 3j, string="a string",
                          bool=True)
        k, v, p, meta = rimuio.load_pairs(f)
        assert np.array_equal(k, keys) and np.array_equal(v, vals)
        assert type(p) is type(proto) and (p.N, p.M) == (proto.N, proto.M)
        assert meta["int"] == 1 and meta["float"] == 2.3 and meta["complex"] == 1.2 + 3j
        assert meta["bool"] is True and meta["string"] == "a string"
        assert meta["RIMU_PACKAGE_VERSION"] == "0.14.0"
        with pa.memory_map(str(f)) as src:
            t = pa.ipc.open_file(src).read_all()
        kf = t.schema.field("key")
        assert kf.type == pa.list_(pa.from_numpy_dtype(dtype), 1)
        kind = "BoseFS" if isinstance(proto, R.BoseFS) else "FermiFS"
        assert kf.metadata[b"ARROW:extension:name"] == f"JuliaLang.Rimu.{kind}.BitString".encode()
        assert kf.metadata[b"ARROW:extension:metadata"] == f"{proto.N}.{proto.M}.{B}".encode()
        assert t.schema.field("value").type in (pa.float64(), pa.int64())


def test_empty_vector(tmp_path):
    f = tmp_path / "empty.arrow"
    rimuio.save_pairs(f, np.zeros(0, dtype=np.uint64), np.zeros(0, dtype=np.int64), R.BoseFS([1, 1, 1]))
    k, v, _, _ = rimuio.load_pairs(f)
    assert len(k) == 0 and len(v) == 0


def test_files_that_are_not_state_files_are_rejected(tmp_path):
    f = tmp_path / "bad.arrow"
    for cols in ({"key": [1, 2, 3], "value": [1, 2, 3], "error": [0, 0, 0]}, {"error": [0, 0, 0]}):
        t = pa.table(cols)
        with pa.ipc.new_file(str(f), t.schema) as w:
            w.write_table(t)
        with pytest.raises(ValueError):
            rimuio.load_pairs(f)


def test_save_and_load_a_product_vector(tmp_path):
    """The reference's "save DVec" case (test/RimuIO.jl:110-115): H * v for
    HubbardReal1D(BoseFS(1,1,1)) and v = {BoseFS(1,1,1) => 1.0, BoseFS(2,1,0) => pi}, saved and
    loaded back equal, key for key and bit for bit.  The product is the oracle's exact step with
    the plain Hamiltonian (IsDeterministic, no transition factor)."""
    import math
    import oracle as O
    m = O.real1d(3, 3, 1.0, 1.0)
    keys = np.array(sorted([R.BoseFS(1, 1, 1).key, R.BoseFS(2, 1, 0).key]), dtype=np.uint64)
    vals = np.array([1.0 if k == R.BoseFS(1, 1, 1).key else math.pi for k in keys])
    hk, hv, _ = O.step(m, O.StepParams(O.STYLE_DETERMINISTIC, op=O.OP_HAMILTONIAN), keys, vals)
    assert len(hk) > 2
    f = tmp_path / "dvec.arrow"
    rimuio.save_pairs(f, hk, hv, R.BoseFS(1, 1, 1))
    k, v, p, _ = rimuio.load_pairs(f)
    o = np.argsort(k)
    assert np.array_equal(k[o], hk) and np.array_equal(np.asarray(v)[o].view(np.uint64), hv.view(np.uint64))
    assert isinstance(p, R.BoseFS) and (p.N, p.M) == (3, 3)


@pytest.mark.parametrize("dtype", [np.int64, np.float64])
def test_empty_vectors_of_both_value_types(tmp_path, dtype):
    """The reference's "save empty vector" case (test/RimuIO.jl:136-145) for integer and float
    values."""
    f = tmp_path / "empty.arrow"
    rimuio.save_pairs(f, np.zeros(0, dtype=np.uint64), np.zeros(0, dtype=dtype), R.BoseFS([1, 1, 1, 1]))
    k, v, _, meta = rimuio.load_pairs(f)
    assert len(k) == 0 and len(v) == 0 and meta["RIMU_PACKAGE_VERSION"] == "0.14.0"


@pytest.mark.parametrize("proto", [R.BoseFS([1] * 50), R.FermiFS([1] * 10 + [0] * 90)],
                         ids=["bose-99", "fermi-100"])
def test_two_chunk_addresses(tmp_path, proto):
    """Addresses of 65-128 bits: a BitString of two UInt64 chunks (num_chunks,
    bitstring.jl:6-18), stored most significant chunk first (:250-252), as a two-element
    fixed-size list; round trip key for key."""
    B = proto.nbits
    assert 64 < B <= 128
    rng = np.random.default_rng(3)
    keys = sorted({int(rng.integers(0, 1 << 62)) | (int(rng.integers(0, 1 << (B - 64))) << 64)
                   for _ in range(300)})
    vals = rng.normal(size=len(keys))
    f = tmp_path / "wide.arrow"
    rimuio.save_pairs(f, np.array(keys, dtype=object), vals, proto, step=12)
    k, v, p, meta = rimuio.load_pairs(f)
    assert [int(x) for x in k] == keys and np.array_equal(v, vals) and meta["step"] == 12
    assert type(p) is type(proto) and (p.N, p.M) == (proto.N, proto.M)
    with pa.memory_map(str(f)) as src:
        t = pa.ipc.open_file(src).read_all()
    kf = t.schema.field("key")
    assert kf.type == pa.list_(pa.uint64(), 2)
    kind = "BoseFS" if isinstance(proto, R.BoseFS) else "FermiFS"
    assert kf.metadata[b"ARROW:extension:metadata"] == f"{proto.N}.{proto.M}.{B}".encode()
    assert kf.metadata[b"ARROW:extension:name"] == f"JuliaLang.Rimu.{kind}.BitString".encode()
    first = t.column("key").combine_chunks()[0].as_py()
    assert first == [keys[0] >> 64, keys[0] & ((1 << 64) - 1)]
