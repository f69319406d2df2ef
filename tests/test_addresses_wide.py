"""Host-side address encodings beyond one 64-bit chunk, and the (lo, hi) word packing the
C ABI uses for them (no GPU needed).  The BoseFS encoding (bitstring.jl:464-472: mode 1 at
the least significant end, n ones then a zero per mode) is checked against the oracle's
independent encoder; unsigned integer order is the reference's isless (bitstring.jl:317-324)."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from rimugpu.dvec import pack_keys, unpack_keys


@pytest.mark.parametrize("onr", [
    [1] * 50,                                   # BoseFS{50,50}: 99 bits
    [0] * 60 + [3, 0, 2] + [1] * 5,             # 10 bosons in 68 modes: 77 bits
    [7] + [0] * 63 + [1],                       # bits at both ends of a 72-bit word
])
def test_wide_bosefs_encoding_matches_the_oracle(onr):
    b = R.BoseFS(onr)
    assert b.nbits == sum(onr) + len(onr) - 1 > 64
    assert b.key == O.bose_key(onr)
    assert b.onr() == tuple(onr)
    assert R.BoseFS.from_key(b.key, b.N, b.M) == b


def test_wide_fermifs_and_order():
    f = R.FermiFS([1, 0] * 50)                  # 100 modes
    assert f.key == sum(1 << k for k in range(0, 100, 2)) and f.nbits == 100
    a, c = R.BoseFS([1] * 40 + [0] * 40), R.BoseFS([0] * 40 + [1] * 40)
    assert (a < c) == (a.key < c.key)
    with pytest.raises(ValueError):
        R.BoseFS([1] * 70)                      # 139 bits
    with pytest.raises(ValueError):
        R.FermiFS([1] * 129)


def test_key_words_round_trip():
    rng = np.random.default_rng(3)
    keys = [int(rng.integers(0, 2 ** 62)) << int(rng.integers(0, 66)) for _ in range(200)]
    words = pack_keys(keys, 2)
    assert words.dtype == np.uint64 and len(words) == 400
    assert words[0] == keys[0] & ((1 << 64) - 1) and words[1] == keys[0] >> 64
    assert list(unpack_keys(words, 2)) == keys
    narrow = np.array([1, 2, 2 ** 63 + 5], dtype=np.uint64)
    assert np.array_equal(unpack_keys(pack_keys(narrow, 1), 1), narrow)


def test_oracle_steps_wide_and_narrow_addresses_alike():
    """A 64-bit-fitting model stepped through the two-word entry point of the oracle gives the
    same step as through the one-word entry point (the address word of the random counters is
    lo ^ mix64(hi), which is the address itself when hi = 0)."""
    m = O.real1d(6, 6, 6.0, 1.0)
    keys = np.array([O.bose_key([1] * 6)], dtype=np.uint64)
    prm = O.StepParams(O.STYLE_DSS, dt=0.01, shift=0.0, seed=7, step=3)
    k1, v1, s1 = O.step(m, prm, keys, np.array([40.0]))
    k2, v2, s2 = O._step_wide(m, prm, [int(keys[0])], np.array([40.0]))
    assert [int(x) for x in k1] == [int(x) for x in k2]
    assert np.array_equal(v1.view(np.uint64), v2.view(np.uint64))
    assert s1 == s2
