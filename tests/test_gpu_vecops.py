"""scale! and add! of device walker lists (VectorInterface on AbstractDVec,
src/DictVectors/abstractdvec.jl:121-208) against the same operations on host dictionaries, bit
for bit: scale!(w, beta) removes the keys whose value becomes zero, then w[key] += alpha*val for
every pair of v, removing zeros again (setindex! of a zero deletes the key).  Float64 lists in
IEEE double arithmetic, Int64 lists with integer factors in wrapping Int64 arithmetic; one- and
two-word addresses; lists of different bucket counts; v aliasing w."""
import numpy as np
import pytest

import rimugpu as R

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def wrap64(x):
    return ((int(x) + (1 << 63)) & M64) - (1 << 63)


def host_scale(v, a, ints):
    if a == 0:
        return {}
    out = {}
    for k, x in v.items():
        y = wrap64(int(a) * x) if ints else float(a) * x
        if y != 0:
            out[k] = y
    return out


def host_add(w, v, a, b, ints):
    out = host_scale(w, b, ints) if b != 1 else dict(w)
    for k, x in v.items():
        y = wrap64(int(a) * x) if ints else float(a) * x
        s = wrap64(out.get(k, 0) + y) if ints else out.get(k, 0.0) + y
        if s == 0:
            out.pop(k, None)
        else:
            out[k] = s
    return out


def make_vec(d, style, addr):
    v = R.GPUDVec(style=style, address_type=addr)
    keys = list(d)
    if addr.nbits > 64:
        v.upload(np.array(keys, dtype=object), np.array([d[k] for k in keys]))
    else:
        v.upload(np.array(keys, dtype=np.uint64),
                 np.array([d[k] for k in keys], dtype=np.int64 if style.valtype is int else np.float64))
    return v


def as_dict(v):
    k, x = v.download()
    return {int(a): (int(b) if v.valtype is int else float(b)) for a, b in zip(k, x)}


def assert_same(got, want, ints):
    assert sorted(got) == sorted(want)
    for k in want:
        if ints:
            assert got[k] == want[k]
        else:
            assert np.float64(got[k]).view(np.uint64) == np.float64(want[k]).view(np.uint64), k


def random_dicts(rng, nw, nv, overlap, wide, ints):
    bits = 100 if wide else 60
    pool = set()
    while len(pool) < nw + nv:
        k = int(rng.integers(0, 1 << 60))
        if wide:
            k |= int(rng.integers(0, 1 << 40)) << 60
        pool.add(k)
    pool = sorted(pool)
    rng.shuffle(pool)
    wk = pool[:nw]
    vk = pool[nw:nw + nv]
    vk[: int(overlap * min(nw, nv))] = wk[: int(overlap * min(nw, nv))]
    assert all(k < (1 << bits) for k in pool)
    if ints:
        wv = rng.integers(-9, 10, nw)
        vv = rng.integers(-9, 10, nv)
        w = {k: int(x) for k, x in zip(wk, wv) if x != 0}
        v = {k: int(x) for k, x in zip(vk, vv) if x != 0}
    else:
        w = {k: float(x) for k, x in zip(wk, rng.normal(size=nw) * 3)}
        v = {k: float(x) for k, x in zip(vk, rng.normal(size=nv) * 3)}
    return w, v


ADDR1 = R.near_uniform(R.BoseFS, 20, 20)            # 39 bits: one word
ADDR2 = R.BoseFS([1] * 50)                           # 99 bits: two words


@pytest.mark.parametrize("wide", [False, True], ids=["one-word", "two-word"])
@pytest.mark.parametrize("a,b", [(0.7, -1.3), (1.0, 1.0), (-2.5, 0.0), (0.0, 3.0), (1.0, -1.0)])
def test_add_float(wide, a, b):
    rng = np.random.default_rng(1)
    w, v = random_dicts(rng, 20000, 15000, 0.4, wide, False)
    addr = ADDR2 if wide else ADDR1
    style = R.IsDynamicSemistochastic()
    gw, gv = make_vec(w, style, addr), make_vec(v, style, addr)
    R.add_(gw, gv, a, b)
    assert_same(as_dict(gw), host_add(w, v, a, b, False), False)
    assert as_dict(gv) == v                          # v is left as it was
    norm, n = gw.walkernumber_and_length()
    want = host_add(w, v, a, b, False)
    assert n == len(want)


def test_add_cancels_to_empty_and_aliasing():
    rng = np.random.default_rng(2)
    w, _ = random_dicts(rng, 5000, 10, 0.0, False, False)
    style = R.IsDynamicSemistochastic()
    gw = make_vec(w, style, ADDR1)
    neg = make_vec({k: -x for k, x in w.items()}, style, ADDR1)
    R.add_(gw, neg)
    assert len(gw) == 0 and as_dict(gw) == {}
    # add!(w, w, a, b): w scaled first, then the scaled w added
    gw = make_vec(w, style, ADDR1)
    R.add_(gw, gw, 0.5, 3.0)
    sw = host_scale(w, 3.0, False)
    assert_same(as_dict(gw), host_add(sw, sw, 0.5, 1.0, False), False)


def test_add_lists_of_different_bucket_counts():
    """A short w and a long v (and the other way round): the lists are brought to a common
    bucket count first."""
    rng = np.random.default_rng(3)
    style = R.IsDynamicSemistochastic()
    for nw, nv in ((50, 60000), (60000, 50)):
        w, v = random_dicts(rng, nw, nv, 0.5, False, False)
        gw, gv = make_vec(w, style, ADDR1), make_vec(v, style, ADDR1)
        R.add_(gw, gv, 1.5, 0.25)
        assert_same(as_dict(gw), host_add(w, v, 1.5, 0.25, False), False)


@pytest.mark.parametrize("a,b", [(3, -2), (1, 1), (-1, 0)])
def test_add_integer_lists(a, b):
    rng = np.random.default_rng(4)
    w, v = random_dicts(rng, 8000, 8000, 0.5, False, True)
    style = R.IsStochasticInteger()
    gw, gv = make_vec(w, style, ADDR1), make_vec(v, style, ADDR1)
    R.add_(gw, gv, a, b)
    assert_same(as_dict(gw), host_add(w, v, a, b, True), True)


def test_add_integer_list_into_float_list():
    rng = np.random.default_rng(5)
    w, _ = random_dicts(rng, 3000, 10, 0.0, False, False)
    _, v = random_dicts(rng, 10, 3000, 0.0, False, True)
    gw = make_vec(w, R.IsDynamicSemistochastic(), ADDR1)
    gv = make_vec(v, R.IsStochasticInteger(), ADDR1)
    R.add_(gw, gv, 0.75, 1.0)
    vf = {k: float(x) for k, x in v.items()}
    assert_same(as_dict(gw), host_add(w, vf, 0.75, 1.0, False), False)


@pytest.mark.parametrize("wide", [False, True], ids=["one-word", "two-word"])
def test_scale(wide):
    rng = np.random.default_rng(6)
    w, _ = random_dicts(rng, 10000, 10, 0.0, wide, False)
    w[next(iter(w))] = 1e-30                         # underflows to zero below: removed
    addr = ADDR2 if wide else ADDR1
    style = R.IsDynamicSemistochastic()
    for a in (1e-300, -3.5, 1.0, 0.0):
        gw = make_vec(w, style, addr)
        R.scale_(gw, a)
        assert_same(as_dict(gw), host_scale(w, a, False) if a != 1.0 else w, False)
    wi, _ = random_dicts(rng, 4000, 10, 0.0, False, True)
    gi = make_vec(wi, R.IsStochasticInteger(), ADDR1)
    R.scale_(gi, -3)
    assert_same(as_dict(gi), host_scale(wi, -3, True), True)


def test_bad_arguments_are_rejected():
    rng = np.random.default_rng(7)
    w, v = random_dicts(rng, 100, 100, 0.5, False, True)
    gi = make_vec(w, R.IsStochasticInteger(), ADDR1)
    gf = make_vec({k: float(x) for k, x in v.items()}, R.IsDynamicSemistochastic(), ADDR1)
    with pytest.raises(R.RimuError):
        R.scale_(gi, 0.5)                            # an Int64 list takes integer factors
    with pytest.raises(R.RimuError):
        R.add_(gi, gf)                               # Float64 values into an Int64 list
    wide = make_vec({1 << 80: 1.0}, R.IsDynamicSemistochastic(), ADDR2)
    with pytest.raises(R.RimuError):
        R.add_(gf, wide)                             # different address widths
