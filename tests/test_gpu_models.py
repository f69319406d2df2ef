"""Matrix elements of the device models against the oracle (bit-exact), on random addresses."""
import numpy as np
import pytest

import oracle as O
import rimugpu as R
from helpers import oracle_model

pytestmark = pytest.mark.gpu


def random_bose(rng, N, M):
    return R.BoseFS(np.bincount(rng.integers(0, M, N), minlength=M).tolist())


def models():
    return [
        R.HubbardReal1D(R.BoseFS(1, 1, 1, 1, 1, 1), u=6.0, t=1.0),
        R.HubbardReal1D(R.near_uniform(R.BoseFS, 20, 20), u=4.0, t=1.0),
        R.HubbardReal1D(R.BoseFS(3, 0, 0, 2, 0), u=1.5, t=0.7),
        R.HubbardRealSpace(R.BoseFS([1] * 16), R.PeriodicBoundaries(4, 4), t=[1.0], u=[[3.0]]),
        R.HubbardRealSpace(R.BoseFS([2, 0, 1, 0, 0, 3]), R.HardwallBoundaries(2, 3), t=[1.3], u=[[2.0]]),
        R.HubbardRealSpace(R.BoseFS([1, 0, 2, 0, 0, 1, 1, 0]), R.LadderBoundaries(2, 4), t=[1.0], u=[[1.0]],
                           v=[0.5, 0.25]),
        R.HubbardRealSpace(R.FermiFS([1, 0, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0, 0, 1, 0, 0]), R.PeriodicBoundaries(4, 4),
                           t=[1.0], u=[[0.0]]),
        R.HubbardRealSpace(R.FermiFS([1, 1, 0, 0, 1, 0, 0, 0, 1]), R.HardwallBoundaries(3, 3), t=[2.0], u=[[0.0]]),
        R.HubbardMom1D(R.BoseFS(3, 2, 1), u=1.0),
        R.HubbardMom1D(R.BoseFS(20, {10: 10}), u=6.0, t=1.0),
        R.HubbardMom1D(R.BoseFS([0, 1, 3, 0, 2, 0, 1]), u=2.5, t=0.5),
    ]


@pytest.mark.parametrize("h", models(), ids=repr)
def test_diagonal_and_offdiagonals_match_oracle(h):
    m = oracle_model(h)
    rng = np.random.default_rng(11)
    addrs = [h.address]
    for _ in range(40):
        if isinstance(h.address, R.FermiFS):
            perm = rng.permutation(h.M)[: h.N]
            onr = [0] * h.M
            for p in perm:
                onr[p] = 1
            addrs.append(R.FermiFS(onr))
        else:
            addrs.append(random_bose(rng, h.N, h.M))
    keys = np.array([a.key for a in addrs], dtype=np.uint64)
    got = h.diagonal_elements(keys)
    want = np.array([O.diagonal(m, int(k)) for k in keys])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    for a in addrs:
        gk, gv = h.offdiagonal_keys(a.key)
        od = O.offdiagonals(m, a.key)
        assert len(gk) == len(od) == h.num_offdiagonals(a)
        for (ok, ov), k, v in zip(od, gk, gv):
            if ov == 0.0:
                assert v == 0.0
            else:
                assert int(k) == ok and v == ov


def test_reference_docstring_offdiagonals_on_gpu():
    h = R.HubbardReal1D(R.BoseFS(3, 2, 1))
    got = [(a.onr(), v) for a, v in h.offdiagonals(h.address)]
    assert got == [((2, 3, 1), -3.0), ((2, 2, 2), -2.449489742783178), ((3, 1, 2), -2.0),
                   ((4, 1, 1), -2.8284271247461903), ((4, 2, 0), -2.0), ((3, 3, 0), -1.7320508075688772)]
    hm = R.HubbardMom1D(R.BoseFS(3, 2, 1))
    assert hm.diagonal_element(hm.address) == 8.666666666666664
    assert hm.num_offdiagonals(hm.address) == 10
    a, v = hm.get_offdiagonal(hm.address, 3)
    assert a.onr() == (2, 1, 3) and v == 1.0
