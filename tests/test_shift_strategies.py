"""The shift strategies of the host step loop (src/strategies_and_params/shiftstrategy.jl)
against their formulas, on the host: the shift update after a step with walker number N
(tnorm) from N_prev (pnorm), time step dτ.  CPU only (the projections of DoubleLogProjected
come from a stand-in vector with the GPU list's dot(dict) method)."""
import math

import pytest

import rimugpu as R
from rimugpu.problem import DefaultShiftParameters


class FakeList:
    """Stands in for a GPUDVec: dot(dict) = sum over the dict's addresses."""

    def __init__(self, values):
        self.values = values

    def dot(self, proj):
        return float(sum(self.values.get(k, 0.0) * p for k, p in proj.items()))


def params(shift=-2.0, pnorm=900.0, dt=1e-3):
    return DefaultShiftParameters(shift, pnorm, dt)


def test_double_log_update():
    """shiftstrategy.jl:174-181: S -= ξ/dτ ln(N/N_t) + ζ/dτ ln(N/N_prev)."""
    sp = params()
    s = R.DoubleLogUpdate(target_walkers=1000, ζ=0.08)
    stats, ok = s.update(sp, 950.0)
    want = -2.0 - (0.08 ** 2 / 4 / 1e-3 * math.log(950 / 1000) + 0.08 / 1e-3 * math.log(950 / 900))
    assert ok and sp.shift == want and sp.pnorm == 950.0 and stats["shift"] == want


def test_log_update_and_after_target():
    """shiftstrategy.jl:100-145: LogUpdate always, LogUpdateAfterTargetWalkers once the walker
    number has passed the target (and from then on)."""
    sp = params()
    R.LogUpdate(ζ=0.1).update(sp, 950.0)
    assert sp.shift == -2.0 - 0.1 / 1e-3 * math.log(950 / 900)
    sp = params()
    s = R.LogUpdateAfterTargetWalkers(target_walkers=1000, ζ=0.1)
    s.update(sp, 950.0)
    assert sp.shift == -2.0 and not sp.shift_mode and sp.pnorm == 950.0
    s.update(sp, 1100.0)
    assert sp.shift_mode and sp.shift == -2.0 - 0.1 / 1e-3 * math.log(1100 / 950)
    s.update(sp, 990.0)                        # stays in shift mode below the target
    assert sp.shift_mode


def test_double_log_projected():
    """shiftstrategy.jl:280-300: S -= ξ/dτ ln(P·ψ_new/target) + ζ/dτ ln(P·ψ_new/P·ψ_old), with
    the projections reported as tp and pp."""
    P = {11: 1.0, 12: 0.5}
    new = FakeList({11: 40.0, 12: 20.0, 13: 5.0})
    old = FakeList({11: 38.0, 12: 22.0})
    sp = params()
    s = R.DoubleLogProjected(target=45.0, projector=P, ζ=0.08)
    stats, ok = s.update(sp, 1000.0, new, old)
    tp, pp = 40.0 + 10.0, 38.0 + 11.0
    want = -2.0 - (0.08 ** 2 / 4 / 1e-3 * math.log(tp / 45.0) + 0.08 / 1e-3 * math.log(tp / pp))
    assert ok and sp.shift == want and stats["tp"] == tp and stats["pp"] == pp
    assert sp.pnorm == 1000.0
    assert getattr(s, "needs_vectors", False)


def test_dont_update():
    sp = params()
    stats, ok = R.DontUpdate(target_walkers=1000).update(sp, 950.0)
    assert sp.shift == -2.0 and ok
    _, ok = R.DontUpdate(target_walkers=1000).update(sp, 1200.0)
    assert not ok                               # DontUpdate stops the run past the target
