"""Shared helpers for the GPU parity tests: build matching oracle models, run one step on
both sides with the same seed/step, compare exactly."""
import numpy as np

import oracle as O
import rimugpu as R


def oracle_model(h):
    if isinstance(h, R.HubbardReal1D):
        return O.real1d(h.N, h.M, h.u, h.t)
    if isinstance(h, R.HubbardMom1D):
        m = O.mom1d(h.N, h.M, h.u, h.t)
        m.kes = np.array(h.kes)
        return m
    g = h.geometry
    return O.realspace(h.N, g.dims, u=h.u, t=h.t, periodic=g.fold,
                       fermion=isinstance(h.address, R.FermiFS), pot=h.potential)


STYLE_CODE = {R.IsStochasticInteger: O.STYLE_INTEGER, R.IsDeterministic: O.STYLE_DETERMINISTIC,
              R.IsDynamicSemistochastic: O.STYLE_DSS}


def oracle_params(style, dt, shift, seed, step, op=O.OP_TRANSITION, boost=1.0, replica=0,
                  initiator=None):
    sp = style.params()
    init = R.NonInitiator() if initiator is None else initiator
    return O.StepParams(STYLE_CODE[type(style)], dt=dt, shift=shift, seed=seed, step=step, op=op,
                        boost=boost, proj_threshold=sp["proj_threshold"],
                        compression=sp["compression"], rel_threshold=sp["rel_spawning_threshold"],
                        abs_threshold=sp["abs_spawning_threshold"], replica=replica,
                        init_rule=init.code, init_threshold=init.threshold)


def gpu_step(h, style, keys, vals, dt, shift, seed, step, boost=1.0, wm=None, initiator=None):
    src = R.GPUDVec(style=style, address_type=h.address, initiator=initiator)
    src.upload(keys, vals)
    dst = src.similar()
    wm = wm or R.GPUWorkingMemory(seed)
    wm.seed = seed
    names, stats, wm, dst = R.apply_operator(wm, dst, src, R.FirstOrderTransitionOperator(h, shift, dt),
                                             boost=boost, step=step)
    k, v = dst.sorted_arrays()
    return k, v, wm.last_stats


STAT_KEYS = ("norm", "len", "len_before", "exact_steps", "inexact_steps", "spawn_attempts",
             "spawns", "clones", "deaths", "zombies")


def assert_same_step(gpu, ora, style):
    gk, gv, gs = gpu
    ok, ov, os_ = ora
    assert len(gk) == len(ok), (len(gk), len(ok))
    assert np.array_equal(gk, ok)
    if isinstance(style, R.IsStochasticInteger):
        assert np.array_equal(gv, ov)
    else:
        assert np.array_equal(gv.view(np.uint64), ov.view(np.uint64)), \
            float(np.max(np.abs(gv - ov) / np.maximum(np.abs(ov), 1e-300)))
    for k in STAT_KEYS:
        assert gs[k] == os_[k], (k, gs[k], os_[k])
