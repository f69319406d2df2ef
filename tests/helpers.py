"""Shared helpers for the GPU parity tests: build matching oracle models, run one step on
both sides with the same seed/step, compare exactly."""
import math

import numpy as np

import oracle as O
import rimugpu as R


def oracle_model(h):
    if isinstance(h, R.HubbardReal1D):
        return O.real1d(h.N, h.M, h.u, h.t)
    if isinstance(h, R.HubbardMom1D):
        if isinstance(h.address, R.CompositeFS):
            a, b = h.address.components
            m = O.mom1d_2c(a.N, b.N, h.M, h.u, h.t)
        else:
            m = O.mom1d(h.N, h.M, h.u, h.t)
        m.kes = np.array(h.kes)
        return m
    g = h.geometry
    if isinstance(h.address, R.CompositeFS):
        comps = tuple((isinstance(c, R.FermiFS), c.N) for c in h.address.components)
        pot = None if h.potential is None else np.asarray(h.potential).reshape(len(comps), h.M)
        return O.realspace_multi(comps, g.dims, t=h.t, u=h.u, periodic=g.fold, pot=pot)
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


def oracle_mem_budget():
    """Bytes the threaded oracle may hold for one step's contributions: a third of the
    memory available, at most 48 GB."""
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    return min(48e9, int(ln.split()[1]) * 1024 / 3)
    except OSError:
        pass
    return 8e9


def popcount64(x):
    """Number of set bits of each element of a uint64 array."""
    x = np.ascontiguousarray(x, dtype=np.uint64)
    table = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)
    return table[x.view(np.uint8)].reshape(-1, 8).sum(axis=1)


def run_trajectory(h, style, start, steps, dt, shift=None, boost=1.0, target=None, seed=0x5EED,
                   threaded=False, wm=None):
    """`steps` steps from `start` on the GPU and in the oracle, compared after every step;
    with `target`, DoubleLogUpdate on the (identical) norm.  `threaded` follows the GPU with
    the oracle's multi-threaded step (the same results, faster on large lists)."""
    m = oracle_model(h)
    wide = h.address.nbits > 64     # two-chunk addresses travel as Python ints
    if isinstance(start, tuple):    # (keys, values) arrays; needs `shift`
        keys, vals = start
        S = float(shift)
    else:
        keys = np.array([a.key for a in start], dtype=object if wide else np.uint64)
        vals = np.array(list(start.values()), dtype=np.int64 if style.valtype is int else np.float64)
        S = h.diagonal_element(next(iter(start))) if shift is None else shift
    pnorm = float(np.abs(vals).sum())
    wm = wm or R.GPUWorkingMemory(seed)
    ostep = (lambda *a: O.step_mt(*a, mem_budget=oracle_mem_budget())) if threaded else O.step
    for step in range(1, steps + 1):
        g = gpu_step(h, style, keys, vals, dt, S, seed, step, boost=boost, wm=wm)
        o = ostep(m, oracle_params(style, dt, S, seed, step, boost=boost), keys, vals)
        assert_same_step(g, o, style)
        keys, vals = o[0], o[1]
        if len(keys) == 0:
            break
        if target is not None:   # DoubleLogUpdate on the (identical) norm
            tn = o[2]["norm"]
            S -= 0.08 ** 2 / 4 / dt * math.log(tn / target) + 0.08 / dt * math.log(tn / pnorm)
            pnorm = tn
    return keys, vals


def oracle_solve(m, style, start_key, population, steps, dt, target, seed, zeta=0.08,
                 initiator=None):
    """The host loop of solve (pmc_simulation.jl:265-310; advance!, fciqmc.jl:126-181) run on
    the oracle's step: one start address with `population` walkers, the initial shift its
    diagonal element, DoubleLogUpdate (shiftstrategy.jl:174-181) after every step, an optional
    initiator rule, and a ProjectedEnergy onto the start address (poststepstrategy.jl:82-121)
    whose frozen H P is the start's diagonal element and offdiagonals.  Same step numbers,
    seed and shift arithmetic as the package's solve, so it is the CPU run of the same
    trajectory.  Returns the report columns shift, vproj and hproj."""
    hp = {int(start_key): O.diagonal(m, start_key)}
    for nk, hv in O.offdiagonals(m, start_key):
        hp[nk] = hp.get(nk, 0.0) + hv
    hp_keys = np.array(sorted(hp), dtype=np.uint64)
    hp_vals = np.array([hp[int(k)] for k in hp_keys])
    integer = style.valtype is int
    keys = np.array([start_key], dtype=np.uint64)
    vals = np.array([population], dtype=np.int64 if integer else np.float64)
    S, pnorm = float(O.diagonal(m, start_key)), float(abs(population))
    xi = zeta ** 2 / 4
    out = {"shift": [], "vproj": [], "hproj": []}
    for step in range(1, steps + 1):
        keys, vals, st = O.step(m, oracle_params(style, dt, S, seed, step, initiator=initiator),
                                keys, vals)
        tn = st["norm"]
        if len(keys):
            S -= xi / dt * math.log(tn / target) + zeta / dt * math.log(tn / pnorm)
            pnorm = tn
        out["shift"].append(S)
        pos = np.minimum(np.searchsorted(keys, hp_keys), max(len(keys) - 1, 0))
        hit = (keys[pos] == hp_keys) if len(keys) else np.zeros(len(hp_keys), bool)
        out["hproj"].append(float(np.sum(hp_vals[hit] * vals[pos[hit]])))
        j = np.searchsorted(keys, np.uint64(start_key))
        out["vproj"].append(float(vals[j]) if j < len(keys) and keys[j] == start_key else 0.0)
        if len(keys) == 0:
            break
    return out
