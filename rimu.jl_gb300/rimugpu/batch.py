"""Many FCIQMC runs stepped together on one GPU (librimu_gpu rimu_batch_*).

The reference runs the replicas of a ProjectorMonteCarloProblem one after another
(pmc_simulation.jl:288-290) and different Hamiltonians as separate problems.
`BatchedReplicas` steps them in one launch per kernel, with the shift update on the device and
segments of steps replayed as CUDA graphs; `solve_batched` takes a list of
ProjectorMonteCarloProblem and returns one simulation-like result per problem, with the same
report columns as `solve`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .problem import DoubleLogUpdate, DontUpdate, ProjectedEnergy, Report

STAT_FIELDS = [f for f, _ in _lib.BatchStats._fields_]


def _u64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


class BatchedReplicas:
    """`hamiltonians[r]` with start vector `starts[r]` (dict address => value), initial shift
    `shifts[r]` and target walker number `targets[r]`.  Replica r draws its random numbers with
    key (seed, r), so its steps equal those of `apply_operator` with `wm.replica = r`."""

    def __init__(self, hamiltonians, style, time_step, targets, starts=None, shifts=None,
                 seed=0, projectors=None, zeta=0.08, xi=None, shift_update=True,
                 segment_steps=64, use_graph=True, autotune=True, launch_shape=None,
                 population=10, annihilation=None):
        self.hamiltonians = list(hamiltonians)
        if any(H.address.nbits > 64 for H in self.hamiltonians):
            raise ValueError("batched runs take addresses of at most 64 bits")
        self.nrep = len(self.hamiltonians)
        self.style = style
        self.time_step = float(time_step)
        self.targets = [float(t) for t in (targets if np.ndim(targets) else [targets] * self.nrep)]
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.zeta = float(zeta)
        self.xi = self.zeta ** 2 / 4 if xi is None else float(xi)
        self.shift_update = bool(shift_update)
        self.segment_steps, self.use_graph, self.autotune = int(segment_steps), bool(use_graph), bool(autotune)
        self.step = 0
        lib = _lib.load()
        self._ctx = _lib.default_context()
        h = C.c_void_p()
        vk = _lib.VAL_I64 if style.valtype is int else _lib.VAL_F64
        _lib.check(lib.rimu_batch_create(self._ctx.handle, self.nrep, vk, C.byref(h)))
        self.handle = h
        self._keep = []
        for r, H in enumerate(self.hamiltonians):
            st = starts[r] if starts is not None else {H.starting_address(): population}
            st = dict(st)
            keys = np.ascontiguousarray([a.key for a in st], dtype=np.uint64)
            vals = np.ascontiguousarray(list(st.values()),
                                        dtype=np.int64 if style.valtype is int else np.float64)
            if shifts is not None:
                s0 = float(shifts[r])
            elif len(st) == 1:
                s0 = H.diagonal_element(next(iter(st)))
            else:
                raise ValueError("give `shifts` for start vectors with more than one address")
            _lib.check(lib.rimu_batch_set_replica(h, r, H.handle, _u64p(keys),
                                                  vals.ctypes.data_as(C.c_void_p), len(keys),
                                                  s0, self.targets[r]))
            if projectors is not None and projectors[r] is not None:
                pe = projectors[r]
                pk = np.ascontiguousarray(pe.keys, dtype=np.uint64)
                pv = np.ascontiguousarray(pe.pvals, dtype=np.float64)
                ph = np.ascontiguousarray(pe.hpvals, dtype=np.float64)
                _lib.check(lib.rimu_batch_set_projector(
                    h, r, _u64p(pk), pv.ctypes.data_as(C.POINTER(C.c_double)),
                    ph.ctypes.data_as(C.POINTER(C.c_double)), len(pk)))
        if launch_shape is not None:
            _lib.check(lib.rimu_batch_set_launch_shape(h, int(launch_shape[0]), int(launch_shape[1])))
        if annihilation is not None:
            m = {"hash": _lib.ANN_HASH, "sort": _lib.ANN_SORT}[annihilation]
            _lib.check(lib.rimu_batch_set_annihilation(h, m))

    def _params(self):
        p = _lib.BatchParams()
        sp = self.style.params()
        p.style = sp["style"]
        p.dt = self.time_step
        p.boost = 1.0
        p.proj_threshold = sp["proj_threshold"]
        p.compression = sp["compression"]
        p.rel_spawning_threshold = sp["rel_spawning_threshold"]
        p.abs_spawning_threshold = sp["abs_spawning_threshold"]
        p.seed = self.seed
        p.shift_update = int(self.shift_update)
        p.zeta, p.xi = self.zeta, self.xi
        p.segment_steps = self.segment_steps
        p.use_graph = int(self.use_graph)
        p.autotune = int(self.autotune)
        return p

    def run(self, nsteps: int) -> dict:
        """Advance every replica by `nsteps` steps; returns a dict of arrays of shape
        (nsteps, nrep), one per field of rimu_batch_stats."""
        out = (_lib.BatchStats * max(nsteps * self.nrep, 1))()
        p = self._params()
        _lib.check(_lib.load().rimu_batch_run(self.handle, C.byref(p), self.step, nsteps,
                                              C.cast(out, C.c_void_p)))
        self.step += nsteps
        rec = np.ctypeslib.as_array(out)[: nsteps * self.nrep]
        return {f: np.array(rec[f]).reshape(nsteps, self.nrep) for f in STAT_FIELDS}

    def download(self, r: int):
        """(keys, values) of replica r, in bucket order."""
        lib = _lib.load()
        n = C.c_int64()
        cap = 1 << 16
        while True:
            keys = np.zeros(cap, dtype=np.uint64)
            vals = np.zeros(cap, dtype=np.int64 if self.style.valtype is int else np.float64)
            rc = lib.rimu_batch_download(self.handle, r, _u64p(keys), vals.ctypes.data_as(C.c_void_p),
                                         cap, C.byref(n))
            if rc == 0:
                return keys[: n.value], vals[: n.value]
            if n.value > cap:
                cap = n.value
                continue
            _lib.check(rc)

    def sorted_arrays(self, r: int):
        k, v = self.download(r)
        o = np.argsort(k, kind="stable")
        return k[o], v[o]

    def info(self) -> dict:
        out = np.zeros(8)
        _lib.check(_lib.load().rimu_batch_info(self.handle, out.ctypes.data_as(C.POINTER(C.c_double))))
        mode = C.c_int()
        _lib.check(_lib.load().rimu_batch_annihilation(self.handle, C.byref(mode)))
        return dict(keys_per_bucket=int(out[0]), table_slots=int(out[1]), buckets=int(out[2]),
                    graph_segments=int(out[3]), eager_segments=int(out[4]), retries=int(out[5]),
                    kernel_ms=float(out[6]), steps=int(out[7]),
                    annihilation="sort" if mode.value == _lib.ANN_SORT else "hash")

    def __del__(self):
        try:
            if self.handle:
                _lib.load().rimu_batch_destroy(self.handle)
        except Exception:
            pass


class BatchedResult:
    """What `solve` returns for one problem of a batch: the report columns (`df`) and the
    final walker list."""

    def __init__(self, problem, report, batch, r):
        self.problem, self.report, self._batch, self._r = problem, report, batch, r
        self.success = True
        self.aborted = False
        self.message = ""

    @property
    def df(self):
        return self.report.columns()

    def state_vector(self):
        return self._batch.sorted_arrays(self._r)


def solve_batched(problems, segment_steps=64, use_graph=True, autotune=True, launch_shape=None,
                  annihilation=None):
    """solve(problem) for each problem of the list, all stepped together (one replica each).
    The problems must share the style, time step, step range and shift strategy
    (DoubleLogUpdate or DontUpdate), and their Hamiltonians the lattice (u may differ)."""
    p0 = problems[0]
    for p in problems:
        if (type(p.style) is not type(p0.style) or p.style.params() != p0.style.params() or
                p.time_step != p0.time_step or p.last_step != p0.last_step or
                p.starting_step != p0.starting_step or p.n_replicas != 1):
            raise ValueError("batched problems need the same style, time step and step range, "
                             "one replica each")
    strat = p0.shift_strategy
    if not isinstance(strat, (DoubleLogUpdate, DontUpdate)) or type(strat) not in (DoubleLogUpdate, DontUpdate):
        raise ValueError("batched runs support DoubleLogUpdate and DontUpdate shift strategies")
    starts, shifts, projs = [], [], []
    for p in problems:
        sa = p.start_at
        st = dict(sa) if isinstance(sa, dict) else {sa: (int(p.population) if p.style.valtype is int
                                                          else float(p.population))}
        starts.append(st)
        if p.shift is not None:
            shifts.append(float(p.shift))
        elif len(st) == 1:
            shifts.append(p.hamiltonian.diagonal_element(next(iter(st))))
        else:
            from .dvec import GPUDVec, dot_operator
            v = GPUDVec(st, style=p.style)
            k, vals = v.download()
            shifts.append(dot_operator(v, p.hamiltonian, v) / float(np.dot(vals.astype(float), vals.astype(float))))
        pe = [s for s in p.post_step_strategy if isinstance(s, ProjectedEnergy)]
        projs.append(pe[0] if pe else None)
    zeta = getattr(strat, "ζ", 0.08)
    xi = getattr(strat, "ξ", zeta ** 2 / 4)
    b = BatchedReplicas([p.hamiltonian for p in problems], p0.style, p0.time_step,
                        [getattr(p.shift_strategy, "target_walkers", 1000) for p in problems],
                        starts=starts, shifts=shifts, seed=p0.random_seed, projectors=projs,
                        zeta=zeta, xi=xi, shift_update=isinstance(strat, DoubleLogUpdate),
                        segment_steps=segment_steps, use_graph=use_graph, autotune=autotune,
                        launch_shape=launch_shape, annihilation=annihilation)
    b.step = p0.starting_step
    nsteps = p0.last_step - p0.starting_step
    res = b.run(nsteps)
    names = p0.style.step_stat_names() + p0.style.compression_names()
    out = []
    steps = np.arange(p0.starting_step + 1, p0.last_step + 1)
    for r, p in enumerate(problems):
        rep = Report()
        rep.data["step"] = list(steps)
        rep.data["len"] = list(res["len"][:, r])
        rep.data["shift"] = list(res["shift"][:, r])
        rep.data["norm"] = list(res["norm"][:, r])
        for n in names:
            rep.data[n] = list(res[n][:, r])
        if projs[r] is not None:
            rep.data[projs[r].vproj_name] = list(res["vproj"][:, r])
            rep.data[projs[r].hproj_name] = list(res["hproj"][:, r])
        out.append(BatchedResult(p, rep, b, r))
    return out
