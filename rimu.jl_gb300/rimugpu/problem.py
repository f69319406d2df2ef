"""ProjectorMonteCarloProblem / PMCSimulation / solve on the GPU walker list.

Host-side orchestration mirroring src/projector_monte_carlo_problem.jl, src/pmc_simulation.jl
and src/fciqmc.jl: every step calls apply_operator on the device, then updates the shift on
the host from the fused walkernumber_and_length.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .dvec import FirstOrderTransitionOperator, GPUDVec, GPUWorkingMemory, apply_operator
from .styles import IsDeterministic, IsDynamicSemistochastic, StochasticStyle


# ----------------------------------------------------------------------------------------
# Shift strategies (src/strategies_and_params/shiftstrategy.jl)
# ----------------------------------------------------------------------------------------
class DefaultShiftParameters:
    def __init__(self, shift, pnorm, time_step, counter=0, shift_mode=False):
        self.shift, self.pnorm, self.time_step = float(shift), float(pnorm), float(time_step)
        self.counter, self.shift_mode = counter, shift_mode


class DontUpdate:
    def __init__(self, target_walkers=1000):
        self.target_walkers = target_walkers

    def update(self, sp, tnorm):
        return {"shift": sp.shift, "norm": tnorm}, tnorm < self.target_walkers


class LogUpdate:
    def __init__(self, ζ=0.08):
        self.ζ = ζ

    def update(self, sp, tnorm):
        sp.shift -= self.ζ / sp.time_step * math.log(tnorm / sp.pnorm)
        sp.pnorm = tnorm
        return {"shift": sp.shift, "norm": tnorm}, True


class LogUpdateAfterTargetWalkers:
    def __init__(self, target_walkers=1000, ζ=0.08):
        self.target_walkers, self.ζ = target_walkers, ζ

    def update(self, sp, tnorm):
        if sp.shift_mode or tnorm > self.target_walkers:
            sp.shift_mode = True
            sp.shift -= self.ζ / sp.time_step * math.log(tnorm / sp.pnorm)
        sp.pnorm = tnorm
        return {"shift": sp.shift, "norm": tnorm, "shift_mode": sp.shift_mode}, True


class DoubleLogUpdate:
    """S -= ξ/dτ ln(N/N_target) + ζ/dτ ln(N/N_prev) (shiftstrategy.jl:161-181)."""

    def __init__(self, target_walkers=1000, ζ=0.08, ξ=None):
        self.target_walkers = target_walkers
        self.ζ = ζ
        self.ξ = ζ ** 2 / 4 if ξ is None else ξ

    def update(self, sp, tnorm):
        dτ = sp.time_step
        sp.shift -= self.ξ / dτ * math.log(tnorm / self.target_walkers) + \
            self.ζ / dτ * math.log(tnorm / sp.pnorm)
        sp.pnorm = tnorm
        return {"shift": sp.shift, "norm": tnorm}, True


class DoubleLogUpdateAfterTargetWalkers(DoubleLogUpdate):
    def update(self, sp, tnorm):
        if sp.shift_mode or tnorm > self.target_walkers:
            sp.shift_mode = True
            dτ = sp.time_step
            sp.shift -= self.ξ / dτ * math.log(tnorm / self.target_walkers) + \
                self.ζ / dτ * math.log(tnorm / sp.pnorm)
        sp.pnorm = tnorm
        return {"shift": sp.shift, "norm": tnorm, "shift_mode": sp.shift_mode}, True


class DoubleLogProjected:
    """S -= ξ/dτ ln(P·ψ_new / target) + ζ/dτ ln(P·ψ_new / P·ψ_old) with a fixed projector P
    (shiftstrategy.jl:280-300); P is a dict address => value, its dot products with the
    device lists are lookups of P's addresses."""

    needs_vectors = True

    def __init__(self, target, projector, ζ=0.08, ξ=None):
        self.target = float(target)
        self.projector = dict(projector)
        self.ζ = ζ
        self.ξ = ζ ** 2 / 4 if ξ is None else ξ

    def update(self, sp, tnorm, v_new=None, v_old=None):
        dτ = sp.time_step
        tp = v_new.dot(self.projector)
        pp = v_old.dot(self.projector)
        sp.shift -= self.ξ / dτ * math.log(tp / self.target) + self.ζ / dτ * math.log(tp / pp)
        sp.pnorm = tnorm
        return {"shift": sp.shift, "norm": tnorm, "tp": tp, "pp": pp}, True


# ----------------------------------------------------------------------------------------
# Post-step strategies
# ----------------------------------------------------------------------------------------
class ProjectedEnergy:
    """ProjectedEnergy(hamiltonian, projector) (poststepstrategy.jl:82-121): reports
    vproj = <P|v> and hproj = <H'P|v>; both dot products are fused into the step kernel."""

    def __init__(self, hamiltonian, projector, vproj="vproj", hproj="hproj"):
        self.hamiltonian = hamiltonian
        if isinstance(projector, GPUDVec):
            projector = projector.to_dict()
        elif isinstance(projector, tuple):
            projector = {projector[0]: projector[1]}
        self.projector = {a: float(v) for a, v in dict(projector).items()}
        self.vproj_name, self.hproj_name = vproj, hproj
        # compute_hproj: H' * P for a Hermitian H (poststepstrategy.jl:106-108)
        hp = {}
        for a, p in self.projector.items():
            hp[a.key] = hp.get(a.key, 0.0) + hamiltonian.diagonal_element(a) * p
            ks, vs = hamiltonian.offdiagonal_keys(a.key)
            for k, h in zip(ks, vs):
                if h != 0.0:
                    hp[int(k)] = hp.get(int(k), 0.0) + h * p
        keys = sorted(set(hp) | {a.key for a in self.projector})
        pv = {a.key: v for a, v in self.projector.items()}
        # addresses of 65-128 bits stay Python ints
        self.key_words = 2 if hamiltonian.address.nbits > 64 else 1
        self.keys = np.array(keys, dtype=object if self.key_words == 2 else np.uint64)
        self.pvals = np.array([pv.get(k, 0.0) for k in keys])
        self.hpvals = np.array([hp.get(k, 0.0) for k in keys])


class ReportDFAndInfo:
    def __init__(self, reporting_interval=1, info_interval=100, io=None, writeinfo=False):
        self.reporting_interval = reporting_interval
        self.info_interval = info_interval


class Report:
    """Column store of per-step results (reportingstrategy.jl:10-170)."""

    def __init__(self):
        self.data: dict[str, list] = {}
        self.meta: dict[str, str] = {}

    def add(self, name, value):
        self.data.setdefault(name, []).append(value)

    def columns(self):
        return {k: np.asarray(v) for k, v in self.data.items()}

    def __getitem__(self, k):
        return np.asarray(self.data[k])

    def __len__(self):
        return len(self.data.get("step", []))


# ----------------------------------------------------------------------------------------
# Replica strategies (replicastrategy.jl)
# ----------------------------------------------------------------------------------------
class NoStats:
    """NoStats(n_replicas) (replicastrategy.jl:53): replicas without cross statistics."""

    def __init__(self, n_replicas=1):
        self.n_replicas = n_replicas

    def replica_stats(self, vectors):
        return (), ()


class AllOverlaps:
    """AllOverlaps(n_replicas=2; operator=nothing, vecnorm=true) (replicastrategy.jl:112-190):
    for every pair i < j of replicas the overlap c{i}_dot_c{j} = dot(v_i, v_j) and, for each
    operator k, c{i}_Op{k}_c{j} = dot(v_i, op_k, v_j), all computed on the device."""

    def __init__(self, n_replicas=2, operator=None, vecnorm=True):
        if not isinstance(n_replicas, int):
            raise ValueError("n_replicas must be an integer")
        if operator is None:
            self.operators = ()
        elif isinstance(operator, (tuple, list)):
            self.operators = tuple(operator)
        else:
            self.operators = (operator,)
        self.n_replicas = n_replicas
        self.vecnorm = vecnorm

    def replica_stats(self, vectors):
        from .dvec import dot_operator
        names, values = [], []
        n = len(vectors)
        for i in range(n):
            for j in range(i + 1, n):
                if self.vecnorm:
                    names.append(f"c{i + 1}_dot_c{j + 1}")
                    values.append(vectors[i].dot(vectors[j]))
                for k, op in enumerate(self.operators):
                    names.append(f"c{i + 1}_Op{k + 1}_c{j + 1}")
                    values.append(dot_operator(vectors[i], op, vectors[j]))
        return tuple(names), tuple(values)


# ----------------------------------------------------------------------------------------
# Problem and simulation
# ----------------------------------------------------------------------------------------
class ProjectorMonteCarloProblem:
    """ProjectorMonteCarloProblem(hamiltonian; kwargs...) (projector_monte_carlo_problem.jl:
    150-290), with the same keyword defaults."""

    def __init__(self, hamiltonian, n_replicas=1, start_at=None, shift=None,
                 style: StochasticStyle | None = None, time_step=0.01, starting_step=0,
                 last_step=100, wall_time=math.inf, target_walkers=1000, ζ=0.08, ξ=None,
                 shift_strategy=None, reporting_strategy=None, post_step_strategy=(),
                 max_length=None, random_seed=True, population=10, replica_strategy=None,
                 initiator=False):
        self.hamiltonian = hamiltonian
        if replica_strategy is None:
            replica_strategy = NoStats(n_replicas)
        elif replica_strategy.n_replicas != n_replicas and n_replicas != 1:
            raise ValueError("n_replicas does not match the replica strategy")
        n_replicas = replica_strategy.n_replicas
        self.replica_strategy = replica_strategy
        self.n_replicas = n_replicas
        self.start_at = start_at if start_at is not None else hamiltonian.starting_address()
        self.shift = shift
        self.style = style if style is not None else IsDynamicSemistochastic()
        self.time_step = float(time_step)
        self.starting_step = starting_step
        self.last_step = last_step
        self.wall_time = wall_time
        ξ = ζ ** 2 / 4 if ξ is None else ξ
        self.shift_strategy = shift_strategy or DoubleLogUpdate(target_walkers, ζ, ξ)
        self.reporting_strategy = reporting_strategy or ReportDFAndInfo()
        if not isinstance(post_step_strategy, (tuple, list)):
            post_step_strategy = (post_step_strategy,)
        self.post_step_strategy = tuple(post_step_strategy)
        tw = getattr(self.shift_strategy, "target_walkers", target_walkers)
        self.max_length = max_length if max_length is not None else round(2 * abs(tw) + 100)
        if random_seed is True:
            random_seed = int.from_bytes(np.random.default_rng().bytes(8), "little")
        elif random_seed is False:
            random_seed = 0
        self.random_seed = int(random_seed) & 0xFFFFFFFFFFFFFFFF
        self.population = population
        from .initiators import initiator_rule
        self.initiator = initiator_rule(initiator)


class SingleState:
    def __init__(self, hamiltonian, v, pv, wm, sp, id=""):
        self.hamiltonian, self.v, self.pv, self.wm, self.shift_parameters, self.id = \
            hamiltonian, v, pv, wm, sp, id


class PMCSimulation:
    """PMCSimulation (pmc_simulation.jl:22-174)."""

    def __init__(self, problem: ProjectorMonteCarloProblem, copy_vectors=True):
        self.problem = problem
        self.report = Report()
        self.modified = self.aborted = self.success = False
        self.message = ""
        self.elapsed_time = 0.0
        self.step = problem.starting_step
        H = problem.hamiltonian
        self.states = []
        pe = [s for s in problem.post_step_strategy if isinstance(s, ProjectedEnergy)]
        for r in range(problem.n_replicas):
            v = self._starting_vector(problem, copy_vectors)
            pv = v.similar()
            wm = GPUWorkingMemory(problem.random_seed)
            wm.replica = r
            if pe:
                wm.set_projector(pe[0].keys, pe[0].pvals, pe[0].hpvals, key_words=pe[0].key_words)
            if problem.shift is None:
                shift = self._initial_shift(H, v)
            else:
                shift = float(problem.shift)
            tnorm, _ = v.walkernumber_and_length()
            sp = DefaultShiftParameters(shift, tnorm, problem.time_step)
            suffix = "" if problem.n_replicas == 1 else f"_{r + 1}"
            self.states.append(SingleState(H, v, pv, wm, sp, suffix))

    @staticmethod
    def _starting_vector(problem, copy_vectors):
        sa = problem.start_at
        if isinstance(sa, GPUDVec):
            return sa.copy() if copy_vectors else sa
        if isinstance(sa, dict):
            return GPUDVec(sa, style=problem.style, initiator=problem.initiator)
        val = problem.population
        return GPUDVec({sa: int(val) if problem.style.valtype is int else float(val)},
                       style=problem.style, initiator=problem.initiator)

    @staticmethod
    def _initial_shift(H, v: GPUDVec) -> float:
        """dot(v, H, v) / dot(v, v) (fciqmc.jl:51-61)."""
        k, vals = v.download()
        vals = vals.astype(float)
        if len(k) == 1:
            return H.diagonal_element(v._addr(k[0]))
        from .dvec import dot_operator
        return dot_operator(v, H, v) / float(np.dot(vals, vals))

    # ---- stepping ----------------------------------------------------------------------
    def _advance(self, s: SingleState) -> bool:
        p = self.problem
        sp = s.shift_parameters
        op = FirstOrderTransitionOperator(s.hamiltonian, sp.shift, sp.time_step)
        names, stats, wm, pv = apply_operator(s.wm, s.pv, s.v, op, step=self.step)
        s.v, s.pv = pv, s.v
        full = s.wm.last_stats
        tnorm, length = full["norm"], full["len"]
        if not length:
            shift_stats, proceed = {"shift": sp.shift, "norm": tnorm}, True
        elif getattr(p.shift_strategy, "needs_vectors", False):
            shift_stats, proceed = p.shift_strategy.update(sp, tnorm, s.v, s.pv)
        else:
            shift_stats, proceed = p.shift_strategy.update(sp, tnorm)
        if self.step % p.reporting_strategy.reporting_interval == 0:
            rep = self.report
            rep.add("len" + s.id, length)
            for k, val in shift_stats.items():
                rep.add(k + s.id, val)
            for n, val in zip(names, stats):
                rep.add(n + s.id, val)
            for pe in p.post_step_strategy:
                if isinstance(pe, ProjectedEnergy):
                    rep.add(pe.vproj_name + s.id, full["vproj"])
                    rep.add(pe.hproj_name + s.id, full["hproj"])
        if length == 0:
            self.message = f"Population in state {s.id} is dead. Aborting."
            return False
        if length > p.max_length:
            self.message = f"`max_length` reached in state {s.id}. Aborting."
            return False
        return proceed

    def step_(self):
        """step!(sm) (pmc_simulation.jl:265-310)."""
        if self.aborted or self.success or self.step >= self.problem.last_step:
            return self
        self.step += 1
        if self.step % self.problem.reporting_strategy.reporting_interval == 0:
            self.report.add("step", self.step)
        proceed = True
        for s in self.states:
            proceed &= self._advance(s)
        if self.step % self.problem.reporting_strategy.reporting_interval == 0:
            names, values = self.problem.replica_strategy.replica_stats([s.v for s in self.states])
            for n, val in zip(names, values):
                self.report.add(n, val)
        self.modified = True
        if not proceed:
            self.aborted = True
            self.message = self.message or f"Aborted in step {self.step}."
            return self
        if self.step == self.problem.last_step:
            self.success = True
        return self

    def solve_(self, last_step=None, wall_time=None):
        """solve!(sm; last_step, wall_time) (pmc_simulation.jl:350-452)."""
        if last_step is not None:
            self.problem.last_step = last_step
            self.aborted = self.success = False
        if wall_time is not None:
            self.problem.wall_time = wall_time
        start = time.time() - self.elapsed_time
        while not self.aborted and not self.success:
            if time.time() - start > self.problem.wall_time:
                self.aborted = True
                self.message = "Wall time limit reached."
                break
            self.step_()
        self.elapsed_time = time.time() - start
        return self

    def DataFrame(self):
        return self.report.columns()

    @property
    def df(self):
        return self.DataFrame()

    def state_vectors(self):
        return [s.v for s in self.states]


def init(problem: ProjectorMonteCarloProblem, copy_vectors=True) -> PMCSimulation:
    return PMCSimulation(problem, copy_vectors)


def solve(problem: ProjectorMonteCarloProblem) -> PMCSimulation:
    return init(problem).solve_()
