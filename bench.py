#!/usr/bin/env python
"""FCIQMC walker-steps/s on one GB300 (plus matrix-free H*v nonzeros/s).

Workload (default): the large plain FCIQMC configuration -- HubbardReal1D, periodic, M = N = 20
(BoseFS in 39 bits of one 64-bit word), u = 4, t = 1, IsDynamicSemistochastic with threshold
1.0 (late ThresholdCompression), target walker norm 1e8, dt = 1e-3, DoubleLogUpdate, seed
0x5EED.  The population is grown from the unit-filling start address and equilibrated for
2 000 untimed steps in all (the configuration's equilibration), then W warm-up steps and K
timed steps are run through rimu_apply_operator.

A "step" is one projector step of the whole walker list (spawn, annihilation, compression,
norm).  value = sum over timed steps of the walker number (1-norm) / device time.  The walker
list (~1e8 walkers, 16-byte records, > 1 GB) is far larger than L2, so no L2 flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "rimu.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "FCIQMC walker-steps/s & H·v nnz/s on 1 GB300; batched/adjoint vs plain, same err"
UNIT = "walker-steps/s"
WORKLOAD = "HubbardReal1D M=N=20 u=4 t=1, IsDynamicSemistochastic(threshold=1), target norm 1e8, dt=1e-3"


# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one k_spawn plus one
# k_ann_warp launch per algorithmic byte (16-byte records read and written), measured at an
# equilibrated norm of 3e7: (568.6 + 571.6 + 864.2 + 358.4) MB / (830 + 1211) MB.
TRAFFIC_PER_ALGORITHMIC_BYTE = (568.6 + 571.6 + 864.2 + 358.4) / (830.0 + 1211.0)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, backend):
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
        return dist
    return None


def reduce_over_ranks(dist, ms, walker_steps, device):
    """Whole-job figures of independent replicas, one per rank: the slowest rank's time and
    the walker-steps of all ranks."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([float(walker_steps)], dtype=torch.float64, device=device)
    dist.all_reduce(w)
    return float(t.item()), float(w.item())


# --------------------------------------------------------------------------------------------
# CPU baseline: the oracle's threaded step (the PDVec step restated in C with OpenMP) on one
# shared walker list, all host cores
# --------------------------------------------------------------------------------------------
def cpu_steps(keys, vals, shift, seconds, min_steps=1, max_steps=10 ** 9, target=None,
              pnorm=None, step0=1, seed=0x5EED):
    """Steps the walker list (keys, vals) with the oracle's threaded step (all host threads)
    until `seconds` have passed (at least `min_steps`, at most `max_steps`), with
    DoubleLogUpdate towards `target` when given.  Returns (walker-steps/s over the steps,
    steps, seconds, final keys, vals, shift, norm)."""
    import numpy as np
    import oracle as O
    m = O.real1d(20, 20, 4.0, 1.0)
    dt = 1e-3
    S = shift
    pn = float(np.abs(vals).sum()) if pnorm is None else pnorm
    walkers, elapsed, steps = 0.0, 0.0, 0
    k, v = keys, vals
    while steps < max_steps and (steps < min_steps or elapsed < seconds):
        p = O.StepParams(O.STYLE_DSS, dt=dt, shift=S, seed=seed, step=step0 + steps,
                         compression=1.0)
        t0 = time.perf_counter()
        k, v, st = O.step_mt(m, p, k, v, sort=False, bits=True, mem_budget=64e9)
        elapsed += time.perf_counter() - t0
        walkers += st["norm"]
        steps += 1
        if target is not None and st["len"]:
            S -= 0.08 ** 2 / 4 / dt * math.log(st["norm"] / target) + 0.08 / dt * math.log(st["norm"] / pn)
            pn = st["norm"]
    return walkers / max(elapsed, 1e-9), steps, elapsed, k, v, S, pn


# --------------------------------------------------------------------------------------------
# Our arm
# --------------------------------------------------------------------------------------------
def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    dist = dist_init(ws, "nccl" if ws > 1 else None)
    torch.cuda.set_device(local)
    if rank == 0:
        from rimugpu import _build
        _build.build()
    if dist:
        dist.barrier()
    import rimugpu as R

    target = args.target
    addr = R.near_uniform(R.BoseFS, 20, 20)
    H = R.HubbardReal1D(addr, u=4.0, t=1.0)
    style = R.IsDynamicSemistochastic(threshold=1.0)
    dt = 1e-3
    p = R.ProjectorMonteCarloProblem(H, style=style, time_step=dt, target_walkers=target,
                                     last_step=10 ** 9, random_seed=0x5EED + rank,
                                     max_length=int(2 * target + 100))
    sim = R.init(p)
    s = sim.states[0]
    if args.shape:
        kpb, slots = (int(x) for x in args.shape.split(","))
        s.wm.set_launch_shape(kpb, slots)
    s.wm.set_annihilation(args.annihilation)
    t_prep = time.time()
    prep = 0
    # growth to the target norm, then equilibration: the list keeps spreading over the
    # Hilbert space (its length grows) long after the norm has reached the target
    while prep < args.max_prep:
        sim.step_()
        prep += 1
        if s.wm.last_stats["norm"] >= 0.9 * target and prep >= max(50, args.equil):
            break
    for _ in range(args.warmup):
        sim.step_()
    torch.cuda.synchronize()
    t_prep = time.time() - t_prep
    s.wm.set_timing(True)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    norms = []
    with ClockSampler(local) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            sim.step_()
            norms.append(s.wm.last_stats["norm"])
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = e0.elapsed_time(e1)
    tim = s.wm.timing()
    lens = list(sim.report.data["len"][-args.steps:])
    walker_steps = float(sum(norms))
    if dist:
        ms, walker_steps = reduce_over_ranks(dist, ms, walker_steps, "cuda")
    value = walker_steps / (ms / 1e3)

    # ---- roofline of spawn + annihilation (the hot path) ----
    peak, peak_kind = peaks()
    k_ms = tim["spawn_ms"] + tim["heavy_ms"] + tim["annihilate_ms"]
    k_bytes = tim["spawn_bytes"] + tim["annihilate_bytes"]
    steps_t = max(tim["steps"], 1)
    achieved = k_bytes / (k_ms / 1e3) / 1e9 if k_ms > 0 else 0.0
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": args.traffic if args.traffic is not None else
                round(TRAFFIC_PER_ALGORITHMIC_BYTE * k_bytes / steps_t),
                "traffic_source": "ncu dram bytes per algorithmic byte of k_spawn + k_ann_warp "
                                  "measured at an equilibrated norm of 3e7, scaled by this run's "
                                  "records per step" if args.traffic is None else "given",
                "peak_source": peak_kind,
                "kernel": "k_spawn + k_spawn_heavy + %s + k_annihilate (one step)"
                          % ("k_ann_sort" if args.annihilation == "sort" else "k_ann_warp"),
                "bytes_per_step": k_bytes / steps_t, "ms_per_step": k_ms / steps_t,
                "spawn": {"ms": tim["spawn_ms"] / steps_t,
                          "gbs": tim["spawn_bytes"] / (tim["spawn_ms"] / 1e3) / 1e9 if tim["spawn_ms"] else 0},
                "annihilate": {"ms": tim["annihilate_ms"] / steps_t,
                               "gbs": tim["annihilate_bytes"] / (tim["annihilate_ms"] / 1e3) / 1e9 if tim["annihilate_ms"] else 0},
                "heavy_ms": tim["heavy_ms"] / steps_t}

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    host_state = None
    if rank == 0 and not args.no_e2e:
        keys, vals = s.v.download()
        n = len(keys)
        hk = torch.empty(n, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
        hv = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        hk[:] = keys
        hv[:] = vals
        ok = torch.empty(max(n * 2, 1), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
        ov = torch.empty(max(n * 2, 1), dtype=torch.float64, pin_memory=True).numpy()
        sp = s.shift_parameters
        shift0, pnorm0 = sp.shift, sp.pnorm
        # The main run's device buffers go back to the library's memory pool, which keeps
        # them, so the timed region measures the copies and the steps rather than the first
        # mapping of fresh device memory (an allocation a long run makes once).
        host_state = (keys, vals, shift0)
        s.v = s.pv = s.wm = None
        __import__("gc").collect()
        torch.cuda.synchronize()
        t0 = time.time()
        v = R.GPUDVec(style=style, address_type=addr, capacity=n)
        v.upload(hk, hv)
        pv = v.similar()
        wm = R.GPUWorkingMemory(0x5EED + 77)
        e2e_norm = 0.0
        S, pn = shift0, pnorm0
        strat = p.shift_strategy
        from rimugpu.problem import DefaultShiftParameters
        spp = DefaultShiftParameters(S, pn, dt)
        for k in range(args.steps):
            R.apply_operator(wm, pv, v, R.FirstOrderTransitionOperator(H, spp.shift, dt), step=10 ** 6 + k)
            v, pv = pv, v
            st = wm.last_stats
            e2e_norm += st["norm"]
            strat.update(spp, st["norm"])
        got = __import__("ctypes").c_int64()
        import ctypes as C
        from rimugpu import _lib
        _lib.check(_lib.load().rimu_vec_download(v.handle, ok.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                  ov.ctypes.data_as(C.c_void_p), len(ok), C.byref(got)))
        torch.cuda.synchronize()
        wall = time.time() - t0
        from rimugpu._lib import StepParams, StepStats
        e2e = {"value": e2e_norm / wall, "unit": UNIT,
               "h2d_bytes_per_step": int((16 * n) / args.steps + C.sizeof(StepParams) + 8),
               "d2h_bytes_per_step": int((16 * got.value) / args.steps + 136 + 4 * 2),
               "how": "upload of the walker list from pinned host memory, K steps through "
                      "rimu_apply_operator (parameters in, statistics out every step), download "
                      "of the final list to pinned host memory; host wall clock; device buffers "
                      "from the library's memory pool, which holds those of the main run "
                      "(released before the timed region)"}

    # ---- matrix-free H*v on the full basis (M = N = 14, D = 20 058 300) ----
    hv_res = None
    if rank == 0 and not args.no_hv:
        hv_res = bench_hv(R, torch, peak, with_cpu=not args.no_cpu)

    # ---- the small and the momentum-space configurations ----
    c1_res = c3_res = None
    if rank == 0 and not args.no_configs:
        c1_res = bench_c1(R, torch)
        c3_res = bench_c3(R, torch)

    # ---- batched replicas (64 runs in one launch per kernel) ----
    batch_res = None
    if rank == 0 and not args.no_batch:
        batch_res = bench_batched(R, torch)

    # ---- CPU baseline: the threaded oracle step on this run's own list ----
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        import numpy as np
        if host_state is not None:          # the main run's list, downloaded for the e2e run
            keys, vals, shift_c = host_state
        else:
            keys, vals = s.v.download()
            shift_c = s.shift_parameters.shift
        import oracle
        oracle.build()
        thr, nsteps, secs, *_ = cpu_steps(keys, vals, shift_c, args.cpu_seconds, min_steps=1,
                                          max_steps=4, step0=10 ** 7)
        cpu = {"value": thr, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{nsteps} step(s) of the GPU run's own steady-state list ({len(keys)} "
                         f"entries, norm {float(np.abs(vals).sum()):.3g}) by the oracle's threaded "
                         f"step (PDVec restated in C/OpenMP, one shared list, "
                         f"{os.cpu_count()} threads), {secs:.1f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "target_walkers": target,
                       "walkers_per_step": walker_steps / args.steps / ws,
                       "entries_per_step": float(np.mean(lens)) if lens else None,
                       "prep_steps": prep, "prep_seconds": round(t_prep, 2),
                       "equilibration": f"{prep} untimed steps from the unit-filling start address",
                       "l2": "inputs larger than L2 (walker list > 1 GB), no flush",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                       "launch_shape": args.shape or "default (at most 448 contributions per bucket on "
                                       "average, one warp per bucket)",
                       "annihilation": args.annihilation},
            "gpu_launches": 4 * args.steps,
            "roofline": roofline,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "hv": hv_res,
            "batched": batch_res,
            "c1": c1_res,
            "c3": c3_res,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def bench_batched(R, torch, prep_steps=1200, batched_steps=256, seq_steps=32):
    """64 independent FCIQMC runs (HubbardRealSpace 4x4 periodic, N=16, U_i = 1 + 15 i/63,
    targets log-uniform in [1e4, 1e6], IsDynamicSemistochastic, dt = 1e-3) stepped together by
    rimu_batch_run, against the same 64 runs stepped one by one with rimu_apply_operator from
    the same equilibrated states.  walker-steps/s = sum over steps and replicas of the walker
    number / wall time (host included on both sides)."""
    import numpy as np
    nrep = 64
    geo = R.PeriodicBoundaries(4, 4)
    addr = R.BoseFS([1] * 16)
    us = [1.0 + 15.0 * i / 63 for i in range(nrep)]
    hs = [R.HubbardRealSpace(addr, geo, u=[[u]], t=[1.0]) for u in us]
    targets = list(10.0 ** np.random.default_rng(2024).uniform(4.0, 6.0, nrep))
    style = R.IsDynamicSemistochastic()
    dt = 1e-3
    b = R.BatchedReplicas(hs, style, dt, targets=targets, starts=[{addr: 10.0}] * nrep,
                          shifts=[0.0] * nrep, seed=0x5EED, segment_steps=64, use_graph=True,
                          autotune=True)
    t0 = time.time()
    b.run(prep_steps)
    t_prep = time.time() - t0
    torch.cuda.synchronize()
    info0 = b.info()
    t0 = time.time()
    res = b.run(batched_steps)
    wall_b = time.time() - t0
    info1 = b.info()
    walkers_b = float(res["norm"].sum())
    kernel_ms = info1["kernel_ms"] - info0["kernel_ms"]
    # the same runs one at a time with the plain step (host shift update, one sync per step)
    last_shift = res["shift"][-1]
    last_norm = res["norm"][-1]
    walkers_s, wall_s = 0.0, 0.0
    for r in range(nrep):
        k, v = b.download(r)
        src = R.GPUDVec(style=style, address_type=addr, capacity=len(k))
        src.upload(k, v)
        dst = src.similar()
        wm = R.GPUWorkingMemory(0x5EED)
        wm.replica = r
        sp = R.problem.DefaultShiftParameters(last_shift[r], last_norm[r], dt)
        strat = R.DoubleLogUpdate(targets[r])
        torch.cuda.synchronize()
        t0 = time.time()
        for s in range(seq_steps):
            R.apply_operator(wm, dst, src, R.FirstOrderTransitionOperator(hs[r], sp.shift, dt),
                             step=b.step + 1 + s)
            src, dst = dst, src
            tn = wm.last_stats["norm"]
            strat.update(sp, tn)
            walkers_s += tn
        torch.cuda.synchronize()
        wall_s += time.time() - t0
    value_b = walkers_b / wall_b
    value_s = walkers_s / wall_s
    return {"workload": "64 x HubbardRealSpace 4x4 periodic N=16, U_i = 1+15i/63, targets "
                        "log-uniform [1e4, 1e6], IsDynamicSemistochastic, dt=1e-3",
            "unit": "walker-steps/s", "value": value_b, "sequential_value": value_s,
            "batched_over_sequential": value_b / value_s,
            "walkers_per_step": walkers_b / batched_steps,
            "entries_per_step": float(res["len"].sum()) / batched_steps,
            "prep_steps": prep_steps, "prep_seconds": round(t_prep, 2),
            "batched_steps": batched_steps, "sequential_steps_per_replica": seq_steps,
            "batched_ms_per_step": wall_b / batched_steps * 1e3,
            "batched_kernel_ms_per_step": kernel_ms / batched_steps,
            "launch_shape": {"keys_per_bucket": info1["keys_per_bucket"],
                             "table_slots": info1["table_slots"], "buckets": info1["buckets"],
                             "autotuned": True},
            "graph_segments": info1["graph_segments"] - info0["graph_segments"],
            "rerun_segments": info1["retries"],
            "how": "batched: rimu_batch_run, segments of 64 steps replayed as CUDA graphs, shift "
                   "update on the device; sequential: rimu_apply_operator per replica and step "
                   "with the host DoubleLogUpdate; both from the same equilibrated states; equal "
                   "step counts give equal blocking error bars (the steps are the same process)"}


def bench_c1(R, torch):
    """The small plain configuration.  (a) The reference's published example
    (scripts/BHM-example.jl: HubbardReal1D(near_uniform(BoseFS{6,6}); u=6, t=1),
    IsDynamicSemistochastic, 1 000 target walkers, dt=1e-3, 3 000 steps, ProjectedEnergy onto
    the start vector), whose main computation the reference reports at 2.69 s on one process
    (docs/src/index.md:100-103): wall time of `solve` here, host loop included.  (b) The same
    Hamiltonian with IsStochasticInteger walkers for 20 000 steps: walker-steps/s through
    `solve`, and the shift and projected energy with blocking errors against E0 = -4.0215."""
    import numpy as np
    addr = R.near_uniform(R.BoseFS, 6, 6)
    H = R.HubbardReal1D(addr, u=6.0, t=1.0)
    out = {"workload": "HubbardReal1D M=N=6 u=6 t=1"}
    style = R.IsDynamicSemistochastic()
    start = {addr: 10.0}
    p = R.ProjectorMonteCarloProblem(H, start_at=start, style=style, last_step=3000,
                                     time_step=1e-3, target_walkers=1000, random_seed=0x5EED,
                                     post_step_strategy=R.ProjectedEnergy(H, start))
    R.solve(p)                                  # warm-up (first-use allocations)
    torch.cuda.synchronize()
    t0 = time.time()
    sim = R.solve(p)
    torch.cuda.synchronize()
    out["bhm_example_seconds"] = time.time() - t0
    out["bhm_example_reference_seconds"] = 2.69
    df = sim.report.data
    out["bhm_example_steps"] = len(df["shift"])
    out["bhm_example_shift"] = list(R.mean_and_se(np.asarray(df["shift"]), skip=1000))
    style = R.IsStochasticInteger()
    start = {addr: 10}
    p = R.ProjectorMonteCarloProblem(H, start_at=start, style=style, last_step=20000,
                                     time_step=1e-3, target_walkers=1000, random_seed=0x5EED + 1,
                                     post_step_strategy=R.ProjectedEnergy(H, start))
    torch.cuda.synchronize()
    t0 = time.time()
    sim = R.solve(p)
    torch.cuda.synchronize()
    wall = time.time() - t0
    df = sim.report.data
    norms = np.asarray(df["norm"], dtype=float)
    out["c1_steps"] = len(norms)
    out["c1_seconds"] = wall
    out["c1_walker_steps_per_s"] = float(norms.sum()) / wall
    out["c1_ms_per_step"] = wall / len(norms) * 1e3
    out["c1_shift"] = list(R.mean_and_se(np.asarray(df["shift"]), skip=5000))
    pe = R.projected_energy(df, skip=5000)
    out["c1_projected_energy"] = [float(pe.mean), float(pe.err)] if hasattr(pe, "mean") else list(pe)
    out["c1_exact_energy"] = -4.0215
    return out


def bench_c3(R, torch, steps=50, max_prep=20000):
    """The momentum-space configuration: HubbardMom1D(BoseFS(20, k=0 => 10); u=6, t=1),
    IsStochasticInteger, target 1e7, dt=5e-4.  The run grows from 100 walkers on the k=0
    address until its norm reaches 0.9 of the target and 500 more steps have passed; then
    `steps` steps are timed (device time of the whole loop, host shift update and statistics
    read-back included)."""
    import numpy as np
    addr = R.BoseFS(20, {10: 10})
    H = R.HubbardMom1D(addr, u=6.0, t=1.0)
    p = R.ProjectorMonteCarloProblem(H, start_at={addr: 100}, style=R.IsStochasticInteger(),
                                     time_step=5e-4, target_walkers=1e7, last_step=10 ** 9,
                                     random_seed=0x5EED, max_length=10 ** 8)
    sim = R.init(p)
    s = sim.states[0]
    prep, reached = 0, None
    while prep < max_prep and (reached is None or prep < reached + 500):
        sim.step_()
        prep += 1
        if reached is None and s.wm.last_stats["norm"] >= 0.9e7:
            reached = prep
    prep_steps = prep
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    norms = []
    e0.record()
    for _ in range(steps):
        sim.step_()
        norms.append(s.wm.last_stats["norm"])
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"workload": "HubbardMom1D M=20 N=10 (all in k=0) u=6 t=1, IsStochasticInteger, "
                        "target 1e7, dt=5e-4",
            "prep_steps": prep_steps, "steps": steps, "ms_per_step": ms / steps,
            "walker_steps_per_s": float(np.sum(norms)) / (ms / 1e3),
            "walkers_per_step": float(np.mean(norms)),
            "entries": int(s.wm.last_stats["len"])}


def bench_c5_full(R, torch, steps=5000, skip=2000, lanczos_i=(0, 21, 42, 63), krylovdim=24,
                  seed=0x5EED):
    """The batched configuration at its full length, both ways.  64 x HubbardRealSpace 4x4
    periodic, N=16, u_i = 1 + 15 i/63, targets log-uniform in [1e4, 1e6],
    IsDynamicSemistochastic, dt=1e-3, 5 000 steps from 10 walkers on the unit filling, with a
    ProjectedEnergy onto it: once stepped together (solve_batched) and once one problem after
    another with the plain step (solve).  Per replica the shift and projected energy with
    blocking errors (after `skip` steps); walker-steps/s of both; the error-bar ratio; and
    Lanczos ground energies (tol 1e-10) of some u_i on the full basis (D = 300 540 195)."""
    import numpy as np
    nrep = 64
    geo = R.PeriodicBoundaries(4, 4)
    addr = R.BoseFS([1] * 16)
    us = [1.0 + 15.0 * i / 63 for i in range(nrep)]
    hs = [R.HubbardRealSpace(addr, geo, u=[[u]], t=[1.0]) for u in us]
    targets = list(10.0 ** np.random.default_rng(2024).uniform(4.0, 6.0, nrep))
    style = R.IsDynamicSemistochastic()

    def problem(i, seed):
        return R.ProjectorMonteCarloProblem(
            hs[i], style=style, time_step=1e-3, last_step=steps, target_walkers=targets[i],
            start_at={addr: 10.0}, random_seed=seed, max_length=int(4 * targets[i] + 1000),
            post_step_strategy=R.ProjectedEnergy(hs[i], {addr: 1.0}))

    R.solve_batched([problem(i, 1) for i in range(nrep)][:2], segment_steps=64)  # warm-up
    torch.cuda.synchronize()
    t0 = time.time()
    sims_b = R.solve_batched([problem(i, seed) for i in range(nrep)], segment_steps=64)
    torch.cuda.synchronize()
    wall_b = time.time() - t0
    sims_s, wall_s = [], 0.0
    for i in range(nrep):
        p = problem(i, seed + 1 + i)
        torch.cuda.synchronize()
        t0 = time.time()
        sims_s.append(R.solve(p))
        torch.cuda.synchronize()
        wall_s += time.time() - t0

    def estimates(sim):
        df = sim.df
        r = R.shift_estimator(df, skip=skip)
        pe, pe_err = R.projected_energy(df, skip=skip)
        proj = [float(pe), float(pe_err)] if math.isfinite(pe) else None
        return {"shift": [float(r.mean), float(r.err)], "projected": proj,
                "walker_steps": float(np.sum(np.asarray(df["norm"], dtype=float)))}
    eb = [estimates(x) for x in sims_b]
    es = [estimates(x) for x in sims_s]
    wb = sum(e["walker_steps"] for e in eb) / wall_b
    ws = sum(e["walker_steps"] for e in es) / wall_s
    ratio_err = [eb[i]["shift"][1] / es[i]["shift"][1] for i in range(nrep)]
    lanczos = {}
    for i in lanczos_i:
        op = R.BasisOperator(hs[i])
        E, _, info = R.eigsolve(op, tol=1e-10, krylovdim=krylovdim)
        zb = (eb[i]["shift"][0] - E[0]) / eb[i]["shift"][1]
        zs = (es[i]["shift"][0] - E[0]) / es[i]["shift"][1]
        lanczos[i] = {"u": us[i], "E0": E[0], "converged": info["converged"],
                      "batched_shift_z": zb, "sequential_shift_z": zs,
                      "numops": info["numops"], "batched_shift": eb[i]["shift"],
                      "batched_projected": eb[i]["projected"],
                      "sequential_shift": es[i]["shift"],
                      "sequential_projected": es[i]["projected"]}
        del op
        torch.cuda.empty_cache()
    # 2-sigma agreement of each replica's batched and sequential estimates
    def within(a, b):
        return a is not None and b is not None and abs(a[0] - b[0]) <= 2 * (a[1] ** 2 + b[1] ** 2) ** 0.5
    agree_shift = sum(within(eb[i]["shift"], es[i]["shift"]) for i in range(nrep))
    agree_pe = sum(within(eb[i]["projected"], es[i]["projected"]) for i in range(nrep))
    n_pe = sum(eb[i]["projected"] is not None and es[i]["projected"] is not None for i in range(nrep))
    med = float(np.median(ratio_err))
    return {"workload": "64 x HubbardRealSpace 4x4 periodic N=16, u_i = 1+15i/63, targets "
                        "log-uniform [1e4, 1e6], IsDynamicSemistochastic, dt=1e-3, 5000 steps",
            "steps": steps, "skip": skip,
            "batched_seconds": wall_b, "sequential_seconds": wall_s,
            "batched_walker_steps_per_s": wb, "sequential_walker_steps_per_s": ws,
            "batched_over_sequential": wb / ws,
            "shift_error_ratio_median": med,
            "shift_error_ratio_range": [float(np.min(ratio_err)), float(np.max(ratio_err))],
            "batched_over_sequential_at_equal_error": wb / ws / med ** 2,
            "replicas_shift_within_2sigma": agree_shift,
            "replicas_projected_within_2sigma": agree_pe,
            "replicas_with_projected_energy": n_pe,
            "lanczos": lanczos,
            "per_replica": [{"u": us[i], "target": targets[i], "batched": eb[i],
                             "sequential": es[i]} for i in range(nrep)]}


def bench_hv(R, torch, peak, with_cpu=True):
    """H*v nonzeros/s on HubbardReal1D M=N=14 (D = 20 058 300), forward and adjoint."""
    h = R.HubbardReal1D(R.BoseFS([1] * 14), u=4.0, t=1.0)
    op = R.BasisOperator(h)
    D = op.dim
    # offdiagonal nonzeros of HubbardReal1D(14,14): two hops per occupied site, and
    # C(N+M-2, N-1) = C(26,13) basis states have a given site occupied: 2 M C(26,13)
    nnz_off = 2 * 14 * math.comb(26, 13)
    nnz = D + nnz_off
    g = torch.Generator(device="cuda").manual_seed(3)
    v = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    v /= torch.linalg.norm(v)
    gw = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    w = torch.empty_like(v)
    for _ in range(3):
        op(v, out=w)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        op(v, out=w)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    for _ in range(2):
        op.adjoint(v, gw)
    torch.cuda.synchronize()
    t0 = time.time()
    for _ in range(3):
        op.adjoint(v, gw)
    torch.cuda.synchronize()
    adj_ms = (time.time() - t0) / 3 * 1e3
    bytes_fwd = 8 * D * 2 + 8 * nnz_off
    # the oracle's H*v on the same basis and vector, all host threads (rows in parallel)
    cpu = None
    if with_cpu:
        import numpy as np
        import oracle as O
        O.build()
        m = O.real1d(14, 14, 4.0, 1.0)
        keys = O.basis(m)
        x = v.cpu().numpy()
        t0 = time.perf_counter()
        O.hv_basis(m, keys, x)
        secs = time.perf_counter() - t0
        cpu = {"value": nnz / secs, "unit": "nnz/s", "seconds": secs, "cores": os.cpu_count(),
               "kind": "port", "sample": "one full-basis product by the oracle (rows in parallel; "
                                         "addresses looked up by binary search in the sorted basis)"}
    # FP64 floor: one FP64 operation per nonzero (the diagonal term a multiply, each hop a
    # fused multiply-add) at GB300's 2 FP64 lanes per cycle per SM and the maximum SM clock
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    fp64_per_s = 2 * props.multi_processor_count * 2.07e9
    floor_ms = nnz / fp64_per_s * 1e3
    return {"workload": "HubbardReal1D M=N=14 full basis, D=20058300", "value": nnz / (ms / 1e3),
            "fp64_floor_ms": floor_ms, "frac_fp64": floor_ms / ms,
            # the adjoint: one fused multiply-add per hop and about five FP64 operations per row
            "adjoint_fp64_floor_ms": (nnz_off + 5 * D) / fp64_per_s * 1e3,
            "unit": "nnz/s", "ms": ms, "nnz": nnz,
            "achieved_gbs": bytes_fwd / (ms / 1e3) / 1e9, "frac_hbm": bytes_fwd / (ms / 1e3) / 1e9 / peak,
            "fp64_fma_per_s": nnz / (ms / 1e3),
            "adjoint_ms": adj_ms, "adjoint_over_forward": adj_ms / ms, "cpu_baseline": cpu}


# --------------------------------------------------------------------------------------------
# Reference arm: the CPU restatement of the reference step, all host cores
# --------------------------------------------------------------------------------------------
def run_reference(args, ws, rank, local):
    """The reference's CPU step restated: the oracle's threaded step (perform_spawns!,
    collect_local!, move_and_compress! of the PDVec, pdworkingmemory.jl:191-309, in C with
    OpenMP) on one shared walker list on every host core.  The population is grown from the
    unit-filling address by the same step (DoubleLogUpdate towards --ref-target, bounded by
    --ref-prep-seconds); then W untimed and K timed steps, each one full step of the list."""
    if rank != 0:
        return
    import numpy as np
    import oracle as O
    O.build()
    target = args.ref_target
    k0 = O.bose_key([1] * 20)
    m = O.real1d(20, 20, 4.0, 1.0)
    keys, vals = np.array([k0], dtype=np.uint64), np.array([target])
    S = O.diagonal(m, k0)
    t0 = time.time()
    _, prep, _, keys, vals, S, pn = cpu_steps(keys, vals, S, args.ref_prep_seconds, min_steps=1,
                                             max_steps=args.ref_prep_steps, target=target)
    t_prep = time.time() - t0
    _, _, _, keys, vals, S, pn = cpu_steps(keys, vals, S, 0.0, min_steps=args.warmup,
                                           max_steps=args.warmup, target=target, pnorm=pn,
                                           step0=prep + 1)
    value, nsteps, secs, keys, vals, S, pn = cpu_steps(
        keys, vals, S, 0.0, min_steps=args.steps, max_steps=args.steps, target=target, pnorm=pn,
        step0=prep + args.warmup + 1)
    threads = os.cpu_count() or 1
    sample = (f"{nsteps} full steps of one shared list grown by the same step from the "
              f"unit-filling address for {prep} steps ({t_prep:.0f} s) towards norm {target:.3g}; "
              f"{len(keys)} entries, norm {pn:.3g} at the end; {threads} threads")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs / max(nsteps, 1) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD + f" at target norm {target:.3g}",
                       "target_walkers": target, "entries": len(keys),
                       "note": "the GPU arm's list (norm 1e8) would need ~2000 growth steps of "
                               "~10 s each on these cores; the same routine on that list is "
                               "the GPU arm's cpu_baseline"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Julia is not installed; this is the C/OpenMP restatement of the reference's "
                    "PDVec step (oracle/)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--target", type=float, default=1e8)
    ap.add_argument("--max-prep", type=int, default=4000)
    ap.add_argument("--equil", type=int, default=2000,
                    help="untimed steps (growth + equilibration) before the warm-up steps")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="bound on the CPU baseline's timed steps of the GPU run's list")
    ap.add_argument("--ref-target", type=float, default=2e6,
                    help="walker norm of the reference arm's list")
    ap.add_argument("--ref-prep-seconds", type=float, default=90.0)
    ap.add_argument("--ref-prep-steps", type=int, default=400)
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per step of the roofline kernels, if measured for this run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-hv", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--c5-full", action="store_true",
                    help="only the batched configuration at full length, batched and one by one "
                         "(about ten minutes), as its own JSON line")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the small (C1) and momentum-space (C3) configuration lines")
    ap.add_argument("--shape", default=None,
                    help="launch shape KEYS_PER_BUCKET,TABLE_SLOTS of the step kernels (0 slots = automatic)")
    ap.add_argument("--annihilation", default="hash", choices=["hash", "sort"],
                    help="how the one-warp buckets group their spawns: shared-memory hash table "
                         "(default) or bitonic sort")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_setup()
    if args.c5_full:
        import torch
        sys.path.insert(0, os.path.join(ROOT, "rimu.jl_gb300"))
        from rimugpu import _build
        _build.build()
        import rimugpu as R
        print(json.dumps(bench_c5_full(R, torch)), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
