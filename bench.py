"""Throughput benchmark of the BCM per-cube dual-time sub-iteration path.

Default workload (``--workload batch``): 16 independent sphere flows with
immersed-boundary ghost cells on two cube levels, advanced together in one
batched context over a flat cube list; cube counts drawn from seed 2024 in
[64, 2048] (15,508 cubes of 16^3 cells, 63,516,672 cells), Mach uniform in
[0.1, 0.6], Re uniform in [100, 1000], per-case dT.  Seeded synthetic
fields; no dataset exists for this metric.  One bench step = one dual-time
step of SUBITERS pseudo-time sub-iterations (3 RK stages each: BCs, IBM
ghosts, interface, flux/RK, interface) plus the time-level shift, over
every cube of every case.  Other workloads (``tgv``, ``vortex``,
``sphere``, ``tgv32``) are the single-case configurations.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|split] [--workload batch|tgv|...]

Prints one JSON line (rank 0).  For N > 1 run under torchrun: every rank
advances its own replica of the case (weak scaling, no data-path
collective; the barrier and the max-over-ranks timing use the process
group).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("cell-subiters/s FP64 vs split-FP32 at ≤1e-5 L2 err; HBM GB/s vs peak")
UNIT = "cell-subiters/s"
SUBITERS = 10
# Contexts the batch is split into for the overlapped end-to-end figure
# (measured on GB300: two 1.50-1.71e9 cell-subiters/s from run to run,
# three 1.73e9, four and six 1.73e9; fewer contexts leave a larger share of
# the first copies and the last read-back exposed).
E2E_GROUPS = 4
# Dual-time steps from the initial state after which the split path is
# compared with the FP64 path (the FP64 leg times these same steps).
ACC_STEPS = 3
# Algorithmic bytes per cell-stage of the flux/RK kernel: read U1_, U1, U1q
# (40 B each) and the flag (4 B), write U1_ (40 B).
BYTES_PER_CELL_STAGE = 164


WORKLOADS = {
    # viscous Taylor-Green vortex, one case
    "tgv": ("taylor-green vortex, periodic 2pi box, 8x8x8 cubes of 24^3 cells "
            "(7,077,888 cells), M=0.1, Re=1600, Pr=0.72, dT=1e-4, dTau=dT/200"),
    # the reference's CPU-runnable case
    "vortex": ("inviscid isentropic vortex, periodic unit box, 4x4x4 cubes of 16^3 cells "
               "(262,144 cells), M=0.5, strength 5, dT=1e-3, dTau=dT/200"),
    # immersed-boundary sphere on two cube levels
    "sphere": ("sphere D=1 with IBM ghost cells, domain [-10,20]x[-10,10]^2, coarse cubes of "
               "2 refined 2:1 in [-2,4]x[-2,2]^2, 1584 cubes of 16^3 (6,488,064 cells), "
               "M=0.3, Re=300, inflow/outflow/slip boundaries, dT=1e-4, dTau=dT/200"),
    # large single case
    "tgv32": ("taylor-green vortex, periodic 2pi box, 16x16x16 cubes of 32^3 cells "
              "(134,217,728 cells), M=0.1, Re=1600, dT=1e-4, dTau=dT/200"),
    # batched uneven cases in one context: the configuration the metric's
    # split-precision target is quoted on (default)
    "batch": ("16 independent sphere flows (D=1, IBM ghost cells, two cube levels) in one "
              "batched context over a flat cube list; cube counts drawn from seed 2024 in "
              "[64, 2048] (realised mx*my*mz+56, 16^3 cells each), Mach uniform in [0.1, 0.6], "
              "Re uniform in [100, 1000], per-case dT (convective CFL 0.5 on the fine cells), "
              "dTau=dT/200"),
}
WORKLOAD = "batch"


class TimedPreprocess:
    """IBM preprocessing of the sphere workloads (the 20,480-triangle
    icosphere through BCM_Immersed_boundary's algorithm), with its wall time
    summed over the cases it builds."""

    def __init__(self, fn, where):
        self.fn, self.where, self.seconds, self.calls = fn, where, 0.0, 0

    def __call__(self, case, tris):
        t0 = time.perf_counter()
        out = self.fn(case, tris)
        self.seconds += time.perf_counter() - t0
        self.calls += 1
        return out


def workload_case(preprocess=None):
    """The workload's case; preprocess (a TimedPreprocess) builds the IBM
    tables of the sphere workloads from the triangulated body."""
    from bcm_cgli_gb300 import cases
    if WORKLOAD == "vortex":
        return cases.isentropic_vortex(ncx=4, n=16)
    if WORKLOAD == "sphere":
        case = cases.sphere_ibm(preprocess=preprocess)
    elif WORKLOAD == "batch":
        case = cases.CaseBatch(cases.sphere_batch(ncase=16, seed=2024, n=16,
                                                  preprocess=preprocess), name="batch")
    elif WORKLOAD == "tgv32":
        return cases.taylor_green(ncx=16, n=32)
    else:
        return cases.taylor_green(ncx=8, n=24)
    if preprocess is not None:
        case.meta["ibm_preprocess"] = {
            "triangles": 20 * 4 ** 5, "cases": preprocess.calls, "where": preprocess.where,
            "seconds": round(preprocess.seconds, 4)}
    return case


def is_batch(case):
    return hasattr(case, "cases")


def make_context(api, case, precision):
    if is_batch(case):
        return api.BatchContext(case.cases, precision=precision)
    return api.CaseContext(case, precision=precision)


def workload_config(case):
    """The workload's description, the same for both arms (no precision or
    setup details: those are keys of the line itself)."""
    extra = {}
    if is_batch(case):
        extra = {"cases": len(case.cases), "cubes": [c.ncube - 1 for c in case.cases],
                 "mach": [round(c.phys.U0 / np.sqrt(1.4 * c.phys.P0 / c.phys.rho0), 4)
                          for c in case.cases],
                 "reynolds": [round(c.phys.rho0 * c.phys.U0 / c.phys.mu_L, 1)
                              for c in case.cases]}
    return {"workload": WORKLOADS[WORKLOAD] + f"; {SUBITERS} sub-iterations x 3 RK stages per "
                                              "dual-time step",
            **extra,
            "cells": int(case.n_cells),
            "subiters_per_step": SUBITERS,
            "l2": (f"inputs larger than L2: each state array is {case.U.nbytes / 1e6:.0f} MB "
                   "(L2 is 129 MB)" if case.U.nbytes > 129e6 else
                   f"each state array is {case.U.nbytes / 1e6:.0f} MB, under the 129 MB L2 "
                   "(no flush between steps)"),
            "parallelism": "replica per GPU"}


# ---------------------------------------------------------------------------
# distributed helpers (timing only)
# ---------------------------------------------------------------------------
class Dist:
    """Rank bookkeeping of a torchrun launch.  Every rank advances its own
    replica of the case (the path has no data exchange between replicas);
    the process group only brackets the timed region with barriers and takes
    the maximum time over ranks.  NCCL on GPUs, gloo where there is none."""

    def __init__(self, gpus: int, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = "cuda"
            dist.init_process_group(backend)
            self.pg = dist
            self.torch = torch

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, ms: float) -> float:
        """Whole-job rate: the units all ranks processed over the slowest
        rank's time (ms already max-reduced)."""
        return units_per_rank * self.world / (ms * 1e-3)

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.p = None
        self.out = []

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.out.append(line.strip())

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU arm: the reference's algorithm on the host cores (oracle port here,
# since the reference sources are not present on the GPU host)
# ---------------------------------------------------------------------------
def _oracle_preprocess():
    """The reference arm builds its sphere tables with the oracle's C
    restatement of BCM_Immersed_boundary (the same tables as the GPU)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    port = O.Port()
    return TimedPreprocess(lambda case, tris: port.ibm(case, case.fws, tris),
                           "CPU, C restatement of BCM_Immersed_boundary (1 thread)")


def _port(threads=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    runner = O.Port()
    threads = threads or os.cpu_count() or 1
    runner.set_threads(threads)
    return O, runner, threads


# The CPU arms time the C restatement of the reference loop: the reference's
# own sources are not on the GPU host.  On an x86 host where both build, the
# restatement runs at 0.77-0.81 of the reference's compiled code on one thread
# and 0.71-0.93 on 8 over repeated runs (vortex and Taylor-Green cubes;
# oracle/time_port_vs_reference.py), so this baseline understates the
# reference's CPU rate by up to about a quarter.
PORT_NOTE = ("C restatement of the reference loop (the reference's sources are not on this "
             "host); on an x86 host it ran at 0.77-0.81 (1 thread) and 0.71-0.93 (8 threads) of "
             "the reference's own compiled code "
             "(oracle/time_port_vs_reference.py)")


def host_cpu():
    """CPU model and logical core count of this host."""
    import platform
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return f"{model} ({platform.machine()}), {os.cpu_count()} logical cores"


def cpu_sample(case, subiters=1, threads=None):
    """The C restatement of the reference loop on the host cores (OpenMP over
    cubes, one process): one dual-time step of `subiters` sub-iterations over
    every case of the workload (about 10-15 s for the batch)."""
    O, runner, threads = _port(threads)
    dt = 0.0
    for c in (case.cases if is_batch(case) else [case]):
        st = O.State(c)
        t0 = time.perf_counter()
        runner.run(c, st, 1, subiters)
        dt += time.perf_counter() - t0
        del st
    return {"value": case.n_cells * subiters / dt, "unit": UNIT, "cores": threads, "ranks": 1,
            "kind": "port", "host": host_cpu(), "note": PORT_NOTE,
            "sample": f"1 dual-time step x {subiters} sub-iteration(s) of the full workload "
                      f"({case.n_cells} cells) through the C restatement of the reference "
                      f"loop, {threads} OpenMP threads over cubes in 1 process (1 rank), "
                      f"{dt:.2f} s"}


def cpu_single_thread(case):
    """The same restatement on one thread (the setting the reference's
    parity runs use): one sub-iteration of the workload's smallest case."""
    O, runner, _ = _port(1)
    c = min(case.cases if is_batch(case) else [case], key=lambda m: m.n_cells)
    st = O.State(c)
    t0 = time.perf_counter()
    runner.run(c, st, 1, 1)
    dt = time.perf_counter() - t0
    return {"value": c.n_cells / dt, "unit": UNIT, "cores": 1,
            "sample": f"1 sub-iteration of the workload's smallest case ({c.n_cells} cells), "
                      f"1 OpenMP thread, {dt:.2f} s"}


def run_reference_arm(args, dist):
    """The reference's CPU algorithm (C restatement of the reference loop;
    the reference's own sources are not on the GPU host) on all host cores.
    Each bench step is one bounded sample: one sub-iteration of one case of
    the workload, the cases taken in turn (for the single-case workloads, one
    sub-iteration of the case).  ms_per_step is the measured time of those
    samples, so ms_per_step x steps is the timed region."""
    if dist.rank != 0:
        return
    case = workload_case(_oracle_preprocess())
    O, runner, threads = _port()
    members = case.cases if is_batch(case) else [case]
    timed_cells, timed_s, sampled = 0, 0.0, []
    st = None
    for i in range(max(0, args.warmup) + max(1, args.steps)):
        q = i % len(members)
        c = members[q]
        if st is None or len(members) > 1:
            st = None  # one case's arrays on the host at a time
            st = O.State(c)
        t0 = time.perf_counter()
        runner.run(c, st, 1, 1)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            timed_cells += c.n_cells
            timed_s += dt
            sampled.append(q)
    steps = max(1, args.steps)
    v = timed_cells / timed_s
    cpu = {"value": v, "unit": UNIT, "cores": threads, "ranks": 1, "kind": "port",
           "host": host_cpu(), "note": PORT_NOTE,
           "sample": (f"per step: 1 sub-iteration of one case (cases {sampled[0]}.. in turn"
                      f", {timed_cells} cell-subiters over {steps} steps)" if is_batch(case)
                      else f"per step: 1 sub-iteration of the case ({case.n_cells} cells)") +
                     f"; C restatement of the reference loop, {threads} OpenMP threads over "
                     f"cubes in 1 process (1 rank); {timed_s:.2f} s timed"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "ms_per_step": timed_s / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(case), "cpu_baseline": cpu,
            "timed_sample": {"subiters_per_step": 1, "cell_subiters": timed_cells,
                             "cases_per_step": 1 if is_batch(case) else None},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def pinned_like(a):
    try:
        import torch
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        out = t.numpy().reshape(a.shape)
        out[...] = a
        return out, t
    except Exception:
        return np.ascontiguousarray(a.copy()), None


def measure(api, case, precision_name, args, dist, clocks_on=True, method=None, steps=None,
            warmup=None, from_initial=False, prof_subiters=SUBITERS, prof_steps=2):
    """Timed region for one precision: `steps` dual-time steps resident in
    HBM (default args.steps), each one captured-graph launch, device-timed
    with CUDA events on the context's stream, after `warmup` untimed steps
    (the last one captures the step graph).  from_initial: the timed steps
    start from the initial state (so their result is comparable across
    precisions; the final state and er are returned).  Then `prof_steps`
    eager profiled steps of `prof_subiters` sub-iterations bracket every
    flux launch with events for the kernel's average duration."""
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    precision = api.PRECISION_SPLIT if precision_name == "split" else api.PRECISION_FP64
    ctx = make_context(api, case, precision)
    meth = method or getattr(args, "method", "rk3")
    if meth == "lusgs":
        ctx.set_method(api.METHOD_LUSGS, cfl=0.0, omega=1.5)
    # launch shapes from the committed autotuner table (bcm_cgli_gb300/autotune.py)
    from bcm_cgli_gb300 import autotune
    shape = autotune.lookup(case.n, precision_name, meth)
    if getattr(args, "flux_form", None) is not None:
        shape = dict(shape or {"flux_tile": 0, "lusgs_threads": 0})
        shape["flux_form"] = args.flux_form
    if shape:
        ctx.set_tuning(shape["flux_tile"], shape["lusgs_threads"], shape.get("flux_form", 0))
    ctx.set_state(case.U, case.U, case.U)
    for _ in range(max(1, warmup)):  # the last warm-up step captures the step graph
        ctx.advance(1, SUBITERS, use_graph=True)
    if from_initial:
        ctx.set_state(case.U, case.U, case.U)
        ctx.emax[...] = 0
    clocks = Clocks(dist.local) if clocks_on else None
    if clocks:
        clocks.start()
    launches = 0
    er = None
    dist.barrier()
    ctx.sync()
    ctx.timer_mark(0)
    for _ in range(steps):  # one graph launch per dual-time step
        er = ctx.advance(1, SUBITERS, use_graph=True)
        launches += ctx.launch_count()
    ctx.timer_mark(1)
    ctx.sync()
    dist.barrier()
    ms = dist.max(ctx.timer_elapsed(0, 1))
    clk = clocks.stop() if clocks else None
    final = ctx.get_state()[0] if from_initial else None
    # flux kernel duration: events around each flux launch in eager profiled
    # steps of the same kind (graphs are not profiled)
    ctx.set_profiling(True)
    for _ in range(max(1, min(prof_steps, steps))):
        ctx.advance(1, prof_subiters, use_graph=False)
    flux_ms, flux_n = ctx.profile()
    ctx.set_profiling(False)
    out = {"tuning": ({"flux_tile": shape["flux_tile"], "lusgs_threads": shape["lusgs_threads"],
                       "flux_form": shape.get("flux_form", 0),
                       "ghost_fill_beside_boundary_fill": ctx.concurrent_ghosts(),
                       "from": "bcm_cgli_gb300/tuning_gb300.json"} if shape else None),
           "value": dist.throughput(case.n_cells * SUBITERS * steps, ms),
           "ms_per_step": ms / steps, "steps": steps, "warmup": max(1, warmup),
           "launches": launches, "flux_ms_avg": flux_ms / max(1, flux_n), "flux_launches": flux_n,
           "clocks": clk, "ctx": ctx, "er": er, "final": final}
    return out


def measure_e2e(ctx, case, args, dist, cell_subiters):
    """Per step: host (pinned) -> device state (U1_, U1, U1q: the three time
    levels a host-held solver passes), one dual-time step, device -> host of
    the step's result, the new state U1_ (after the time shift U1 equals it
    on the interior and U1q is the previous U1, which the host holds),
    through the public C ABI; device-timed, and the host clock over the same
    region (returned second)."""
    hU, hold = pinned_like(case.U)
    hU1, hold1 = pinned_like(case.U)
    hU1q, hold1q = pinned_like(case.U)
    oU, ohold = pinned_like(case.U)
    dist.barrier()
    ctx.sync()
    t0 = time.perf_counter()
    ctx.timer_mark(2)
    for _ in range(args.steps):
        ctx.set_state(hU, hU1, hU1q)
        ctx.advance(1, SUBITERS, use_graph=True)
        ctx.get_result(oU)
    ctx.timer_mark(3)
    ctx.sync()
    wall = dist.max(time.perf_counter() - t0)
    dist.barrier()
    ms_e2e = dist.max(ctx.timer_elapsed(2, 3))
    return cell_subiters / (ms_e2e * 1e-3), cell_subiters / wall


def measure_twins(api, case, precision_name, subiters=2):
    """The drop-in twins end to end: sub-iterations in main.cpp's call order
    (main.cpp:1161-1241: X/Y/Z boundary conditions, IBM ghost cells,
    interface, flux/RK stage, interface; three stages) on host arrays, each
    call copying its arrays to the GPU and back as the reference's routines
    are replaced one for one.  The reference runs one case per process, so
    this times one case: the workload's largest.  Wall clock, after one
    untimed sub-iteration (which page-locks the arrays and sizes the device
    buffers)."""
    c = max(case.cases, key=lambda x: x.n_cells) if is_batch(case) else case
    api.reference_config_for(c)
    api.set_reference_precision(api.PRECISION_SPLIT if precision_name == "split"
                                else api.PRECISION_FP64)
    api.set_twin_scratch_kept(True)  # main.cpp keeps its scratch arrays
    api.set_host_pinning(True)       # and its arrays for the whole run
    U1_, U1, U1q = c.U.copy(), c.U.copy(), c.U.copy()
    U1p1, U1p2, Rku1, Res = (np.zeros_like(c.U) for _ in range(4))
    er = np.zeros(8)
    lists = [api._one_based(x) for x in c.bc_lists()]
    tables = [(f, t) for f, t in ((api.BCM_Ghostcell_minus, c.ibm_minus),
                                  (api.BCM_Ghostcell_plus, c.ibm_plus)) if t is not None]

    def subiteration():
        xl, xu, yl, yu, zl, zu = lists
        for RK in (1, 2, 3):
            api.BCM_X_boundary_condition(0, len(xl) - 1, len(xu) - 1, xl, xu, U1_)
            api.BCM_Y_boundary_condition(len(yl) - 1, len(yu) - 1, yl, yu, U1_)
            api.BCM_Z_boundary_condition(len(zl) - 1, len(zu) - 1, zl, zu, U1_)
            for f, (W, Gi, I) in tables:
                f(0, (len(Gi) - 1) // 4, W, Gi, I, c.fws, U1_)
            api.BCM_Interface_for_case(c, U1_)
            api.BCM_Flux_XYZ_Viscous_Runge_kutta(0, c.ncube, RK, c.dT, c.dTau, c.e, c.fws, c.csl,
                                                 c.cube_size, U1_, U1, U1q, U1p1, U1p2, Rku1,
                                                 Res, er)
            api.BCM_Interface_for_case(c, U1_)

    try:
        subiteration()
        t0 = time.perf_counter()
        for _ in range(subiters):
            subiteration()
        dt = time.perf_counter() - t0
    finally:
        api.release_host_arrays()  # before the arrays go
        api.set_host_pinning(False)
        api.set_reference_precision(api.PRECISION_FP64)
        api.set_twin_scratch_kept(False)
    return {"value": c.n_cells * subiters / dt, "unit": UNIT, "precision": precision_name,
            "case": f"{c.name}: {c.ncube - 1} cubes, {c.n_cells} cells",
            "subiters": subiters, "seconds": dt,
            "note": "drop-in twins in main.cpp's call order on host arrays (page-locked once, "
                    "scratch arrays kept), wall clock"}


def measure_e2e_pipelined(api, case, precision_name, args, dist, ngroups=None):
    """End to end with the host link overlapped: the batch's cases in
    ngroups contexts of about equal cells (consecutive cases), each on its
    own stream; per step and group, the host -> device copies of its three
    time levels (U1_, U1, U1q, from page-locked memory), one dual-time step
    (a graph launch) and the device -> host copy of its new U1_ are enqueued
    asynchronously, so one group's copies run while the others step.  Same
    bytes per step as measure_e2e; device-timed (events on every stream, the
    longest span), and the host clock from before the first copy is enqueued
    until every stream has finished (returned second)."""
    ngroups = ngroups or E2E_GROUPS
    cs = case.cases
    cells = np.cumsum([c.n_cells for c in cs])
    cuts = [0]
    for g in range(1, ngroups):
        k = int(np.argmin(np.abs(cells - cells[-1] * g / ngroups))) + 1
        if k > cuts[-1] and k < len(cs):
            cuts.append(k)
    cuts.append(len(cs))
    groups = [cs[a:b] for a, b in zip(cuts[:-1], cuts[1:])]
    precision = api.PRECISION_SPLIT if precision_name == "split" else api.PRECISION_FP64
    from bcm_cgli_gb300 import autotune
    shape = autotune.lookup(case.n, precision_name, "rk3")
    halves, keep = [], []
    for g in groups:
        ctx = api.BatchContext(g, precision=precision)
        if shape:
            ctx.set_tuning(shape["flux_tile"], shape["lusgs_threads"], shape.get("flux_form", 0))
        U = cases_flat(g)
        held = [pinned_like(U) for _ in range(4)]  # (array, page-locked tensor) pairs
        keep.append(held)
        ins, out = [h[0] for h in held[:3]], held[3][0]
        ctx.set_state(U, U, U)
        for _ in range(max(1, args.warmup)):
            ctx.advance(1, SUBITERS, use_graph=True)  # the first captures the step graph
        halves.append((ctx, ins, out))
    dist.barrier()
    for ctx, _, _ in halves:
        ctx.sync()
    t0 = time.perf_counter()
    for ctx, _, _ in halves:
        ctx.timer_mark(6)
    for _ in range(args.steps):
        for ctx, ins, out in halves:
            ctx.copy_state_async(True, *ins)
            ctx.advance_async(1, SUBITERS)
            ctx.copy_state_async(False, out)
    for ctx, _, _ in halves:
        ctx.timer_mark(7)
    for ctx, _, _ in halves:
        ctx.sync()
    wall = dist.max(time.perf_counter() - t0)
    dist.barrier()
    ms = dist.max(max(ctx.timer_elapsed(6, 7) for ctx, _, _ in halves))
    for ctx, _, _ in halves:
        ctx.close()
    done = case.n_cells * SUBITERS * args.steps * dist.world
    return done / (ms * 1e-3), cuts, done / wall


def cases_flat(group):
    """The flat batch state of a list of cases (slot 0 unused)."""
    from bcm_cgli_gb300 import cases as cz
    return cz.CaseBatch(group).U


def measure_converged(api, case, precision_name, method, args, dist, steps=2, max_subiters=50,
                      tol=0.02):
    """Physical steps with the reference's convergence test (main.cpp:1249-
    1271: every E-normalised change norm below tol, else max_subiters), one
    graph launch per step with the sub-iteration loop on the device; from
    the initial state, after one untimed step that builds the graph."""
    precision = api.PRECISION_SPLIT if precision_name == "split" else api.PRECISION_FP64
    ctx = make_context(api, case, precision)
    ctx.set_method(api.METHOD_LUSGS if method == "lusgs" else api.METHOD_RK3)
    ctx.set_state(case.U, case.U, case.U)
    ctx.advance_converged(1, max_subiters, tol)
    ctx.set_state(case.U, case.U, case.U)
    ctx.emax[...] = 0
    dist.barrier()
    ctx.sync()
    ctx.timer_mark(4)
    _, its = ctx.advance_converged(steps, max_subiters, tol)
    ctx.timer_mark(5)
    ctx.sync()
    ms = dist.max(ctx.timer_elapsed(4, 5))
    ctx.close()
    its = np.asarray(its).reshape(steps, -1)
    return {"ms_per_physical_step": ms / steps,
            "subiters_per_step": its.max(axis=1).tolist(),
            "converged": bool((its < max_subiters).all())}


def rel_l2(a, b, n):
    """Relative L2 error per conservative variable over interior cells; the
    momentum components are also given relative to the momentum magnitude
    (rho w of a 2-D or symmetric flow is ~0, so its own norm is no scale)."""
    ai = a[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    bi = b[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    d = ai - bi
    own = [float(np.linalg.norm(d[:, v]) / max(np.linalg.norm(bi[:, v]), 1e-300)) for v in range(5)]
    mom = float(np.linalg.norm(bi[:, 1:4]))
    scaled = [own[0]] + [float(np.linalg.norm(d[:, v]) / mom) for v in (1, 2, 3)] + [own[4]]
    return own, scaled


def accuracy(case, split, fp64, steps):
    """Split-precision state and forces against the FP64 path after `steps`
    dual-time steps from the same initial state: relative L2 per variable
    over the interior cells of every case, and per case the drag and lift
    coefficients from the force integrals er[6], er[7] (the reference
    normalises them by 0.5 rho0 U0^2 * 2.602, BCM_Flux_XYZ_Viscous_Runge_
    kutta.cpp:2609-2650; re-scaled here to the body's frontal area).  A
    sphere's lift is ~0 in these flows, so its error is stated relative to
    the drag as well as absolutely."""
    (us, ers), (uf, erf) = split, fp64
    own, scaled = rel_l2(us, uf, case.n)
    acc = {"rel_l2_per_variable": own, "rel_l2_momentum_scaled": scaled,
           "max_rel_l2": max(scaled), "bound": 1e-5, "drag_bound": 1e-3,
           "after": f"{steps} dual-time step(s) x {SUBITERS} sub-iterations from the same "
                    "initial state"}
    members = case.cases if is_batch(case) else [case]
    if "area_ratio" not in members[0].meta:
        return acc
    ers = np.asarray(ers).reshape(len(members), 8)
    erf = np.asarray(erf).reshape(len(members), 8)
    rows = []
    for q, c in enumerate(members):
        r = c.meta["area_ratio"]
        cd_s, cl_s, cd_f, cl_f = -ers[q, 6] * r, -ers[q, 7] * r, -erf[q, 6] * r, -erf[q, 7] * r
        rows.append({"cd_fp64": cd_f, "cd_split": cd_s, "cl_fp64": cl_f, "cl_split": cl_s,
                     "cd_rel_err": abs(cd_s - cd_f) / abs(cd_f),
                     "cl_abs_err": abs(cl_s - cl_f),
                     "cl_err_rel_to_cd": abs(cl_s - cl_f) / abs(cd_f)})
    acc["forces_per_case"] = rows
    acc["cd_rel_err_max"] = max(x["cd_rel_err"] for x in rows)
    acc["cl_err_rel_to_cd_max"] = max(x["cl_err_rel_to_cd"] for x in rows)
    return acc


def run_gpu_arm(args, dist):
    from bcm_cgli_gb300 import api
    # the FP64 probe also creates the CUDA context, which the preprocessing
    # time below should not include
    fp64_gflops = api.probe_fp64_gflops()
    case = workload_case(TimedPreprocess(api.ibm_preprocess, "GPU, bcmg_ibm_preprocess"))
    head = args.precision
    other = "fp64" if head == "split" else "split"
    m_head = measure(api, case, head, args, dist, clocks_on=True)
    # The other precision: a bounded sample (an FP64 dual-time step of the
    # batch takes about 10 s) whose timed steps start from the initial state,
    # so they also give the accuracy comparison below.
    m_other = None
    acc_steps = max(1, args.acc_steps)
    if not args.quick:
        m_other = measure(api, case, other, args, dist, clocks_on=False, steps=acc_steps,
                          warmup=1, from_initial=True,
                          prof_subiters=1 if other == "fp64" else SUBITERS, prof_steps=1)

    # Accuracy of the split form against the FP64 path after acc_steps
    # dual-time steps from the same initial state (bounds: 1e-5 relative L2,
    # 0.1% drag).
    acc = None
    if m_other is not None:
        ctx = m_head["ctx"]
        ctx.set_state(case.U, case.U, case.U)
        ctx.emax[...] = 0
        for _ in range(acc_steps):
            er_h = ctx.advance(1, SUBITERS, use_graph=True)
        res = {head: (ctx.get_state()[0], er_h), other: (m_other["final"], m_other["er"])}
        acc = accuracy(case, res["split"], res["fp64"], acc_steps)
        m_other["final"] = None

    ctx = m_head["ctx"]
    cell_subiters = case.n_cells * SUBITERS * args.steps * dist.world
    e2e = e2e_serial = e2e_wall = None
    e2e_how = None
    if not args.no_e2e:
        e2e_serial, e2e_wall = measure_e2e(ctx, case, args, dist, cell_subiters)
        e2e, e2e_how = e2e_serial, "one context: copy in, step, copy out, in series"
        if is_batch(case) and len(case.cases) >= 2:
            piped, cuts, piped_wall = measure_e2e_pipelined(api, case, head, args, dist)
            if piped > e2e:
                e2e, e2e_wall = piped, piped_wall
                parts = ", ".join(f"{a}..{b - 1}" for a, b in zip(cuts[:-1], cuts[1:]))
                e2e_how = (f"{len(cuts) - 1} contexts (cases {parts}) on their own streams: "
                           "each one's copies overlap the others' steps")
    peaks = {}

    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))

    def roofline(m, prec):
        alg_bytes = BYTES_PER_CELL_STAGE * case.n_cells
        achieved = alg_bytes / (m["flux_ms_avg"] * 1e-3) / 1e9
        traffic, traffic_src = None, None
        # DRAM bytes per cell-stage from an ncu capture of the same kernel on a
        # smaller case of the same cube resolution (scaled by cells: a launch's
        # traffic grows with its cells), else of another resolution
        for fn in (f"flux_{prec}_traffic_n{case.n}.json", f"flux_{prec}_traffic.json"):
            prof = os.path.join(ROOT, "profiles", fn)
            if os.path.isfile(prof):
                try:
                    t = json.load(open(prof))
                    traffic = t["dram_bytes_per_cell_stage"] * case.n_cells
                    traffic_src = f"profiles/{fn}"
                    break
                except Exception:
                    traffic = None
        return {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic, "kernel": f"k_flux_{prec}",
                "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": m["flux_ms_avg"],
                "launches": m["flux_launches"], "traffic_from": traffic_src,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}

    line = {"metric": METRIC, "value": m_head["value"], "unit": UNIT, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": m_head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == "fp64" else "f32+f64",
            "data": "synthetic", "config": workload_config(case), "precision": head,
            "roofline": roofline(m_head, head),
            "e2e": ({"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 3 * case.U.nbytes,
                     "d2h_bytes_per_step": case.U.nbytes, "how": e2e_how,
                     "serial_value": e2e_serial, "wall_value": e2e_wall}
                    if e2e is not None else None),
            "gpu_launches": m_head["launches"], "clocks": m_head["clocks"],
            "launch_shapes": m_head["tuning"],
            "fp64_alu": {"measured_fma_gflops": fp64_gflops,
                         "note": "FP64 FMA rate of this GPU, measured by bcmg_probe_fp64_rate"}}
    if "ibm_preprocess" in getattr(case, "meta", {}):
        line["setup"] = {"ibm_preprocess": case.meta["ibm_preprocess"]}
    if m_other is not None:
        line[other] = {"value": m_other["value"], "ms_per_step": m_other["ms_per_step"],
                       "steps": m_other["steps"], "warmup": m_other["warmup"],
                       "timed_from": "the initial state (the accuracy comparison's steps)",
                       "roofline": roofline(m_other, other), "gpu_launches": m_other["launches"]}
        line["split_vs_fp64_speedup"] = (line["value"] / m_other["value"] if head == "split"
                                         else m_other["value"] / line["value"])
    if acc is not None:
        line["accuracy"] = acc
    line["method"] = args.method
    if args.method == "rk3" and not args.quick:
        # the same workload with LU-SGS sub-iterations (no reference
        # counterpart; converges further per sub-iteration)
        m_lu = measure(api, case, head, args, dist, clocks_on=False, method="lusgs")
        line["lusgs"] = {"value": m_lu["value"], "ms_per_step": m_lu["ms_per_step"],
                         "precision": head, "gpu_launches": m_lu["launches"],
                         "note": "LU-SGS sub-iterations (hyperplane sweeps) instead of the "
                                 "reference's 3-stage RK, same residual and workload"}
        m_lu["ctx"].close()
    if not args.no_e2e and not args.quick:
        line["e2e_twins"] = {p: measure_twins(api, case, p) for p in ("split", "fp64")}
    if not args.no_converged and not args.quick:
        conv = {m: measure_converged(api, case, head, m, args, dist) for m in ("rk3", "lusgs")}
        conv["tol"] = 0.02
        conv["max_subiters"] = 50
        conv["precision"] = head
        conv["note"] = ("physical steps with the reference's convergence test "
                        "(main.cpp:1249-1271); RK3 at the reference's dTau=dT/200")
        conv["lusgs_speedup_per_physical_step"] = (conv["rk3"]["ms_per_physical_step"] /
                                                   conv["lusgs"]["ms_per_physical_step"])
        line["converged_step"] = conv
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(case, subiters=1)
        line["cpu_baseline"]["single_thread"] = cpu_single_thread(case)
    for m in (m_head, m_other):
        if m is not None:
            m["ctx"].close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def run_accuracy(args):
    """Accuracy over a configuration's own horizon: the FP64 and the split
    path advance the workload from the same initial state for
    args.accuracy dual-time steps (args.method sub-iterations, SUBITERS
    each, one graph launch per step); at every checkpoint (a quarter of the
    run) the split state and forces are compared with the FP64 path's
    (relative L2 per variable, per-case drag and lift).  Prints one JSON
    line; not the benchmark line."""
    from bcm_cgli_gb300 import api
    case = workload_case(TimedPreprocess(api.ibm_preprocess, "GPU, bcmg_ibm_preprocess"))
    steps = args.accuracy
    ctxs = {}
    for p in ("fp64", "split"):
        ctx = make_context(api, case, api.PRECISION_SPLIT if p == "split" else api.PRECISION_FP64)
        if args.method == "lusgs":
            ctx.set_method(api.METHOD_LUSGS, cfl=0.0, omega=1.5)
        ctx.set_state(case.U, case.U, case.U)
        ctxs[p] = ctx
    marks = sorted({max(1, (steps * q) // 4) for q in (1, 2, 3, 4)})
    out, done, secs = [], 0, {"fp64": 0.0, "split": 0.0}
    for m in marks:
        res = {}
        for p, ctx in ctxs.items():
            t0 = time.perf_counter()
            er = None
            for _ in range(m - done):
                er = ctx.advance(1, SUBITERS, use_graph=True)
            secs[p] += time.perf_counter() - t0
            res[p] = (ctx.get_state()[0], er)
        done = m
        acc = accuracy(case, res["split"], res["fp64"], m)
        out.append(acc)
        print(json.dumps({"checkpoint": m, "max_rel_l2": acc["max_rel_l2"],
                          "cd_rel_err_max": acc.get("cd_rel_err_max")}), file=sys.stderr,
              flush=True)
    for ctx in ctxs.values():
        ctx.close()
    print(json.dumps({"accuracy_horizon": WORKLOAD, "workload": WORKLOADS[WORKLOAD],
                      "method": args.method, "subiters_per_step": SUBITERS, "steps": steps,
                      "checkpoints": out, "seconds": secs}), flush=True)


def run_flux_only(args):
    """Profiling target: the flux kernel alone on a Taylor-Green case of
    ncx^3 cubes of n^3 cells (ncx=6, n=24: 216 cubes, 3.0 M cells, 190 MB per
    state array, above the 129 MB L2), one warm-up launch and `steps` timed
    launches.  Used by the ncu commands recorded under profiles/."""
    from bcm_cgli_gb300 import api, cases
    case = cases.taylor_green(ncx=args.ncx, n=args.n)
    prec = api.PRECISION_SPLIT if args.precision == "split" else api.PRECISION_FP64
    ctx = api.CaseContext(case, precision=prec)
    if args.flux_form is not None:
        ctx.set_tuning(0, 0, args.flux_form)
    ctx.set_state(case.U, case.U, case.U)
    ms = ctx.time_flux(reps=max(1, args.steps))
    ctx.close()
    print(json.dumps({"flux_only": args.precision, "cells": case.n_cells, "ms_per_launch": ms,
                      "cell_stages_per_s": case.n_cells / (ms * 1e-3)}), flush=True)


def run_step_only(args):
    """Profiling target of the kernels around the flux: one eager dual-time
    step of one sub-iteration (split precision) on a Taylor-Green case of
    ncx^3 cubes of n^3 cells, or with --workload sphere on the two-level
    sphere with IBM ghost cells (1,584 cubes of 16^3, 260 MB per state
    array), after one untimed step."""
    from bcm_cgli_gb300 import api, cases
    case = (cases.sphere_ibm() if args.workload == "sphere"
            else cases.taylor_green(ncx=args.ncx, n=args.n))
    ctx = api.CaseContext(case, precision=api.PRECISION_SPLIT)
    ctx.set_state(case.U, case.U, case.U)
    ctx.advance(1, 1, use_graph=False)
    ctx.sync()
    ctx.timer_mark(0)
    ctx.advance(1, 1, use_graph=False)
    ctx.timer_mark(1)
    ms = ctx.timer_elapsed(0, 1)
    ctx.close()
    print(json.dumps({"step_only": case.name, "cells": case.n_cells, "ms_per_step": ms}),
          flush=True)


def run_lusgs_only(args):
    """Profiling target: LU-SGS sub-iterations (residual + sweeps) on a
    Taylor-Green case of ncx^3 cubes of n^3 cells, `steps` sub-iterations
    after one warm-up step."""
    from bcm_cgli_gb300 import api, cases
    case = cases.taylor_green(ncx=args.ncx, n=args.n)
    prec = api.PRECISION_SPLIT if args.precision == "split" else api.PRECISION_FP64
    ctx = api.CaseContext(case, precision=prec)
    ctx.set_method(api.METHOD_LUSGS)
    ctx.set_state(case.U, case.U, case.U)
    ctx.advance(1, 1, use_graph=False)
    ctx.sync()
    ctx.timer_mark(0)
    ctx.advance(1, max(1, args.steps), use_graph=False)
    ctx.timer_mark(1)
    ms = ctx.timer_elapsed(0, 1)
    ctx.close()
    print(json.dumps({"lusgs_only": args.precision, "cells": case.n_cells,
                      "ms_per_subiter": ms / max(1, args.steps)}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split", choices=["fp64", "split"],
                    help="path whose throughput is the headline value (the other is "
                         "reported beside it)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end measurement")
    ap.add_argument("--no-converged", action="store_true",
                    help="skip the convergence-test (RK3 vs LU-SGS) physical-step timing")
    ap.add_argument("--quick", action="store_true",
                    help="headline path only (no second precision, no accuracy check)")
    ap.add_argument("--flux-only", action="store_true",
                    help="time the flux kernel alone on a smaller case (profiling target)")
    ap.add_argument("--step-only", action="store_true",
                    help="one eager step of one sub-iteration (profiling target of the "
                         "interface, boundary and IBM kernels)")
    ap.add_argument("--lusgs-only", action="store_true",
                    help="LU-SGS sub-iterations alone on a smaller case (profiling target)")
    ap.add_argument("--ncx", type=int, default=6,
                    help="cubes per edge for --flux-only / --lusgs-only")
    ap.add_argument("--n", type=int, default=24,
                    help="cells per cube edge for --flux-only / --lusgs-only")
    ap.add_argument("--method", default="rk3", choices=["rk3", "lusgs"],
                    help="sub-iteration method (rk3: the reference's RK; lusgs: LU-SGS sweeps)")
    ap.add_argument("--workload", default="batch", choices=sorted(WORKLOADS),
                    help="batch (default: 16 batched sphere cases, the configuration the "
                         "metric's split-precision target is quoted on), tgv, vortex, sphere, "
                         "tgv32")
    ap.add_argument("--flux-form", type=int, default=None, choices=[0, 1, 2],
                    help="override the split flux form of the tuning table (1 packed face "
                         "pairs, 2 one face at a time)")
    ap.add_argument("--accuracy", type=int, default=0, metavar="STEPS",
                    help="accuracy over STEPS dual-time steps (split vs FP64 from the same "
                         "state, checkpoints at each quarter) instead of the benchmark")
    ap.add_argument("--acc-steps", type=int, default=ACC_STEPS,
                    help="dual-time steps of the split-vs-FP64 accuracy comparison")
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = args.workload
    if args.flux_only:
        run_flux_only(args)
        return
    if args.accuracy > 0:
        run_accuracy(args)
        return
    if args.lusgs_only:
        run_lusgs_only(args)
        return
    if args.step_only:
        run_step_only(args)
        return
    if args.impl == "reference":
        # Rank 0 alone times the CPU implementation; other ranks exit at once.
        class R0:
            rank = int(os.environ.get("RANK", "0"))
        run_reference_arm(args, R0())
        return
    dist = Dist(args.gpus)
    run_gpu_arm(args, dist)
    dist.close()


if __name__ == "__main__":
    main()
