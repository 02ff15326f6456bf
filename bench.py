"""Benchmark of the GB300 gas-phase step (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A step is one gas-phase time step of every scenario of the workload, with the
pressure solve run to a relative residual of 1e-8 (max|r| <= 1e-8 max|b|).
value = cell-updates/s (cells x steps / device seconds) with all state resident
in HBM, timed with CUDA events on the solver's stream, L2 flushed before each
step when the working set fits in L2. e2e = the same metric through the C ABI
per step: phx_batch_step with every scenario's dtMax copied from pinned host
memory, then every scenario's stats (phx_stats: time, dt, heat-release rate,
CG iterations, residual, ...) read back to the host. cpu_baseline = the
reference's own FP32 solver (oracle/_ref) on the host cores, on a bounded
sample of the same workload. plain_c1 / plain_c2: the plain FP64 method on the
36x24x24 single room and the 72x52x44 house, each with the reference's FP32
and FP64 CPU builds timed on the same grid.

--impl reference times the reference's own CPU step (oracle/_ref) on the same
workload: every scenario of the batch, stepped by one reference solver thread
each, as many scenarios at a time as the host has threads. With --gpus N > 1
(torchrun) the work is replicated: every rank steps its own copy, no
collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s, mixed+batched vs FP64 GPU @1e-8 resid; p50/p99 scenario latency"
REL_TOL = 1e-8


def tol_str(x: float) -> str:
    """1e-08 -> 1e-8"""
    return ("%g" % x).replace("e-0", "e-")
SPINUP_STEPS = 100   # untimed steps that develop the plume before warm-up


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(t_s: float) -> float:
    """The timed region of the slowest rank (replicas: each rank steps its own
    batch; the whole job's rate is all ranks' cell-updates over this time)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return t_s
    import torch
    t = torch.tensor([t_s], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def whole_job_rate(cells: int, steps: int, world: int, t_s: float) -> float:
    """cell-updates/s of N replicas of the workload over the slowest rank's time"""
    return cells * steps * world / t_s


def make_workloads(name: str):
    """list of cases of a workload"""
    from photon_gb300 import casegen
    if name == "batch64":
        cs = casegen.batch_scenarios(64)
        for c in cs:
            c.profile.tol = 0.0
            c.profile.rel_tol = REL_TOL
            c.profile.maxIters = 400
        return cs
    return [make_workload(name)]


def make_workload(name: str):
    from photon_gb300 import casegen
    if name == "house_72x52x44":
        c = casegen.house_small(1)
    elif name == "single_room_36x24x24":
        c = casegen.single_room()
    elif name == "house_144x104x88":
        c = casegen.house_fine(1)
    else:
        raise SystemExit("unknown workload " + name)
    c.profile.tol = 0.0
    c.profile.rel_tol = REL_TOL
    c.profile.maxIters = 400
    return c


# Algorithmic bytes per unit of each kernel's domain for storage width w
# (8 for FP64 fields, 4 for the mixed path): each input array read once and
# each output written once per launch; uint8 masks count 1 B, int32 maps 4 B.
# The mixed path's level-0 kernels read one coefficient-code byte per cell in
# place of the diagonal and the three coefficient arrays.
def kernel_bytes(name: str, w: int):
    coded = w == 4
    table = {
        "k_advect": 18 * w + 1 + 10 * w,        # 10 scalars + u,v,w + fx,fy,fz + Pb,nu + blocked -> 10 scalars
        "k_momentum": 9 * w,                    # vel, 2 other components, fo, Pb, T, nu, p -> vel' (per face)
        "k_gs_pre": 2 * w + 1 if coded else 6 * w,                 # r, code (diag, 3 coefficients) -> z
        "k_gs_black": 3 * w + 4 + 1 if coded else 6.5 * w + 4,     # r, z, agg, code -> z (black)
        "k_gs_red_dot": 3 * w + 1 if coded else 6.5 * w,           # r, z, code -> z (red), r.z
        "k_cg_apply": 4 * w + 1 if coded else 8 * w,               # z, d, code -> d, q
        "k_cg_update": 7 * w,                   # p, d, r, q, diag -> p, r
        "k_res_restrict": 2 * w + 4 + 1 if coded else 6 * w + 4,   # r, z, agg, code -> level-1 b
        "k_rhs": 13 * w + 1,
        "k_heat": 8 * w + 1,
        "k_energy": 6 * w + 1,
        "k_combust": 6 * w + 3,
        "k_turb_filter": 6 * w + 1,             # three components along one axis -> three components
        "k_turb_center": 6 * w + 1,
        "k_turb_nu": 5 * w + 1,
        "k_velcorr": 5 * w,
        "k_stats": 4 * w + 1,
        "k_mx_res64": 8 + 3 * w + 1,            # p64, b, code -> r, e
        "k_mx_update": 8 + 8 + 2 * w,
    }
    return table.get(name)


# DRAM bytes (read + write) per cell of each level-0 kernel, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum of the first full-batch launch
# on the 64-scenario batch, mixed path, divided by its 7,964,799 cells)
NCU_BYTES_PER_CELL = {"k_gs_pre": 22.7, "k_res_restrict": 30.0, "k_gs_black": 32.3, "k_gs_red_dot": 26.8,
                      "k_cg_apply": 25.6, "k_cg_update": 23.5, "k_mx_res64": 34.5}


def jacobi_step_bytes(levels, iters, w: int) -> float:
    """Algorithmic bytes of one step's coarse-level damped Jacobi sweeps
    (k_jacobi): every scenario runs it + 1 V-cycles, each with three sweeps of
    each level 1..L-2 (one on the way down -- the from-zero sweep is fused into
    the restriction -- and two on the way up); a sweep of a level with n rows
    and nnz stored off-diagonal entries reads diag, b, the input vector and
    rowStart per row and col and val per entry and writes one value per row
    (4w + 4 per row, 4 + w per entry); the prolongating sweep also reads agg."""
    total = 0.0
    for (rows, nnz), it in zip(levels, iters):
        per_cycle = sum(rows[l] * (12 * w + 16) + 3 * (4 + w) * nnz[l] for l in range(1, len(rows) - 1))
        total += (it + 1) * per_cycle
    return total


def launched_cells(name: str, launches: int, iters, sizes) -> int:
    """Cells processed by all launches of one kernel in one step. A scenario
    that stopped after it CG iterations took part in it launches of q = A d and
    of the update, and in it + 1 V-cycles (level-0 sweeps and residual);
    every other kernel runs over every cell at each launch."""
    if name in ("k_cg_apply", "k_cg_update"):
        return sum(i * n for i, n in zip(iters, sizes))
    if name in ("k_gs_pre", "k_gs_black", "k_gs_red_dot", "k_res_restrict"):
        return sum((i + 1) * n for i, n in zip(iters, sizes))
    return launches * sum(sizes)


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    def __init__(self, gpu_index: int):
        self.proc = None
        # raw samples: PHX_CLOCKS_DIR if set, else the system temporary directory
        import tempfile
        self.path = os.path.join(os.environ.get("PHX_CLOCKS_DIR", tempfile.gettempdir()),
                                 "bench_clocks_%d.csv" % os.getpid())
        self.gpu = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return out
        sm, mxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mxs.append(float(r[1]))
                for n, v in zip(names, r[2:6]):
                    if v.strip().lower() in ("active", "1", "yes"):
                        reasons.add(n)
            except Exception:
                continue
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mxs), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def cpu_reference_rate(case, steps: int, warm: int, threads: int, bits: int = 32, budget_s: float = 20.0,
                       spinup: int = 0):
    """cell-updates/s of the reference's own CPU step on this case (oracle/_ref),
    or of the FP64 oracle port when the reference build is absent."""
    from oracle import refpy
    kind = "reference"
    if refpy.available(bits):
        s = refpy.RefSolver(case, bits, threads)
        stepf = lambda: s.step_relative(case.profile.dtMax, REL_TOL)
    else:
        from oracle.oraclepy import OracleSolver
        s = OracleSolver(case)
        kind, threads = "port", 1
        stepf = lambda: s.step(case.profile.dtMax)
    for _ in range(spinup + warm):
        stepf()
    t0 = time.perf_counter()
    n = 0
    while n < steps and (n == 0 or time.perf_counter() - t0 < budget_s):
        stepf()
        n += 1
    el = time.perf_counter() - t0
    return case.N * n / el, kind, threads, n, el


def cpu_model() -> str:
    """the host CPU's model name (lscpu, else /proc/cpuinfo)"""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        info = open("/proc/cpuinfo").read()
        for line in info.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
        imp = [l.split(":")[1].strip() for l in info.splitlines() if l.startswith("CPU implementer")]
        part = [l.split(":")[1].strip() for l in info.splitlines() if l.startswith("CPU part")]
        if imp and part:
            return "Arm implementer %s part %s" % (imp[0], part[0])
    except Exception:
        pass
    return "unknown"


def balance(sizes, workers):
    """scenario indices per worker, largest first onto the least-loaded worker"""
    load = [0] * workers
    out = [[] for _ in range(workers)]
    for i in sorted(range(len(sizes)), key=lambda i: -sizes[i]):
        w = min(range(workers), key=lambda k: load[k])
        out[w].append(i)
        load[w] += sizes[i]
    return [o for o in out if o]


def run_reference(args, rank, world):
    """The reference's own FP32 CPU step on every scenario of the workload,
    spun up like our arm. The scenarios are independent: each gets its own
    reference solver with one thread, and as many run at a time as the host
    has threads (measured faster than one scenario at a time with a thread per
    core, which leaves cores idle in the solver's serial parts)."""
    if rank != 0:
        return 0
    import threading
    cases = make_workloads(args.workload)
    threads = os.cpu_count() or 1
    from oracle import refpy
    if not refpy.available(32):
        print(json.dumps({"impl": "reference", "unavailable": "reference CPU build (oracle/_ref) is not present"}))
        return 0
    solvers = []
    for c in cases:
        # the reference has only an absolute CG stop: step_relative sets it before each step to
        # REL_TOL times the previous step's max|b|, the relative stop of our arm (1e-8 1/s for the
        # first step)
        c.profile.tol = 1e-8
        solvers.append(refpy.RefSolver(c, 32, 1))
    groups = balance([c.N for c in cases], threads)

    def phase(nsteps):
        def work(idx):
            for _ in range(nsteps):
                for k in idx:
                    solvers[k].step_relative(cases[k].profile.dtMax, REL_TOL)
        ths = [threading.Thread(target=work, args=(g,)) for g in groups]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    phase(args.spinup + args.warmup)
    t0 = time.perf_counter()
    phase(args.steps)
    el = time.perf_counter() - t0
    cells = sum(c.N for c in cases)
    v = cells * args.steps / el
    desc = ("%d steps of all %d scenarios (%d cells) after %d spin-up and %d warm-up steps; one reference solver "
            "thread per scenario, %d scenarios at a time" % (args.steps, len(cases), cells, args.spinup,
                                                               args.warmup, len(groups)))
    line = {"metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded house generator)",
            "config": {"workload": args.workload, "scenarios": len(cases), "cells": cells,
                       "pressure_stop": "relative %s: the reference's absolute stop set each step to %s max|b| of its "
                                        "previous step" % (tol_str(REL_TOL), tol_str(REL_TOL)), "threads": threads,
                       "spinup_steps": args.spinup,
                       "cpu_model": cpu_model(),
                       "hardware": "host CPU cores of rank 0 (the reference has no GPU path)"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "reference",
                             "sample": desc},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def step_bytes_model(k: float, w: int) -> float:
    """Algorithmic bytes per cell-update of one plain step with k CG
    iterations: every pass of the reference's step reads each input array once
    and writes each output once (153 + 61 k words of width w, 24 + 25 (k + 1)
    bytes of masks and maps)."""
    return (153 + 61 * k) * w + 24 + 25 * (k + 1)


def measure_plain(args, name: str):
    """The plain method on one grid: the FP64 GPU step (and the mixed one) timed
    with CUDA events after the same spin-up as the batch, with its roofline by
    the step's byte model, beside the reference's CPU builds on the same grid:
    FP32 with every host thread and with the default hardware threads - 2
    (Solver(), src/sim/solver.cpp:41), and the FP64 build."""
    from photon_gb300 import _lib
    from photon_gb300.solver import Batch
    out = {"workload": name}
    peak, peak_kind = measured_peak()
    for pname, prec, w in (("fp64", _lib.PREC_FP64, 8), ("mixed", _lib.PREC_MIXED, 4)):
        c = make_workload(name)
        g = Batch([c], prec)
        dtMax = c.profile.dtMax
        g.run(args.spinup + max(3, args.warmup), dtMax)
        flush = g.device_bytes() < (200 << 20)
        g.sync()
        ms, iters = [], []
        for _ in range(args.steps):
            t, _n = g.time_steps(1, dtMax, flush_l2=flush)
            ms.append(t)
            iters.append(g.stats(0)["pressure_iters"])
        value = c.N * args.steps / (sum(ms) / 1e3)
        k = float(np.mean(iters))
        achieved = step_bytes_model(k, w) * value / 1e9
        out[pname] = {"value": value, "unit": "cell-updates/s", "ms_per_step": sum(ms) / len(ms),
                      "cg_iters_mean": k, "cells": c.N,
                      "max_rel_residual_last_step": g.stats(0)["pressure_rel_residual"],
                      "roofline": {"bound": "hbm", "model": "step bytes per cell-update (153 + 61 k) w + 24 + 25 (k + 1)",
                                   "bytes_per_cell_update": step_bytes_model(k, w), "achieved": achieved,
                                   "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind},
                      "l2": "flushed before each step" if flush else "inputs larger than L2"}
        g.close()
    if not args.no_cpu_baseline:
        nproc = os.cpu_count() or 1
        cpu = {"cores": nproc, "cpu_model": cpu_model()}
        for key, bits, thr in (("ref32_all_threads", 32, nproc), ("ref32_default_threads", 32, max(1, nproc - 2)),
                               ("ref64_all_threads", 64, nproc)):
            c = make_workload(name)
            c.profile.tol = 1e-8
            v, kind, t_used, nst, el = cpu_reference_rate(c, steps=20, warm=2, threads=thr, bits=bits,
                                                          budget_s=args.cpu_budget, spinup=args.spinup)
            cpu[key] = {"value": v, "unit": "cell-updates/s", "threads": t_used, "kind": kind,
                        "sample": "%d steps after %d spin-up and 2 warm-up steps (%.1f s)" % (nst, args.spinup, el)}
        out["cpu_baseline"] = cpu
        out["fp64_over_ref32_all_threads"] = out["fp64"]["value"] / cpu["ref32_all_threads"]["value"]
    return out


def measure(args, precision, L, world, clocks: bool):
    """Timed steps of one precision on the workload: value, launches, per-kernel
    profile and roofline of the dominant kernel, e2e through the C ABI."""
    import ctypes
    from photon_gb300 import _lib
    from photon_gb300.solver import Batch
    cases = make_workloads(args.workload)
    cells = sum(c.N for c in cases)
    g = Batch(cases, precision)
    dtMax = cases[0].profile.dtMax
    if args.spinup > 0:
        g.run(args.spinup, dtMax)
    vcycle = None
    if precision == _lib.PREC_MIXED and not args.no_tune:
        # the V-cycle schedule per size bucket, tuned on the developed batch (state restored)
        t0 = time.perf_counter()
        stops = g.tune_vcycle(3, dtMax)
        vcycle = {"coarsening_stop_per_bucket": stops, "coarse_jacobi_sweeps_per_leg": g.coarse_sweeps,
                  "tuning_s": round(time.perf_counter() - t0, 2),
                  "buckets": "bucket b: [20000 * 2^b, 20000 * 2^(b+1)) cells"}
    g.run(max(3, args.warmup), dtMax)
    # a working set that fits in L2 is flushed before every timed step
    flush = g.device_bytes() < (200 << 20)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    g.sync()
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    if clocks:
        clk.__enter__()
    step_ms = []
    launches = 0
    for _ in range(args.steps):
        ms, nl = g.time_steps(1, dtMax, flush_l2=flush)
        step_ms.append(ms)
        launches += nl
    if clocks:
        clk.__exit__()
    g.sync()
    t_s = max_over_ranks(sum(step_ms) / 1e3)
    value = whole_job_rate(cells, args.steps, world, t_s)
    iters = [g.stats(s)["pressure_iters"] for s in range(len(cases))]
    rels = [g.stats(s)["pressure_rel_residual"] for s in range(len(cases))]
    # e2e through the C ABI: per step, the dtMax of every scenario goes down
    # from pinned memory and every scenario's stats (phx_stats) come back
    n = len(cases)
    h2d = L.phx_alloc_host(8 * n)
    dtm = (ctypes.c_double * n).from_address(h2d)
    for i in range(n):
        dtm[i] = dtMax
    dts = (ctypes.c_double * n)()
    st = _lib.PhxStats()
    for _ in range(2):
        L.phx_batch_step(g.h, ctypes.c_void_p(h2d), 0.0, dts)
    g.sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if L.phx_batch_step(g.h, ctypes.c_void_p(h2d), 0.0, dts) != 0:
            raise SystemExit(L.phx_last_error(g.h).decode())
        for s in range(n):
            L.phx_batch_get_stats(g.h, s, ctypes.byref(st))
    e2e_s = time.perf_counter() - t0
    L.phx_free_host(ctypes.c_void_p(h2d))
    e2e_value = cells * args.steps * world / e2e_s
    # per-kernel device times of one step (outside the timed region) for the roofline
    prof = g.profile_step(dtMax, flush_l2=flush)
    prof_iters = [g.stats(s)["pressure_iters"] for s in range(len(cases))]
    tot_prof = sum(p[2] for p in prof)
    w = 8 if precision == _lib.PREC_FP64 else 4
    # the dominant kernel of the step; the coarse-level Jacobi sweeps are
    # modelled per multigrid row, the other kernels per cell
    modelled = [p for p in prof if kernel_bytes(p[0], w) or p[0] == "k_jacobi"]
    top = max(modelled or prof, key=lambda p: p[2])
    per_unit = kernel_bytes(top[0], w)
    peak, peak_kind = measured_peak()
    roof = None
    if top[0] == "k_jacobi":
        levels = [(g.mg_levels(s), g.mg_nnz(s)) for s in range(len(cases))]
        total = jacobi_step_bytes(levels, prof_iters, w)
        bytes_per_launch = total / top[1]
        achieved = bytes_per_launch / (top[2] / top[1] / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "kernel": top[0], "kernel_share": top[2] / tot_prof,
                "algorithmic_bytes_per_launch": bytes_per_launch, "peak_kind": peak_kind,
                "model": "per V-cycle and level 1..L-2: rows (12w + 16) + 3 (4 + w) nnz (three sweeps)"}
    elif per_unit:
        # cells the kernel's launches of the profiled step processed: the CG
        # kernels skip scenarios that have stopped iterating
        units = launched_cells(top[0], top[1], prof_iters, [c.N for c in cases])
        bytes_per_launch = per_unit * units / top[1]
        achieved = bytes_per_launch / (top[2] / top[1] / 1e3) / 1e9
        traffic = None
        if precision == _lib.PREC_MIXED and top[0] in NCU_BYTES_PER_CELL and args.workload == "batch64":
            traffic = NCU_BYTES_PER_CELL[top[0]] * units / top[1]
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": top[0], "kernel_share": top[2] / tot_prof,
                "algorithmic_bytes_per_launch": bytes_per_launch, "peak_kind": peak_kind}
    g.close()
    sm = sorted(step_ms)
    pct = lambda q: sm[min(len(sm) - 1, int(round(q * (len(sm) - 1))))]
    return {"cases": cases, "cells": cells, "value": value, "t_s": t_s, "iters": iters, "rels": rels,
            "launches": launches, "roofline": roof, "clk": clk, "prof": prof, "e2e": e2e_value,
            "h2d": 8 * n, "d2h": n * ctypes.sizeof(_lib.PhxStats) + 8 * n, "flush": flush,
            "p50_ms": pct(0.5), "p99_ms": pct(0.99), "vcycle": vcycle}


def measure_serving(args, precision):
    """Serving form: a Poisson stream of house requests (20k-1.32M cells,
    seeded geometry, 10-500 kW burners) submitted by client threads at their
    arrival times, admitted under a 150 GB HBM budget and stepped together by
    one serving loop (continuous batching). The simulated durations of
    30-300 s are scaled by args.serve_scale (0.01 in the default line, so the
    run ends in about a minute; --serving-only --serve-scale 1 runs them
    unscaled). Returns throughput and p50/p99 step and completion latency."""
    import threading
    from photon_gb300 import casegen
    from photon_gb300.serve import Server
    reqs = casegen.serving_requests(args.serve_requests, args.serve_rate, seed=7)
    for _, c in reqs:
        c.profile.tol = 0.0
        c.profile.rel_tol = REL_TOL
    srv = Server(precision, hbm_budget_bytes=150 << 30)
    ids = [None] * len(reqs)
    arrival = [0.0] * len(reqs)
    t0 = time.monotonic() + 0.5
    lock = threading.Lock()
    nxt = [0]

    def client():
        while True:
            with lock:
                k = nxt[0]
                nxt[0] += 1
            if k >= len(reqs):
                return
            at, c = reqs[k]
            wait = t0 + at - time.monotonic()
            if wait > 0:
                time.sleep(wait)
            arrival[k] = time.monotonic()
            ids[k] = srv.submit(c, c.duration * args.serve_scale, c.profile.dtMax)

    clients = [threading.Thread(target=client) for _ in range(4)]
    for th in clients:
        th.start()
    step_ms = []
    done = set()
    tfirst = None
    while len(done) < len(reqs):
        c = srv.counts()
        if c["queued"] == 0 and c["running"] == 0:
            time.sleep(0.001)
        else:
            a = time.monotonic()
            tfirst = tfirst or a
            srv.step()
            step_ms.append((time.monotonic() - a) * 1e3)
        for k, rid in enumerate(ids):
            if rid is not None and k not in done and srv.poll(rid)["state"] in ("done", "rejected"):
                done.add(k)
    tend = time.monotonic()
    for th in clients:
        th.join()
    infos = [srv.poll(rid) for rid in ids]
    cell_updates = srv.counts()["cell_updates"]
    srv.close()
    comp = sorted(i["t_done"] - a for i, a in zip(infos, arrival))
    st = sorted(step_ms)
    pct = lambda v, q: v[min(len(v) - 1, int(round(q * (len(v) - 1))))]
    return {"value": cell_updates / (tend - tfirst), "unit": "cell-updates/s", "requests": len(reqs),
            "rejected": sum(1 for i in infos if i["state"] == "rejected"),
            "steps": len(step_ms), "wall_s": tend - tfirst,
            "step_p50_ms": pct(st, 0.5), "step_p99_ms": pct(st, 0.99),
            "completion_p50_s": pct(comp, 0.5), "completion_p99_s": pct(comp, 0.99),
            "config": {"arrivals": "Poisson, %.1f requests/s" % args.serve_rate,
                       "cells": "20k-1.32M log-uniform", "hbm_budget_gb": 150,
                       "duration": "30-300 s simulated x %g" % args.serve_scale,
                       "pressure_stop": "relative %s" % tol_str(REL_TOL)}}


def measure_radiation(args, cpu_baseline: bool):
    """The radiation trace (phx_rad_trace; Solver::traceRadiation,
    src/sim/radiation.cpp:181-319) on the seeded 144x104x88 house at 0.1 m
    (1.32 M cells) with its synthetic element set (casegen.rad_workload): device
    time of the trace kernels (CUDA events) and the end-to-end call with its
    host copies, per precision; the oracle's single-threaded restatement on a
    sample of the elements as the CPU baseline."""
    from photon_gb300 import _lib, casegen
    from photon_gb300.solver import Solver
    c = casegen.house_fine(1) if args.extras_case == "fine" else casegen.house_small(1)
    w = casegen.rad_workload(c)
    el, wl = _lib.rad_elements(w["elements"]), _lib.rad_walls(w["walls"])
    rays = int(32 * np.count_nonzero(el["sphere"])) + 16 * int(np.count_nonzero(el["sphere"] == 0))
    out = {"workload": "house %dx%dx%d at %.1f m (%d cells), %d elements, %d walls" % (
        c.nx, c.ny, c.nz, c.dx, c.N, len(el), len(wl)), "rays_per_trace_approx": rays}
    for name, prec in (("mixed", _lib.PREC_MIXED), ("fp64", _lib.PREC_FP64)):
        g = Solver(c, prec)
        for f, a in w["gas"].items():
            g.set(f, a)
        for _ in range(max(3, args.warmup)):
            g.rad_trace(el, wl, w["solidT"])
        dev, wall = [], []
        for _ in range(10):
            t = time.perf_counter()
            g.rad_trace(el, wl, w["solidT"])
            wall.append((time.perf_counter() - t) * 1e3)
            dev.append(g.rad_last_ms())
        g.close()
        out[name] = {"device_ms": float(np.median(dev)), "e2e_ms": float(np.median(wall)),
                     "traces_per_s": 1e3 / float(np.median(dev)),
                     "h2d_bytes": int(el.nbytes + wl.nbytes + w["solidT"].nbytes),
                     "d2h_bytes": int(len(el) * 8 + c.N * 8)}
    if cpu_baseline:
        from oracle import oraclepy
        k = max(1, len(el) // 16)
        sub = w["elements"][:k]
        t = time.perf_counter()
        oraclepy.rad_trace((c.nx, c.ny, c.nz), (c.dx, c.ox, c.oy, c.oz), c.blocked, w["gas"], sub, w["walls"],
                           w["solidT"])
        ms = (time.perf_counter() - t) * 1e3 * len(el) / k
        out["cpu_baseline"] = {"ms_per_trace": ms, "cores": 1, "kind": "port",
                               "sample": "oracle restatement, first %d of %d elements, scaled by element count" %
                                         (k, len(el))}
    return out


def measure_volume(args, cpu_baseline: bool):
    """The headless smoke and flame render (phx_vol_render; the viewer's
    VOL_FS shader) of the 1.32 M-cell house with the synthetic trace fields at
    1280x720: device time (CUDA events) and the end-to-end call; the oracle's
    C restatement of the shader on a band of rows as the CPU baseline."""
    from photon_gb300 import _lib, casegen, render
    from photon_gb300.solver import Solver
    c = casegen.house_fine(1) if args.extras_case == "fine" else casegen.house_small(1)
    w = casegen.rad_workload(c)
    g = Solver(c, _lib.PREC_MIXED)
    gas = dict(w["gas"])
    gas["Ys"] = gas["Ys"] * 0.01
    for f, a in gas.items():
        g.set(f, a)
    g.set("Ya", 0.5 * gas["Ys"])
    cx, cy = c.ox + c.nx * c.dx / 2, c.oy + c.ny * c.dx / 2
    p = render.camera(c, eye=(cx - 14, cy - 16, 9.0), target=(cx, cy, 2.0), width=1280, height=720,
                      lights=render.fire_lights(c, gas["hrr"]), slice_z=1.5)
    for _ in range(max(3, args.warmup)):
        g.vol_render(p)
    dev, wall = [], []
    for _ in range(10):
        t = time.perf_counter()
        g.vol_render(p)
        wall.append((time.perf_counter() - t) * 1e3)
        dev.append(g.vol_last_ms())
    out = {"workload": "house %dx%dx%d at %.1f m, 1280x720, smoke + fire + slice, step 0.3 dx" % (
        c.nx, c.ny, c.nz, c.dx), "device_ms": float(np.median(dev)), "e2e_ms": float(np.median(wall)),
        "frames_per_s": 1e3 / float(np.median(dev)), "d2h_bytes": 1280 * 720 * 12}
    if cpu_baseline:
        from oracle import oraclepy
        vol = oraclepy.pack_volume(c.blocked, g.get("T"), g.get("Ys"), g.get("Ya"), g.get("Pb"), g.get("hrr"))
        r0, r1 = 360 - 24, 360 + 24
        t = time.perf_counter()
        oraclepy.vol_render(c, vol, p, rows=(r0, r1))
        out["cpu_baseline"] = {"ms_per_frame": (time.perf_counter() - t) * 1e3 * 720 / (r1 - r0), "cores": 1,
                               "kind": "port", "sample": "oracle restatement of the shader, rows %d-%d of 720, "
                                                         "scaled by row count" % (r0, r1)}
    g.close()
    return out


def precision_study(args):
    """The precision form's outputs on the seeded house at 10 cm (144x104x88 =
    1.32 M cells): the per-step pressure error of the mixed path against the
    converged FP64 answer (an FP64 step from the same state with the pressure
    solved to a relative residual of 1e-12), sampled along an FP64 run; the
    same for the FP64 path at the 1e-8 stop; the mixed solve's divergence
    residual on every step; and the layer-averaged temperature profile of the
    mixed and FP64 runs after args.study_seconds simulated. The FP64 GPU path
    tracks the oracle within 1e-9 per step at these grid sizes."""
    from photon_gb300 import _lib, casegen
    from photon_gb300.solver import Solver

    def case(rel):
        c = casegen.house_fine(1)
        c.profile.tol = 0.0
        c.profile.rel_tol = rel
        return c
    c = case(REL_TOL)
    dt_max = c.profile.dtMax
    f64, mx = Solver(c, _lib.PREC_FP64), Solver(c, _lib.PREC_MIXED)
    probe, probe64, conv = Solver(c, _lib.PREC_MIXED), Solver(c, _lib.PREC_FP64), Solver(case(1e-12), _lib.PREC_FP64)
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    p_err, p_err64, n64 = [], [], 0
    while f64.stats()["time"] < args.study_seconds:
        if n64 % args.study_every == args.study_every // 2:
            for dst in (probe, probe64, conv):   # identical state, then one step each
                f64.export_state(dst)
            probe.step(dt_max)
            probe64.step(dt_max)
            conv.step(dt_max)
            pc = conv.get("p")
            p_err.append(rel(probe.get("p"), pc))
            p_err64.append(rel(probe64.get("p"), pc))
        f64.step(dt_max)
        n64 += 1
    rres, nmx = [], 0
    while mx.stats()["time"] < args.study_seconds:
        mx.step(dt_max)
        rres.append(mx.stats()["pressure_rel_residual"])
        nmx += 1
    gas = c.blocked.reshape(c.nz, c.ny, c.nx) == 0
    def layers(g):
        T = g.get("T").reshape(c.nz, c.ny, c.nx)
        return np.array([T[k][gas[k]].mean() if gas[k].any() else np.nan for k in range(c.nz)])
    lf, lm = layers(f64), layers(mx)
    ok = ~np.isnan(lf)
    lerr = np.abs(lm[ok] - lf[ok]) / lf[ok]
    return {"workload": "house %dx%dx%d at %.1f m (%d cells), seed 1" % (c.nx, c.ny, c.nz, c.dx, c.N),
            "simulated_s": args.study_seconds, "steps": {"fp64": n64, "mixed": nmx},
            "pressure_rel_l2_vs_converged": {
                "reference": "FP64 step from the same state, pressure solved to a relative residual of 1e-12",
                "samples": len(p_err), "mixed_max": max(p_err), "mixed_median": float(np.median(p_err)),
                "fp64_at_1e-8_max": max(p_err64), "fp64_at_1e-8_median": float(np.median(p_err64)),
                "mixed_all": [float("%.3e" % e) for e in p_err]},
            "pressure_stop": "relative %s (both paths' probe steps and the mixed run)" % tol_str(REL_TOL),
            "mixed_rel_residual": {"max": max(rres), "steps_above_stop": int(sum(r > REL_TOL for r in rres))},
            "layer_T_rel_err": {"max": float(lerr.max()), "mean": float(lerr.mean())},
            "layer_T_K": {"fp64": [round(float(v), 2) for v in lf[ok]], "mixed": [round(float(v), 2) for v in lm[ok]]}}


def main():
    global REL_TOL
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the reference's V-cycle schedule (no autotuning)")
    ap.add_argument("--cpu-budget", type=float, default=8.0, help="seconds of timed CPU steps per CPU baseline")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 lines on the 36x24x24 room and the "
                                                           "72x52x44 house")
    ap.add_argument("--spinup", type=int, default=SPINUP_STEPS, help="untimed steps before warm-up")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-rate", type=float, default=8.0, help="request arrivals per second (Poisson)")
    ap.add_argument("--serve-scale", type=float, default=0.01, help="scale of the 30-300 s simulated durations")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--rel-tol", type=float, default=REL_TOL,
                    help="the pressure solve's relative stop max|r| <= rel_tol max|b| for every arm (default 1e-8)")
    ap.add_argument("--serving-only", action="store_true",
                    help="only the serving form, per --precision (one JSON line; e.g. --serve-scale 1 for the "
                         "unscaled 30-300 s durations)")
    ap.add_argument("--no-radiation", action="store_true", help="skip the radiation trace and volume render")
    ap.add_argument("--extras-only", action="store_true",
                    help="time only the radiation trace and the volume render (one JSON line)")
    ap.add_argument("--precision-study", action="store_true",
                    help="the precision form's error outputs on the 1.32 M-cell house (one JSON line)")
    ap.add_argument("--study-seconds", type=float, default=60.0)
    ap.add_argument("--study-every", type=int, default=200, help="FP64 steps between pressure-error samples")
    ap.add_argument("--extras-case", default="fine", choices=["fine", "small"],
                    help="house for the trace and the render: 144x104x88 at 0.1 m, or 72x52x44 at 0.2 m")
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64"],
                    help="which paths to time (the line's value is the mixed path unless only fp64 runs)")
    args = ap.parse_args()
    REL_TOL = args.rel_tol
    rank, world, local = rank_info()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    from photon_gb300 import _lib
    L = _lib.load()
    if L.phx_select_device(local) != 0:
        raise SystemExit("cannot select device %d" % local)
    if args.precision_study:
        if rank == 0:
            print(json.dumps(precision_study(args)))
        return 0
    if args.serving_only:
        if rank == 0:
            out = {}
            if args.precision in ("both", "mixed"):
                out["mixed"] = measure_serving(args, _lib.PREC_MIXED)
            if args.precision in ("both", "fp64"):
                out["fp64"] = measure_serving(args, _lib.PREC_FP64)
            print(json.dumps({"serving": out}))
        return 0
    if args.extras_only:
        if rank == 0:
            print(json.dumps({"radiation_trace": measure_radiation(args, not args.no_cpu_baseline),
                              "volume_render": measure_volume(args, not args.no_cpu_baseline)}))
        return 0

    mixed = measure(args, _lib.PREC_MIXED, L, world, clocks=True) if args.precision in ("both", "mixed") else None
    fp64 = measure(args, _lib.PREC_FP64, L, world, clocks=mixed is None) if args.precision in ("both", "fp64") else None
    if mixed is None:           # FP64 only: it is the line's measurement
        mixed = fp64
    if fp64 is None:
        fp64 = mixed
    cases = mixed["cases"]
    serving = None
    if not args.no_serving:
        serving = {}
        if args.precision in ("both", "mixed"):
            serving["mixed"] = measure_serving(args, _lib.PREC_MIXED)
        if args.precision in ("both", "fp64"):
            serving["fp64"] = measure_serving(args, _lib.PREC_FP64)

    plain = {}
    if rank == 0 and not args.no_plain:
        plain["plain_c1"] = measure_plain(args, "single_room_36x24x24")
        plain["plain_c2"] = measure_plain(args, "house_72x52x44")

    radiation = volume = None
    if rank == 0 and not args.no_radiation:
        radiation = measure_radiation(args, not args.no_cpu_baseline)
        volume = measure_volume(args, not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the reference's FP32 CPU step on a sample of the workload: its
        # median-size scenario, spun up like the GPU arm
        sample = sorted(make_workloads(args.workload), key=lambda c: c.N)[len(cases) // 2]
        sample.profile.tol = 1e-8
        threads = os.cpu_count() or 1
        v, kind, thr, nst, el = cpu_reference_rate(sample, steps=20, warm=2, threads=threads, spinup=args.spinup)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": thr, "kind": kind,
               "sample": "%d steps of scenario %s (%d cells, %.1f s) after %d spin-up and 2 warm-up steps, FP32 "
                         "reference build, relative pressure stop 1e-8 (the absolute stop set each step from the previous max|b|)" % (nst, sample.name, sample.N, el, args.spinup)}
    if rank == 0:
        import ctypes
        line = {"metric": METRIC, "value": mixed["value"], "unit": "cell-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": mixed["t_s"] / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
                "data": "synthetic (seeded house generator; no dataset)",
                "config": {"workload": args.workload, "scenarios": len(cases), "cells": mixed["cells"],
                           "precision": "mixed: FP32 fields and stencils, FP32 MG-CG inside FP64 refinement",
                           "pressure_stop": "relative %s (max|r| <= %s max|b|, FP64)" % (tol_str(REL_TOL), tol_str(REL_TOL)),
                           "l2": "flushed before each step" if mixed["flush"] else "inputs larger than L2",
                           "spinup_steps": args.spinup,
                           "vcycle_schedule": mixed.get("vcycle"),
                           "cg_iters_last_step": {"min": min(mixed["iters"]), "max": max(mixed["iters"])},
                           "max_rel_residual_last_step": max(mixed["rels"]),
                           "parallelism": "replicas" if world > 1 else "single GPU, batched"},
                "latency": {"step_p50_ms": mixed["p50_ms"], "step_p99_ms": mixed["p99_ms"]},
                "e2e": {"value": mixed["e2e"], "unit": "cell-updates/s", "h2d_bytes_per_step": mixed["h2d"],
                        "d2h_bytes_per_step": mixed["d2h"]},
                "fp64": {"value": fp64["value"], "ms_per_step": fp64["t_s"] / args.steps * 1e3,
                         "cg_iters_last_step": {"min": min(fp64["iters"]), "max": max(fp64["iters"])},
                         "max_rel_residual_last_step": max(fp64["rels"]),
                         "gpu_launches": fp64["launches"], "roofline": fp64["roofline"], "e2e": fp64["e2e"],
                         "latency": {"step_p50_ms": fp64["p50_ms"], "step_p99_ms": fp64["p99_ms"]},
                         "kernels": [{"name": p[0], "launches": p[1], "ms": round(p[2], 4)} for p in
                                     sorted(fp64["prof"], key=lambda p: -p[2])[:10]]},
                "mixed_over_fp64": mixed["value"] / fp64["value"],
                **plain,
                "gpu_launches": mixed["launches"],
                "roofline": mixed["roofline"],
                "cpu_baseline": cpu,
                "serving": serving,
                "radiation_trace": radiation,
                "volume_render": volume,
                "clocks": mixed["clk"].summary(),
                "kernels": [{"name": p[0], "launches": p[1], "ms": round(p[2], 4)} for p in
                            sorted(mixed["prof"], key=lambda p: -p[2])]}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
