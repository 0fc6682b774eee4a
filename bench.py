"""Benchmark of the GB300 L-sweeps path: FGMRES + checkerboard L-sweep
preconditioner solves.  Default workload C4: 4127^2 elements, seeded
piecewise-smooth medium c in [1.5, 5.0], 32 x 32 cells of 128^2, PML 20,
8 points per wavelength at c_min, one centred source; `--config C1..C3`
selects the other workloads.

A step is one complete solve to true relative residual 1e-6 with the cell
factors resident in HBM (the workload's factor arithmetic -- BF16-split
tensor-core products for C4, complex64 for C1-C3 -- inside FP64 flexible
GMRES(30)); the plain FP64 GPU path (complex128 factors) is measured beside it.
Prints one JSON line (see the keys below).  `--impl reference` times the CPU
oracle's restatement of the reference instead (the reference itself cannot be
built: no Eigen / libconfig++ / MPI)."""
from __future__ import annotations

import argparse
import re
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "l-sweeps-2d_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "time-to-solution & solves/s at rel. residual 1e-6: mixed vs FP64 on GB300; p50/p99"
UNIT = "solves/s"
WORKLOADS = {
    "C1": "C1: 2D Helmholtz, 259^2 elements, c = 1, 10 ppw, 4x4 checkerboard of 64^2 cells, PML 10, "
          "1 point source, FGMRES(30) tol 1e-6",
    "C2": "C2: 2D Helmholtz, 1031^2 elements (1062^2 DOFs with PML), Gaussian lens c=1-0.4exp(-r^2/0.02), "
          "8 ppw at c_min, 8x8 checkerboard of 128^2 cells, PML 16, 1 point source, FGMRES(30) tol 1e-6",
    "C3": "C3: 2D Helmholtz, 2063^2 elements, 12 seeded layers c in [1.5,4.5] + 5% smoothed perturbation, "
          "8 ppw, 16x16 checkerboard of 128^2 cells, PML 20, 64 sources on a line solved as one batch of "
          "64 right-hand sides, FGMRES(30) tol 1e-6",
    "C4": "C4: 2D Helmholtz, 4127^2 elements, seeded piecewise-smooth c in [1.5,5.0] (sigma 8 cells), "
          "8 ppw at c_min, 32x32 checkerboard of 128^2 cells, PML 20, 1 centred source, FGMRES(30) tol 1e-6",
}
WORKLOAD = WORKLOADS["C4"]
# factor and sweep arithmetic per workload: complex FP32 where the workload names it, the
# BF16-split tensor-core products (hi + lo bf16 terms, FP32 accumulation) for the 4096^2 case
PRECISION = {"C1": "c64", "C2": "c64", "C3": "c64", "C4": "bf16x2"}
DATA = {"C1": "synthetic (constant medium)", "C2": "synthetic (seeded Gaussian-lens medium)",
        "C3": "synthetic (seeded layered medium)", "C4": "synthetic (seeded piecewise-smooth random medium)"}
# how L2 is kept out of the timing: every workload streams more factor bytes per apply than L2 holds
L2_NOTE = {n: f"inputs larger than L2 (129 MB): {gb} of cell factors streamed per preconditioner apply"
           for n, gb in (("C1", "0.1 GB"), ("C2", "2.3 GB (c64)"), ("C3", "10.7 GB (c64)"),
                         ("C4", "43.9 GB (bf16x2)"))}
DTYPE = {"c64": "c64 factors/applies + f64 Krylov",
         "bf16x2": "bf16-split factor products (hi+lo, fp32 accumulate) + f64 Krylov",
         "c128": "c128 factors/applies + f64 Krylov"}


def pctl(v, q):
    s = sorted(v)
    if not s:
        return None
    k = (len(s) - 1) * q
    f = int(k)
    c = min(f + 1, len(s) - 1)
    return s[f] + (s[c] - s[f]) * (k - f)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        if self.p is None:
            return None
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (SuperLU local solves) on a bounded sample
# ---------------------------------------------------------------------------
def max_over_ranks(x: float, dist=None, device="cpu") -> float:
    """The maximum of x over the ranks of the process group (x itself without
    one); the tensor lives on `device` (the GPU for NCCL, the CPU for gloo)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_iterations(name: str) -> dict:
    """The reference GMRES's iteration count on a workload (committed fixture,
    tests/golden/make_reference_iterations.py)."""
    f = ROOT / "tests" / "golden" / "reference_gmres_iterations.json"
    return json.loads(f.read_text())[name]


def reference_sample(spec, name: str, med, parts: int, warmup_parts: int = 0, procs: int | None = None,
                     log=None) -> dict:
    """Time the oracle's restatement of the reference on the host cores: the
    DDCheckerboard apply (DDCheckerboard::applyPrecond, DDCheckerboard.cpp:
    687-739) with its cell solves spread over worker processes that own rows
    of cells round-robin (the reference's MPI layout,
    DDCheckerboard.cpp:126-177; SuperLU, one thread each), front by front as
    the reference's pipelined sweeps run them.  `parts` timed shifted parts
    (one of the four shifted decompositions each, in turn) give the apply time;
    the DD matvec, the Arnoldi dot and axpy on the global vectors are timed
    once.  A reference solve of k iterations (GlobalIterativeSolverGMRES.cpp:
    65-203) costs k + 2 applies (75, 82, 255), k + 1 matvecs and
    sum_{j<k} (j + 1) dot + axpy pairs."""
    import numpy as np
    from oracle.parallel import ParallelOracle
    procs = procs or os.cpu_count() or 1
    k = reference_iterations(name)["iterations"]
    t0 = time.perf_counter()
    with ParallelOracle(spec.N, spec.m, spec.p, spec.h, spec.omega, med, procs=procs) as Q:
        setup_s = time.perf_counter() - t0
        procs = Q.procs   # at most one worker per row of cells, as the reference's ranks
        rng = np.random.default_rng(0)
        n2 = Q.n_dof ** 2
        xc = Q.cells_of(rng.standard_normal(n2) + 1j * rng.standard_normal(n2))
        per_q = {0: [], 1: [], 2: [], 3: []}
        steps = []
        for i in range(warmup_parts + parts):
            q = i % 4
            t = time.perf_counter()
            res = Q.dd.apply_precond_part(xc, q)
            dt = time.perf_counter() - t
            if i >= warmup_parts:
                per_q[q].append(dt)
                steps.append(dt)
            if log:
                log(f"part {q}: {dt:.2f} s")
        for q in range(4):   # parts never timed: their warm-up times
            if not per_q[q]:
                t = time.perf_counter()
                Q.dd.apply_precond_part(xc, q)
                per_q[q].append(time.perf_counter() - t)
        t = time.perf_counter()
        ax = Q.dd.apply_system_matrix(xc)
        t_mv = time.perf_counter() - t
        del res, ax
    a = np.concatenate(xc)
    b = a[::-1].copy()
    td, ta = [], []
    for _ in range(3):
        t = time.perf_counter()
        np.vdot(a, b)
        td.append(time.perf_counter() - t)
        t = time.perf_counter()
        b = b - 0.5 * a
        ta.append(time.perf_counter() - t)
    t_dot, t_axpy = statistics.median(td), statistics.median(ta)
    t_apply = sum(statistics.median(per_q[q]) for q in range(4))
    t_krylov = (k + 1) * t_mv + sum(j + 1 for j in range(k)) * (t_dot + t_axpy)
    t_solve = (k + 2) * t_apply + t_krylov
    return {
        "value": 1.0 / t_solve, "unit": UNIT, "cores": procs, "kind": "port",
        "sample": (f"timed apply: the oracle's restatement of DDCheckerboard::applyPrecond on {name} "
                   f"({spec.N}x{spec.N} cells, {Q.n_dof}^2 DOFs) with its SuperLU cell solves on {procs} "
                   f"worker processes owning rows of cells round-robin (the reference's MPI layout), front by "
                   f"front; {len(steps)} timed shifted parts (one of the four shifted decompositions each): "
                   f"apply {t_apply:.2f} s; DD matvec {t_mv:.2f} s, dot {t_dot * 1e3:.1f} ms, axpy "
                   f"{t_axpy * 1e3:.1f} ms on the global vectors; a reference GMRES solve of {k} iterations "
                   f"(committed count) = {k + 2} applies + {k + 1} matvecs + {k * (k + 1) // 2} MGS dot/axpy "
                   f"pairs = {t_solve:.1f} s; cell factorisation ({Q.factorize_s:.1f} s per worker) not "
                   f"included (factors resident on both sides)"),
        "t_apply_s": t_apply, "t_solve_s": t_solve, "iterations": k, "setup_s": setup_s,
        "step_s": steps, "t_matvec_s": t_mv,
    }


def bench_config(name: str, nrhs: int, world: int) -> dict:
    """The workload description shared by both arms."""
    from lsweeps.problems import config as _cfg
    return {"workload": WORKLOADS[name], "restart": 30, "tol": 1e-6, "parallelism": f"replicas x{world}",
            "nrhs": nrhs, "l2": L2_NOTE[name]}


def run_reference(args):
    """--impl reference: the CPU restatement of the reference path, timed on
    the host cores (every core, one worker process each); rank 0 only.  Each
    step is one shifted part of a preconditioner apply of the workload (see
    reference_sample)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from lsweeps.problems import config
    name = args.config.upper()
    spec, med = config(name)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    smp = reference_sample(spec, name, med, parts=args.steps, warmup_parts=args.warmup,
                           log=lambda m: print(m, file=sys.stderr, flush=True))
    v = smp["value"]
    nrhs = len(spec.sources) if name == "C3" else 1
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(smp["step_s"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": DATA[name], "config": bench_config(name, nrhs, world),
        "precision": "fp64 (reference arithmetic)", "iterations": smp["iterations"],
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": smp["cores"], "kind": "port", "sample": smp["sample"]},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def run_gpu(args):
    import numpy as np
    import torch
    from lsweeps.problems import config
    from lsweeps.solver import Solver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    spec, med = config(args.config)
    prec = args.precision or PRECISION[args.config.upper()]
    S = Solver(spec, med, precision=prec, device=local)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    S.factorize()
    e1.record(st)
    torch.cuda.synchronize()
    fact_s = e0.elapsed_time(e1) / 1e3
    if args.config.upper() == "C3":
        # one right-hand side per source, solved as one batch
        b = torch.cat([S.assemble_rhs([src]) for src in spec.sources])
    else:
        b = S.assemble_rhs(spec.sources)
    nrhs = b.numel() // S.n2
    x = torch.empty_like(b)
    # the sweep-front launch shapes of this batch size are measured (or read
    # from the tuner's cache) before anything is timed
    S.front_shapes(nrhs)

    def solve():
        return S.gmres(b, mode="flexible", tol=args.tol, max_iter=300, restart=30, x=x)

    for _ in range(args.warmup):
        _, rep = solve()
    launches0 = S.info()["kernel_launches"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    reps = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            ev[i][0].record(st)
            _, rep = solve()
            ev[i][1].record(st)
            reps.append(rep)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
    if dist:
        dist.barrier()
    gpu_launches = S.info()["kernel_launches"] - launches0
    step_ms = [a.elapsed_time(c) for a, c in ev]
    dev_total = max_over_ranks(sum(step_ms) / 1e3, dist, dev)
    value = world * args.steps * nrhs / dev_total   # right-hand sides solved per second

    # end to end through the host-buffer C call (H2D of b, D2H of x in the timed region)
    # (pinned host buffers for every right-hand side of the batch; the device
    # solves' workspaces are released first so that a large batch fits)
    S.release_workspace()
    bh = torch.empty(b.numel(), dtype=torch.complex128, pin_memory=True)
    bh.copy_(b.cpu())
    bnp = bh.numpy()
    xnp = torch.empty(b.numel(), dtype=torch.complex128, pin_memory=True).numpy()
    for _ in range(1):
        S.solve_host(bnp, tol=args.tol, max_iter=300, restart=30, x_host=xnp)
    torch.cuda.synchronize()
    te = []
    for _ in range(args.e2e_steps):
        t = time.perf_counter()
        xh, rep_h = S.solve_host(bnp, tol=args.tol, max_iter=300, restart=30, x_host=xnp)
        te.append(time.perf_counter() - t)
    e2e_value = world * len(te) * nrhs / sum(te)

    # roofline of the dominant kernel (sweep fronts) from CUDA events
    # the solves' Krylov bases go first: a many-right-hand-side batch would not
    # leave room for the apply's pools otherwise
    S.release_workspace()
    prof_runs = []
    v = torch.randn(S.n2 * nrhs, dtype=torch.complex128, device=dev)
    for _ in range(3):
        _, pr = S.apply_precond_profiled(v)
        prof_runs.append(pr)
    front_ms = statistics.median(p["front_ms"] for p in prof_runs)
    pr = prof_runs[-1]

    # launch shapes: the tuner's per-front choice against the cost model's, and
    # one apply replayed as a CUDA graph against its kernels launched one by one
    def apply_ms(reps=3):
        ts = []
        for _ in range(reps + 1):
            a1, a2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a1.record(st)
            S.apply_precond(v)
            a2.record(st)
            torch.cuda.synchronize()
            ts.append(a1.elapsed_time(a2))
        return statistics.median(ts[1:])
    shapes, tune_s = S.front_shapes(nrhs)
    t_tuned_graph = apply_ms()
    S.set_graphs(False)
    t_tuned_eager = apply_ms()
    S.set_graphs(True)
    S.set_tuning(False)
    t_model_graph = apply_ms()
    model_shapes, _ = S.front_shapes(nrhs)
    S.set_tuning(True)
    apply_ms(1)
    # with per-sweep launches (batches of one or two right-hand sides): the
    # apply with one launch per sweep step beside it, on the same context
    steps_per_apply = 3 * spec.N - 3
    t_step_graph = None
    if len(shapes) > steps_per_apply:
        S.set_sweep_lanes(0)
        S.front_shapes(nrhs)
        t_step_graph = apply_ms()
        S.set_sweep_lanes(sweep_lanes_default())
        apply_ms(1)
    launch = {
        "apply_ms_tuned_graph": t_tuned_graph, "apply_ms_tuned_eager": t_tuned_eager,
        "apply_ms_model_graph": t_model_graph, "tune_s": tune_s,
        "per_sweep_launches": len(shapes) > steps_per_apply, "launches_per_apply": len(shapes),
        "apply_ms_one_launch_per_step_graph": t_step_graph,
        "fronts_changed_by_tuner": sum(1 for a, b in zip(shapes, model_shapes)
                                       if (a["slots_cap"], a["cluster"]) != (b["slots_cap"], b["cluster"])),
        "tuned_shapes": " ".join(f"{f['slots_cap']}x{f['cluster']}" for f in shapes),
    }
    # achieved: the apply's algorithmic bytes over the device time of the
    # apply as the solves run it (the captured graph, whose fronts run as one
    # launch per shifted decomposition on concurrent streams), CUDA events on
    # the launching stream; the fronts one by one (profiled, sequential) beside it
    achieved = pr["alg_bytes"] / (t_tuned_graph / 1e3) / 1e9
    achieved_sequential = pr["alg_bytes"] / (front_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    # DRAM traffic of the fronts: the ncu capture's traffic per algorithmic
    # byte (a full C2 apply of the same kernel and precision) times this
    # apply's algorithmic bytes
    # (the capture of the same schedule kind: per-sweep launches or one launch
    # per step, where one exists)
    traffic, traffic_key = None, None
    tf = ROOT / "profiles" / "k_front_dram_traffic.md"
    if tf.exists() and prec in ("c64", "bf16x2"):
        keys = ([prec + "_per_sweep"] if launch["per_sweep_launches"] else []) + [prec]
        for key in keys:
            m = re.search(r"traffic_per_alg_byte_%s:\s*([0-9.eE+]+)" % key, tf.read_text())
            if m:
                traffic, traffic_key = float(m.group(1)) * pr["alg_bytes"], key
                break

    # plain FP64 GPU path
    S64 = None
    fp64 = None
    if args.fp64_steps > 0:
        S64 = Solver(spec, med, precision="c128", device=local)
        e0.record(st)
        S64.factorize()
        e1.record(st)
        torch.cuda.synchronize()
        f64_fact = e0.elapsed_time(e1) / 1e3
        S64.front_shapes(nrhs)
        x64 = torch.empty_like(b)
        if args.fp64_warmup:
            S64.gmres(b, mode="flexible", tol=args.tol, max_iter=300, restart=30, x=x64)
        t64, r64 = [], None
        for _ in range(args.fp64_steps):
            a1, a2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a1.record(st)
            _, r64 = S64.gmres(b, mode="flexible", tol=args.tol, max_iter=300, restart=30, x=x64)
            a2.record(st)
            torch.cuda.synchronize()
            t64.append(a1.elapsed_time(a2))
        fp64 = {"p50_ms": pctl(t64, 0.5), "p99_ms": pctl(t64, 0.99), "iterations": r64.iterations,
                "true_rel_res": r64.true_rel_res, "factorize_s": f64_fact, "steps": len(t64),
                "warmup_solves": args.fp64_warmup}
        # the mixed and FP64 solutions of the same right-hand side agree
        fp64["rel_diff_vs_mixed"] = float((x - x64).norm() / x64.norm())
        S64.close()
        S64 = None
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu:
        # the Krylov bases and factors go first: the oracle's workers hold the
        # cell factors in host memory, not on the GPU, but this keeps the
        # process's footprint to the solver it timed
        cpu = reference_sample(spec, args.config.upper(), med, parts=4)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}

    clocks = clk.summary()
    if rank == 0:
        p50 = pctl(step_ms, 0.5)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_total * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[prec],
            "data": DATA[args.config.upper()],
            "config": bench_config(args.config.upper(), nrhs, world),
            "precision": "mixed" if prec != "c128" else "fp64", "factor_precision": prec,
            "factor_bytes": S.info()["factor_bytes"],
            "p50_ms": p50, "p99_ms": pctl(step_ms, 0.99), "iterations": reps[-1].iterations,
            "true_rel_res": reps[-1].true_rel_res, "factorize_s": fact_s,
            "time_to_solution_s": fact_s + p50 / 1e3,
            "fp64": fp64,
            "mixed_vs_fp64_speedup": (fp64["p50_ms"] / p50) if fp64 else None,
            "mixed_vs_fp64_tts_speedup": ((fp64["factorize_s"] + fp64["p50_ms"] / 1e3) / (fact_s + p50 / 1e3))
            if fp64 else None,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "traffic_source": "ncu DRAM bytes per algorithmic byte of a full C2 apply of this kernel "
                                           "(traffic_per_alg_byte_%s in profiles/k_front_dram_traffic.md), times "
                                           "this apply's algorithmic bytes" % traffic_key if traffic else None,
                         "kernel": "k_front (sweep-front cell solves), all fronts of one apply (graph replay)",
                         # the launches one by one on one stream (profiled): no overlap between
                         # launches, so below the replayed apply, far below with per-sweep launches
                         "achieved_launches_serialised": achieved_sequential,
                         "peak_kind": peak_kind, "alg_bytes_per_apply": pr["alg_bytes"],
                         "streamed_bytes_per_apply": pr["streamed_bytes"],
                         "launch_ms_per_apply_serialised": front_ms, "launches": pr["fronts"],
                         "items": pr["items"],
                         "slots": pr["slots"], "apply_ms": pr["total_ms"]},
            "launch_shapes": launch,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": S.n2 * 16 * nrhs,
                    "d2h_bytes_per_step": S.n2 * 16 * nrhs, "steps": len(te)},
            "clocks": clocks,
            "gpu_launches": gpu_launches,
            "wall_s_timed": elapsed,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def run_apply_only(args):
    """Set up and factorise one configuration, then run `--warmup` + `--steps`
    preconditioner applies on a random vector (the workload of the ncu captures)."""
    import torch
    from lsweeps.problems import config
    from lsweeps.solver import Solver
    spec, med = config(args.config)
    prec = args.precision or PRECISION[args.config.upper()]
    S = Solver(spec, med, precision=prec)
    S.factorize()
    shapes, tune_s = S.front_shapes(args.nrhs)   # tuned before anything is timed
    v = torch.randn(S.n2 * args.nrhs, dtype=torch.complex128, device="cuda")
    y = torch.empty_like(v)
    for _ in range(args.warmup):
        S.apply_precond(v, out=y)
    st = torch.cuda.current_stream()
    ts = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        S.apply_precond(v, out=y)
        e1.record(st)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    line = {"apply_only": args.config, "precision": prec, "nrhs": args.nrhs,
            "applies": args.warmup + args.steps, "steps_per_apply": 3 * spec.N - 3,
            "launches_per_apply": len(shapes), "tune_s": round(tune_s, 2),
            "shapes": " ".join("%dx%d%s" % (f["slots_cap"], f["cluster"], "t" if f["tensor_cores"] else "")
                               for f in shapes)}
    if ts:
        # graph-replayed applies, CUDA events on the launching stream
        med_ms = statistics.median(ts)
        line.update({"apply_ms": round(med_ms, 3), "apply_ms_per_rhs": round(med_ms / args.nrhs, 3)})
        if len(shapes) > 3 * spec.N - 3:
            # per-sweep launches: the same applies with one launch per sweep step
            S.set_sweep_lanes(0)
            S.front_shapes(args.nrhs)
            S.apply_precond(v, out=y)
            t1 = []
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                S.apply_precond(v, out=y)
                e1.record(st)
                torch.cuda.synchronize()
                t1.append(e0.elapsed_time(e1))
            line["apply_ms_one_launch_per_step"] = round(statistics.median(t1), 3)
            S.set_sweep_lanes(sweep_lanes_default())
    if args.warmup + args.steps > 0:
        # the algorithmic and streamed bytes of one apply (one more, profiled, apply)
        _, pr = S.apply_precond_profiled(v)
        line.update({k: pr[k] for k in ("alg_bytes", "streamed_bytes", "front_ms", "fronts", "items")})
    print(json.dumps(line))


def sweep_lanes_default() -> int:
    """The context's per-sweep launch threshold as created (LSW_SWEEP_LANES or 2)."""
    return max(0, int(os.environ.get("LSW_SWEEP_LANES", "2")))


def run_serve(args):
    """Serving stream (grids 256^2-2048^2 of 128^2 cells, 6-10 points per
    wavelength, lens/layered media with 30 % repeats, 1-16 sources, Poisson
    arrivals): one JSON line per arrival rate with p50/p99 latency and
    solves/s.  The stream is a scaled-down instance (`--serve-requests`) of
    the 2,000-request workload."""
    from lsweeps.serving import GpuBackend, ServeEngine, serving_stream
    rates = [float(r) for r in args.serve_rates.split(",")]
    for i, rate in enumerate(rates):
        # every rate starts from an empty factor cache with its own stream
        eng = ServeEngine(GpuBackend(0), slots=args.serve_slots, max_batch=8)
        # --serve-window caps the stream by time: the requests of that many
        # seconds of Poisson arrivals at this rate
        n_req = max(1, int(round(rate * args.serve_window))) if args.serve_window > 0 else args.serve_requests
        reqs = serving_stream(n_req, rate_hz=rate, seed=3 + i)
        st = eng.run(reqs, realtime=True)
        res = [r.true_rel_res for r in reqs if r.error is None]
        errs = {}
        for r in reqs:
            if r.error is not None:
                k = r.error[:160]
                errs[k] = errs.get(k, 0) + 1
        print(json.dumps({"metric": "serving: p50/p99 latency and solves/s at rel. residual 1e-6",
                          "rate_hz": rate, "requests": len(reqs), "unit": "solves/s",
                          "value": st.solves_per_s, **st.as_dict(),
                          "max_true_rel_res": max(res) if res else None,
                          "errors": errs,
                          "config": {"workload": "serving stream: grids {256,512,1024,2048}^2 of 128^2 cells, "
                                                 "6-10 ppw, lens/layered media with 30% repeats, 1-16 sources, "
                                                 "Poisson arrivals", "precision": "mixed", "slots": args.serve_slots,
                                     "max_batch": 8}}), flush=True)
        eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--fp64-warmup", type=int, default=None,
                    help="untimed FP64 solves before the timed ones (default 1, 0 for C4: ~85 s each)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--apply-only", action="store_true", help="only preconditioner applies (profiling workload)")
    ap.add_argument("--serve", action="store_true", help="serving stream at the rates of --serve-rates")
    ap.add_argument("--serve-rates", default="1,4,16")
    ap.add_argument("--serve-requests", type=int, default=40)
    ap.add_argument("--serve-window", type=float, default=0.0,
                    help="seconds of arrivals per rate (overrides --serve-requests when > 0)")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--config", default="C4")
    ap.add_argument("--precision", default=None, choices=["c64", "bf16x2", "c128"],
                    help="factor/sweep arithmetic (default: the workload's, c64 for C1-C3, bf16x2 for C4)")
    ap.add_argument("--nrhs", type=int, default=1)
    args = ap.parse_args()
    if args.fp64_warmup is None:
        args.fp64_warmup = 0 if args.config.upper() == "C4" else 1
    if args.serve:
        run_serve(args)
        return
    if args.apply_only:
        run_apply_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
