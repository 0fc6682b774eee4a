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


def _interior_cell(spec, med):
    """One interior C2-shaped cell (column/row 1: interior domain [a - 2h, b + 4h],
    (m + 6 + 2p - 1)^2 DOFs), assembled by the oracle."""
    from oracle.lsweeps_oracle import AssemblerHelmholtz2DFD, SubdomainStructured, grid_medium
    h, m = spec.h, spec.m
    a = (m + 1) * h
    dom = ((a - 2 * h, a + m * h + 4 * h), (a - 2 * h, a + m * h + 4 * h))
    asm = AssemblerHelmholtz2DFD(spec.omega, spec.p * h, grid_medium(med, h, spec.p))
    asm.set_domain(dom)
    asm.set_n((m + 6, m + 6))
    cell = SubdomainStructured(asm, 1, 1)
    cell.A = asm.assemble_system_matrix()
    cell.size = cell.A.shape[0]
    return cell


def _cell_solve_worker(spec, med, budget_s: float, barrier, results) -> None:
    """A worker process of the all-core sample: factorise the cell, wait for
    every worker, then solve for `budget_s`; reports the solves done."""
    import numpy as np
    cell = _interior_cell(spec, med)
    cell.factorize()
    rng = np.random.default_rng(os.getpid())
    b = rng.standard_normal(cell.size) + 1j * rng.standard_normal(cell.size)
    barrier.wait()
    t_end = time.perf_counter() + budget_s
    k = 0
    while time.perf_counter() < t_end:
        cell.solve(b)
        k += 1
    results.put(k)


def cpu_sample(spec, med, iterations: int, budget_s: float = 25.0, procs: int | None = None) -> dict:
    """Time the oracle's cell solves (SuperLU) on a sample of the C2 cells and
    extrapolate to one preconditioner apply (the apply is a sum of cell solves:
    N^2 + 4N(N-1) + 4(N-1)^2 per shifted decomposition, x4) and to one solve of
    `iterations` FGMRES iterations (iterations + 1 applies).  With procs > 1,
    `procs` spawned processes (one thread each) solve concurrently for the
    budget and their aggregate rate gives the per-solve time: the solves of a
    sweep front are independent (C2: >= 64 per front step), as the
    reference's ranks run them."""
    import numpy as np
    procs = procs if procs is not None else (os.cpu_count() or 1)
    t0 = time.perf_counter()
    cell = _interior_cell(spec, med)
    setup_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    cell.factorize()
    fact_s = time.perf_counter() - t1
    rng = np.random.default_rng(0)
    n = cell.size
    ts, k = [], 0
    t2 = time.perf_counter()
    single_s = min(3.0, budget_s / 3) if procs > 1 else budget_s
    while time.perf_counter() - t2 < single_s and k < 400:
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        t = time.perf_counter()
        cell.solve(b)
        ts.append(time.perf_counter() - t)
        k += 1
    t_solve = statistics.median(ts)
    N = spec.N
    n_solves = 4 * (N * N + 4 * N * (N - 1) + 4 * (N - 1) ** 2)
    par = ""
    cores = 1
    t_cell = t_solve
    if procs > 1:
        import multiprocessing as mp
        # spawned workers (never forked after a GPU call), one BLAS thread each
        par_s = budget_s / 2
        ctx = mp.get_context("spawn")
        saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        for v in saved:
            os.environ[v] = "1"
        try:
            barrier, results = ctx.Barrier(procs), ctx.Queue()
            ws = [ctx.Process(target=_cell_solve_worker, args=(spec, med, par_s, barrier, results))
                  for _ in range(procs)]
            for w in ws:
                w.start()
            counts = [results.get(timeout=600) for _ in ws]
            for w in ws:
                w.join()
        finally:
            for v, old in saved.items():
                if old is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = old
        total = sum(counts)
        if total > 0:
            t_cell = par_s / total               # amortised per-solve time with every worker busy
            cores = procs
            par = (f"; all-core rate: {procs} processes x {par_s:.1f} s, {total} solves "
                   f"({t_cell * 1e3:.3f} ms per solve amortised, {t_solve / t_cell:.1f}x one process)")
    t_apply = n_solves * t_cell
    t_sol = (iterations + 1) * t_apply
    return {
        "value": 1.0 / t_sol, "unit": UNIT, "cores": cores, "kind": "port",
        "sample": (f"oracle (numpy/SciPy SuperLU, one thread per process): {k} single-process solves of one "
                   f"interior C2-shaped cell ({n} DOFs, median {t_solve * 1e3:.2f} ms){par}; x {n_solves} cell "
                   f"solves per apply x {iterations + 1} applies per solve; cell factorisation {fact_s:.2f} s "
                   f"x {N * N} cells not included (factors resident on both sides)"),
        "t_apply_s": t_apply, "t_solve_s": t_sol, "cell_factorize_s": fact_s, "setup_s": setup_s,
    }


def run_reference(args):
    """--impl reference: the CPU restatement of the reference path, timed on
    the host cores; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from lsweeps.problems import config
    spec, med = config("C2")
    its = args.ref_iterations
    samples = []
    for _ in range(max(1, args.warmup)):
        cpu_sample(spec, med, its, budget_s=2.0, procs=1)
    for _ in range(args.steps):
        samples.append(cpu_sample(spec, med, its, budget_s=args.ref_budget))
    vals = [s["value"] for s in samples]
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "iterations_assumed": its},
        "cpu_baseline": {k: samples[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
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
    WORKLOAD = WORKLOADS[args.config.upper()]
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
    peak, peak_kind = measured_peaks()
    achieved = pr["alg_bytes"] / (front_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "k_front_C2_dram_traffic.md"
    if tf.exists() and args.config.upper() == "C2" and nrhs == 1:
        m = re.search(r"traffic_bytes_per_apply_c2:\s*([0-9.eE+]+)", tf.read_text())
        traffic = float(m.group(1)) if m else None

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
        cpu = cpu_sample(spec, med, reps[-1].iterations, budget_s=args.ref_budget)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}

    clocks = clk.summary()
    if rank == 0:
        p50 = pctl(step_ms, 0.5)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_total * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[prec],
            "data": {"C1": "synthetic (constant medium)", "C2": "synthetic (seeded Gaussian-lens medium)",
                     "C3": "synthetic (seeded layered medium)",
                     "C4": "synthetic (seeded piecewise-smooth random medium)"}[args.config.upper()],
            "config": {"workload": WORKLOAD, "precision": "mixed" if prec != "c128" else "fp64",
                       "factor_precision": prec, "restart": 30, "tol": args.tol,
                       "parallelism": f"replicas x{world}",
                       "nrhs": nrhs,
                       "l2": f"inputs larger than L2: {S.info()['factor_bytes'] / 1e9:.1f} GB of {prec} factors "
                             "streamed per apply (L2 129 MB)"},
            "p50_ms": p50, "p99_ms": pctl(step_ms, 0.99), "iterations": reps[-1].iterations,
            "true_rel_res": reps[-1].true_rel_res, "factorize_s": fact_s,
            "time_to_solution_s": fact_s + p50 / 1e3,
            "fp64": fp64,
            "mixed_vs_fp64_speedup": (fp64["p50_ms"] / p50) if fp64 else None,
            "mixed_vs_fp64_tts_speedup": ((fp64["factorize_s"] + fp64["p50_ms"] / 1e3) / (fact_s + p50 / 1e3))
            if fp64 else None,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "kernel": "k_front (sweep-front cell solves), all fronts of one apply",
                         "peak_kind": peak_kind, "alg_bytes_per_apply": pr["alg_bytes"],
                         "streamed_bytes_per_apply": pr["streamed_bytes"],
                         "front_ms_per_apply": front_ms, "fronts": pr["fronts"], "items": pr["items"],
                         "slots": pr["slots"], "apply_ms": pr["total_ms"]},
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
    v = torch.randn(S.n2 * args.nrhs, dtype=torch.complex128, device="cuda")
    for _ in range(args.warmup + args.steps):
        S.apply_precond(v)
    torch.cuda.synchronize()
    print(json.dumps({"apply_only": args.config, "precision": prec, "nrhs": args.nrhs,
                      "applies": args.warmup + args.steps, "fronts_per_apply": 3 * spec.N - 3 + 1}))


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
        reqs = serving_stream(args.serve_requests, rate_hz=rate, seed=3 + i)
        st = eng.run(reqs, realtime=True)
        res = [r.true_rel_res for r in reqs if r.error is None]
        print(json.dumps({"metric": "serving: p50/p99 latency and solves/s at rel. residual 1e-6",
                          "rate_hz": rate, "requests": len(reqs), "unit": "solves/s",
                          "value": st.solves_per_s, **st.as_dict(),
                          "max_true_rel_res": max(res) if res else None,
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
    ap.add_argument("--ref-budget", type=float, default=15.0)
    # the reference GMRES (the oracle's restatement, reference arithmetic) reaches
    # its 1e-6 log on the C2 workload in 5 iterations: 6 preconditioner applies
    ap.add_argument("--ref-iterations", type=int, default=5)
    ap.add_argument("--apply-only", action="store_true", help="only preconditioner applies (profiling workload)")
    ap.add_argument("--serve", action="store_true", help="serving stream at the rates of --serve-rates")
    ap.add_argument("--serve-rates", default="1,4,16")
    ap.add_argument("--serve-requests", type=int, default=40)
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
