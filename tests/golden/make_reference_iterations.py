"""Writes reference_gmres_iterations.json: the iteration count of the
reference GMRES (GlobalIterativeSolverGMRES::solve restated: left
preconditioning, no restart, the reference's Givens bookkeeping; tolerance
1e-6 on its logged residual, MaxIter 40 as the reference's default, raised to
100 where 40 does not reach it) on the workloads, in FP64.  The CPU baseline
of bench.py reads these counts: a reference solve costs iterations + 2
preconditioner applies.

    python tests/golden/make_reference_iterations.py --oracle C1 C2   # CPU
    python tests/golden/make_reference_iterations.py --gpu C3 C4      # a GPU

--oracle runs the oracle's restatement (gmres_reference on the process-
parallel executor, every host core).  --gpu runs the library's reference mode
in complex128 (`lsw_gmres` with LSW_GMRES_REFERENCE), whose iteration count
and residual log are pinned to the oracle's by the GPU parity tests (small
fixtures and C2); it stands in where the oracle's solve would take too long.
--out PATH writes elsewhere (default: beside this script).
"""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "l-sweeps-2d_gb300"):
    sys.path.insert(0, str(p))


def _source_rhs(spec, name):
    # C3 is a line of 64 sources solved one at a time by the reference: its middle source
    return [spec.sources[len(spec.sources) // 2]] if name == "C3" else spec.sources


def run_gpu(name):
    import torch
    from lsweeps.problems import config
    from lsweeps.solver import Solver
    spec, med = config(name)
    S = Solver(spec, med, precision="c128")
    S.factorize()
    b = S.assemble_rhs(_source_rhs(spec, name))
    for cap in (40, 100):
        x, rep = S.gmres(b, mode="reference", tol=1e-6, max_iter=cap)
        if rep.converged:
            break
    out = {"iterations": int(rep.iterations), "max_iter": cap, "converged": bool(rep.converged),
           "final_log": float(rep.final_log), "true_rel_res": float(rep.true_rel_res),
           "source": "library reference mode, complex128 (GPU)"}
    S.close()
    del x, b
    torch.cuda.empty_cache()
    return out


def run_oracle(name):
    from lsweeps.problems import config
    from oracle.lsweeps_oracle import gaussian_rhs, gmres_reference
    from oracle.parallel import ParallelOracle
    spec, med = config(name)
    with ParallelOracle(spec.N, spec.m, spec.p, spec.h, spec.omega, med) as Q:
        b = [gaussian_rhs(c.X, c.Y, _source_rhs(spec, name), Q.dd.mesh_size()) for c in Q.dd.cells]
        b = Q.dd.reduce(b)
        for cap in (40, 100):
            x, rep = gmres_reference(Q.dd, b, tol=1e-6, max_iter=cap)
            if rep.log[-1] <= 1e-6:
                break
    return {"iterations": int(rep.iterations), "max_iter": cap, "converged": bool(rep.log[-1] <= 1e-6),
            "final_log": float(rep.log[-1]), "source": "oracle restatement (CPU)"}


def main(argv):
    out = ROOT / "tests" / "golden" / "reference_gmres_iterations.json"
    mode, names = None, []
    it = iter(argv)
    for a in it:
        if a in ("--gpu", "--oracle"):
            mode = a[2:]
        elif a == "--out":
            out = Path(next(it))
        else:
            names.append(a.upper())
    if mode is None or not names:
        raise SystemExit(__doc__)
    data = json.loads(out.read_text()) if out.exists() else {}
    for name in names:
        data[name] = run_gpu(name) if mode == "gpu" else run_oracle(name)
        print(name, data[name], flush=True)
        out.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:])
