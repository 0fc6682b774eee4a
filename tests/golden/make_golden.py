"""Generate the golden fixtures of tests/golden from the CPU oracle.

The reference ships no golden vectors and cannot be built or run here (Eigen,
libconfig++ and MPI are absent), so these fixtures are outputs of the oracle's
restatement of it.  Each .npz holds one seeded small problem: the squared
slowness grid, a random vector v with M^-1 v and A v, the source right-hand
side b, the global direct solution, and the reference-GMRES iteration count and
residual log.  Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np
import scipy.sparse.linalg as spla

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "l-sweeps-2d_gb300")]

from lsweeps.problems import small  # noqa: E402
from oracle.lsweeps_oracle import OracleProblem, gmres_reference  # noqa: E402

CASES = [
    dict(N=2, m=10, p=4, medium="lens", ppw=10.0, seed=0),
    dict(N=3, m=12, p=5, medium="layered", ppw=8.0, seed=4),
    dict(N=4, m=8, p=3, medium="random", ppw=8.0, seed=7),
]


def main():
    for c in CASES:
        spec, med = small(N=c["N"], m=c["m"], p=c["p"], medium=c["medium"], ppw=c["ppw"], seed=c["seed"])
        P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
        P.dd.factorize()
        rng = np.random.default_rng(100 + c["seed"])
        v = rng.standard_normal(P.n_dof ** 2) + 1j * rng.standard_normal(P.n_dof ** 2)
        b = P.global_rhs(spec.sources)
        A = P.global_matrix()
        xd = spla.splu(A.tocsc()).solve(b)
        xs, rep = gmres_reference(P.dd, P.C(b), tol=1e-6, max_iter=40)
        name = f"N{c['N']}_m{c['m']}_p{c['p']}_{c['medium']}.npz"
        np.savez_compressed(HERE / name, Nmp=np.array([c["N"], c["m"], c["p"]]), h=spec.h, omega=spec.omega,
                            m_grid=med, v=v, Mv=P.apply_precond_global(v), Av=A @ v, b=b, x_direct=xd,
                            gmres_ref_iters=rep.iterations, gmres_ref_log=np.array(rep.log),
                            gmres_ref_x=P.G(xs), sources=np.array(spec.sources))
        print(name, "iters", rep.iterations)


if __name__ == "__main__":
    main()
