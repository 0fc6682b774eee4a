"""The process-parallel executor of the oracle (worker processes owning rows
of cells round-robin, as the reference's MPI ranks do) gives the serial
oracle's results bit for bit: preconditioner, DD matvec and the reference
GMRES."""
import numpy as np
import pytest

from lsweeps.problems import small
from oracle.lsweeps_oracle import OracleProblem, gmres_reference
from oracle.parallel import ParallelOracle


@pytest.fixture(scope="module")
def pair():
    spec, med = small(N=3, m=10, p=4, medium="layered", seed=4)
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    P.dd.factorize()
    with ParallelOracle(spec.N, spec.m, spec.p, spec.h, spec.omega, med, procs=2) as Q:
        yield spec, P, Q


def test_parallel_precond_and_matvec_are_bit_identical(pair):
    spec, P, Q = pair
    rng = np.random.default_rng(3)
    v = rng.standard_normal(P.n_dof ** 2) + 1j * rng.standard_normal(P.n_dof ** 2)
    assert np.array_equal(Q.apply_precond_global(v), P.apply_precond_global(v))
    xc = P.C(v)
    a = Q.dd.apply_system_matrix(xc)
    b = P.dd.apply_system_matrix(xc)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    # the four shifted parts sum to the apply
    parts = [Q.dd.apply_precond_part(xc, q) for q in range(4)]
    full = P.dd.apply_precond(xc)
    assert all(np.array_equal(parts[0][i] + (parts[1][i] + parts[2][i] + parts[3][i]), full[i])
               for i in range(len(full)))


def test_parallel_reference_gmres_matches_serial(pair):
    spec, P, Q = pair
    b = P.C(P.global_rhs(spec.sources))
    xs, rs = gmres_reference(P.dd, b, tol=1e-6, max_iter=40)
    xp, rp = gmres_reference(Q.dd, b, tol=1e-6, max_iter=40)
    assert rs.iterations == rp.iterations
    assert rs.log == rp.log
    assert all(np.array_equal(x, y) for x, y in zip(xs, xp))
