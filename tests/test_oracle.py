"""Pins of the CPU oracle (no GPU).  The reference ships no tests or golden
vectors and cannot be built here, so the oracle restatement is pinned by
properties the reference's algorithm must satisfy, and by the committed
fixtures in tests/golden (generated from the oracle by tests/golden/make_golden.py)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from lsweeps.problems import small, ProblemSpec, constant_medium
from oracle.lsweeps_oracle import OracleProblem, gmres_reference, fgmres, fd_weights

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def _problem(N, m=10, p=4, medium="lens", ppw=10.0):
    spec, med = small(N=N, m=m, p=p, medium=medium, ppw=ppw)
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    return spec, med, P


def test_fd_weights_central():
    # FDweights (FiniteDifferences.cpp:11-54) for Order 2: [1,-2,1] and [-1/2,0,1/2]
    assert np.allclose(fd_weights(1, np.arange(3.0), 2), [1, -2, 1])
    assert np.allclose(fd_weights(1, np.arange(3.0), 1), [-0.5, 0, 0.5])


@pytest.mark.parametrize("N,m,p", [(1, 10, 4), (2, 10, 4), (3, 10, 4), (4, 7, 2), (5, 6, 3)])
def test_ownership_partition(N, m, p):
    _, _, P = _problem(N, m=m, p=p)
    for key, keep in P.dd.keep.items():
        from oracle.lsweeps_oracle import global_indices
        g = np.concatenate(global_indices(P.dd, P.h, P.p, P.n_dof, *key))
        assert g.size == P.n_dof ** 2 and np.unique(g).size == g.size


@pytest.mark.parametrize("N,m,p,medium", [(2, 10, 4, "lens"), (3, 10, 4, "lens"), (4, 7, 2, "layered"),
                                          (3, 9, 5, "random")])
def test_dd_matvec_equals_global_operator(N, m, p, medium):
    _, _, P = _problem(N, m=m, p=p, medium=medium)
    A = P.global_matrix()
    rng = np.random.default_rng(0)
    v = rng.standard_normal(P.n_dof ** 2) + 1j * rng.standard_normal(P.n_dof ** 2)
    assert np.linalg.norm(P.apply_A_global(v) - A @ v) <= 1e-14 * np.linalg.norm(A @ v)


@pytest.mark.parametrize("N,m,p", [(3, 10, 4), (2, 7, 2), (4, 6, 3)])
def test_windows_partition(N, m, p):
    _, _, P = _problem(N, m=m, p=p)
    rng = np.random.default_rng(1)
    x = P.C(rng.standard_normal(P.n_dof ** 2) + 0j)
    parts = [P.dd.get_separated_rhs(x, a, b) for a, b in ((0, 0), (1, 0), (0, 1), (1, 1))]
    tot = [sum(p[i] for p in parts) for i in range(len(x))]
    ref = P.dd.expand(x)
    assert all(np.array_equal(t, r) for t, r in zip(tot, ref))


def test_one_cell_precond_is_exact_inverse():
    _, _, P = _problem(1)
    P.dd.factorize()
    A = P.global_matrix()
    rng = np.random.default_rng(2)
    v = rng.standard_normal(P.n_dof ** 2) + 1j * rng.standard_normal(P.n_dof ** 2)
    z = P.apply_precond_global(v)
    assert np.linalg.norm(A @ z - v) <= 1e-12 * np.linalg.norm(v)


@pytest.mark.parametrize("N,medium", [(3, "lens"), (4, "layered")])
def test_precond_is_linear(N, medium):
    """applyPrecond is a linear operator (sums of exact local solves of windows,
    equivalent sources and traces that depend linearly on the input), as GMRES
    requires: M(a x + b y) = a M x + b M y to rounding."""
    _, _, P = _problem(N, medium=medium)
    P.dd.factorize()
    rng = np.random.default_rng(5)
    n2 = P.n_dof ** 2
    x = rng.standard_normal(n2) + 1j * rng.standard_normal(n2)
    y = rng.standard_normal(n2) + 1j * rng.standard_normal(n2)
    a, b = 0.7 - 0.2j, -1.3 + 0.4j
    z = P.apply_precond_global(a * x + b * y)
    w = a * P.apply_precond_global(x) + b * P.apply_precond_global(y)
    assert np.linalg.norm(z - w) <= 1e-12 * np.linalg.norm(z)


def test_shift_conversions_are_identity_on_global_vectors():
    _, _, P = _problem(3)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(P.n_dof ** 2) + 1j * rng.standard_normal(P.n_dof ** 2)
    from oracle.lsweeps_oracle import global_indices, to_global
    for sud in (False, True):
        x = P.dd.reduce(P.dd.expand(P.C(v)))
        if sud:
            x = P.dd.convert_nonshifted_to_shifted_ud(x, False)
        y = P.dd.convert_nonshifted_to_shifted_lr(x, sud)
        g = to_global(y, global_indices(P.dd, P.h, P.p, P.n_dof, True, sud), P.n_dof ** 2)
        assert np.array_equal(g, v)


@pytest.mark.parametrize("N", [2, 3])
def test_gmres_paths(N):
    spec, _, P = _problem(N)
    P.dd.factorize()
    A = P.global_matrix()
    b = P.global_rhs(spec.sources)
    xd = spla.splu(A.tocsc()).solve(b)
    # reference GMRES: its own log converges; its true residual is not small (quirks)
    xs, rep = gmres_reference(P.dd, P.C(b), tol=1e-6, max_iter=40)
    assert rep.log[-1] <= 1e-6 and rep.iterations < 40
    # flexible GMRES with the same preconditioner reaches the true tolerance
    xf, it, hist = fgmres(lambda u: A @ u, P.apply_precond_global, b, tol=1e-6, restart=30)
    assert np.linalg.norm(b - A @ xf) <= 1e-6 * np.linalg.norm(b)
    assert np.linalg.norm(xf - xd) <= 1e-5 * np.linalg.norm(xd)


def test_golden_fixtures_reproduce():
    files = sorted(GOLDEN.glob("*.npz"))
    assert files, "tests/golden has no fixtures"
    for f in files:
        d = np.load(f)
        N, m, p = (int(v) for v in d["Nmp"])
        spec = ProblemSpec(N=N, m=m, p=p, h=float(d["h"]), omega=float(d["omega"]))
        P = OracleProblem(N, m, p, spec.h, spec.omega, d["m_grid"])
        P.dd.factorize()
        assert np.allclose(P.apply_precond_global(d["v"]), d["Mv"], rtol=0, atol=1e-12 * np.abs(d["Mv"]).max())
        assert np.allclose(P.apply_A_global(d["v"]), d["Av"], rtol=0, atol=1e-12 * np.abs(d["Av"]).max())
