"""GPU parity of the CUDA path (through the C ABI) against the oracle.

Tolerances: FP64 (complex128) factors and applies must match the oracle's
SuperLU-based restatement to 1e-10 relative (different but exact-arithmetic-
equivalent factorisations, so only rounding separates them); the complex64
mixed path and the bf16-split path (factor entries as bf16 hi + lo terms,
three tensor-core products, FP32 accumulation; about 16 significant bits per
entry) to 2e-4 relative on the preconditioner.  Solves: true relative
residual <= 1e-6 and relative difference <= 1e-5 against the global direct
solve; reference-mode GMRES iteration count within +-1 of the oracle."""
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps.problems import ProblemSpec, small, config  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("*.npz"))


def _solver(spec, med, prec):
    from lsweeps.solver import Solver
    S = Solver(spec, med, precision=prec)
    S.factorize()
    return S


def _load(f):
    d = np.load(f)
    N, m, p = (int(v) for v in d["Nmp"])
    spec = ProblemSpec(N=N, m=m, p=p, h=float(d["h"]), omega=float(d["omega"]))
    spec.sources = [tuple(s) for s in d["sources"]]
    return spec, d


def _dev(v):
    return torch.from_numpy(np.ascontiguousarray(v)).to("cuda")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
def test_apply_A_matches_oracle(f):
    spec, d = _load(f)
    S = _solver(spec, d["m_grid"], "c128")
    y = S.apply_A(_dev(d["v"])).cpu().numpy()
    assert rel(y, d["Av"]) <= 1e-13


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c64", 2e-4), ("bf16x2", 2e-4)])
def test_precond_matches_oracle(f, prec, tol):
    spec, d = _load(f)
    S = _solver(spec, d["m_grid"], prec)
    y = S.apply_precond(_dev(d["v"])).cpu().numpy()
    assert rel(y, d["Mv"]) <= tol


@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c64", 2e-4), ("bf16x2", 2e-4)])
def test_local_solve_matches_superlu(prec, tol):
    from oracle.lsweeps_oracle import OracleProblem
    spec, med = small(N=3, m=12, p=5, medium="layered", seed=2)
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    S = _solver(spec, med, prec)
    rng = np.random.default_rng(5)
    for c in (0, 4, 8):
        cell = P.dd.cells[c]
        cell.factorize()
        n = cell.size
        b = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
        x = S.local_solve(c, _dev(b.ravel())).cpu().numpy().reshape(2, n)
        for r in range(2):
            assert rel(x[r], cell.solve(b[r])) <= tol


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
def test_reference_gmres_iteration_count(f):
    spec, d = _load(f)
    S = _solver(spec, d["m_grid"], "c128")
    x, rep = S.gmres(_dev(d["b"]), mode="reference", tol=1e-6, max_iter=40)
    assert abs(rep.iterations - int(d["gmres_ref_iters"])) <= 1
    n = min(len(rep.log), len(d["gmres_ref_log"]))
    assert np.allclose(rep.log[:n], d["gmres_ref_log"][:n], rtol=1e-6, atol=1e-12)
    if rep.iterations == int(d["gmres_ref_iters"]):
        assert rel(x.cpu().numpy(), d["gmres_ref_x"]) <= 1e-8


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
@pytest.mark.parametrize("prec", ["c128", "c64", "bf16x2"])
def test_fgmres_solves_to_tolerance(f, prec):
    spec, d = _load(f)
    S = _solver(spec, d["m_grid"], prec)
    x, rep = S.gmres(_dev(d["b"]), mode="flexible", tol=1e-6, max_iter=100, restart=30)
    assert rep.converged and rep.true_rel_res <= 1e-6
    assert rel(x.cpu().numpy(), d["x_direct"]) <= 1e-5


@pytest.mark.parametrize("N,m,p,medium", [(5, 7, 2, "layered"), (2, 20, 8, "random"), (6, 5, 1, "lens")])
def test_precond_more_geometries(N, m, p, medium):
    """The preconditioner against the oracle on decompositions beyond the
    fixtures: a thin PML, more cells, odd cell sizes, all three media."""
    from oracle.lsweeps_oracle import OracleProblem
    spec, med = small(N=N, m=m, p=p, medium=medium)
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    P.dd.factorize()
    rng = np.random.default_rng(N * 100 + m)
    v = rng.standard_normal(P.n_dof ** 2) + 1j * rng.standard_normal(P.n_dof ** 2)
    y_or = P.apply_precond_global(v)
    for prec, tol in (("c128", 1e-10), ("c64", 2e-4), ("bf16x2", 2e-4)):
        S = _solver(spec, med, prec)
        assert rel(S.apply_precond(_dev(v)).cpu().numpy(), y_or) <= tol, prec
        S.close()


def test_one_cell_precond_is_the_exact_inverse():
    """N = 1: the only cell is the whole domain, so the L-sweep preconditioner
    is A^-1 (the other three shifted windows are empty); FGMRES then converges
    in one iteration."""
    spec, med = small(N=1, m=30, p=6, medium="lens")
    S = _solver(spec, med, "c128")
    rng = np.random.default_rng(17)
    v = rng.standard_normal(S.n2) + 1j * rng.standard_normal(S.n2)
    y = S.apply_precond(_dev(v))
    assert rel(S.apply_A(y).cpu().numpy(), v) <= 1e-10
    b = S.assemble_rhs(spec.sources)
    x, rep = S.gmres(b, mode="flexible", tol=1e-8, max_iter=10, restart=10)
    assert rep.iterations <= 1 and rep.true_rel_res <= 1e-8


def test_batched_rhs_equal_single():
    """A batch of right-hand sides gives each one's single result; only the
    summation order inside a cell solve may differ (the number of consumer
    warps per row group depends on the slots per front)."""
    f = FIXTURES[-1]
    spec, d = _load(f)
    for prec, tol in (("c128", 1e-13), ("c64", 1e-5), ("bf16x2", 1e-4)):
        S = _solver(spec, d["m_grid"], prec)
        rng = np.random.default_rng(9)
        V = rng.standard_normal((3, S.n2)) + 1j * rng.standard_normal((3, S.n2))
        Y = S.apply_precond(_dev(V.ravel())).cpu().numpy().reshape(3, -1)
        for r in range(3):
            y = S.apply_precond(_dev(V[r])).cpu().numpy()
            assert rel(Y[r], y) <= tol


def test_krylov_sub_batches_equal_one_batch(monkeypatch):
    """A right-hand-side batch solved as sub-batches (as when the Krylov bases
    of the whole batch do not fit in device memory) gives the one-batch
    solutions and a merged report."""
    f = FIXTURES[-1]
    spec, d = _load(f)
    rng = np.random.default_rng(21)
    S = _solver(spec, d["m_grid"], "c64")
    B = rng.standard_normal((5, S.n2)) + 1j * rng.standard_normal((5, S.n2))
    x1, r1 = S.gmres(_dev(B.ravel()), mode="flexible", tol=1e-8, max_iter=100, restart=30)
    S.close()
    monkeypatch.setenv("LSW_KRYLOV_BATCH", "2")
    S2 = _solver(spec, d["m_grid"], "c64")
    x2, r2 = S2.gmres(_dev(B.ravel()), mode="flexible", tol=1e-8, max_iter=100, restart=30)
    # the complex64 sweeps round differently with the batch composition, so
    # the two solutions agree to the solve tolerance, not bit for bit
    assert r2.converged and r2.true_rel_res <= 1e-8
    assert abs(r2.iterations - r1.iterations) <= 1
    assert r2.precond_applies > r1.precond_applies     # three sub-batches
    assert rel(x2.cpu().numpy(), x1.cpu().numpy()) <= 1e-6


def test_release_workspace_returns_memory_and_keeps_factors():
    f = FIXTURES[0]
    spec, d = _load(f)
    S = _solver(spec, d["m_grid"], "c64")
    b = _dev(d["b"])
    x1, r1 = S.gmres(b, mode="flexible", tol=1e-6, max_iter=100, restart=30)
    held = S.info()["device_bytes"]
    S.release_workspace()
    assert S.info()["device_bytes"] < held
    assert S.info()["device_bytes"] >= S.info()["factor_bytes"]
    x2, r2 = S.gmres(b, mode="flexible", tol=1e-6, max_iter=100, restart=30)
    # the rebuilt schedule and pools give the same arithmetic: the same bits
    assert r2.iterations == r1.iterations and r2.true_rel_res <= 1e-6
    assert np.array_equal(x2.cpu().numpy(), x1.cpu().numpy())


def test_c1_precond_and_solve_match_oracle():
    """Configuration C1 (4x4 cells of 64^2, PML 10, c = 1, 10 ppw) in FP64."""
    import scipy.sparse.linalg as spla
    from oracle.lsweeps_oracle import OracleProblem
    spec, med = config("C1")
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    P.dd.factorize()
    S = _solver(spec, med, "c128")
    rng = np.random.default_rng(11)
    v = rng.standard_normal(S.n2) + 1j * rng.standard_normal(S.n2)
    y_or = P.apply_precond_global(v)
    assert rel(S.apply_precond(_dev(v)).cpu().numpy(), y_or) <= 1e-10
    # 64-DOF cells on the tensor-core split path (eight 16-row tiles per cell)
    Ss = _solver(spec, med, "bf16x2")
    assert rel(Ss.apply_precond(_dev(v)).cpu().numpy(), y_or) <= 2e-4
    b = S.assemble_rhs(spec.sources)
    bo = P.global_rhs(spec.sources)
    assert rel(b.cpu().numpy(), bo) <= 1e-12
    x, rep = S.gmres(b, mode="flexible", tol=1e-6, max_iter=100, restart=20)
    xd = spla.splu(P.global_matrix().tocsc()).solve(bo)
    assert rep.true_rel_res <= 1e-6 and rel(x.cpu().numpy(), xd) <= 1e-5


def test_largest_cells_batched_fp64():
    """Cells at the 192-DOF limit (190-192 per side) with 8 right-hand sides
    in complex128: the widest shared-memory layout of the sweep kernel.  The
    batched preconditioner equals the single applies and the oracle."""
    from oracle.lsweeps_oracle import OracleProblem
    spec, med = small(N=2, m=149, p=20, ppw=8.0, medium="lens")
    S = _solver(spec, med, "c128")
    rng = np.random.default_rng(13)
    V = rng.standard_normal((8, S.n2)) + 1j * rng.standard_normal((8, S.n2))
    Y = S.apply_precond(_dev(V.ravel())).cpu().numpy().reshape(8, -1)
    for r in (0, 5, 7):
        assert rel(Y[r], S.apply_precond(_dev(V[r])).cpu().numpy()) <= 1e-13
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    P.dd.factorize()
    assert rel(Y[3], P.apply_precond_global(V[3])) <= 1e-10


def test_error_paths():
    from lsweeps import capi
    from lsweeps.solver import Solver
    spec, med = small(N=2, m=10, p=4)
    S = Solver(spec, med, precision="c64")
    v = torch.zeros(S.n2, dtype=torch.complex128, device="cuda")
    with pytest.raises(capi.LswError) as e:
        S.apply_precond(v)
    assert e.value.status == 5   # LSW_ERR_NOT_FACTORIZED
    with pytest.raises(ValueError):
        Solver(spec, med[:-1], precision="c64")


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
@pytest.mark.parametrize("prec", ["c64", "bf16x2"])
def test_tensor_core_factorisation_matches_cuda_core(f, prec, monkeypatch):
    """The complex64 / split factorisation with each pivot block's update on
    the tensor cores (3 x TF32 tcgen05.mma into a TMEM accumulator) gives the
    preconditioner of the CUDA-core factorisation within 1e-5 (FP32 rounding
    of the factors), and both stay within the oracle tolerance."""
    spec, d = _load(f)
    v = _dev(d["v"])
    monkeypatch.setenv("LSW_FACTOR_TC", "0")
    S0 = _solver(spec, d["m_grid"], prec)
    y0 = S0.apply_precond(v).cpu().numpy()
    S0.close()
    monkeypatch.setenv("LSW_FACTOR_TC", "1")
    S1 = _solver(spec, d["m_grid"], prec)
    y1 = S1.apply_precond(v).cpu().numpy()
    S1.close()
    assert rel(y1, y0) <= 1e-5
    assert rel(y1, d["Mv"]) <= 2e-4


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
@pytest.mark.parametrize("prec,tol,tol_single", [("c64", 2e-4, 1e-5), ("bf16x2", 2e-4, 1e-4)])
def test_sixteen_slot_items_match_oracle(f, prec, tol, tol_single, monkeypatch):
    """Items of 16 right-hand-side slots on clusters of 2 x 2 CTAs (imposed
    with LSW_FRONT_SHAPE) solve every vector of a 16-vector batch (phase
    rotations of the fixture's vector) like the oracle and like a single-
    vector apply with the tuner's shapes (only the summation order of a cell
    solve changes with the slots per item and the CTAs per half: 1e-5 for
    complex64, 1e-4 for the bf16 hi/lo terms, as for batched right-hand
    sides)."""
    spec, d = _load(f)
    monkeypatch.setenv("LSW_FRONT_SHAPE", "16x2")
    S = _solver(spec, d["m_grid"], prec)
    monkeypatch.delenv("LSW_FRONT_SHAPE")
    S1 = _solver(spec, d["m_grid"], prec)
    ph = np.exp(2j * np.pi * np.arange(16) / 16)
    V = ph[:, None] * d["v"][None, :]
    Y = S.apply_precond(_dev(V.ravel())).cpu().numpy().reshape(16, -1)
    shapes, _ = S.front_shapes(16)
    assert all(fr["slots_cap"] == 16 for fr in shapes if fr["items"] > 0)
    y1 = S1.apply_precond(_dev(d["v"])).cpu().numpy()
    for r in range(16):
        assert rel(Y[r], ph[r] * d["Mv"]) <= tol
        assert rel(Y[r], ph[r] * y1) <= tol_single
    S.close()
    S1.close()
