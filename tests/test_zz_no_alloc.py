"""The allocation-free cell solve (lsw_local_solve_noalloc) gives the same
result as lsw_local_solve, through the C ABI, on two calls in a row: bit for
bit (the same kernel and launch shape; only where the scratch lives differs),
and within the precision's tolerance of the oracle's SuperLU cell solve.

It serves callers that cannot call cudaMalloc (a fixed device-memory budget
owned by their own pool, or loops that cannot afford an allocation's device
synchronisation); its scratch sits in a fixed 8 MiB array of the library.
This file is collected last so that a failure here does not stop the rest of
a run that stops at the first failure."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps import capi  # noqa: E402
from lsweeps.problems import small  # noqa: E402

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c64", 2e-4), ("bf16x2", 2e-4)])
def test_noalloc_local_solve_matches_local_solve(prec, tol):
    from lsweeps.solver import Solver, _stream_ptr
    from oracle.lsweeps_oracle import OracleProblem
    spec, med = small(N=3, m=12, p=5, medium="layered", seed=2)
    S = Solver(spec, med, precision=prec)
    S.factorize()
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    L = capi.lib()
    rng = np.random.default_rng(21)
    for call, (cell, nrhs) in enumerate(((4, 3), (0, 5))):   # two calls in a row
        ci = S.cell_info(cell)
        n = ci["nx"] * ci["ny"]
        b = rng.standard_normal(nrhs * n) + 1j * rng.standard_normal(nrhs * n)
        bd = torch.from_numpy(b).cuda()
        ref = S.local_solve(cell, bd).cpu().numpy()
        x = torch.full_like(bd, complex(np.nan, np.nan))
        st = L.lsw_local_solve_noalloc(S.ctx, cell, C.c_void_p(bd.data_ptr()), C.c_void_p(x.data_ptr()), nrhs,
                                       _stream_ptr(None))
        capi.check(st, S.ctx)
        torch.cuda.synchronize()
        got = x.cpu().numpy()
        assert np.isfinite(got).all()
        # the same kernel and launch shape as lsw_local_solve: identical bits
        assert np.array_equal(got, ref), f"call {call}: {_rel(got, ref):.3e}"
        # and the oracle's SuperLU solve of the same cell
        oc = P.dd.cells[cell]
        oc.factorize()
        assert oc.size == n
        want = np.concatenate([oc.solve(b[r * n:(r + 1) * n]) for r in range(nrhs)])
        assert _rel(got, want) <= tol, f"call {call} vs SuperLU"


def test_noalloc_rejects_oversized_request():
    from lsweeps.solver import Solver, _stream_ptr
    spec, med = small(N=2, m=10, p=4)
    S = Solver(spec, med, precision="c128")
    S.factorize()
    ci = S.cell_info(0)
    n = ci["nx"] * ci["ny"]
    nrhs = (8 << 20) // (n * 16) + 8          # more forward storage than the fixed buffer holds
    b = torch.zeros(nrhs * n, dtype=torch.complex128, device="cuda")
    x = torch.empty_like(b)
    st = capi.lib().lsw_local_solve_noalloc(S.ctx, 0, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), nrhs,
                                            _stream_ptr(None))
    assert st == 1   # LSW_ERR_INVALID_ARGUMENT
    assert b"fixed buffer" in capi.lib().lsw_ctx_last_error(S.ctx)
