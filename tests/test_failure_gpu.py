"""Failure paths of the GPU library, made on the host: nothing here faults,
traps or hangs the GPU.

* A non-finite squared slowness (injected in the host array) reaches the
  factorisation as a non-finite pivot: lsw_factorize returns
  LSW_ERR_SINGULAR_BLOCK (the reference prints and exits when Eigen's
  factorisation fails, LocalLinearSolverEigenSparseLU.cpp:54-58).
* A bounded wait that runs out returns LSW_ERR_CUDA and leaves the context
  usable: lsw_selftest_bounded_wait waits, with the context's limit, on a
  barrier that nothing completes (the same wait routine as the sweep
  kernels), and the error is reported once."""
import ctypes as C
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps import capi  # noqa: E402
from lsweeps.problems import small  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["c128", "c64", "bf16x2"])
def test_nan_medium_returns_singular_block(prec):
    from lsweeps.solver import Solver
    spec, med = small(N=2, m=10, p=4, medium="lens")
    bad = med.copy()
    bad[bad.shape[0] // 2, bad.shape[1] // 2] = np.nan
    S = Solver(spec, bad, precision=prec)
    with pytest.raises(capi.LswError) as ei:
        S.factorize()
    assert ei.value.status == 6, str(ei.value)   # LSW_ERR_SINGULAR_BLOCK
    S.close()
    # a healthy problem in a fresh context still factorises and applies
    S2 = Solver(spec, med, precision=prec)
    S2.factorize()
    v = torch.ones(S2.n2, dtype=torch.complex128, device="cuda")
    y = S2.apply_precond(v)
    torch.cuda.synchronize()
    assert torch.isfinite(torch.view_as_real(y)).all()


def test_bounded_wait_runs_out_and_context_stays_usable():
    from lsweeps.solver import Solver, _stream_ptr
    spec, med = small(N=2, m=10, p=4, medium="lens")
    S = Solver(spec, med, precision="c64")
    S.factorize()
    L = capi.lib()
    with pytest.raises(capi.LswError):
        capi.check(L.lsw_ctx_set_wait_limit(S.ctx, C.c_double(0.0)), S.ctx)
    capi.check(L.lsw_ctx_set_wait_limit(S.ctx, C.c_double(0.002)), S.ctx)   # 2 ms
    t = time.perf_counter()
    st = L.lsw_selftest_bounded_wait(S.ctx, _stream_ptr(None))
    dt = time.perf_counter() - t
    assert st == 2, capi.lib().lsw_ctx_last_error(S.ctx)   # LSW_ERR_CUDA
    assert b"bounded wait" in L.lsw_ctx_last_error(S.ctx)
    assert dt < 5.0
    # the error is reported once: the default limit back, a sweep runs and
    # its synchronous check reports success
    capi.check(L.lsw_ctx_set_wait_limit(S.ctx, C.c_double(2.0)), S.ctx)
    ci = S.cell_info(0)
    b = torch.ones(ci["nx"] * ci["ny"], dtype=torch.complex128, device="cuda")
    x = S.local_solve(0, b)
    torch.cuda.synchronize()
    assert torch.isfinite(torch.view_as_real(x)).all()
    v = torch.ones(S.n2, dtype=torch.complex128, device="cuda")
    _, prof = S.apply_precond_profiled(v)
    assert prof["fronts"] > 0
