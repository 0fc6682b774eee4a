"""High-level Python handle on one L-sweeps problem on the GPU.

Device memory for vectors comes from torch (complex128 tensors on cuda); every
operation is a call into the C ABI of liblsweeps_gb300.so.  There is no CPU
fallback: without a GPU and the built library this module raises."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .problems import ProblemSpec


def _torch():
    import torch
    return torch


def _stream_ptr(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


@dataclass
class SolveReport:
    iterations: int
    converged: bool
    final_log: float
    true_rel_res: float
    seconds: float
    precond_applies: int
    log: list


class Solver:
    """DDCheckerboard + LocalLinearSolverCUDA + GlobalIterativeSolverGMRES on one GPU.

    precision: "c128" / "fp64" (complex double factors and sweeps, the
    reference's arithmetic), "c64" / "mixed" (complex float, FP32 accumulation)
    or "bf16x2" / "split" (factor entries as bf16 hi + lo terms, tensor-core
    products, FP32 accumulation); the Krylov solver is FP64 in every case.
    """

    def __init__(self, spec: ProblemSpec, m_grid: np.ndarray, precision: str = "c64", device: int = 0):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("lsweeps.Solver needs a CUDA GPU (the GPU path has no CPU fallback)")
        self.L = capi.lib()
        self.spec = spec
        self.device = device
        self.precision = precision
        ctx = C.c_void_p()
        capi.check(self.L.lsw_ctx_create(C.byref(ctx), device))
        self.ctx = ctx
        g = capi.Geom(spec.N, spec.m, spec.p, 2, spec.h)
        mg = np.ascontiguousarray(m_grid, dtype=np.float64)
        if mg.shape != (spec.n_dof, spec.n_dof):
            raise ValueError(f"m_grid must be {spec.n_dof}x{spec.n_dof}")
        capi.check(self.L.lsw_problem_setup(ctx, C.byref(g), mg.ctypes.data_as(C.POINTER(C.c_double)),
                                            float(spec.omega), capi.PREC[precision]), ctx)
        self.n_dof = spec.n_dof
        self.n2 = spec.n_dof * spec.n_dof

    def close(self):
        if getattr(self, "ctx", None):
            self.L.lsw_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- info -----------------------------------------------------------------
    def info(self) -> dict:
        o = capi.ProblemInfo()
        capi.check(self.L.lsw_problem_info_get(self.ctx, C.byref(o)), self.ctx)
        return {k: getattr(o, k) for k, _ in capi.ProblemInfo._fields_}

    def cell_info(self, cell: int) -> dict:
        o = capi.CellInfo()
        capi.check(self.L.lsw_cell_info_get(self.ctx, cell, C.byref(o)), self.ctx)
        return o.as_dict()

    # ---- operations -------------------------------------------------------------
    def _vec(self, x, nrhs=None):
        torch = _torch()
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.complex128 and x.is_contiguous()):
            raise TypeError("expected a contiguous complex128 CUDA tensor")
        if x.numel() % self.n2:
            raise ValueError("tensor size is not a multiple of n_dof^2")
        return x.numel() // self.n2

    def factorize(self, stream=None):
        capi.check(self.L.lsw_factorize(self.ctx, _stream_ptr(stream)), self.ctx)

    def front_shapes(self, nrhs: int = 1, stream=None) -> tuple[list[dict], float]:
        """The sweep fronts' launch shapes for a batch of nrhs right-hand sides
        (lsw_front_shapes) and the context's tuning time in seconds."""
        n = C.c_int(0)
        ts = C.c_double(0.0)
        cap = 16 * self.spec.N + 16   # one launch per step, or per (step, sweep) for small batches
        buf = (capi.FrontShape * cap)()
        capi.check(self.L.lsw_front_shapes(self.ctx, nrhs, buf, cap, C.byref(n), C.byref(ts), _stream_ptr(stream)),
                   self.ctx)
        return [{k: getattr(buf[i], k) for k, _ in capi.FrontShape._fields_} for i in range(n.value)], ts.value

    def set_tuning(self, enable: bool):
        """Measure sweep-front shapes on first use (lsw_ctx_set_tuning)."""
        capi.check(self.L.lsw_ctx_set_tuning(self.ctx, 1 if enable else 0), self.ctx)

    def set_sweep_lanes(self, max_rhs: int):
        """Per-sweep launches for batches of at most max_rhs right-hand sides
        (lsw_ctx_set_sweep_lanes; 0 turns them off)."""
        capi.check(self.L.lsw_ctx_set_sweep_lanes(self.ctx, int(max_rhs)), self.ctx)

    def set_graphs(self, enable: bool):
        """Replay applies as CUDA graphs (lsw_ctx_set_graphs)."""
        capi.check(self.L.lsw_ctx_set_graphs(self.ctx, 1 if enable else 0), self.ctx)

    def release_workspace(self):
        """Free the Krylov bases and sweep pools (lsw_release_workspace); the factors stay."""
        capi.check(self.L.lsw_release_workspace(self.ctx), self.ctx)

    def apply_precond(self, x, out=None, stream=None):
        torch = _torch()
        nr = self._vec(x)
        y = torch.empty_like(x) if out is None else out
        capi.check(self.L.lsw_apply_precond(self.ctx, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), nr,
                                            _stream_ptr(stream)), self.ctx)
        return y

    def apply_precond_profiled(self, x, out=None, stream=None) -> tuple:
        torch = _torch()
        nr = self._vec(x)
        y = torch.empty_like(x) if out is None else out
        prof = capi.ApplyProfile()
        capi.check(self.L.lsw_apply_precond_profiled(self.ctx, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                     nr, _stream_ptr(stream), C.byref(prof)), self.ctx)
        return y, {k: getattr(prof, k) for k, _ in capi.ApplyProfile._fields_}

    def apply_A(self, x, out=None, stream=None):
        torch = _torch()
        nr = self._vec(x)
        y = torch.empty_like(x) if out is None else out
        capi.check(self.L.lsw_apply_A(self.ctx, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), nr,
                                      _stream_ptr(stream)), self.ctx)
        return y

    def assemble_rhs(self, sources, amplitudes=None, stream=None):
        torch = _torch()
        b = torch.empty(self.n2, dtype=torch.complex128, device=f"cuda:{self.device}")
        src = np.ascontiguousarray(np.asarray(sources, dtype=np.float64).reshape(-1))
        amp = None if amplitudes is None else np.ascontiguousarray(np.asarray(amplitudes, dtype=np.float64))
        capi.check(self.L.lsw_assemble_rhs(
            self.ctx, src.ctypes.data_as(C.POINTER(C.c_double)),
            None if amp is None else amp.ctypes.data_as(C.POINTER(C.c_double)),
            len(src) // 2, C.c_void_p(b.data_ptr()), _stream_ptr(stream)), self.ctx)
        return b

    def gmres(self, b, mode: str = "flexible", tol: float = 1e-6, max_iter: int = 200, restart: int = 30,
              verbose: bool = False, x=None, stream=None):
        torch = _torch()
        nr = self._vec(b)
        x = torch.empty_like(b) if x is None else x
        opts = capi.GmresOpts(capi.GMRES_MODE[mode], tol, max_iter, restart, int(verbose))
        logbuf = (C.c_double * 512)()
        rep = capi.GmresReport()
        rep.log = C.cast(logbuf, C.POINTER(C.c_double))
        rep.log_capacity = 512
        capi.check(self.L.lsw_gmres(self.ctx, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), nr,
                                    C.byref(opts), C.byref(rep), _stream_ptr(stream)), self.ctx)
        return x, SolveReport(rep.iterations, bool(rep.converged), rep.final_log, rep.true_rel_res, rep.seconds,
                              rep.precond_applies, [logbuf[i] for i in range(rep.log_len)])

    def solve_host(self, b_host: np.ndarray, mode: str = "flexible", tol: float = 1e-6, max_iter: int = 200,
                   restart: int = 30, stream=None, x_host: np.ndarray | None = None):
        """GlobalIterativeSolver::solve on host buffers (copies included); x_host:
        an optional (pinned) output buffer of b's size."""
        b = np.ascontiguousarray(b_host, dtype=np.complex128)
        nr = b.size // self.n2
        if x_host is not None and (x_host.dtype != np.complex128 or x_host.size != b.size
                                   or not x_host.flags.c_contiguous):
            raise ValueError("x_host must be a contiguous complex128 array of b's size")
        x = np.empty_like(b) if x_host is None else x_host
        opts = capi.GmresOpts(capi.GMRES_MODE[mode], tol, max_iter, restart, 0)
        rep = capi.GmresReport()
        capi.check(self.L.lsw_solve_host(self.ctx, b.ctypes.data_as(C.POINTER(C.c_double)),
                                         x.ctypes.data_as(C.POINTER(C.c_double)), nr, C.byref(opts), C.byref(rep),
                                         _stream_ptr(stream)), self.ctx)
        return x, SolveReport(rep.iterations, bool(rep.converged), rep.final_log, rep.true_rel_res, rep.seconds,
                              rep.precond_applies, [])

    def local_solve(self, cell: int, b, stream=None):
        torch = _torch()
        ci = self.cell_info(cell)
        n = ci["nx"] * ci["ny"]
        if b.numel() % n:
            raise ValueError("cell vector size mismatch")
        x = torch.empty_like(b)
        capi.check(self.L.lsw_local_solve(self.ctx, cell, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                                          b.numel() // n, _stream_ptr(stream)), self.ctx)
        return x
