"""ctypes binding of the C ABI in include/lsweeps.h (liblsweeps_gb300.so).

This is the same surface a reference-side FFI would bind; the library is loaded
from this package directory and a missing or stale build fails loudly."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "liblsweeps_gb300.so"

LSW_OK = 0
STATUS_NAMES = ["LSW_OK", "LSW_ERR_INVALID_ARGUMENT", "LSW_ERR_CUDA", "LSW_ERR_OUT_OF_MEMORY",
                "LSW_ERR_NOT_SET_UP", "LSW_ERR_NOT_FACTORIZED", "LSW_ERR_SINGULAR_BLOCK",
                "LSW_ERR_NOT_CONVERGED", "LSW_ERR_UNSUPPORTED"]
PREC = {"c128": 0, "fp64": 0, "c64": 1, "mixed": 1, "bf16x2": 2, "split": 2}
GMRES_MODE = {"reference": 0, "flexible": 1}

# every entry point declared in include/lsweeps.h
EXPORTS = [
    "lsw_ctx_create", "lsw_ctx_destroy", "lsw_status_string", "lsw_ctx_last_error", "lsw_geometry_cell",
    "lsw_problem_setup", "lsw_problem_info_get", "lsw_cell_info_get", "lsw_factorize", "lsw_apply_precond",
    "lsw_apply_A", "lsw_assemble_rhs", "lsw_gmres", "lsw_solve_host", "lsw_local_solve",
    "lsw_apply_precond_profiled", "lsw_local_solve_noalloc", "lsw_release_workspace",
    "lsw_ctx_set_wait_limit", "lsw_selftest_bounded_wait", "lsw_ctx_set_graphs", "lsw_ctx_set_tuning",
    "lsw_ctx_set_sweep_lanes", "lsw_front_shapes",
]


class Geom(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_els_in_cell", C.c_int), ("pml", C.c_int), ("order", C.c_int),
                ("h", C.c_double)]


class ProblemInfo(C.Structure):
    _fields_ = [("n_g", C.c_int), ("n_dof", C.c_int), ("n_cells_total", C.c_int), ("max_cell_side", C.c_int),
                ("precision", C.c_int), ("factorized", C.c_int), ("factor_bytes", C.c_longlong),
                ("device_bytes", C.c_longlong), ("omega", C.c_double), ("pml_C", C.c_double),
                ("kernel_launches", C.c_longlong)]


class ApplyProfile(C.Structure):
    _fields_ = [("fronts", C.c_int), ("items", C.c_int), ("slots", C.c_int), ("front_ms", C.c_double),
                ("total_ms", C.c_double), ("alg_bytes", C.c_double), ("alg_flops", C.c_double),
                ("streamed_bytes", C.c_double)]


class CellInfo(C.Structure):
    _fields_ = [("I", C.c_int), ("J", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("lo_x", C.c_int),
                ("lo_y", C.c_int), ("lines_x", (C.c_int * 4) * 2), ("lines_y", (C.c_int * 4) * 2),
                ("own_x", (C.c_int * 2) * 2), ("own_y", (C.c_int * 2) * 2)]

    def as_dict(self):
        return dict(I=self.I, J=self.J, nx=self.nx, ny=self.ny, lo_x=self.lo_x, lo_y=self.lo_y,
                    lines_x=[list(r) for r in self.lines_x], lines_y=[list(r) for r in self.lines_y],
                    own_x=[list(r) for r in self.own_x], own_y=[list(r) for r in self.own_y])


class FrontShape(C.Structure):
    _fields_ = [("items", C.c_int), ("max_slots", C.c_int), ("slots_cap", C.c_int), ("cluster", C.c_int),
                ("tuned_ms", C.c_float), ("tensor_cores", C.c_int)]


class GmresOpts(C.Structure):
    _fields_ = [("mode", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int), ("restart", C.c_int),
                ("verbose", C.c_int)]


class GmresReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("final_log", C.c_double),
                ("true_rel_res", C.c_double), ("seconds", C.c_double), ("precond_applies", C.c_int),
                ("log", C.POINTER(C.c_double)), ("log_capacity", C.c_int), ("log_len", C.c_int)]


class LswError(RuntimeError):
    def __init__(self, status: int, msg: str):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {msg}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                          "(the CUDA library is the only implementation of this path)")
    L = C.CDLL(str(LIB_PATH))
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "lsw_ctx_create": (i, [C.POINTER(vp), i]),
        "lsw_ctx_destroy": (i, [vp]),
        "lsw_status_string": (C.c_char_p, [i]),
        "lsw_ctx_last_error": (C.c_char_p, [vp]),
        "lsw_geometry_cell": (i, [C.POINTER(Geom), i, C.POINTER(CellInfo)]),
        "lsw_problem_setup": (i, [vp, C.POINTER(Geom), C.POINTER(d), d, i]),
        "lsw_problem_info_get": (i, [vp, C.POINTER(ProblemInfo)]),
        "lsw_cell_info_get": (i, [vp, i, C.POINTER(CellInfo)]),
        "lsw_factorize": (i, [vp, vp]),
        "lsw_apply_precond": (i, [vp, vp, vp, i, vp]),
        "lsw_apply_A": (i, [vp, vp, vp, i, vp]),
        "lsw_assemble_rhs": (i, [vp, C.POINTER(d), C.POINTER(d), i, vp, vp]),
        "lsw_gmres": (i, [vp, vp, vp, i, C.POINTER(GmresOpts), C.POINTER(GmresReport), vp]),
        "lsw_solve_host": (i, [vp, C.POINTER(d), C.POINTER(d), i, C.POINTER(GmresOpts), C.POINTER(GmresReport), vp]),
        "lsw_local_solve": (i, [vp, i, vp, vp, i, vp]),
        "lsw_apply_precond_profiled": (i, [vp, vp, vp, i, vp, C.POINTER(ApplyProfile)]),
        "lsw_local_solve_noalloc": (i, [vp, i, vp, vp, i, vp]),
        "lsw_release_workspace": (i, [vp]),
        "lsw_ctx_set_wait_limit": (i, [vp, d]),
        "lsw_selftest_bounded_wait": (i, [vp, vp]),
        "lsw_ctx_set_graphs": (i, [vp, i]),
        "lsw_ctx_set_tuning": (i, [vp, i]),
        "lsw_ctx_set_sweep_lanes": (i, [vp, i]),
        "lsw_front_shapes": (i, [vp, i, C.POINTER(FrontShape), i, C.POINTER(i), C.POINTER(d), vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int, ctx=None):
    if status != LSW_OK:
        msg = lib().lsw_ctx_last_error(ctx).decode() if ctx else ""
        raise LswError(status, msg)


def geometry_cell(N: int, m: int, p: int, h: float, cell: int) -> dict:
    """Host-only geometry query (no GPU needed)."""
    g = Geom(N, m, p, 2, h)
    out = CellInfo()
    check(lib().lsw_geometry_cell(C.byref(g), cell, C.byref(out)))
    return out.as_dict()
