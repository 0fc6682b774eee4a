"""C ABI checks that need no GPU: the library loads, exports every entry point
of include/lsweeps.h, and its integer-grid geometry equals the oracle's
floating-point restatement of DDCheckerboard::setUp / assignIndexSets."""
import re
from pathlib import Path

import numpy as np
import pytest

from lsweeps import capi
from lsweeps.problems import small
from oracle.lsweeps_oracle import OracleProblem

ROOT = Path(__file__).resolve().parent.parent


def test_library_loads_and_exports_header_symbols():
    L = capi.lib()
    header = (ROOT / "include" / "lsweeps.h").read_text()
    declared = set(re.findall(r"\b(lsw_[A-Za-z_]+)\s*\(", header))
    assert declared == set(capi.EXPORTS)
    for name in declared:
        assert hasattr(L, name), name


def test_status_strings():
    L = capi.lib()
    assert L.lsw_status_string(0) == b"LSW_OK"
    assert L.lsw_status_string(6) == b"LSW_ERR_SINGULAR_BLOCK"


def test_geometry_rejects_bad_input():
    with pytest.raises(capi.LswError):
        capi.geometry_cell(2, 4, 3, 0.01, 0)        # m <= 4 (DDCheckerboard.cpp:106-111)
    with pytest.raises(capi.LswError):
        capi.geometry_cell(2, 10, 3, 0.01, 4)       # cell index out of range


def _oracle_geometry(P, c_idx):
    c = P.dd.cells[c_idx]
    nx, ny = c.asm.N[0] - 1, c.asm.N[1] - 1
    gx = int(np.rint(c.X[0] / P.h)) + P.p - 1
    gy = int(np.rint(c.Y[0] / P.h)) + P.p - 1
    out = dict(I=c.I, J=c.J, nx=nx, ny=ny, lo_x=gx, lo_y=gy)
    for d, key, div in (("x", "LeftRight", True), ("y", "UpDown", False)):
        lines, own = [], []
        for s in (False, True):
            sets = c.get_index_sets(key, s)
            row = []
            for k in (1, 2, 4, 5):
                idx = sets[k]
                if idx.size == 0:
                    row.append(-1)
                else:
                    v = np.unique(idx // ny if div else idx % ny)
                    assert v.size == 1
                    row.append(int(v[0]))
            lines.append(row)
            keep = P.dd.keep[(s, False) if d == "x" else (False, s)][c_idx]
            v = keep // ny if div else keep % ny
            own.append([int(v.min()), int(v.max())])
        out[f"lines_{d}"] = lines
        out[f"own_{d}"] = own
    return out


@pytest.mark.parametrize("N,m,p", [(1, 6, 2), (2, 10, 4), (3, 12, 5), (4, 8, 3),
                                   # odd and even cell sizes, thin and thick PML, more cells,
                                   # and the 192-DOF limit
                                   (5, 7, 2), (6, 5, 1), (3, 31, 9), (8, 16, 6), (2, 149, 20)])
def test_geometry_matches_oracle(N, m, p):
    spec, med = small(N=N, m=m, p=p)
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    for c in range(N * N):
        assert capi.geometry_cell(N, m, p, spec.h, c) == _oracle_geometry(P, c)
