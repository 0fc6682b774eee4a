"""The C++ host layer's Subdomain interface (SubdomainStructured on the
library's integer-grid geometry, no GPU) against the oracle's cells
(src/SubdomainStructured.cpp restated): the volume and L-trace index sets,
the cell operator A x, the equivalent sources of every trace type and shift,
the L-shaped traces; the element sets and element corners against the
reference's rules (element midpoints against the trace lines; corners
counter-clockwise from the bottom-left) evaluated on the probe's own points.
Also the GMRES settings of a problem file (Tol / MaxIter 0 keep the
reference's defaults 1e-6 / 40, Verbose defaults to true)."""
import json
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from lsweeps.problems import small
from oracle.lsweeps_oracle import OracleProblem

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "l-sweeps-2d_gb300" / "lsweeps"


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    if not (LIBDIR / "liblsweeps_gb300.so").exists():
        pytest.skip("library not built")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("probe") / "host_probe"
    cmd = [cxx, "-std=c++17", "-O1", str(ROOT / "tests" / "host" / "host_probe.cpp"), "-I", str(ROOT / "include"),
           "-L", str(LIBDIR), "-llsweeps_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _vals(n, seed):
    k = np.arange(n)
    return np.cos(seed + 0.7 * k) + 1j * np.sin(2.0 * seed + 0.3 * k)


def _cx(a):
    a = np.asarray(a, dtype=float)
    return a[:, 0] + 1j * a[:, 1] if a.size else np.zeros(0, complex)


@pytest.fixture(scope="module")
def problem():
    spec, med = small(N=3, m=10, p=4, medium="layered", seed=3)
    P = OracleProblem(spec.N, spec.m, spec.p, spec.h, spec.omega, med)
    return spec, med, P


def _cell(probe, problem, tmp_path, c):
    spec, med, P = problem
    gf = tmp_path / "m.bin"
    np.ascontiguousarray(med, dtype=np.float64).tofile(gf)
    r = subprocess.run([str(probe), "cell", str(spec.N), str(spec.m), str(spec.p), repr(spec.h), repr(spec.omega),
                        str(c), str(gf)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


@pytest.mark.parametrize("c", [0, 1, 4, 5, 8])
def test_subdomain_matches_oracle_cell(probe, problem, tmp_path, c):
    spec, med, P = problem
    d = _cell(probe, problem, tmp_path, c)
    oc = P.dd.cells[c]
    assert d["size"] == oc.size
    for direction in ("LeftRight", "UpDown"):
        for sh in (0, 1):
            got = d[f"sets_{direction}_{sh}"]
            want = oc.get_index_sets(direction, bool(sh))
            assert len(got) == 7
            for k in range(7):
                assert np.array_equal(np.asarray(got[k], dtype=np.int64), np.sort(want[k])), (direction, sh, k)
    for lt in ("BottomLeft", "BottomRight", "TopRight", "TopLeft"):
        for a in (0, 1):
            for b in (0, 1):
                got = d[f"ltr_{lt}_{a}{b}"]
                want = oc.ltr[(lt, bool(a), bool(b))]
                assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (lt, a, b)
    # the cell operator: the oracle's assembled matrix
    x = _vals(oc.size, 0.25)
    ax = _cx(d["Ax"])
    want = oc.A @ x
    assert np.linalg.norm(ax - want) <= 1e-12 * np.linalg.norm(want)
    # equivalent sources of every trace type present in this cell
    seen = 0
    for key, v in d.items():
        if not key.startswith("eqs_"):
            continue
        _, tt, ab = key.split("_")
        a, b = bool(int(ab[0])), bool(int(ab[1]))
        r0, r1 = _cx(v[0]), _cx(v[1])
        if tt in ("Left", "Right", "Bottom", "Top"):
            okey = (tt, b) if tt in ("Bottom", "Top") else (tt, a)
        else:
            okey = (tt, a, b)
        A01 = oc.A01[okey]
        w0, w1 = oc.get_equivalent_sources(tt, a, b, _vals(A01.shape[0], 0.5), _vals(A01.shape[1], 1.5))
        assert np.allclose(r0, w0, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(w0).max(initial=0))), key
        assert np.allclose(r1, w1, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(w1).max(initial=0))), key
        seen += 1
    assert seen > 0
    for key, v in d.items():
        if not key.startswith("ltraces_"):
            continue
        _, lt, ab = key.split("_")
        a, b = bool(int(ab[0])), bool(int(ab[1]))
        s1, s2 = oc.get_index_sets("LeftRight", a), oc.get_index_sets("UpDown", b)
        left, bottom = lt in ("BottomLeft", "TopLeft"), lt in ("BottomLeft", "BottomRight")
        n = [len(s1[1] if left else s1[5]), len(s1[2] if left else s1[4]),
             len(s2[1] if bottom else s2[5]), len(s2[2] if bottom else s2[4])]
        w = oc.extract_ltraces(lt, a, b, _vals(n[0], 2.0), _vals(n[1], 2.5), _vals(n[2], 3.0), _vals(n[3], 3.5))
        assert np.array_equal(_cx(v[0]), w[0]) and np.array_equal(_cx(v[1]), w[1]), key


@pytest.mark.parametrize("c", [0, 4, 8])
def test_subdomain_points_elements_and_corners(probe, problem, tmp_path, c):
    spec, med, P = problem
    d = _cell(probe, problem, tmp_path, c)
    oc = P.dd.cells[c]
    pts = np.asarray(d["phys"])
    n = oc.size
    # DOF points first, as the oracle's cell (x-major, y fastest)
    assert np.allclose(pts[:n, 0], oc.X, atol=1e-12) and np.allclose(pts[:n, 1], oc.Y, atol=1e-12)
    h = spec.h
    xs, ys = np.unique(np.round(oc.X / h, 6)), np.unique(np.round(oc.Y / h, 6))
    ex, ey = len(xs) + 1, len(ys) + 1
    assert d["nels"] == ex * ey and len(pts) == n + 2 * ex + 2 * ey
    # every element: four corners counter-clockwise from the bottom-left, an h x h square
    cen = np.zeros((ex * ey, 2))
    for e, cr in enumerate(d["corners"]):
        q = pts[cr]
        J, I = divmod(e, ey)
        assert np.allclose(q[1] - q[0], [h, 0], atol=1e-9) and np.allclose(q[2] - q[1], [0, h], atol=1e-9)
        assert np.allclose(q[3] - q[2], [-h, 0], atol=1e-9)
        cen[e] = q.mean(axis=0)
        if e:
            assert np.allclose(cen[e] - cen[0], [J * h, I * h], atol=1e-9)
    # element sets: the element midpoint against the trace-line coordinates
    # ([1], [2], [4], [5] of the volume sets), nine sets, all in [4] without lines
    for direction, comp in (("LeftRight", 0), ("UpDown", 1)):
        for sh in (0, 1):
            sets = oc.get_index_sets(direction, bool(sh))
            X = pts[:, comp]
            lo, hi = X.min(), X.max()

            def lim(k, fb):
                return X[sets[k]].min() if len(sets[k]) else fb

            lims = [lim(1, lo - 1), lim(2, lo - 1), lim(4, hi + 1), lim(5, hi + 1)]
            want = np.full(ex * ey, 8)
            for e in range(ex * ey):
                v = cen[e, comp]
                for k, L in enumerate(lims):
                    if v < L:
                        want[e] = 2 * k
                        break
            if all(len(sets[k]) == 0 for k in (1, 2, 4, 5)):
                want[:] = 4
            got = d[f"elsets_{direction}_{sh}"]
            for k in range(9):
                assert np.array_equal(got[k], np.nonzero(want == k)[0]), (direction, sh, k)


def test_gmres_defaults_from_problem_file(probe, tmp_path):
    def settings(body):
        f = tmp_path / "p.cfg"
        f.write_text('Problems = ( { Solver = "g"; } );\nGlobalSolvers = { g = { Type = "GMRES"; ' + body + ' }; };\n')
        r = subprocess.run([str(probe), "gmres", str(f)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        t = r.stdout.split()
        return float(t[1]), int(t[3]), int(t[5])

    assert settings("") == (1e-6, 40, 1)
    assert settings("MaxIter = 0; Tol = 0.0;") == (1e-6, 40, 1)
    assert settings("MaxIter = 12; Tol = 1e-8; Verbose = false;") == (1e-8, 12, 0)


def test_driver_against_abstract_interfaces_compiles(tmp_path):
    """A driver written only against the reference's abstract classes (DD,
    Subdomain, Assembler, PML, Function, RHS, LocalLinearSolver,
    GlobalIterativeSolver, Output) compiles and links against the library."""
    if not (LIBDIR / "liblsweeps_gb300.so").exists():
        pytest.skip("library not built")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path / "abstract_driver"
    cmd = [cxx, "-std=c++17", "-O0", "-Wall", "-Werror", str(ROOT / "tests" / "host" / "abstract_driver.cpp"),
           "-I", str(ROOT / "include"), "-L", str(LIBDIR), "-llsweeps_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
