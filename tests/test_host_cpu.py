"""The C++ host layer's CPU parts (include/lsweeps_host.hpp): the libconfig
subset parser, FunctionCSV sampling and RHSSrcPts, through a small probe
program compiled against the header and the library."""
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

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


def _run(probe, *args, stdin=""):
    return subprocess.run([str(probe), *map(str, args)], input=stdin, capture_output=True, text=True)


def _tree(dump: str):
    """Dump lines 'indent name kind [value]' back into nested tuples."""
    lines = [l for l in dump.splitlines() if l.strip()]
    pos = 0

    def node(depth):
        nonlocal pos
        l = lines[pos]
        pos += 1
        parts = l.strip().split(" ", 2)
        name, kind = parts[0], parts[1]
        val = parts[2] if len(parts) > 2 else None
        kids = []
        while pos < len(lines) and (len(lines[pos]) - len(lines[pos].lstrip(" "))) // 2 == depth + 1:
            kids.append(node(depth + 1))
        return (name, kind, val, kids)

    return node(0)


CONFIG = r'''
# reference-style problem file
Problems = ( { DomainDecomposition = "CheckerboardDD"; DomainDecompositionID = 0;
               RHS = "center"; Solver = "gmres"; Output = "vtk"; } );
/* block
   comment */
Domains : { unit = { Dim = 2; ax = 0.0; bx = 1.0; ay = -0.5; by = 5e-1; }; };
RHSs = { center = ( { Dim = 2; x = 0.5; y = 0.25 }, { Dim = 2; x = -1.25E+1; y = 3 } ); };
GlobalSolvers = { gmres = { Type = "GMRES"; Tol = 1e-6; MaxIter = 0x20; Verbose = TRUE; }; };  // trailing
Misc = { arr = [1, 2, 3]; empty = (); s = "a\"b" "c"; big = 123456789012L; neg = -7; };
'''


def test_libconfig_subset(probe, tmp_path):
    f = tmp_path / "p.cfg"
    f.write_text(CONFIG)
    r = _run(probe, "parse", f)
    assert r.returncode == 0, r.stderr
    root = _tree(r.stdout)

    def get(n, *path):
        for p in path:
            n = [c for c in n[3] if c[0] == p][0] if isinstance(p, str) else n[3][p]
        return n

    pr = get(root, "Problems")
    assert pr[1] == "list" and len(pr[3]) == 1
    assert get(pr, 0, "DomainDecomposition")[2] == "CheckerboardDD"
    assert get(pr, 0, "DomainDecompositionID")[1:3] == ("int", "0")
    assert float(get(root, "Domains", "unit", "by")[2]) == 0.5
    assert float(get(root, "Domains", "unit", "ay")[2]) == -0.5
    srcs = get(root, "RHSs", "center")
    assert len(srcs[3]) == 2 and float(get(srcs, 1, "x")[2]) == -12.5 and get(srcs, 1, "y")[1:3] == ("int", "3")
    g = get(root, "GlobalSolvers", "gmres")
    assert get(g, "MaxIter")[1:3] == ("int", "32") and get(g, "Verbose")[1:3] == ("bool", "true")
    assert float(get(g, "Tol")[2]) == 1e-6
    m = get(root, "Misc")
    assert get(m, "arr")[1] == "array" and [k[2] for k in get(m, "arr")[3]] == ["1", "2", "3"]
    assert get(m, "empty")[1] == "list" and get(m, "empty")[3] == []
    assert get(m, "s")[2] == 'a"bc'
    assert get(m, "big")[2] == "123456789012" and get(m, "neg")[2] == "-7"


@pytest.mark.parametrize("text,where", [('a = "x;', "line 1"), ("a = 1;\nb = ;", "line 2"),
                                        ("a = { b = 1; ", "end of file"), ("@include \"x\"", "include")])
def test_libconfig_errors(probe, tmp_path, text, where):
    f = tmp_path / "bad.cfg"
    f.write_text(text)
    r = _run(probe, "parse", f)
    assert r.returncode == 2 and where in r.stderr, r.stderr


def _csv_reference(vel, fdom, dom, pts):
    """FunctionCSV (src/FunctionCSV.cpp:46-236) restated: velocity file, row 0
    at the top, window of the domain, nearest file cell after clamping."""
    rows, cols = vel.shape
    hx = (fdom[0][1] - fdom[0][0]) / cols
    hy = (fdom[1][1] - fdom[1][0]) / rows
    d = [[max(dom[0][0], fdom[0][0]), min(dom[0][1], fdom[0][1])],
         [max(dom[1][0], fdom[1][0]), min(dom[1][1], fdom[1][1])]]
    r0 = int((fdom[1][1] - d[1][1]) / hy)
    r1 = min(int((fdom[1][1] - d[1][0]) / hy), rows - 1)
    c0 = int((d[0][0] - fdom[0][0]) / hx)
    c1 = min(int((d[0][1] - fdom[0][0]) / hx), cols - 1)
    da = [[fdom[0][0] + c0 * hx, fdom[0][0] + (c1 + 1) * hx], [fdom[1][1] - (r1 + 1) * hy, fdom[1][1] - r0 * hy]]
    A = 1.0 / vel[r0:r1 + 1, c0:c1 + 1].astype(np.float64) ** 2
    out = []
    for x in pts:
        x = list(x)
        for i in range(2):
            if x[i] <= da[i][0] + 0.5 * hx:
                x[i] = da[i][0] + 0.5 * hx
        for i in range(2):
            if x[i] >= da[i][1] - 0.5 * hy:
                x[i] = da[i][1] - 0.5 * hy
        col = int((x[0] - da[0][0]) / hx)
        row = int((da[1][1] - x[1]) / hy)
        out.append(A[row, col])
    return np.array(out), A.min(), A.max()


def test_function_csv_matches_the_reference_sampling(probe, tmp_path):
    rng = np.random.default_rng(4)
    vel = rng.uniform(1.5, 4.5, size=(5, 7)).astype(np.float32)
    f = tmp_path / "v.csv"
    f.write_text("\n".join(",".join(f"{v:.6f}" for v in row) for row in vel) + "\n")
    vel = np.array([[np.float32(f"{v:.6f}") for v in row] for row in vel], dtype=np.float32)
    fdom = [[0.0, 7.0], [0.0, 5.0]]
    dom = [[0.5, 6.2], [0.3, 4.9]]
    pts = np.concatenate([rng.uniform(-1, 8, size=(60, 2)), [[0.5, 0.3], [6.2, 4.9], [3.0, 2.0]]])
    r = _run(probe, "csv", f, 0.0, 7.0, 0.0, 5.0, 0.5, 6.2, 0.3, 4.9,
             stdin="\n".join(f"{float(x)!r} {float(y)!r}" for x, y in pts))
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    mn, mx = float(lines[0].split()[1]), float(lines[0].split()[3])
    got = np.array([float(v) for v in lines[1:] if v.strip()])
    want, _, _ = _csv_reference(vel, fdom, dom, pts)
    assert np.array_equal(got, want)
    a = 1.0 / vel.astype(np.float64) ** 2
    assert mn == a.min() and mx == a.max()


def test_rhs_src_pts(probe):
    pts = [(0.3, 0.4), (0.31, 0.45), (0.9, 0.1)]
    r = _run(probe, "rhs", 0.01, 0.3, 0.4, 0.32, 0.44, stdin="\n".join(f"{x} {y}" for x, y in pts))
    assert r.returncode == 0, r.stderr
    got = [float(v) for v in r.stdout.split()]
    for (x, y), g in zip(pts, got):
        want = sum(math.exp(-((x - a) ** 2 + (y - b) ** 2) / 1e-4) / (math.pi * 1e-4)
                   for a, b in ((0.3, 0.4), (0.32, 0.44)))
        assert g == pytest.approx(want, rel=1e-14, abs=1e-300)
