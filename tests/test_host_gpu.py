"""The reference's driver flow on the GPU: lsweeps_gb300_main reads a
libconfig problem file (Input), sets up DDCheckerboard with
LocalLinearSolverCUDA, solves with GlobalIterativeSolverGMRES and writes the
wavefield with OutputVTK.  The VTK values must equal the Python solver's
solution of the same problem (same geometry, PML, medium sampling and
source) within the VTK text precision (6 significant digits) and the solve
tolerance."""
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps.problems import ProblemSpec  # noqa: E402

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
MAIN = ROOT / "l-sweeps-2d_gb300" / "lsweeps" / "lsweeps_gb300_main"

N, M, P = 3, 12, 5
N_G = N * M + N - 1
L = 1.0
H = L / N_G


def _csv_grid(vel, fdom, dom, xs):
    """Squared slowness at the DOF points (FunctionCSV with the problem domain)."""
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
    g = np.empty((len(xs), len(xs)))
    for i, x in enumerate(xs):
        for j, y in enumerate(xs):
            p = [x, y]
            for k in range(2):
                if p[k] <= da[k][0] + 0.5 * hx:
                    p[k] = da[k][0] + 0.5 * hx
            for k in range(2):
                if p[k] >= da[k][1] - 0.5 * hy:
                    p[k] = da[k][1] - 0.5 * hy
            g[i, j] = A[int((da[1][1] - p[1]) / hy), int((p[0] - da[0][0]) / hx)]
    return g


def _problem_file(tmp_path, omega, min_m, medium_block, sources, extra_dd="", extra_solver=""):
    # MinWavelengthsInPML chosen so that the PML rounds to P elements
    wavelength = L * 2 * math.pi / omega / math.sqrt(min_m)
    minwl = P * H / wavelength
    src = ", ".join(f"{{ Dim = 2; x = {x!r}; y = {y!r}; }}" for x, y in sources)
    text = f"""
Problems = ( {{ DomainDecomposition = "CheckerboardDD"; DomainDecompositionID = 0;
               RHS = "src"; Solver = "gmres"; Output = "out"; }} );
DomainDecompositions = {{ CheckerboardDD = ( {{ Dim = 2; Domain = "unit"; PDE = "Helmholtz";
    NX = {M}; NY = {M}; NCellsX = {N}; NCellsY = {N}; Solver = "CUDA"; Omega = {omega!r};
    MinWavelengthsInPML = {minwl!r}; SquaredSlowness = "med"; Order = 2; {extra_dd} }} ); }};
Domains = {{ unit = {{ Dim = 2; ax = 0.0; bx = {L!r}; ay = 0.0; by = {L!r}; }};
            file = {{ Dim = 2; ax = 0.0; bx = {L!r}; ay = 0.0; by = {L!r}; }}; }};
SquaredSlownesses = {{ med = {medium_block}; }};
RHSs = {{ src = ( {src} ); }};
GlobalSolvers = {{ gmres = {{ Type = "GMRES"; Tol = 1e-6; MaxIter = 80; Verbose = false; {extra_solver} }}; }};
Outputs = {{ out = {{ Type = "VTK"; Filename = "{tmp_path / 'wave'}"; }}; }};
"""
    f = tmp_path / "problem.cfg"
    f.write_text(text)
    return f


def _read_vtk(path):
    lines = Path(path).read_text().splitlines()
    assert lines[0] == "# vtk DataFile Version 1.0" and lines[2] == "ASCII"
    assert lines[4] == "DATASET UNSTRUCTURED_GRID"
    npts = int(lines[5].split()[1])
    pts = np.array([[float(v) for v in l.split()[:2]] for l in lines[6:6 + npts]])
    k = lines.index(f"SCALARS wavefield_re float")
    re_ = np.array([float(v) for v in lines[k + 2:k + 2 + npts]])
    k2 = lines.index(f"SCALARS wavefield_im float")
    im_ = np.array([float(v) for v in lines[k2 + 2:k2 + 2 + npts]])
    cells = [l for l in lines if l.startswith("CELLS ")][0].split()
    return pts, re_ + 1j * im_, int(cells[1])


def _python_solution(omega, m_grid, sources, prec, mode):
    from lsweeps.solver import Solver
    spec = ProblemSpec(N=N, m=M, p=P, h=H, omega=omega)
    S = Solver(spec, m_grid, precision=prec)
    S.factorize()
    b = S.assemble_rhs(sources)
    x, rep = S.gmres(b, mode=mode, tol=1e-6, max_iter=80, restart=80 if mode == "reference" else 30)
    u = x.cpu().numpy().reshape(spec.n_dof, spec.n_dof)
    S.close()
    return u[P - 1:N_G + P, P - 1:N_G + P]


def _run_main(cfg):
    r = subprocess.run([str(MAIN), str(cfg)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Time to factorize system:" in r.stdout and "Time to run the GMRES:" in r.stdout
    return r.stdout


def test_driver_constant_medium_fp64_reference_gmres(tmp_path):
    omega = 2 * math.pi * 4.0
    sources = [(0.5, 0.5)]
    cfg = _problem_file(tmp_path, omega, 1.0, '{ Type = "Constant"; }', sources)
    _run_main(cfg)
    pts, vals, ncell = _read_vtk(tmp_path / "wave.vtk")
    assert len(vals) == (N_G + 1) ** 2 and ncell == N_G * N_G
    assert np.allclose(pts[:, 0].reshape(N_G + 1, N_G + 1)[:, 0], np.arange(N_G + 1) * H, atol=1e-6)
    nd = N_G + 2 * P - 1
    u = _python_solution(omega, np.ones((nd, nd)), sources, "c128", "reference")
    d = np.linalg.norm(vals - u.ravel()) / np.linalg.norm(u)
    assert d <= 1e-4, d


def test_driver_csv_medium_mixed_fgmres(tmp_path):
    rng = np.random.default_rng(3)
    vel = rng.uniform(1.0, 2.0, size=(8, 8)).astype(np.float32)
    csv = tmp_path / "vel.csv"
    csv.write_text("\n".join(",".join(f"{v:.6f}" for v in row) for row in vel) + "\n")
    vel = np.array([[np.float32(f"{v:.6f}") for v in row] for row in vel], dtype=np.float32)
    min_m = float((1.0 / vel.astype(np.float64) ** 2).min())
    omega = 2 * math.pi * 5.0
    sources = [(0.3, 0.6), (0.7, 0.35)]
    cfg = _problem_file(tmp_path, omega, min_m,
                        f'{{ Type = "CSV"; Filename = "{csv.name}"; Dim = 2; Domain = "file"; }}', sources,
                        extra_dd='Precision = "mixed";', extra_solver='Mode = "flexible"; Restart = 30;')
    _run_main(cfg)
    pts, vals, _ = _read_vtk(tmp_path / "wave.vtk")
    nd = N_G + 2 * P - 1
    xs = (np.arange(nd) + 1 - P) * H
    m_grid = _csv_grid(vel, [[0, L], [0, L]], [[0, L], [0, L]], xs)
    u = _python_solution(omega, m_grid, sources, "c64", "flexible")
    d = np.linalg.norm(vals - u.ravel()) / np.linalg.norm(u)
    assert d <= 1e-4, d


def test_driver_split_precision(tmp_path):
    omega = 2 * math.pi * 4.0
    sources = [(0.4, 0.55)]
    cfg = _problem_file(tmp_path, omega, 1.0, '{ Type = "Constant"; }', sources,
                        extra_dd='Precision = "split";', extra_solver='Mode = "flexible"; Restart = 30;')
    _run_main(cfg)
    _, vals, _ = _read_vtk(tmp_path / "wave.vtk")
    nd = N_G + 2 * P - 1
    u = _python_solution(omega, np.ones((nd, nd)), sources, "c128", "flexible")
    d = np.linalg.norm(vals - u.ravel()) / np.linalg.norm(u)
    assert d <= 1e-4, d


def test_driver_reports_input_errors(tmp_path):
    f = tmp_path / "bad.cfg"
    f.write_text('Problems = ( { DomainDecomposition = "CheckerboardDD"; } );')
    r = subprocess.run([str(MAIN), str(f)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "DomainDecompositionID" in r.stderr


def test_abstract_interface_driver_runs(tmp_path):
    """A driver written only against the abstract plugin classes (DD,
    Subdomain, Assembler, PML, LocalLinearSolver, GlobalIterativeSolver,
    Output; tests/host/abstract_driver.cpp) builds, solves on the GPU, copies
    its decomposition (DD::copy) and writes the wavefield."""
    import shutil
    lib = ROOT / "l-sweeps-2d_gb300" / "lsweeps"
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "abstract_driver"
    r = subprocess.run([cxx, "-std=c++17", "-O1", str(ROOT / "tests" / "host" / "abstract_driver.cpp"), "-I",
                        str(ROOT / "include"), "-L", str(lib), "-llsweeps_gb300", f"-Wl,-rpath,{lib}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "wave"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    vtk = (tmp_path / "wave.vtk").read_text().splitlines()
    i = vtk.index("SCALARS wavefield_re float")
    vals = np.array([float(v) for v in vtk[i + 2:i + 2 + 48 * 48]])
    assert np.isfinite(vals).all() and np.abs(vals).max() > 0
