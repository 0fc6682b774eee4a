"""CPU oracle: a restatement of L-Sweeps-2D's checkerboard L-sweep preconditioner inside GMRES.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module, and only as the reference results or the timed CPU baseline.  The product path
(the CUDA library behind ``include/lsweeps.h``) never calls it.

Parity status: **parity unpinned by the reference.**  The reference ships no
tests, fixtures or golden vectors, and it cannot be compiled in this container
(Eigen 3, libconfig++ and MPI are absent).  This restatement is pinned instead
by self-consistency properties that hold for the reference's algorithm
(DD matvec == globally assembled operator, N=1 preconditioner == exact inverse,
window partition, ownership partition, GMRES solution == global direct solve),
see ``tests/test_oracle.py``.

Third-party arithmetic the reference delegates to Eigen 3 (version unpinned,
not vendored): ``SparseLU`` with COLAMD ordering for the local solves
(LocalLinearSolverEigenSparseLU.cpp:50,75) is restated with SciPy's SuperLU
(``splu``, COLAMD column ordering); the final Hessenberg solve
``colPivHouseholderQr`` (GlobalIterativeSolverGMRES.cpp:199) is restated with
``numpy.linalg.lstsq`` on the same square block; Eigen's ``dot`` (conjugate on
the first argument) and ``norm`` are restated with numpy.

Structure and names follow the reference (paths relative to the reference root):
  * AssemblerHelmholtz2DFD (src/AssemblerHelmholtz2DFD.cpp), PMLCubic2D
    (src/PMLCubic2D.cpp), FDweights / DerivativeDifferenceMatrix1D
    (src/FiniteDifferences.cpp), RHSSrcPts (src/RHSSrcPts.cpp)
  * SubdomainStructured (src/SubdomainStructured.cpp)
  * DDCheckerboard (src/DDCheckerboard.cpp), single process: every cell is
    local, so the MPI send/receive branches reduce to the local copies.
  * GlobalIterativeSolverGMRES (src/GlobalIterativeSolverGMRES.cpp) including
    its arithmetic quirks.
Geometry is computed in floating point exactly as the reference does (trace
limits between DOF rows, PML width rounded to whole cells), independently of
the integer-grid geometry used by the CUDA library, so the two cross-check.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PI = math.pi  # include/utils.h:12


# ----------------------------------------------------------------------------
# Finite differences  (src/FiniteDifferences.cpp)
# ----------------------------------------------------------------------------
def fd_weights(z: float, x: np.ndarray, m: int) -> np.ndarray:
    """Fornberg's weights for the m-th derivative at z on nodes x
    (src/FiniteDifferences.cpp:11-54)."""
    n = len(x) - 1
    c1 = 1.0
    c4 = x[0] - z
    c = np.zeros((m + 1, n + 1))
    c[0, 0] = 1.0
    for i in range(n):
        mn = min(i + 1, m)
        c2 = 1.0
        c5 = c4
        c4 = x[i + 1] - z
        for j in range(i + 1):
            c3 = x[i + 1] - x[j]
            c2 *= c3
            if j == i:
                for k in range(mn - 1, -1, -1):
                    c[k + 1, i + 1] = c1 * ((k + 1) * c[k, i] - c5 * c[k + 1, i]) / c2
                c[0, i + 1] = -c1 * c5 * c[0, i] / c2
            for k in range(mn - 1, -1, -1):
                c[k + 1, j] = (c4 * c[k + 1, j] - (k + 1) * c[k, j]) / c3
            c[0, j] = c4 * c[0, j] / c3
        c1 = c2
    return c[m].copy()


def derivative_difference_matrix_1d(nx: int, h: float, approx_order: int, der_order: int) -> sp.csr_matrix:
    """1D FD derivative matrix with one-sided end stencils
    (src/FiniteDifferences.cpp:57-122)."""
    assert nx >= approx_order + 1
    center = approx_order // 2
    nodes = np.arange(approx_order + 1, dtype=float)
    rows, cols, vals = [], [], []
    for i in range(center):
        w = fd_weights(i, nodes, der_order)
        for k in range(approx_order + 1):
            rows.append(i); cols.append(k); vals.append(w[k])
    w = fd_weights(center, nodes, der_order)
    for i in range(max(0, center), nx - max(center, approx_order - center)):
        for k in range(approx_order + 1):
            rows.append(i); cols.append(i - max(center, 0) + k); vals.append(w[k])
    for i in range(nx - max(center, approx_order - center), nx):
        w2 = fd_weights(nx - 1 - i + approx_order, nodes, der_order)
        for k in range(approx_order + 1):
            rows.append(i); cols.append(nx - (approx_order + 1) + k); vals.append(w2[k])
    vals = np.asarray(vals) / h ** der_order
    return sp.csr_matrix((vals, (rows, cols)), shape=(nx, nx))


# ----------------------------------------------------------------------------
# PML  (src/PMLCubic2D.cpp, src/PML.cpp)
# ----------------------------------------------------------------------------
@dataclass
class PMLCubic2D:
    """Cubic PML sigma = C*(dist/delta)^3, alpha = 1/(1+i*sigma)
    (src/PMLCubic2D.cpp:35-236)."""
    C: float
    omega: float
    width: float = 0.0
    int_domain: tuple = ((0.0, 1.0), (0.0, 1.0))

    @property
    def comp_domain(self):
        (a0, b0), (a1, b1) = self.int_domain
        w = self.width
        return ((a0 - w, b0 + w), (a1 - w, b1 + w))

    def _sigma(self, x, d):
        ia, ib = self.int_domain[d]
        ca, cb = self.comp_domain[d]
        s = np.zeros_like(x)
        ds = np.zeros_like(x)
        left = (x >= ca) & (x < ia)
        right = (x > ib) & (x < cb)
        inside = (x >= ia) & (x <= ib)
        if not np.all(left | right | inside):
            raise ValueError("ERROR: Evaluation point out of range!")  # PMLCubic2D.cpp:144
        dl = ia - ca
        dr = cb - ib
        s[left] = self.C * ((ia - x[left]) / dl) ** 3
        ds[left] = -3.0 * self.C * (ia - x[left]) ** 2 / dl ** 3
        s[right] = self.C * ((x[right] - ib) / dr) ** 3
        ds[right] = 3.0 * self.C * (x[right] - ib) ** 2 / dr ** 3
        return s, ds

    def diffusion(self, X, Y):
        s1, _ = self._sigma(X, 0)
        s2, _ = self._sigma(Y, 1)
        a1 = 1.0 / (1.0 + 1j * s1)
        a2 = 1.0 / (1.0 + 1j * s2)
        return a1 ** 2, a2 ** 2

    def convection(self, X, Y):
        s1, d1 = self._sigma(X, 0)
        s2, d2 = self._sigma(Y, 1)
        a1 = 1.0 / (1.0 + 1j * s1)
        a2 = 1.0 / (1.0 + 1j * s2)
        a1dx = -1j * d1 / (1.0 + 1j * s1) ** 2
        a2dy = -1j * d2 / (1.0 + 1j * s2) ** 2
        return a1dx * a1, a2dy * a2


# ----------------------------------------------------------------------------
# Assembler  (src/AssemblerHelmholtz2DFD.cpp)
# ----------------------------------------------------------------------------
class AssemblerHelmholtz2DFD:
    """5-point FD Helmholtz operator with cubic PML on one rectangle."""

    def __init__(self, omega: float, pml_width: float, mfunc, order: int = 2):
        self.omega = omega
        self.order = order
        self.mfunc = mfunc  # squared slowness m(X, Y), vectorised
        self.pml = PMLCubic2D(C=math.log(omega), omega=omega, width=pml_width)  # Input.cpp:836
        self.int_domain = None
        self.N = None

    def copy(self):
        a = AssemblerHelmholtz2DFD(self.omega, self.pml.width, self.mfunc, self.order)
        return a

    def set_domain(self, dom):
        self.int_domain = (tuple(dom[0]), tuple(dom[1]))
        self.pml.int_domain = self.int_domain

    def set_n(self, n):
        """AssemblerHelmholtz2DFD::setN (src/AssemblerHelmholtz2DFD.cpp:67-114)."""
        (a0, b0), (a1, b1) = self.int_domain
        h1 = (b0 - a0) / n[0]
        h2 = (b1 - a1) / n[1]
        h = min(h1, h2)
        w = self.pml.width
        ratio = w / h
        els = int(ratio)
        if ratio - els > 0.5:
            els += 1
        w = h * els
        self.pml.width = w
        cd = self.pml.comp_domain
        self.comp_domain = cd
        self.N = (int((cd[0][1] - cd[0][0] + 0.5 * h1) / h1),
                  int((cd[1][1] - cd[1][0] + 0.5 * h2) / h2))

    def mesh_size(self):
        cd = self.comp_domain
        h1 = (cd[0][1] - cd[0][0]) / self.N[0]
        h2 = (cd[1][1] - cd[1][0]) / self.N[1]
        return math.sqrt(h1 * h2)

    def dof_pts(self):
        """DOF ordering index = i*(ny-1)+j, y fastest (AssemblerHelmholtz2DFD.cpp:147-181)."""
        nx, ny = self.N
        cd = self.comp_domain
        hx = (cd[0][1] - cd[0][0]) / nx
        hy = (cd[1][1] - cd[1][0]) / ny
        i = np.arange(nx - 1)
        j = np.arange(ny - 1)
        X = np.repeat(cd[0][0] + (i + 1) * hx, ny - 1)
        Y = np.tile(cd[1][0] + (j + 1) * hy, nx - 1)
        return X, Y

    def assemble_system_matrix(self) -> sp.csc_matrix:
        """-(L1 Dxx + L2 Dyy) - (b1 Dx + b2 Dy) - w^2 m  (AssemblerHelmholtz2DFD.cpp:371-457)."""
        nx, ny = self.N
        cd = self.comp_domain
        hx = (cd[0][1] - cd[0][0]) / nx
        hy = (cd[1][1] - cd[1][0]) / ny
        A1 = derivative_difference_matrix_1d(nx + 1, hx, self.order, 2)[1:nx, 1:nx]
        A2 = derivative_difference_matrix_1d(ny + 1, hy, self.order, 2)[1:ny, 1:ny]
        I1 = sp.identity(nx - 1, format="csr")
        I2 = sp.identity(ny - 1, format="csr")
        X, Y = self.dof_pts()
        L1, L2 = self.pml.diffusion(X, Y)
        res = -(sp.diags(L1) @ sp.kron(A1, I2)) - sp.diags(L2) @ sp.kron(I1, A2)
        B1 = derivative_difference_matrix_1d(nx + 1, hx, self.order, 1)[1:nx, 1:nx]
        B2 = derivative_difference_matrix_1d(ny + 1, hy, self.order, 1)[1:ny, 1:ny]
        b1, b2 = self.pml.convection(X, Y)
        res = res - (sp.diags(b1) @ sp.kron(B1, I2) + sp.diags(b2) @ sp.kron(I1, B2))
        mval = self.mfunc(X, Y)
        res = res - sp.diags(self.omega * self.omega * mval * 1.0)  # reaction coeff = 1
        return sp.csc_matrix(res.astype(np.complex128))


def gaussian_rhs(X, Y, sources, eps, amplitudes=None):
    """RHSSrcPts::eval / deltaFunction (src/RHSSrcPts.cpp:87-112); source coeff = 1."""
    res = np.zeros(X.shape, dtype=np.complex128)
    for s, (x0, y0) in enumerate(sources):
        a = 1.0 if amplitudes is None else amplitudes[s]
        res += a * (1.0 / (PI * eps ** 2) * np.exp(-((x0 - X) ** 2 + (y0 - Y) ** 2) / eps ** 2))
    return res


# ----------------------------------------------------------------------------
# Subdomain  (src/SubdomainStructured.cpp)
# ----------------------------------------------------------------------------
class SubdomainStructured:
    def __init__(self, assembler: AssemblerHelmholtz2DFD, I: int, J: int):
        self.asm = assembler
        self.I, self.J = I, J
        self.lu = None

    def set_limits(self, lims_lr, lims_ud):
        """setLimits (SubdomainStructured.cpp:315-397): index sets in both
        directions, non-shifted and shifted, plus the L-trace index sets."""
        X, Y = self.asm.dof_pts()
        self.X, self.Y = X, Y
        self.size = X.size
        self.idx = {}
        self.idx["LeftRight"] = self._compute_volume_index_sets(X, lims_lr)
        self.idx["UpDown"] = self._compute_volume_index_sets(Y, lims_ud)
        self.ltr = {}
        for lt in ("BottomLeft", "BottomRight", "TopRight", "TopLeft"):
            for slr in (False, True):
                for sud in (False, True):
                    self.ltr[(lt, slr, sud)] = self._compute_ltrace_index_sets(lt, slr, sud)

    @staticmethod
    def _assign_index_sets(Xc, lims):
        """assignIndexSets (SubdomainStructured.cpp:1019-1116): first limit above the point."""
        cmp = Xc[:, None] < np.asarray(lims)[None, :]
        dom = np.where(cmp.any(axis=1), cmp.argmax(axis=1), 10)
        return [np.nonzero(dom == k)[0] for k in range(11)]

    def _compute_volume_index_sets(self, Xc, lims):
        """computeVolumeIndexSets (SubdomainStructured.cpp:749-801)."""
        s = self._assign_index_sets(Xc, lims)
        cat = lambda *a: np.sort(np.concatenate([s[k] for k in a]))
        non = [s[0], s[1], s[2], cat(3, 4, 5), s[6], s[7], cat(8, 9, 10)]
        shf = [cat(0, 1, 2), s[3], s[4], cat(5, 6, 7), s[8], s[9], s[10]]
        return {False: non, True: shf}

    def get_index_sets(self, direction, shifted):
        return self.idx[direction][shifted]

    def _compute_ltrace_index_sets(self, lt, slr, sud):
        """computeLTraceIndexSets (SubdomainStructured.cpp:1119-1277)."""
        s1 = self.get_index_sets("LeftRight", slr)
        s2 = self.get_index_sets("UpDown", sud)
        cat = np.concatenate
        if lt == "BottomLeft":
            i0v, i1v, i0h, i1h = s1[1], s1[2], s2[1], s2[2]
            n0v, n0h = s1[0], s2[0]
            n1v, n1h = cat([s1[0], s1[1]]), cat([s2[0], s2[1]])
        elif lt == "BottomRight":
            i0v, i1v, i0h, i1h = s1[5], s1[4], s2[1], s2[2]
            n0v, n0h = s1[6], s2[0]
            n1v, n1h = cat([s1[5], s1[6]]), cat([s2[0], s2[1]])
        elif lt == "TopRight":
            i0v, i1v, i0h, i1h = s1[5], s1[4], s2[5], s2[4]
            n0v, n0h = s1[6], s2[6]
            n1v, n1h = cat([s1[5], s1[6]]), cat([s2[5], s2[6]])
        elif lt == "TopLeft":
            i0v, i1v, i0h, i1h = s1[1], s1[2], s2[5], s2[4]
            n0v, n0h = s1[0], s2[6]
            n1v, n1h = cat([s1[0], s1[1]]), cat([s2[5], s2[6]])
        else:
            raise ValueError("ERROR: Invalid LTrace type!")
        res = []
        for on, off in (((i0v, i0h), (n0v, n0h)), ((i1v, i1h), (n1v, n1h))):
            t = np.zeros(self.size, dtype=bool)
            t[on[0]] = True
            t[on[1]] = True
            t[off[0]] = False
            t[off[1]] = False
            res.append(np.nonzero(t)[0])
        return res

    def assemble_system_matrix(self):
        """assembleSystemMatrix (SubdomainStructured.cpp:549-654): the matrix and
        the 48 coupling slices A[trace0,trace1] / A[trace1,trace0]."""
        self.A = self.asm.assemble_system_matrix()
        A = sp.csr_matrix(self.A)
        sl = lambda r, c: sp.csr_matrix(A[r][:, c])
        self.A01, self.A10 = {}, {}
        for shifted in (False, True):
            s1 = self.get_index_sets("LeftRight", shifted)
            s2 = self.get_index_sets("UpDown", shifted)
            self.A01[("Bottom", shifted)] = sl(s2[1], s2[2]); self.A10[("Bottom", shifted)] = sl(s2[2], s2[1])
            self.A01[("Right", shifted)] = sl(s1[5], s1[4]); self.A10[("Right", shifted)] = sl(s1[4], s1[5])
            self.A01[("Top", shifted)] = sl(s2[5], s2[4]); self.A10[("Top", shifted)] = sl(s2[4], s2[5])
            self.A01[("Left", shifted)] = sl(s1[1], s1[2]); self.A10[("Left", shifted)] = sl(s1[2], s1[1])
        for key, (l0, l1) in self.ltr.items():
            self.A01[key] = sl(l0, l1)
            self.A10[key] = sl(l1, l0)

    def factorize(self):
        """LocalLinearSolverEigenSparseLU::factorize (LocalLinearSolverEigenSparseLU.cpp:40-62),
        restated with SuperLU + COLAMD."""
        if self.lu is None:
            self.lu = spla.splu(sp.csc_matrix(self.A), permc_spec="COLAMD")

    def solve(self, b):
        if self.lu is None:
            raise RuntimeError("ERROR: The linear system has to be factorized before it can be solved!")
        return self.lu.solve(np.asarray(b, dtype=np.complex128))

    def get_equivalent_sources(self, trace_type, slr, sud, vals0, vals1):
        """getEquivalentSources (SubdomainStructured.cpp:1304-1465)."""
        if trace_type in ("Bottom", "Top"):
            key = (trace_type, sud)
        elif trace_type in ("Left", "Right"):
            key = (trace_type, slr)
        else:
            key = (trace_type, slr, sud)
        A01, A10 = self.A01[key], self.A10[key]
        assert vals0.size == A01.shape[0] and vals1.size == A01.shape[1]
        return [A01 @ vals1, -(A10 @ vals0)]

    def extract_ltraces(self, lt, slr, sud, lr0, lr1, ud0, ud1):
        """extractLTraces (SubdomainStructured.cpp:1468-1539): writes LR1, UD1, LR0,
        UD0 in that order into one cell vector, then gathers the L sets."""
        s1 = self.get_index_sets("LeftRight", slr)
        s2 = self.get_index_sets("UpDown", sud)
        if lt == "BottomLeft":
            iLR0, iLR1, iUD0, iUD1 = s1[1], s1[2], s2[1], s2[2]
        elif lt == "BottomRight":
            iLR0, iLR1, iUD0, iUD1 = s1[5], s1[4], s2[1], s2[2]
        elif lt == "TopRight":
            iLR0, iLR1, iUD0, iUD1 = s1[5], s1[4], s2[5], s2[4]
        else:
            iLR0, iLR1, iUD0, iUD1 = s1[1], s1[2], s2[5], s2[4]
        tmp = np.full(self.size, np.nan + 0j)  # Eigen leaves it uninitialised
        tmp[iLR1] = lr1
        tmp[iUD1] = ud1
        tmp[iLR0] = lr0
        tmp[iUD0] = ud0
        l0, l1 = self.ltr[(lt, slr, sud)]
        r0, r1 = tmp[l0], tmp[l1]
        assert not (np.isnan(r0).any() or np.isnan(r1).any())
        return [r0, r1]


# ----------------------------------------------------------------------------
# Domain decomposition  (src/DDCheckerboard.cpp)
# ----------------------------------------------------------------------------
class DDCheckerboard:
    """Single-process restatement: cell index i*N+j has row I=i, column J=j
    (DDCheckerboard.cpp:185-205 with nprocs = 1)."""

    def setup(self, assembler: AssemblerHelmholtz2DFD, domain, n_cells, n_els_in_cell, verbose=False,
              assemble=True):
        """DDCheckerboard::setUp (src/DDCheckerboard.cpp:87-645).  ``assemble``
        (True, False or a predicate of (I, J)) selects the cells whose matrices
        and coupling slices are assembled; the others get their geometry and
        index sets only (a process that owns some cells, as a rank of the
        reference owns its rows)."""
        order = assembler.order
        tt = int(math.ceil(order / 2.0))
        if n_els_in_cell[0] <= 4 * tt or n_els_in_cell[1] <= 4 * tt:
            raise ValueError("ERROR: Not enough elements in cell!")
        self.N1, self.N2 = n_cells
        n1 = n_cells[0] * n_els_in_cell[0] + n_cells[0] - 1
        n2 = n_cells[1] * n_els_in_cell[1] + n_cells[1] - 1
        h1 = (domain[0][1] - domain[0][0]) / n1
        h2 = (domain[1][1] - domain[1][0]) / n2
        self.cells = []
        self.keep = {}
        for I in range(n_cells[0]):
            for J in range(n_cells[1]):
                l1 = np.zeros(10)
                l2 = np.zeros(10)
                a = domain[0][0] + (n_els_in_cell[1] + 1) * J * h1
                if J > 0:
                    l1[0:5] = [a - tt * h1 - 0.5 * h1, a - 0.5 * h1, a + tt * h1 - 0.5 * h1,
                               a + 2 * tt * h1 - 0.5 * h1, a + 3 * tt * h1 - 0.5 * h1]
                    a -= 2 * tt * h1
                    if a < domain[0][0]:
                        a = domain[0][0]
                b = domain[0][0] + (n_els_in_cell[1] + 1) * J * h1 + n_els_in_cell[1] * h1
                if J < n_cells[1] - 1:
                    l1[5:10] = [b - tt * h1 + 0.5 * h1, b + 0.5 * h1, b + tt * h1 + 0.5 * h1,
                                b + 2 * tt * h1 + 0.5 * h1, b + 3 * tt * h1 + 0.5 * h1]
                    b += 4 * tt * h1
                    if b > domain[0][1]:
                        b = domain[0][1]
                dx = (a, b)
                a = domain[1][0] + (n_els_in_cell[0] + 1) * I * h2
                if I > 0:
                    l2[0:5] = [a - tt * h2 - 0.5 * h2, a - 0.5 * h2, a + tt * h2 - 0.5 * h2,
                               a + 2 * tt * h2 - 0.5 * h2, a + 3 * tt * h2 - 0.5 * h2]
                    a -= 2 * tt * h2
                    if a < domain[1][0]:
                        a = domain[1][0]
                b = domain[1][0] + (n_els_in_cell[0] + 1) * I * h2 + n_els_in_cell[0] * h2
                if I < n_cells[0] - 1:
                    l2[5:10] = [b - tt * h2 + 0.5 * h2, b + 0.5 * h2, b + tt * h2 + 0.5 * h2,
                                b + 2 * tt * h2 + 0.5 * h2, b + 3 * tt * h2 + 0.5 * h2]
                    b += 4 * tt * h2
                    if b > domain[1][1]:
                        b = domain[1][1]
                dy = (a, b)
                nn = (int((dx[1] - dx[0] + 0.5 * h1) / h1), int((dy[1] - dy[0] + 0.5 * h2) / h2))
                asm = assembler.copy()
                asm.set_domain((dx, dy))
                asm.set_n(nn)
                cell = SubdomainStructured(asm, I, J)
                X, Y = asm.dof_pts()
                minx, maxx = min(0.0, X.min()), max(0.0, X.max())
                miny, maxy = min(0.0, Y.min()), max(0.0, Y.max())
                if J == 0:
                    l1[0:5] = minx - h1
                if J == n_cells[1] - 1:
                    l1[5:10] = maxx + h1
                if I == 0:
                    l2[0:5] = miny - h2
                if I == n_cells[0] - 1:
                    l2[5:10] = maxy + h2
                cell.set_limits(l1, l2)
                if assemble is True or (callable(assemble) and assemble(I, J)):
                    cell.assemble_system_matrix()
                self.cells.append(cell)
                if verbose:
                    print("set up", I, "/", J)
        # owned-DOF masks  (DDCheckerboard.cpp:446-634)
        for key in ((False, False), (True, False), (False, True), (True, True)):
            self.keep[key] = []
        for c in self.cells:
            s1, s1s = c.get_index_sets("LeftRight", False), c.get_index_sets("LeftRight", True)
            s2, s2s = c.get_index_sets("UpDown", False), c.get_index_sets("UpDown", True)

            def mask(sa, sb):
                v = np.zeros(c.size, dtype=bool)
                for k in (2, 3, 4):
                    v[sa[k]] = True
                for k in (0, 1, 5, 6):
                    v[sb[k]] = False
                return np.nonzero(v)[0]

            self.keep[(False, False)].append(mask(s1, s2))
            self.keep[(True, False)].append(mask(s1s, s2))
            self.keep[(False, True)].append(mask(s1, s2s))
            self.keep[(True, True)].append(mask(s1s, s2s))
        self._loc = {(c.I, c.J): k for k, c in enumerate(self.cells)}
        return self

    # ---- bookkeeping --------------------------------------------------------
    def loc(self, I, J):
        return self._loc[(I, J)]

    def factorize(self):
        """DDCheckerboard::factorize (DDCheckerboard.cpp:648-665)."""
        for c in self.cells:
            c.factorize()

    def mesh_size(self):
        return min(c.asm.mesh_size() for c in self.cells)

    def assemble_rhs(self, sources, amplitudes=None):
        """assembleRHS (DDCheckerboard.cpp:668-684) with RHSSrcPts, eps = DD mesh size
        (Input.cpp:243)."""
        eps = self.mesh_size()
        full = [gaussian_rhs(c.X, c.Y, sources, eps, amplitudes) for c in self.cells]
        return self.reduce(full)

    def reduce(self, x, slr=False, sud=False):
        keep = self.keep[(slr, sud)]
        return [np.asarray(x[i])[keep[i]].copy() for i in range(len(self.cells))]

    def expand(self, x, slr=False, sud=False):
        keep = self.keep[(slr, sud)]
        out = []
        for i, c in enumerate(self.cells):
            v = np.zeros(c.size, dtype=np.complex128)
            v[keep[i]] = x[i]
            out.append(v)
        return out

    # ---- preconditioner -----------------------------------------------------
    def get_separated_rhs(self, rhs, slr, sud):
        """getSeparatedRHS (DDCheckerboard.cpp:3564-3674)."""
        res = self.expand(rhs)
        for i, c in enumerate(self.cells):
            s1 = c.get_index_sets("LeftRight", False)
            s2 = c.get_index_sets("UpDown", False)
            lr_lines = (1, 2, 4, 5)
            lr_rest = (0, 3, 6)
            ks1 = lr_rest if slr else lr_lines
            ks2 = lr_rest if sud else lr_lines
            for k in ks1:
                res[i][s1[k]] = 0.0
            for k in ks2:
                res[i][s2[k]] = 0.0
        return res

    def apply_precond(self, x):
        """applyPrecond (DDCheckerboard.cpp:687-739)."""
        res1, res2, res3, res4 = (self.apply_precond_part(x, q) for q in range(4))
        return [res1[i] + (res2[i] + res3[i] + res4[i]) for i in range(len(self.cells))]

    def apply_precond_part(self, x, q):
        """The q-th of the four shifted decompositions of applyPrecond
        (DDCheckerboard.cpp:687-739): q = 0 non-shifted, 1 shifted left-right,
        2 shifted up-down, 3 shifted both; window, conversion to the shifted
        ownership, sweep, conversion back."""
        slr, sud = bool(q & 1), bool(q & 2)
        r = self.reduce(self.get_separated_rhs(x, slr, sud))
        if q == 0:
            return self.apply_sweep(r, False, False)
        if q == 1:
            r = self.convert_nonshifted_to_shifted_lr(r, False)
            return self.convert_shifted_to_nonshifted_lr(self.apply_sweep(r, True, False), False)
        if q == 2:
            r = self.convert_nonshifted_to_shifted_ud(r, False)
            return self.convert_shifted_to_nonshifted_ud(self.apply_sweep(r, False, True), False)
        r = self.convert_nonshifted_to_shifted_lr(r, False)
        r = self.convert_nonshifted_to_shifted_ud(r, True)
        res = self.convert_shifted_to_nonshifted_ud(self.apply_sweep(r, True, True), True)
        return self.convert_shifted_to_nonshifted_lr(res, False)

    def apply_sweep(self, x, slr, sud):
        """applySweep (DDCheckerboard.cpp:812-880)."""
        xt = self.expand(x, slr, sud)
        res = [np.zeros_like(v) for v in xt]
        tLRloc, tUDloc = self.add_loc_sol(xt, res, slr, sud)
        tUDright = self.add_right_sweep(res, tLRloc, slr, sud)
        tUDleft = self.add_left_sweep(res, tLRloc, slr, sud)
        tLRup = self.add_up_sweep(res, tUDloc, slr, sud)
        tLRdown = self.add_down_sweep(res, tUDloc, slr, sud)
        self.add_bl2tr_sweep(res, tLRup, tUDright, slr, sud)
        self.add_tr2bl_sweep(res, tLRdown, tUDleft, slr, sud)
        self.add_br2tl_sweep(res, tLRup, tUDleft, slr, sud)
        self.add_tl2br_sweep(res, tLRdown, tUDright, slr, sud)
        return self.reduce(res, slr, sud)

    @staticmethod
    def _traces(sol, sets):
        return [sol[sets[1]].copy(), sol[sets[2]].copy(), sol[sets[4]].copy(), sol[sets[5]].copy()]

    def _order(self, key):
        """getSortedIndices on the diagonal index (utils.cpp:242-260); std::sort of
        (value, index) pairs == lexicographic sort."""
        d = [key(c.I, c.J) for c in self.cells]
        return sorted(range(len(self.cells)), key=lambda i: (d[i], i))

    def _fronts(self, key):
        """The cells of _order(key) grouped by equal key: one group is one step of
        the reference's pipelined sweep (cells on one anti-diagonal, whose solves
        depend only on groups before it), in the same order."""
        d = [key(c.I, c.J) for c in self.cells]
        groups = []
        for i in self._order(key):
            if groups and d[groups[-1][0]] == d[i]:
                groups[-1].append(i)
            else:
                groups.append([i])
        return groups

    def solve_many(self, jobs):
        """Local solves of one sweep front: jobs = [(cell index, rhs)], returns
        the solutions in order.  Serial here; a process-parallel executor
        replaces it (the solves of a front are independent)."""
        return [self.cells[i].solve(r) for i, r in jobs]

    def matvec_many(self, jobs):
        """Cell operator products [(cell index, x)] -> [A_cell x] (serial here)."""
        return [self.cells[i].A @ x for i, x in jobs]

    def add_loc_sol(self, x, res, slr, sud):
        """addLocSol (DDCheckerboard.cpp:883-973)."""
        tLR, tUD = [None] * len(self.cells), [None] * len(self.cells)
        sols = self.solve_many([(i, x[i]) for i in range(len(self.cells))])
        for i, c in enumerate(self.cells):
            sol = sols[i]
            res[i] += sol
            tUD[i] = self._traces(sol, c.get_index_sets("UpDown", sud))
            tLR[i] = self._traces(sol, c.get_index_sets("LeftRight", slr))
        return tLR, tUD

    def _dir_sweep(self, res, tin, slr, sud, order_key, active, nb, trace_type, rows_in, out_dir, own_sets, ins):
        """One directional sweep (addLeft/Right/Up/DownSweep) front by front: for
        each cell, the neighbour's outgoing pair becomes this cell's incoming
        pair, its equivalent sources are solved, the solution is added to res,
        its cross-direction traces recorded and its outgoing pair accumulated.
        ins: the (in0, in1) slots of tmp taken from the neighbour's (out0, out1)
        slots and the order of the trace values given to getEquivalentSources."""
        tmp = [list(t) for t in tin]
        tout = [None] * len(self.cells)
        (i0, i1), (o0, o1), eq_args = ins
        for group in self._fronts(order_key):
            jobs, meta = [], []
            for idx in group:
                c = self.cells[idx]
                s1, s2 = c.get_index_sets("LeftRight", slr), c.get_index_sets("UpDown", sud)
                so = s1 if out_dir == "LR" else s2        # sets of the cross-direction traces
                si = s1 if out_dir == "UD" else s2        # sets along the sweep direction
                tout[idx] = [np.zeros(so[k].size, dtype=np.complex128) for k in (1, 2, 4, 5)]
                if not active(c):
                    continue
                p = nb(c)
                tmp[idx][i0] = tmp[p][o0]
                tmp[idx][i1] = tmp[p][o1]
                eq = c.get_equivalent_sources(trace_type, slr, sud, tmp[idx][eq_args[0]], tmp[idx][eq_args[1]])
                rhs = np.zeros(c.size, dtype=np.complex128)
                rhs[si[rows_in[0]]] = eq[rows_in[2]]
                rhs[si[rows_in[1]]] = eq[rows_in[3]]
                jobs.append((idx, rhs))
                meta.append((so, si))
            for (idx, _), sol, (so, si) in zip(jobs, self.solve_many(jobs), meta):
                res[idx] += sol
                for t, k in zip(range(4), (1, 2, 4, 5)):
                    tout[idx][t] = tout[idx][t] + sol[so[k]]
                tmp[idx][own_sets[0][0]] = tmp[idx][own_sets[0][0]] + sol[si[own_sets[0][1]]]
                tmp[idx][own_sets[1][0]] = tmp[idx][own_sets[1][0]] + sol[si[own_sets[1][1]]]
        return tout

    def add_left_sweep(self, res, tLR, slr, sud):
        """addLeftSweep (DDCheckerboard.cpp:976-1164): from the right neighbour's
        (trace0, trace1) as this cell's (traceN, traceNP); sources on traceN /
        traceNP rows; accumulates trace0 / trace1."""
        N1, N2 = self.N1, self.N2
        return self._dir_sweep(res, tLR, slr, sud, lambda I, J: (N1 - 1 - I) + (N2 - 1 - J),
                               lambda c: c.J < N2 - 1, lambda c: self.loc(c.I, c.J + 1), "Right",
                               (4, 5, 1, 0), "UD", ((0, 1), (1, 2)), ((2, 3), (0, 1), (3, 2)))

    def add_right_sweep(self, res, tLR, slr, sud):
        """addRightSweep (DDCheckerboard.cpp:1168-1350): from the left neighbour's
        (traceN, traceNP) as this cell's (trace0, trace1); accumulates traceN /
        traceNP."""
        return self._dir_sweep(res, tLR, slr, sud, lambda I, J: I + J,
                               lambda c: c.J > 0, lambda c: self.loc(c.I, c.J - 1), "Left",
                               (1, 2, 0, 1), "UD", ((2, 4), (3, 5)), ((0, 1), (2, 3), (0, 1)))

    def add_down_sweep(self, res, tUD, slr, sud):
        """addDownSweep (DDCheckerboard.cpp:1353-1540)."""
        N1, N2 = self.N1, self.N2
        return self._dir_sweep(res, tUD, slr, sud, lambda I, J: (N1 - 1 - I) + (N2 - 1 - J),
                               lambda c: c.I < N1 - 1, lambda c: self.loc(c.I + 1, c.J), "Top",
                               (4, 5, 1, 0), "LR", ((0, 1), (1, 2)), ((2, 3), (0, 1), (3, 2)))

    def add_up_sweep(self, res, tUD, slr, sud):
        """addUpSweep (DDCheckerboard.cpp:1544-1724)."""
        return self._dir_sweep(res, tUD, slr, sud, lambda I, J: I + J,
                               lambda c: c.I > 0, lambda c: self.loc(c.I - 1, c.J), "Bottom",
                               (1, 2, 0, 1), "LR", ((2, 4), (3, 5)), ((0, 1), (2, 3), (0, 1)))

    def _lsweep(self, res, tLR, tUD, slr, sud, lt, order_key, active, pull, extract_args,
                overwrite, overwrite_before_add, push):
        tLR = [list(t) for t in tLR]
        tUD = [list(t) for t in tUD]
        for group in self._fronts(order_key):
            jobs = []
            for idx in group:
                c = self.cells[idx]
                if not active(c.I, c.J):
                    continue
                pull(idx, c, tLR, tUD)
                lr0, lr1, ud0, ud1 = extract_args(idx, tLR, tUD)
                lv = c.extract_ltraces(lt, slr, sud, lr0, lr1, ud0, ud1)
                eq = c.get_equivalent_sources(lt, slr, sud, lv[0], lv[1])
                l0, l1 = c.ltr[(lt, slr, sud)]
                rhs = np.zeros(c.size, dtype=np.complex128)
                rhs[l0] = eq[0]
                rhs[l1] = eq[1]
                jobs.append((idx, rhs))
            for (idx, _), sol in zip(jobs, self.solve_many(jobs)):
                c = self.cells[idx]
                s1, s2 = c.get_index_sets("LeftRight", slr), c.get_index_sets("UpDown", sud)
                if overwrite_before_add:
                    overwrite(idx, sol, s1, s2, tLR, tUD)
                    res[idx] += sol
                else:
                    res[idx] += sol
                    overwrite(idx, sol, s1, s2, tLR, tUD)
                push(idx, sol, s1, s2, tLR, tUD)

    def add_bl2tr_sweep(self, res, tLR, tUD, slr, sud):
        """addBL2TRSweep (DDCheckerboard.cpp:2393-2608); overwrites trace0 entries
        before the accumulation (2520-2526)."""
        loc = self.loc

        def pull(idx, c, LR, UD):
            m = loc(c.I, c.J - 1)
            LR[idx][0] = LR[m][2]; LR[idx][1] = LR[m][3]
            m = loc(c.I - 1, c.J)
            UD[idx][0] = UD[m][2]; UD[idx][1] = UD[m][3]

        def over(idx, sol, s1, s2, LR, UD):
            sol[s1[1]] = LR[idx][0]
            sol[s2[1]] = UD[idx][0]

        def push(idx, sol, s1, s2, LR, UD):
            LR[idx][2] = LR[idx][2] + sol[s1[4]]; LR[idx][3] = LR[idx][3] + sol[s1[5]]
            UD[idx][2] = UD[idx][2] + sol[s2[4]]; UD[idx][3] = UD[idx][3] + sol[s2[5]]

        self._lsweep(res, tLR, tUD, slr, sud, "BottomLeft", lambda I, J: I + J,
                     lambda I, J: I > 0 and J > 0, pull,
                     lambda idx, LR, UD: (LR[idx][0], LR[idx][1], UD[idx][0], UD[idx][1]),
                     over, True, push)

    def add_tr2bl_sweep(self, res, tLR, tUD, slr, sud):
        """addTR2BLSweep (DDCheckerboard.cpp:1949-2170)."""
        N1, N2, loc = self.N1, self.N2, self.loc

        def pull(idx, c, LR, UD):
            p = loc(c.I, c.J + 1)
            LR[idx][2] = LR[p][0]; LR[idx][3] = LR[p][1]
            p = loc(c.I + 1, c.J)
            UD[idx][2] = UD[p][0]; UD[idx][3] = UD[p][1]

        def over(idx, sol, s1, s2, LR, UD):
            sol[s1[5]] = LR[idx][3]
            sol[s2[5]] = UD[idx][3]

        def push(idx, sol, s1, s2, LR, UD):
            LR[idx][0] = LR[idx][0] + sol[s1[1]]; LR[idx][1] = LR[idx][1] + sol[s1[2]]
            UD[idx][0] = UD[idx][0] + sol[s2[1]]; UD[idx][1] = UD[idx][1] + sol[s2[2]]

        self._lsweep(res, tLR, tUD, slr, sud, "TopRight",
                     lambda I, J: (N1 - 1 - I) + (N2 - 1 - J),
                     lambda I, J: I < N1 - 1 and J < N2 - 1, pull,
                     lambda idx, LR, UD: (LR[idx][3], LR[idx][2], UD[idx][3], UD[idx][2]),
                     over, False, push)

    def add_br2tl_sweep(self, res, tLR, tUD, slr, sud):
        """addBR2TLSweep (DDCheckerboard.cpp:2173-2390)."""
        N2, loc = self.N2, self.loc

        def pull(idx, c, LR, UD):
            p = loc(c.I, c.J + 1)
            LR[idx][2] = LR[p][0]; LR[idx][3] = LR[p][1]
            m = loc(c.I - 1, c.J)
            UD[idx][0] = UD[m][2]; UD[idx][1] = UD[m][3]

        def over(idx, sol, s1, s2, LR, UD):
            sol[s1[5]] = LR[idx][3]
            sol[s2[1]] = UD[idx][0]

        def push(idx, sol, s1, s2, LR, UD):
            LR[idx][0] = LR[idx][0] + sol[s1[1]]; LR[idx][1] = LR[idx][1] + sol[s1[2]]
            UD[idx][2] = UD[idx][2] + sol[s2[4]]; UD[idx][3] = UD[idx][3] + sol[s2[5]]

        self._lsweep(res, tLR, tUD, slr, sud, "BottomRight", lambda I, J: I + (N2 - 1 - J),
                     lambda I, J: I > 0 and J < N2 - 1, pull,
                     lambda idx, LR, UD: (LR[idx][3], LR[idx][2], UD[idx][0], UD[idx][1]),
                     over, False, push)

    def add_tl2br_sweep(self, res, tLR, tUD, slr, sud):
        """addTL2BRSweep (DDCheckerboard.cpp:1727-1946)."""
        N1, loc = self.N1, self.loc

        def pull(idx, c, LR, UD):
            m = loc(c.I, c.J - 1)
            LR[idx][0] = LR[m][2]; LR[idx][1] = LR[m][3]
            p = loc(c.I + 1, c.J)
            UD[idx][2] = UD[p][0]; UD[idx][3] = UD[p][1]

        def over(idx, sol, s1, s2, LR, UD):
            sol[s1[1]] = LR[idx][0]
            sol[s2[5]] = UD[idx][3]

        def push(idx, sol, s1, s2, LR, UD):
            LR[idx][2] = LR[idx][2] + sol[s1[4]]; LR[idx][3] = LR[idx][3] + sol[s1[5]]
            UD[idx][0] = UD[idx][0] + sol[s2[1]]; UD[idx][1] = UD[idx][1] + sol[s2[2]]

        self._lsweep(res, tLR, tUD, slr, sud, "TopLeft", lambda I, J: (N1 - 1 - I) + J,
                     lambda I, J: I < N1 - 1 and J > 0, pull,
                     lambda idx, LR, UD: (LR[idx][0], LR[idx][1], UD[idx][3], UD[idx][2]),
                     over, False, push)

    # ---- ownership conversions  (DDCheckerboard.cpp:2995-3515) ---------------
    def _convert(self, x, src_keep, dst_keep, direction, forward):
        """One restatement for the four conversion routines: expand with the source
        ownership, copy the two boundary lines from the neighbour, reduce with the
        destination ownership."""
        xe = self.expand(x, *src_keep)
        N1, N2 = self.N1, self.N2
        for idx, c in enumerate(self.cells):
            nb = None
            if direction == "LR":
                if forward and c.J < N2 - 1:
                    nb = self.loc(c.I, c.J + 1)
                elif not forward and c.J > 0:
                    nb = self.loc(c.I, c.J - 1)
            else:
                if forward and c.I < N1 - 1:
                    nb = self.loc(c.I + 1, c.J)
                elif not forward and c.I > 0:
                    nb = self.loc(c.I - 1, c.J)
            if nb is None:
                continue
            d = "LeftRight" if direction == "LR" else "UpDown"
            s, ss = c.get_index_sets(d, False), c.get_index_sets(d, True)
            n = self.cells[nb]
            t, ts = n.get_index_sets(d, False), n.get_index_sets(d, True)
            if forward:   # non-shifted -> shifted: fill traceNP and traceN-shifted
                xe[idx][s[5]] = xe[nb][t[2]]
                xe[idx][ss[4]] = xe[nb][ts[1]]
            else:         # shifted -> non-shifted: fill trace0-shifted and trace1
                xe[idx][ss[1]] = xe[nb][ts[4]]
                xe[idx][s[2]] = xe[nb][t[5]]
        return self.reduce(xe, *dst_keep)

    def convert_nonshifted_to_shifted_lr(self, x, sud):
        return self._convert(x, (False, sud), (True, sud), "LR", True)

    def convert_nonshifted_to_shifted_ud(self, x, slr):
        return self._convert(x, (slr, False), (slr, True), "UD", True)

    def convert_shifted_to_nonshifted_lr(self, x, sud):
        return self._convert(x, (True, sud), (False, sud), "LR", False)

    def convert_shifted_to_nonshifted_ud(self, x, slr):
        return self._convert(x, (slr, True), (slr, False), "UD", False)

    # ---- DD matvec  (DDCheckerboard.cpp:2611-2992) ----------------------------
    def apply_system_matrix(self, x):
        xe = self.expand(x)
        for idx, c in enumerate(self.cells):
            s1, s2 = c.get_index_sets("LeftRight", False), c.get_index_sets("UpDown", False)
            if c.J > 0:
                m = self.cells[self.loc(c.I, c.J - 1)]
                xe[idx][s1[1]] = xe[self.loc(c.I, c.J - 1)][m.get_index_sets("LeftRight", False)[4]]
            if c.I > 0:
                m = self.cells[self.loc(c.I - 1, c.J)]
                xe[idx][s2[1]] = xe[self.loc(c.I - 1, c.J)][m.get_index_sets("UpDown", False)[4]]
        for idx, c in enumerate(self.cells):
            s1, s2 = c.get_index_sets("LeftRight", False), c.get_index_sets("UpDown", False)
            if c.J < self.N2 - 1:
                p = self.cells[self.loc(c.I, c.J + 1)]
                xe[idx][s1[5]] = xe[self.loc(c.I, c.J + 1)][p.get_index_sets("LeftRight", False)[2]]
            if c.I < self.N1 - 1:
                p = self.cells[self.loc(c.I + 1, c.J)]
                xe[idx][s2[5]] = xe[self.loc(c.I + 1, c.J)][p.get_index_sets("UpDown", False)[2]]
        return self.reduce(self.matvec_many([(i, xe[i]) for i in range(len(self.cells))]))


# ----------------------------------------------------------------------------
# GMRES  (src/GlobalIterativeSolverGMRES.cpp)
# ----------------------------------------------------------------------------
def _cat(x):
    return np.concatenate(x)


def _split(v, like):
    out, o = [], 0
    for a in like:
        out.append(v[o:o + a.size].copy())
        o += a.size
    return out


def givens_rotation_ref(v1, v2):
    """givens_rotation (GlobalIterativeSolverGMRES.cpp:333-348): `v1==(0.0,0.0)` is a
    comma expression (== v1==0); complex squares, no conjugation."""
    if v1 == 0.0:
        return 0.0 + 0j, 1.0 + 0j
    t = (v1 ** 2 + v2 ** 2) ** 0.5
    cs = abs(v1) / t
    sn = cs * v2 / v1
    return cs, sn


def apply_givens_rotation_ref(h, cs, sn, k):
    """apply_givens_rotation (GlobalIterativeSolverGMRES.cpp:313-330): applies only
    rotations 0..k-2 (loop from i=1 to i<k with index i-1)."""
    for i in range(1, k):
        temp = cs[i - 1] * h[i - 1] + sn[i - 1] * h[i]
        h[i] = -sn[i - 1] * h[i - 1] + cs[i - 1] * h[i]
        h[i - 1] = temp
    c, s = givens_rotation_ref(h[k], h[k + 1])
    h[k] = c * h[k] + s * h[k + 1]
    h[k + 1] = 0.0
    cs.append(c)
    sn.append(s)


@dataclass
class GMRESReport:
    iterations: int
    log: list = field(default_factory=list)


def gmres_reference(dd: DDCheckerboard, rhs, tol=1e-6, max_iter=40, verbose=False):
    """GlobalIterativeSolverGMRES::solve (GlobalIterativeSolverGMRES.cpp:65-203):
    left-preconditioned, no restart, x0 = M^-1 b, MGS with Eigen's conjugate-first
    dot, the reference's Givens bookkeeping, and a square solve of H at the end."""
    rhs_prec = dd.apply_precond(rhs)
    res = [v.copy() for v in rhs_prec]
    r = dd.apply_precond(dd.apply_system_matrix(res))
    r = [rhs_prec[i] - r[i] for i in range(len(r))]
    rhs_norm = math.sqrt(sum(np.linalg.norm(v) ** 2 for v in rhs_prec))
    r_norm = math.sqrt(sum(np.linalg.norm(v) ** 2 for v in r))
    log = [r_norm / rhs_norm]
    if verbose:
        print("iteration 0:", log[-1])
    if log[0] < tol or max_iter == 0:
        return res, GMRESReport(0, log)
    Q = [_cat(r) / r_norm]
    beta = [complex(r_norm)]
    H = np.zeros((0, 0), dtype=np.complex128)
    cs, sn = [], []
    lastk = 0
    for k in range(max_iter):
        # arnoldi (GlobalIterativeSolverGMRES.cpp:238-310)
        q = _cat(dd.apply_precond(dd.apply_system_matrix(_split(Q[k], rhs))))
        h = np.zeros(k + 2, dtype=np.complex128)
        for i in range(k + 1):
            h[i] = np.vdot(q, Q[i])  # Eigen a.dot(b) = sum conj(a) b
            q = q - h[i] * Q[i]
        qn = np.linalg.norm(q)
        h[k + 1] = qn
        q = q / h[k + 1]
        apply_givens_rotation_ref(h, cs, sn, k)
        Hn = np.zeros((k + 2, k + 1), dtype=np.complex128)
        Hn[:H.shape[0], :H.shape[1]] = H
        Hn[:, k] = h
        H = Hn
        Q.append(q)
        beta.append(-sn[k] * beta[k])
        beta[k] = beta[k] * cs[k]
        log.append(abs(beta[-1]) / rhs_norm)
        if verbose:
            print(f"iteration {k + 1}:", log[-1])
        if log[-1] <= tol or k == max_iter - 1:
            lastk = k
            break
    k = lastk
    y = np.linalg.lstsq(H[:k + 1, :k + 1], np.asarray(beta[:k + 1]), rcond=None)[0]
    x = _cat(res) + np.stack(Q[:k + 1], axis=1) @ y
    return _split(x, rhs), GMRESReport(k + 1, log)


def fgmres(apply_A, apply_M, b, x0=None, tol=1e-6, restart=30, max_iter=200):
    """Textbook right-preconditioned flexible GMRES(m) (Saad 1993) with modified
    Gram-Schmidt and complex Givens rotations; the CPU model of the device FGMRES.
    Returns (x, iterations, history); history holds the Givens estimates and the
    true relative residual at every restart."""
    b = np.asarray(b, dtype=np.complex128)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.complex128)
    bn = np.linalg.norm(b)
    if bn == 0.0:
        return np.zeros_like(b), 0, [0.0]
    it = 0
    hist = []
    while True:
        r = b - apply_A(x)
        beta = np.linalg.norm(r)
        hist.append(beta / bn)
        if beta / bn <= tol or it >= max_iter:
            return x, it, hist
        V = [r / beta]
        Z = []
        H = np.zeros((restart + 1, restart), dtype=np.complex128)
        cs = np.zeros(restart, dtype=np.complex128)
        sn = np.zeros(restart, dtype=np.complex128)
        g = np.zeros(restart + 1, dtype=np.complex128)
        g[0] = beta
        ncol = 0
        for j in range(restart):
            z = apply_M(V[j])
            Z.append(z)
            w = apply_A(z)
            for i in range(j + 1):
                H[i, j] = np.vdot(V[i], w)
                w = w - H[i, j] * V[i]
            hn = np.linalg.norm(w)
            H[j + 1, j] = hn
            for i in range(j):
                t = np.conj(cs[i]) * H[i, j] + np.conj(sn[i]) * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            a, bb = H[j, j], H[j + 1, j]
            den = math.sqrt(abs(a) ** 2 + abs(bb) ** 2)
            cs[j] = a / den if den > 0 else 1.0
            sn[j] = bb / den if den > 0 else 0.0
            H[j, j] = den
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = np.conj(cs[j]) * g[j]
            it += 1
            ncol = j + 1
            hist.append(abs(g[j + 1]) / bn)
            if abs(g[j + 1]) / bn <= tol or it >= max_iter or hn == 0.0:
                break
            V.append(w / hn)
        y = np.zeros(ncol, dtype=np.complex128)
        for i in range(ncol - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:ncol] @ y[i + 1:ncol]) / H[i, i]
        x = x + np.stack(Z[:ncol], axis=1) @ y


# ----------------------------------------------------------------------------
# Global layout helpers (test infrastructure)
# ----------------------------------------------------------------------------
def grid_medium(m_grid: np.ndarray, h: float, p: int):
    """Squared slowness sampled on the global DOF nodes, nearest-node lookup
    (the FunctionCSV semantics of piecewise-constant sampling, FunctionCSV.cpp:215-236)."""
    n = m_grid.shape[0]

    def f(X, Y):
        gx = np.clip(np.rint(X / h).astype(np.int64) + p - 1, 0, n - 1)
        gy = np.clip(np.rint(Y / h).astype(np.int64) + p - 1, 0, m_grid.shape[1] - 1)
        return m_grid[gx, gy]
    return f


def global_indices(dd: DDCheckerboard, h: float, p: int, n_dof: int, slr=False, sud=False):
    """Global DOF index (x-major, y fastest) of every owned DOF of every cell."""
    out = []
    for i, c in enumerate(dd.cells):
        k = dd.keep[(slr, sud)][i]
        gx = np.rint(c.X[k] / h).astype(np.int64) + p - 1
        gy = np.rint(c.Y[k] / h).astype(np.int64) + p - 1
        out.append(gx * n_dof + gy)
    return out


def to_global(x_cells, gidx, n_total):
    v = np.zeros(n_total, dtype=np.complex128)
    for xc, gi in zip(x_cells, gidx):
        v[gi] = xc
    return v


def to_cells(v, gidx):
    return [np.asarray(v)[gi].copy() for gi in gidx]


@dataclass
class OracleProblem:
    """One L-sweeps problem on the square domain [0, n_g h]^2: N x N cells of m
    interior elements, PML of p cells, squared slowness on the global DOF grid."""
    N: int
    m: int
    p: int
    h: float
    omega: float
    m_grid: np.ndarray

    def __post_init__(self):
        self.n_g = self.N * self.m + self.N - 1
        self.n_dof = self.n_g + 2 * self.p - 1
        self.L = self.n_g * self.h
        self.domain = ((0.0, self.L), (0.0, self.L))
        self.mfunc = grid_medium(self.m_grid, self.h, self.p)
        self.assembler = AssemblerHelmholtz2DFD(self.omega, self.p * self.h, self.mfunc)
        self.dd = DDCheckerboard().setup(self.assembler, self.domain, (self.N, self.N), (self.m, self.m))
        self.gidx = global_indices(self.dd, self.h, self.p, self.n_dof)

    def global_assembler(self):
        a = self.assembler.copy()
        a.set_domain(self.domain)
        a.set_n((self.n_g, self.n_g))
        return a

    def global_matrix(self):
        return self.global_assembler().assemble_system_matrix()

    def global_rhs(self, sources, amplitudes=None):
        X, Y = self.global_assembler().dof_pts()
        return gaussian_rhs(X, Y, sources, self.dd.mesh_size(), amplitudes)

    def G(self, x_cells):
        return to_global(x_cells, self.gidx, self.n_dof * self.n_dof)

    def C(self, v):
        return to_cells(v, self.gidx)

    def apply_precond_global(self, v):
        return self.G(self.dd.apply_precond(self.C(v)))

    def apply_A_global(self, v):
        return self.G(self.dd.apply_system_matrix(self.C(v)))
