"""Problem specifications and seeded synthetic media for the L-sweeps solver.

A problem is the 2D Helmholtz equation -Lap u - omega^2 m(x) u = f on the square
[0, L]^2, L = n_g h, discretised by 5-point finite differences with a cubic PML
of ``p`` cells on every side, and decomposed into an N x N checkerboard of cells
with ``m`` interior elements each.  The global element count per side is
n_g = N m + N - 1 (DDCheckerboard.cpp:119 in the reference) and the global
DOF grid has n_dof = n_g + 2p - 1 nodes per side, node G at coordinate
(G + 1 - p) h, ordered x-major with y fastest (AssemblerHelmholtz2DFD.cpp:166-177).

The squared slowness m = 1/c^2 is given on that global DOF grid, PML included
(FunctionCSV semantics: velocity file -> 1/c^2 per sample, FunctionCSV.cpp:158).
The reference reads its media from CSV files of a companion repository that is
not available here; the generators below are seeded synthetic stand-ins with
the shapes and value ranges of the benchmark configurations.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class ProblemSpec:
    N: int                 # cells per side (NCellsX == NCellsY)
    m: int                 # interior elements per cell (NX == NY)
    p: int                 # PML thickness in cells
    h: float               # mesh size
    omega: float           # angular frequency
    name: str = "custom"
    sources: list = field(default_factory=list)     # [(x, y), ...]
    amplitudes: list | None = None

    @property
    def n_g(self) -> int:
        return self.N * self.m + self.N - 1

    @property
    def n_dof(self) -> int:
        return self.n_g + 2 * self.p - 1

    @property
    def L(self) -> float:
        return self.n_g * self.h

    def coords(self) -> np.ndarray:
        return (np.arange(self.n_dof) + 1 - self.p) * self.h

    def check(self):
        if self.m <= 4:
            raise ValueError("ERROR: Not enough elements in cell!")   # DDCheckerboard.cpp:108
        if self.p < 1 or self.N < 1:
            raise ValueError("need N >= 1 and p >= 1")


def omega_for_ppw(c_min: float, ppw: float, h: float) -> float:
    """Angular frequency at which the shortest wavelength 2 pi c_min / omega spans ppw cells."""
    return 2.0 * math.pi * c_min / (ppw * h)


def _smooth(a: np.ndarray, sigma: float) -> np.ndarray:
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(a, sigma, mode="nearest")


def constant_medium(spec: ProblemSpec, c: float = 1.0) -> np.ndarray:
    return np.full((spec.n_dof, spec.n_dof), 1.0 / (c * c))


def lens_medium(spec: ProblemSpec, amp: float = 0.4, width: float = 0.1) -> np.ndarray:
    """c(x) = 1 - amp exp(-|x - x0|^2 / (2 width^2)) on unit-scaled coordinates, x0 the centre."""
    s = spec.coords() / spec.L
    X, Y = np.meshgrid(s, s, indexing="ij")
    c = 1.0 - amp * np.exp(-((X - 0.5) ** 2 + (Y - 0.5) ** 2) / (2 * width * width))
    return 1.0 / (c * c)


def layered_medium(spec: ProblemSpec, n_layers: int = 12, cmin: float = 1.5, cmax: float = 4.5,
                   pert: float = 0.05, sigma_cells: float = 4.0, seed_layers: int = 0,
                   seed_pert: int = 1) -> np.ndarray:
    """Horizontal layers (velocity depends on depth = L - y) with seeded U[cmin,cmax]
    velocities, times (1 + pert * smoothed unit Gaussian noise)."""
    rl = np.random.default_rng(seed_layers)
    vel = rl.uniform(cmin, cmax, size=n_layers)
    depth = np.clip(1.0 - spec.coords() / spec.L, 0.0, 1.0 - 1e-12)
    layer = np.minimum((depth * n_layers).astype(int), n_layers - 1)
    c = np.broadcast_to(vel[layer][None, :], (spec.n_dof, spec.n_dof)).copy()
    rp = np.random.default_rng(seed_pert)
    noise = _smooth(rp.standard_normal(c.shape), sigma_cells)
    noise /= max(noise.std(), 1e-30)
    c = c * (1.0 + pert * noise)
    return 1.0 / (c * c)


def random_medium(spec: ProblemSpec, cmin: float = 1.5, cmax: float = 5.0, n_regions: int = 48,
                  sigma_cells: float = 8.0, seed: int = 2) -> np.ndarray:
    """Seeded piecewise-smooth medium: Voronoi regions with random velocities plus a
    linear trend per region, Gaussian-smoothed, rescaled to [cmin, cmax]."""
    r = np.random.default_rng(seed)
    n = spec.n_dof
    pts = r.uniform(0, n, size=(n_regions, 2))
    vals = r.uniform(0, 1, size=n_regions)
    grads = r.normal(0, 0.3 / n, size=(n_regions, 2))
    ii = np.arange(n, dtype=np.float64)
    c = np.empty((n, n))
    step = max(1, 4096 * 64 // max(n, 1))
    for a in range(0, n, step):
        xs = ii[a:a + step, None, None]
        ys = ii[None, :, None]
        d = (xs - pts[None, None, :, 0]) ** 2 + (ys - pts[None, None, :, 1]) ** 2
        k = d.argmin(axis=2)
        c[a:a + step] = vals[k] + grads[k, 0] * (xs[..., 0] - pts[k, 0]) + grads[k, 1] * (ys[..., 0] - pts[k, 1])
    c = _smooth(c, sigma_cells)
    c = (c - c.min()) / max(c.max() - c.min(), 1e-30)
    c = cmin + (cmax - cmin) * c
    return 1.0 / (c * c)


def config(name: str) -> tuple[ProblemSpec, np.ndarray]:
    """The benchmark configurations (C1..C4) with their seeded media."""
    name = name.upper()
    if name == "C1":
        h = 1.0 / 256
        spec = ProblemSpec(N=4, m=64, p=10, h=h, omega=omega_for_ppw(1.0, 10, h), name="C1")
        spec.sources = [(spec.L / 2, spec.L / 2)]
        return spec, constant_medium(spec)
    if name == "C2":
        N, m = 8, 128
        n_g = N * m + N - 1
        h = 1.0 / n_g
        spec = ProblemSpec(N=N, m=m, p=16, h=h, omega=omega_for_ppw(0.6, 8, h), name="C2")
        spec.sources = [(0.5, 0.5)]
        return spec, lens_medium(spec)
    if name == "C3":
        N, m = 16, 128
        n_g = N * m + N - 1
        h = 1.0 / n_g
        spec = ProblemSpec(N=N, m=m, p=20, h=h, omega=0.0, name="C3")
        med = layered_medium(spec)
        spec.omega = omega_for_ppw(float(np.sqrt(1.0 / med.max())), 8, h)
        spec.sources = [((k + 0.5) / 64, 1.0 - 0.05) for k in range(64)]
        return spec, med
    if name == "C4":
        N, m = 32, 128
        n_g = N * m + N - 1
        h = 1.0 / n_g
        spec = ProblemSpec(N=N, m=m, p=20, h=h, omega=0.0, name="C4")
        med = random_medium(spec)
        spec.omega = omega_for_ppw(float(np.sqrt(1.0 / med.max())), 8, h)
        spec.sources = [(0.5, 0.5)]
        return spec, med
    raise KeyError(name)


def small(N: int = 2, m: int = 12, p: int = 4, ppw: float = 10.0, medium: str = "lens",
          seed: int = 0) -> tuple[ProblemSpec, np.ndarray]:
    """A small seeded problem for parity tests (solved by the oracle in seconds)."""
    n_g = N * m + N - 1
    h = 1.0 / n_g
    spec = ProblemSpec(N=N, m=m, p=p, h=h, omega=0.0, name=f"small-N{N}-m{m}-p{p}-{medium}")
    if medium == "lens":
        med = lens_medium(spec)
    elif medium == "layered":
        med = layered_medium(spec, seed_layers=seed, seed_pert=seed + 1, sigma_cells=1.0)
    elif medium == "random":
        med = random_medium(spec, seed=seed, sigma_cells=1.5, n_regions=8)
    else:
        med = constant_medium(spec)
    spec.omega = omega_for_ppw(float(np.sqrt(1.0 / med.max())), ppw, h)
    spec.sources = [(0.5 * spec.L, 0.5 * spec.L)]
    return spec, med
