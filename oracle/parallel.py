"""Process-parallel executor of the CPU oracle.

TEST INFRASTRUCTURE AND CPU BASELINE ONLY.  Only ``tests/`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use this
module; the product path (the CUDA library) never calls it.

The reference runs its sweeps on MPI ranks that own rows of cells, dealt
round-robin (src/DDCheckerboard.cpp:126-177), each rank factorising and solving
its own cells and passing interface traces to its neighbours.  This executor
does the same with worker processes on one host: worker w owns the cells of
rows I = w (mod P), assembles and factorises them (SuperLU, one thread per
process) and answers the local solves and cell matvecs of those cells.  The
master process keeps the decomposition's geometry (index sets, ownership
masks, the small coupling slices sent back by the workers) and runs the
oracle's own sweep code (``DDCheckerboard`` in ``lsweeps_oracle``) unchanged:
every sweep front hands its independent cell solves to ``solve_many``, which
this executor spreads over the owners.  Vectors travel through shared memory
(one input and one output slot per owned cell), commands through pipes.

The result is bit-identical to the serial oracle: the same matrices, the same
SuperLU factorisations, the same arithmetic in the same order on the master.
"""
from __future__ import annotations

import math
import multiprocessing as mp
import os
import time
from multiprocessing import shared_memory

import numpy as np

from .lsweeps_oracle import AssemblerHelmholtz2DFD, DDCheckerboard, grid_medium


_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _problem_dd(N, m, p, h, omega, m_grid, assemble):
    n_g = N * m + N - 1
    L = n_g * h
    asm = AssemblerHelmholtz2DFD(omega, p * h, grid_medium(m_grid, h, p))
    return DDCheckerboard().setup(asm, ((0.0, L), (0.0, L)), (N, N), (m, m), assemble=assemble)


def _worker(conn, w, P, N, m, p, h, omega, grid_name, grid_shape, in_name, out_name, slots, max_size):
    """Worker w: own rows I = w (mod P); answer 'solve' / 'matvec' commands."""
    gshm = shared_memory.SharedMemory(name=grid_name)
    ishm = shared_memory.SharedMemory(name=in_name)
    oshm = shared_memory.SharedMemory(name=out_name)
    try:
        m_grid = np.ndarray(grid_shape, dtype=np.float64, buffer=gshm.buf).copy()
        dd = _problem_dd(N, m, p, h, omega, m_grid, assemble=lambda I, J: I % P == w)
        own = [i for i, c in enumerate(dd.cells) if c.I % P == w]
        t0 = time.perf_counter()
        for i in own:
            dd.cells[i].factorize()
        fact_s = time.perf_counter() - t0
        slices = {i: (dd.cells[i].A01, dd.cells[i].A10) for i in own}
        conn.send(("ready", slices, fact_s))
        inb = np.ndarray((slots, max_size), dtype=np.complex128, buffer=ishm.buf)
        outb = np.ndarray((slots, max_size), dtype=np.complex128, buffer=oshm.buf)
        while True:
            msg = conn.recv()
            if msg[0] == "quit":
                break
            kind, jobs = msg
            t = time.perf_counter()
            for cell, slot in jobs:
                c = dd.cells[cell]
                x = inb[slot, :c.size]
                outb[slot, :c.size] = c.solve(x) if kind == "solve" else c.A @ x
            conn.send(("ok", time.perf_counter() - t))
    finally:
        gshm.close()
        ishm.close()
        oshm.close()


class ParallelOracle:
    """The oracle's DDCheckerboard on [0, n_g h]^2 with its cell work spread
    over ``procs`` worker processes (spawned, so safe after a GPU call).

    ``dd`` is the master's DDCheckerboard: its apply_precond /
    apply_precond_part / apply_system_matrix and ``gmres_reference(dd, ...)``
    run the oracle's code with parallel cell solves.  Close with ``close()``
    (or use as a context manager)."""

    def __init__(self, N, m, p, h, omega, m_grid, procs=None):
        self.N, self.m, self.p, self.h, self.omega = N, m, p, h, omega
        self.procs = P = max(1, min(procs or os.cpu_count() or 1, N))
        self.n_g = N * m + N - 1
        self.n_dof = self.n_g + 2 * p - 1
        t0 = time.perf_counter()
        self.dd = _problem_dd(N, m, p, h, omega, m_grid, assemble=False)
        self.geometry_s = time.perf_counter() - t0
        cells = self.dd.cells
        self.owner = [c.I % P for c in cells]
        self.slot = [0] * len(cells)
        count = [0] * P
        for i, c in enumerate(cells):
            self.slot[i] = count[self.owner[i]]
            count[self.owner[i]] += 1
        self.max_size = max(c.size for c in cells)
        grid = np.ascontiguousarray(m_grid, dtype=np.float64)
        self._shms = []

        def shm(nbytes):
            s = shared_memory.SharedMemory(create=True, size=max(1, nbytes))
            self._shms.append(s)
            return s

        gs = shm(grid.nbytes)
        np.ndarray(grid.shape, dtype=np.float64, buffer=gs.buf)[...] = grid
        ctx = mp.get_context("spawn")
        self.conns, self.procs_, self.inb, self.outb = [], [], [], []
        t0 = time.perf_counter()
        # one BLAS thread per worker: the children read these when they import
        # numpy, so they are set in the parent before the processes start
        saved = {v: os.environ.get(v) for v in _THREAD_VARS}
        for v in _THREAD_VARS:
            os.environ[v] = "1"
        try:
            for w in range(P):
                si = shm(count[w] * self.max_size * 16)
                so = shm(count[w] * self.max_size * 16)
                self.inb.append(np.ndarray((count[w], self.max_size), dtype=np.complex128, buffer=si.buf))
                self.outb.append(np.ndarray((count[w], self.max_size), dtype=np.complex128, buffer=so.buf))
                a, b = ctx.Pipe()
                pr = ctx.Process(target=_worker, args=(b, w, P, N, m, p, h, omega, gs.name, grid.shape, si.name,
                                                       so.name, count[w], self.max_size), daemon=True)
                pr.start()
                self.conns.append(a)
                self.procs_.append(pr)
            for v, old in saved.items():
                if old is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = old
            saved = {}
            self.factorize_s = 0.0
            for w in range(P):
                msg = self.conns[w].recv()
                if msg[0] != "ready":
                    raise RuntimeError(f"oracle worker {w} failed to start")
                for i, (a01, a10) in msg[1].items():
                    cells[i].A01, cells[i].A10 = a01, a10
                self.factorize_s = max(self.factorize_s, msg[2])
        except BaseException:
            for v, old in saved.items():
                if old is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = old
            self.close()
            raise
        self.setup_s = time.perf_counter() - t0
        self.dd.solve_many = lambda jobs: self._run("solve", jobs)
        self.dd.matvec_many = lambda jobs: self._run("matvec", jobs)
        self.worker_s = 0.0   # summed busy time of the workers (all calls)

    def _run(self, kind, jobs):
        if not jobs:
            return []
        per = [[] for _ in range(self.procs)]
        for cell, x in jobs:
            w, s = self.owner[cell], self.slot[cell]
            n = self.dd.cells[cell].size
            self.inb[w][s, :n] = x
            per[w].append((cell, s))
        active = [w for w in range(self.procs) if per[w]]
        for w in active:
            self.conns[w].send((kind, per[w]))
        for w in active:
            msg = self.conns[w].recv()
            if msg[0] != "ok":
                raise RuntimeError(f"oracle worker {w}: {msg}")
            self.worker_s += msg[1]
        out = []
        for cell, _ in jobs:
            w, s = self.owner[cell], self.slot[cell]
            out.append(self.outb[w][s, :self.dd.cells[cell].size].copy())
        return out

    # ---- global-vector helpers (the library's layout: x-major, y fastest) ----
    def cells_of(self, v):
        from .lsweeps_oracle import global_indices, to_cells
        if not hasattr(self, "_gidx"):
            self._gidx = global_indices(self.dd, self.h, self.p, self.n_dof)
        return to_cells(v, self._gidx)

    def global_of(self, x_cells):
        from .lsweeps_oracle import global_indices, to_global
        if not hasattr(self, "_gidx"):
            self._gidx = global_indices(self.dd, self.h, self.p, self.n_dof)
        return to_global(x_cells, self._gidx, self.n_dof * self.n_dof)

    def apply_precond_global(self, v):
        return self.global_of(self.dd.apply_precond(self.cells_of(v)))

    def close(self):
        for c in getattr(self, "conns", []):
            try:
                c.send(("quit",))
            except (BrokenPipeError, OSError):
                pass
        for pr in getattr(self, "procs_", []):
            pr.join(timeout=30)
            if pr.is_alive():
                pr.terminate()
        self.conns, self.procs_ = [], []
        for s in getattr(self, "_shms", []):
            try:
                s.close()
                s.unlink()
            except FileNotFoundError:
                pass
        self._shms = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
