"""Request loop for Helmholtz solves on one GPU: admission by device memory,
a factor cache keyed by the operator, continuous batching and p50/p99
latency beside throughput.

The reference solves one problem per MPI job (main.cpp, Problem::solve in
src/Problem.cpp:94-158); this module runs a stream of such solves on the
sweep engine.  A request is one right-hand side (the sum of its point
sources, RHSSrcPts::eval, src/RHSSrcPts.cpp:87-99) for an operator given by
the geometry (cells, cell size, PML), the frequency, the medium and the
precision.

* Operators are factorised once and stay resident (``FactorCache``); a later
  request with the same key reuses the factors.  Device memory is the
  admission budget: a request whose operator is not resident is admitted when
  its estimated footprint fits after evicting idle operators (least recently
  used first); otherwise it waits until running work frees memory.  An
  operator with no request waiting returns its solve workspace (Krylov bases,
  sweep pools) when its batch ends and is charged only its factors while
  idle; its next batch is admitted for the growth back to the batch
  footprint, so far more operators stay resident than their peak sizes allow.
* Continuous batching: every slot (a host thread with its own CUDA stream)
  takes the oldest admissible request and every other waiting request for
  the same operator (up to ``max_batch``), and solves them as one
  multi-right-hand-side flexible GMRES, so each sweep-front launch carries
  all of their slots.  Requests that arrive while a batch runs join the next
  batch of their operator; batches of different operators run at the same
  time on different slots, and their kernels overlap on the device.
* Each request records its arrival, start and completion times; ``ServeStats``
  reports latency percentiles, throughput and cache behaviour.

The GPU path goes through ``lsweeps.solver.Solver`` (the C ABI); the
scheduling logic takes any backend with the same small interface, which is
how it is tested without a GPU.
"""
from __future__ import annotations

import hashlib
import math
import threading
import time
from collections import OrderedDict
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from .problems import ProblemSpec, layered_medium, lens_medium, random_medium, constant_medium, omega_for_ppw


# ---------------------------------------------------------------------------
# Requests and operators
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Medium:
    """A seeded medium generator (``kind`` in lens / layered / random /
    constant with its parameters) or an explicit slowness grid (``kind`` =
    "array", ``grid`` = 1/c^2 on the DOF grid)."""
    kind: str
    params: tuple = ()
    grid: Optional[np.ndarray] = field(default=None, compare=False, hash=False)

    def digest(self, spec: ProblemSpec) -> str:
        h = hashlib.sha1()
        h.update(repr((self.kind, self.params, spec.n_dof)).encode())
        if self.grid is not None:
            h.update(np.ascontiguousarray(self.grid, dtype=np.float64).tobytes())
        return h.hexdigest()[:16]

    def build(self, spec: ProblemSpec) -> np.ndarray:
        if self.kind == "array":
            return np.ascontiguousarray(self.grid, dtype=np.float64)
        p = dict(self.params)
        if self.kind == "lens":
            return lens_medium(spec, **p)
        if self.kind == "layered":
            return layered_medium(spec, **p)
        if self.kind == "random":
            return random_medium(spec, **p)
        if self.kind == "constant":
            return constant_medium(spec, **p)
        raise ValueError(f"unknown medium kind {self.kind!r}")


@dataclass(frozen=True)
class OperatorKey:
    N: int
    m: int
    p: int
    h: float
    omega: float
    medium: str
    precision: str


@dataclass
class Request:
    rid: int
    spec: ProblemSpec
    medium: Medium
    sources: list
    amplitudes: Optional[list] = None
    arrival: float = 0.0          # seconds after the stream starts
    tol: float = 1e-6
    precision: str = "c64"
    # filled in by the engine
    x: Optional[np.ndarray] = None
    iterations: int = 0
    true_rel_res: float = float("nan")
    batch_size: int = 0
    cache_hit: bool = False
    t_start: float = float("nan")
    t_done: float = float("nan")
    error: Optional[str] = None

    def key(self) -> OperatorKey:
        k = self.__dict__.get("_key")
        if k is None:
            s = self.spec
            k = OperatorKey(s.N, s.m, s.p, float(s.h), float(s.omega), self.medium.digest(s), self.precision)
            self.__dict__["_key"] = k
        return k

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def estimate_bytes(spec: ProblemSpec, precision: str, max_batch: int, restart: int = 30) -> int:
    """Device footprint of a resident operator: the factors of every cell
    (nx x ny x ldn complex values) plus the per-problem vectors, the Krylov
    basis of a batch and the sweep buffers, with 25 % headroom."""
    cs = 16 if precision in ("c128", "fp64") else 8
    side = spec.m + 6 + 2 * spec.p - 1          # interior cell DOFs per side (the largest)
    ldn = (side + 3) // 4 * 4
    factors = spec.N * spec.N * side * side * ldn * cs
    n2 = spec.n_dof * spec.n_dof
    vectors = n2 * 8 + 16 * n2 * max_batch * (2 * (restart + 1) + 8) + 4 * cs * n2 * max_batch * 2
    return int(1.25 * (factors + vectors))


# ---------------------------------------------------------------------------
# Backends
# ---------------------------------------------------------------------------
class GpuOperator:
    """A resident operator on the GPU: set up and factorised on creation."""

    def __init__(self, spec: ProblemSpec, m_grid: np.ndarray, precision: str, device: int, stream):
        from .solver import Solver
        self.solver = Solver(spec, m_grid, precision=precision, device=device)
        # several slots run operators from their own host threads: a CUDA-graph
        # capture in one thread can be invalidated by another thread's
        # allocations, frees or synchronous copies (and invalidate their
        # calls), so serving launches every apply's kernels directly (launch
        # overhead is < 1 % of an apply)
        self.solver.set_graphs(False)
        try:
            self.solver.factorize(stream=stream)
        except BaseException:
            # a failed factorisation (e.g. out of device memory) returns its
            # context and buffers now, not when the exception is collected
            self.solver.close()
            raise
        self.bytes = int(self.solver.info()["device_bytes"])

    def solve(self, reqs: list, stream, restart: int = 30, max_iter: int = 400) -> None:
        import torch
        S = self.solver
        with torch.cuda.stream(stream):
            b = torch.cat([S.assemble_rhs(r.sources, r.amplitudes, stream=stream) for r in reqs])
            tol = min(r.tol for r in reqs)
            x, rep = S.gmres(b, mode="flexible", tol=tol, max_iter=max_iter, restart=restart, stream=stream)
            # true relative residual of every request
            ax = S.apply_A(x, stream=stream)
            res = (b - ax).view(len(reqs), -1).norm(dim=1) / b.view(len(reqs), -1).norm(dim=1)
            xh = x.view(len(reqs), -1).cpu().numpy()
            resh = res.cpu().numpy()
        self.bytes = max(self.bytes, int(S.info()["device_bytes"]))
        for i, r in enumerate(reqs):
            r.x = xh[i].copy()
            r.iterations = rep.iterations
            r.true_rel_res = float(resh[i])

    def release(self) -> int:
        """Return the Krylov bases and sweep pools to the device (the factors
        stay); the bytes the operator still holds."""
        self.solver.release_workspace()
        return int(self.solver.info()["device_bytes"])

    def close(self) -> None:
        self.solver.close()


class GpuBackend:
    def __init__(self, device: int = 0):
        self.device = device

    def free_bytes(self) -> int:
        import torch
        return int(torch.cuda.mem_get_info(self.device)[0])

    def new_stream(self):
        import torch
        return torch.cuda.Stream(device=self.device)

    def create(self, req: Request, stream):
        return GpuOperator(req.spec, req.medium.build(req.spec), req.precision, self.device, stream)

    def trim(self) -> None:
        """Return torch's cached, unused device blocks to the driver (before an
        out-of-memory retry)."""
        import torch
        torch.cuda.empty_cache()


# ---------------------------------------------------------------------------
# Factor cache
# ---------------------------------------------------------------------------
@dataclass
class CacheEntry:
    key: OperatorKey
    bytes: int
    op: object = None
    busy: bool = False
    ready: bool = False
    last_used: float = 0.0
    uses: int = 0


class FactorCache:
    """Resident operators under a byte budget; idle entries are evicted least
    recently used first."""

    def __init__(self, budget: int):
        self.budget = int(budget)
        self.entries: "OrderedDict[OperatorKey, CacheEntry]" = OrderedDict()
        self.evictions = 0

    @property
    def used(self) -> int:
        return sum(e.bytes for e in self.entries.values())

    def can_admit(self, nbytes: int, keep=None) -> bool:
        """Whether `nbytes` fit after evicting every idle entry but `keep`."""
        idle = sum(e.bytes for e in self.entries.values() if not e.busy and e is not keep)
        return self.used - idle + nbytes <= self.budget

    def make_room(self, nbytes: int, keep=None) -> list:
        """Evict idle entries but `keep` (LRU first) until `nbytes` fit; returns
        the evicted entries (their operators still have to be closed)."""
        out = []
        for k in sorted(self.entries, key=lambda k: self.entries[k].last_used):
            if self.used + nbytes <= self.budget:
                break
            e = self.entries[k]
            if e.busy or e is keep:
                continue
            del self.entries[k]
            out.append(e)
            self.evictions += 1
        return out


# ---------------------------------------------------------------------------
# Engine
# ---------------------------------------------------------------------------
@dataclass
class ServeStats:
    n: int
    makespan_s: float
    solves_per_s: float
    p50_ms: float
    p99_ms: float
    mean_ms: float
    wait_p50_ms: float
    cache_hits: int
    factorisations: int
    evictions: int
    batches: int
    mean_batch: float
    max_in_flight: int
    failures: int
    oom_retries: int = 0

    def as_dict(self) -> dict:
        return dict(self.__dict__)


def _pct(v, q):
    v = sorted(v)
    if not v:
        return float("nan")
    i = q * (len(v) - 1)
    lo, hi = int(math.floor(i)), int(math.ceil(i))
    return v[lo] + (v[hi] - v[lo]) * (i - lo)


class ServeEngine:
    """Continuous-batching request loop (see the module docstring)."""

    def __init__(self, backend=None, slots: int = 4, max_batch: int = 8, budget: Optional[int] = None,
                 reserve: int = 4 << 30, restart: int = 30, clock: Callable[[], float] = time.perf_counter):
        self.backend = backend if backend is not None else GpuBackend()
        self.slots = slots
        self.max_batch = max_batch
        self.restart = restart
        if budget is None:
            budget = max(0, self.backend.free_bytes() - reserve)
        self.cache = FactorCache(budget)
        self.clock = clock
        self._cv = threading.Condition()
        self._pending: list = []
        self._done: list = []
        self._closing = False
        self._in_flight = 0
        self._max_in_flight = 0
        self._batches = 0
        self._batched = 0
        self._hits = 0
        self._factorisations = 0
        self._oom_retries = 0
        self._t0 = 0.0

    # -- scheduling (called with the lock held) --------------------------------
    def _pick(self):
        """The oldest waiting request that can run now, with every waiting
        request for the same operator (up to max_batch).  A request whose
        operator alone exceeds the budget fails at once."""
        for r in list(self._pending):
            if r.key() not in self.cache.entries:
                need = estimate_bytes(r.spec, r.precision, self.max_batch, self.restart)
                if need > self.cache.budget:
                    self._pending.remove(r)
                    r.error = f"operator needs ~{need} device bytes, budget is {self.cache.budget}"
                    r.t_start = r.t_done = self.clock() - self._t0
                    self._done.append(r)
        for r in self._pending:
            k = r.key()
            e = self.cache.entries.get(k)
            if e is not None:
                if e.busy:
                    continue
                # an idle operator that returned its workspace grows back to
                # the batch footprint: admit the growth like a new operator
                need = estimate_bytes(r.spec, r.precision, self.max_batch, self.restart)
                grow = need - e.bytes
                if grow > 0:
                    if not self.cache.can_admit(grow, keep=e):
                        continue
                    for ev in self.cache.make_room(grow, keep=e):
                        if ev.op is not None:
                            ev.op.close()
                    e.bytes = need
                hit = True
            else:
                need = estimate_bytes(r.spec, r.precision, self.max_batch, self.restart)
                if not self.cache.can_admit(need):
                    continue
                evicted = self.cache.make_room(need)
                e = CacheEntry(k, need)
                self.cache.entries[k] = e
                hit = False
                for ev in evicted:
                    if ev.op is not None:
                        ev.op.close()
            e.busy = True
            batch = [q for q in self._pending if q.key() == k][: self.max_batch]
            for q in batch:
                self._pending.remove(q)
                q.cache_hit = hit and e.ready
            return e, batch
        return None

    def _oom_retry(self, e, fn):
        """Run fn; if the device ran out of memory (the footprint estimate was
        low), evict every idle operator but e and run it once more."""
        oom = False
        try:
            return fn()
        except Exception as ex:
            if "OUT_OF_MEMORY" not in str(ex) and "out of memory" not in str(ex).lower():
                raise
            oom = True
        # retried outside the handler: the failed call's frames (and the device
        # buffers they hold) are released with the exception before the retry
        assert oom
        with self._cv:
            victims = [x for x in self.cache.entries.values() if not x.busy and x is not e]
            for v in victims:
                del self.cache.entries[v.key]
                self.cache.evictions += 1
            self._oom_retries += 1
        for v in victims:
            if v.op is not None:
                v.op.close()
        trim = getattr(self.backend, "trim", None)
        if trim is not None:
            trim()
        return fn()

    def _worker(self, slot: int):
        stream = self.backend.new_stream()
        while True:
            with self._cv:
                job = None
                while job is None:
                    if self._closing and not self._pending:
                        return
                    job = self._pick()
                    if job is None:
                        self._cv.wait(timeout=0.05)
                e, batch = job
                self._in_flight += 1
                self._max_in_flight = max(self._max_in_flight, self._in_flight)
                self._batches += 1
                self._batched += len(batch)
            t_start = self.clock() - self._t0
            for r in batch:
                r.t_start = t_start
                r.batch_size = len(batch)
            err = None
            try:
                if e.op is None:
                    e.op = self._oom_retry(e, lambda: self.backend.create(batch[0], stream))
                    self._factorisations += 1
                    e.ready = True
                else:
                    self._hits += len(batch)
                self._oom_retry(e, lambda: e.op.solve(batch, stream, restart=self.restart))
            except Exception as ex:  # a failed solve fails its requests, not the loop
                err = f"{type(ex).__name__}: {ex}"
            t_done = self.clock() - self._t0
            # nothing waiting for this operator: it returns its solve workspace
            # (outside the lock: freeing device memory waits for the device) and
            # is charged only the bytes it keeps while idle
            resident = None
            with self._cv:
                idle_next = err is None and not any(q.key() == e.key for q in self._pending)
            if idle_next and e.op is not None and hasattr(e.op, "release"):
                try:
                    resident = int(e.op.release())
                except Exception:
                    resident = None
            with self._cv:
                for r in batch:
                    r.t_done = t_done
                    r.error = err
                    self._done.append(r)
                if e.op is not None:
                    e.bytes = max(e.bytes, int(getattr(e.op, "bytes", e.bytes)))
                if resident is not None:
                    e.bytes = resident
                if err is not None and not e.ready:
                    self.cache.entries.pop(e.key, None)
                    if e.op is not None:
                        e.op.close()
                e.busy = False
                e.last_used = t_done
                e.uses += 1
                self._in_flight -= 1
                self._cv.notify_all()

    def run(self, requests: list, realtime: bool = True) -> ServeStats:
        """Serve `requests` (arrival times in seconds from now when
        `realtime`, otherwise all at once) and return the statistics."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        # statistics are per run; resident factors carry over
        self._done, self._batches, self._batched, self._hits, self._factorisations = [], 0, 0, 0, 0
        self._max_in_flight = 0
        self._evictions0 = self.cache.evictions
        self._t0 = self.clock()
        self._closing = False
        workers = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(self.slots)]
        for w in workers:
            w.start()
        for r in reqs:
            if realtime:
                delay = r.arrival - (self.clock() - self._t0)
                if delay > 0:
                    time.sleep(delay)
            else:
                r.arrival = self.clock() - self._t0
            with self._cv:
                self._pending.append(r)
                self._cv.notify_all()
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        for w in workers:
            w.join()
        return self.stats()

    def stats(self) -> ServeStats:
        done = [r for r in self._done if r.error is None]
        lat = [1e3 * r.latency for r in done]
        waits = [1e3 * (r.t_start - r.arrival) for r in done]
        span = (max(r.t_done for r in done) - min(r.arrival for r in done)) if done else float("nan")
        return ServeStats(
            n=len(done), makespan_s=span, solves_per_s=len(done) / span if done and span > 0 else float("nan"),
            p50_ms=_pct(lat, 0.5), p99_ms=_pct(lat, 0.99), mean_ms=float(np.mean(lat)) if lat else float("nan"),
            wait_p50_ms=_pct(waits, 0.5), cache_hits=self._hits, factorisations=self._factorisations,
            evictions=self.cache.evictions - getattr(self, "_evictions0", 0), batches=self._batches,
            mean_batch=self._batched / self._batches if self._batches else 0.0,
            max_in_flight=self._max_in_flight, failures=len(self._done) - len(done),
            oom_retries=self._oom_retries)

    def close(self) -> None:
        for e in list(self.cache.entries.values()):
            if e.op is not None:
                e.op.close()
        self.cache.entries.clear()


# ---------------------------------------------------------------------------
# Synthetic request streams
# ---------------------------------------------------------------------------
def serving_stream(n: int, rate_hz: float, grids=(256, 512, 1024, 2048), m: int = 128, p: int = 16,
                   ppw=(6.0, 10.0), repeat_frac: float = 0.3, max_sources: int = 16, seed: int = 3,
                   precision: str = "c64", tol: float = 1e-6) -> list:
    """The serving workload: Poisson arrivals at `rate_hz`, grids drawn from
    `grids` (nominal sides, checkerboards of m x m cells), frequencies for
    6-10 points per wavelength at the medium's minimum velocity, lens or
    layered media of which `repeat_frac` repeat an earlier medium (same
    generator, seed and frequency, so the cached factors are reused), and
    1-`max_sources` point sources per request."""
    rng = np.random.default_rng(seed)
    t = 0.0
    seen: list = []
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate_hz) if rate_hz > 0 else 0.0
        if seen and rng.uniform() < repeat_frac:
            spec0, med = seen[rng.integers(len(seen))]
            spec = ProblemSpec(N=spec0.N, m=spec0.m, p=spec0.p, h=spec0.h, omega=spec0.omega, name=spec0.name)
        else:
            side = int(rng.choice(grids))
            N = max(1, side // m)
            n_g = N * m + N - 1
            h = 1.0 / n_g
            spec = ProblemSpec(N=N, m=m, p=p, h=h, omega=0.0, name=f"serve-{side}")
            if rng.uniform() < 0.5:
                med = Medium("lens", (("amp", float(rng.uniform(0.2, 0.5))), ("width", 0.1)))
                cmin = 1.0 - dict(med.params)["amp"]
            else:
                s = int(rng.integers(0, 1000))
                med = Medium("layered", (("seed_layers", s), ("seed_pert", s + 1)))
                cmin = float(np.sqrt(1.0 / med.build(spec).max()))
            spec.omega = omega_for_ppw(cmin, float(rng.uniform(*ppw)), h)
            seen.append((spec, med))
        k = int(rng.integers(1, max_sources + 1))
        srcs = [(float(rng.uniform(0.2, 0.8)) * spec.L, float(rng.uniform(0.2, 0.8)) * spec.L) for _ in range(k)]
        out.append(Request(rid=i, spec=spec, medium=med, sources=srcs, arrival=t, precision=precision, tol=tol))
    return out
