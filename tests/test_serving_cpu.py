"""Scheduling logic of the serving loop (admission by memory budget, factor
cache, continuous batching, statistics) with a fake backend, on the CPU."""
import threading
import time

import numpy as np
import pytest

from lsweeps.problems import ProblemSpec
from lsweeps.serving import (FactorCache, Medium, Request, ServeEngine, _pct, estimate_bytes,
                             serving_stream)


class FakeOp:
    def __init__(self, req, log, factor_s):
        self.key = req.key()
        self.log = log
        self.bytes = 1
        time.sleep(factor_s)
        log.append(("create", self.key))

    def solve(self, reqs, stream, restart=30):
        time.sleep(0.01)
        with threading.Lock():
            self.log.append(("solve", self.key, tuple(r.rid for r in reqs)))
        for r in reqs:
            r.x = np.array([float(r.rid)])
            r.iterations = 1
            r.true_rel_res = 0.0

    def close(self):
        self.log.append(("close", self.key))


class FakeBackend:
    def __init__(self, factor_s=0.02):
        self.log = []
        self.factor_s = factor_s

    def free_bytes(self):
        return 1 << 40

    def new_stream(self):
        return None

    def create(self, req, stream):
        return FakeOp(req, self.log, self.factor_s)


def _spec(N=2, m=12, p=4):
    n_g = N * m + N - 1
    return ProblemSpec(N=N, m=m, p=p, h=1.0 / n_g, omega=30.0)


def _req(rid, medium_seed, arrival=0.0, N=2):
    return Request(rid=rid, spec=_spec(N=N), medium=Medium("lens", (("amp", 0.1 + 0.01 * medium_seed),)),
                   sources=[(0.5, 0.5)], arrival=arrival)


def one_op_bytes(max_batch=4):
    return estimate_bytes(_spec(), "c64", max_batch)


def test_same_operator_requests_are_batched():
    be = FakeBackend()
    eng = ServeEngine(be, slots=2, max_batch=4, budget=10 * one_op_bytes())
    reqs = [_req(i, 0) for i in range(8)]
    st = eng.run(reqs, realtime=False)
    assert st.n == 8 and st.failures == 0
    assert st.factorisations == 1
    assert st.mean_batch > 1.0
    assert all(r.x[0] == r.rid for r in reqs)
    solves = [e for e in be.log if e[0] == "solve"]
    assert max(len(e[2]) for e in solves) <= 4


def test_distinct_operators_run_concurrently_and_are_cached():
    be = FakeBackend(factor_s=0.05)
    eng = ServeEngine(be, slots=3, max_batch=4, budget=10 * one_op_bytes())
    reqs = [_req(i, i % 3) for i in range(9)]
    st = eng.run(reqs, realtime=False)
    assert st.n == 9
    assert st.factorisations == 3
    assert st.max_in_flight >= 2
    # a second stream over the same media reuses every factor
    more = [_req(100 + i, i % 3) for i in range(6)]
    st2 = eng.run(more, realtime=False)
    assert st2.factorisations == 0 and st2.cache_hits == 6
    assert all(r.cache_hit for r in more)


def test_budget_evicts_least_recently_used_idle_operator():
    be = FakeBackend()
    b1 = one_op_bytes()
    eng = ServeEngine(be, slots=1, max_batch=4, budget=2 * b1 + 10)
    seq = [_req(0, 0, 0.00), _req(1, 1, 0.05), _req(2, 0, 0.10), _req(3, 2, 0.15)]
    st = eng.run(seq, realtime=True)
    assert st.n == 4
    # medium 1 was used least recently when medium 2 needed room
    closed = [e[1] for e in be.log if e[0] == "close"]
    assert closed == [seq[1].key()]
    assert st.evictions == 1
    assert set(eng.cache.entries) == {seq[0].key(), seq[3].key()}


class ReleasingOp(FakeOp):
    """A fake operator that keeps only a small resident part when idle."""

    def release(self):
        self.log.append(("release", self.key))
        return 10


class ReleasingBackend(FakeBackend):
    def create(self, req, stream):
        return ReleasingOp(req, self.log, self.factor_s)


def test_idle_operators_return_their_workspace_and_stay_resident():
    be = ReleasingBackend()
    b1 = one_op_bytes()
    # the budget of the eviction test above: without the release one operator
    # had to go, with it all three stay and the repeat is a cache hit
    eng = ServeEngine(be, slots=1, max_batch=4, budget=2 * b1 + 10)
    seq = [_req(0, 0, 0.00), _req(1, 1, 0.05), _req(2, 2, 0.10), _req(3, 1, 0.15)]
    st = eng.run(seq, realtime=True)
    assert st.n == 4 and st.failures == 0
    assert st.evictions == 0 and st.factorisations == 3 and st.cache_hits == 1
    assert len([e for e in be.log if e[0] == "release"]) == 4
    # idle entries are charged their resident bytes
    assert all(e.bytes == 10 for e in eng.cache.entries.values())


class OomOnceOp(FakeOp):
    """Fails its first solve as the device would when memory runs out."""
    tripped = False

    def solve(self, reqs, stream, restart=30):
        if not OomOnceOp.tripped:
            OomOnceOp.tripped = True
            raise RuntimeError("LSW_ERR_OUT_OF_MEMORY: cudaMalloc(Z): out of memory")
        super().solve(reqs, stream, restart)


class OomOnceBackend(FakeBackend):
    def create(self, req, stream):
        if req.rid == 2:
            return OomOnceOp(req, self.log, self.factor_s)
        return FakeOp(req, self.log, self.factor_s)


def test_out_of_memory_evicts_idle_operators_and_retries():
    be = OomOnceBackend()
    eng = ServeEngine(be, slots=1, max_batch=4, budget=10 * one_op_bytes())
    seq = [_req(0, 0, 0.00), _req(1, 1, 0.05), _req(2, 2, 0.10)]
    st = eng.run(seq, realtime=True)
    assert st.n == 3 and st.failures == 0 and st.oom_retries == 1
    # the two idle operators were evicted to make room for the retry
    assert st.evictions == 2 and {e[1] for e in be.log if e[0] == "close"} >= {seq[0].key(), seq[1].key()}
    assert seq[2].x is not None


def test_busy_operator_is_never_evicted():
    c = FactorCache(budget=100)
    from lsweeps.serving import CacheEntry, OperatorKey
    k1 = OperatorKey(1, 1, 1, 1.0, 1.0, "a", "c64")
    k2 = OperatorKey(1, 1, 1, 1.0, 1.0, "b", "c64")
    c.entries[k1] = CacheEntry(k1, 60, busy=True, last_used=0.0)
    c.entries[k2] = CacheEntry(k2, 30, busy=False, last_used=1.0)
    assert not c.can_admit(50)        # 60 busy + 50 > 100
    assert c.can_admit(40)
    ev = c.make_room(40)
    assert [e.key for e in ev] == [k2] and k1 in c.entries


def test_regrowth_never_evicts_the_operator_itself():
    c = FactorCache(budget=100)
    from lsweeps.serving import CacheEntry, OperatorKey
    k1 = OperatorKey(1, 1, 1, 1.0, 1.0, "a", "c64")
    k2 = OperatorKey(1, 1, 1, 1.0, 1.0, "b", "c64")
    e1 = CacheEntry(k1, 10, busy=False, last_used=0.0)     # released, about to regrow
    e2 = CacheEntry(k2, 50, busy=False, last_used=1.0)
    c.entries[k1], c.entries[k2] = e1, e2
    assert not c.can_admit(95, keep=e1)     # 10 kept + 95 > 100 even with e2 evicted
    assert c.can_admit(80, keep=e1)
    ev = c.make_room(80, keep=e1)
    assert [e.key for e in ev] == [k2] and k1 in c.entries


def test_oversized_request_fails_and_loop_ends():
    be = FakeBackend()
    eng = ServeEngine(be, slots=2, max_batch=4, budget=one_op_bytes() // 2)
    reqs = [_req(0, 0)]
    st = eng.run(reqs, realtime=False)
    assert st.n == 0 and st.failures == 1
    assert "budget" in reqs[0].error


def test_requests_arriving_during_a_batch_join_the_next_one():
    be = FakeBackend(factor_s=0.1)
    eng = ServeEngine(be, slots=1, max_batch=8, budget=10 * one_op_bytes())
    # the first request starts the factorisation; the others arrive while it runs
    reqs = [_req(0, 0, 0.0)] + [_req(i, 0, 0.02 + 0.005 * i) for i in range(1, 6)]
    st = eng.run(reqs, realtime=True)
    assert st.n == 6
    solves = [e[2] for e in be.log if e[0] == "solve"]
    assert solves[0] == (0,) and sorted(solves[1]) == [1, 2, 3, 4, 5]


def test_percentiles_and_stream_generator():
    assert _pct([1, 2, 3, 4], 0.5) == 2.5
    assert _pct([5.0], 0.99) == 5.0
    s = serving_stream(40, rate_hz=10.0, grids=(256, 512), seed=3)
    assert len(s) == 40
    arr = [r.arrival for r in s]
    assert arr == sorted(arr) and arr[0] > 0
    keys = [r.key() for r in s]
    assert len(set(keys)) < len(keys)          # some media repeat
    assert all(1 <= len(r.sources) <= 16 for r in s)
    assert {r.spec.N for r in s} <= {2, 4}


class PartialCreateBackend(FakeBackend):
    """create() allocates (a handle that must be closed) and then runs out of
    memory once, as a factorisation would; the retry succeeds."""

    def __init__(self):
        super().__init__()
        self.failed = False
        self.trims = 0

    def create(self, req, stream):
        if req.rid == 1 and not self.failed:
            self.failed = True
            self.log.append(("alloc-partial", req.key()))
            try:
                raise RuntimeError("LSW_ERR_OUT_OF_MEMORY: cudaMalloc(factors): out of memory")
            except RuntimeError:
                self.log.append(("close-partial", req.key()))
                raise
        return FakeOp(req, self.log, self.factor_s)

    def trim(self):
        self.trims += 1
        self.log.append(("trim",))


def test_out_of_memory_on_create_closes_partial_operator_before_retry():
    be = PartialCreateBackend()
    eng = ServeEngine(be, slots=1, max_batch=4, budget=10 * one_op_bytes())
    seq = [_req(0, 0, 0.00), _req(1, 1, 0.05)]
    st = eng.run(seq, realtime=True)
    assert st.n == 2 and st.failures == 0 and st.oom_retries == 1
    kinds = [e[0] for e in be.log]
    # the partial operator is closed, the cache trimmed, and only then created again
    i_close = kinds.index("close-partial")
    i_trim = kinds.index("trim")
    i_create = max(i for i, e in enumerate(be.log) if e[0] == "create" and e[1] == seq[1].key())
    assert i_close < i_trim < i_create
    assert seq[1].x is not None


def test_gpu_operator_closes_its_solver_when_factorisation_fails(monkeypatch):
    """GpuOperator returns its context when factorize raises (no GPU: the
    Solver is replaced by a recording fake)."""
    import lsweeps.solver as solver_mod
    from lsweeps.serving import GpuOperator
    events = []

    class FakeSolver:
        def __init__(self, *a, **k):
            events.append("init")

        def set_graphs(self, enable):
            events.append(f"graphs {int(enable)}")

        def factorize(self, stream=None):
            raise RuntimeError("LSW_ERR_OUT_OF_MEMORY: cudaMalloc(factors): out of memory")

        def close(self):
            events.append("close")

    monkeypatch.setattr(solver_mod, "Solver", FakeSolver)
    with pytest.raises(RuntimeError):
        GpuOperator(_spec(), np.ones((1, 1)), "c64", 0, None)
    # serving operators launch directly (no graph capture across slots)
    assert events == ["init", "graphs 0", "close"]
