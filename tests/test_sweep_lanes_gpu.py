"""Per-sweep launches (the schedule of one or two right-hand sides): every
stage-2 sweep and every L-sweep runs as its own chain of launches on its own
stream, the L-sweeps starting while stage 2 still runs, with one output plane
per stage-2 sweep summed at the end.

They solve the same cells with the same inputs as one launch per sweep step
(LSW_SWEEP_LANES=0); only the order of the final sums differs, so the two
agree to rounding (complex128 1e-13, complex64 1e-5, bf16 split 1e-4, the
tolerances of batched against single right-hand sides) and both match the
oracle.  The per-sweep launches give identical bits however they run: graph
replay on concurrent streams, eager launches on concurrent streams, and the
launches one by one on one stream (the per-front timing)."""
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps import capi  # noqa: E402
from lsweeps.problems import ProblemSpec  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("*.npz"))


def _load(f):
    d = np.load(f)
    N, m, p = (int(v) for v in d["Nmp"])
    spec = ProblemSpec(N=N, m=m, p=p, h=float(d["h"]), omega=float(d["omega"]))
    return spec, d


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("f", FIXTURES, ids=lambda p: p.stem)
@pytest.mark.parametrize("prec,tol,tol_oracle", [("c128", 1e-13, 1e-10), ("c64", 1e-5, 2e-4),
                                                 ("bf16x2", 1e-4, 2e-4)])
def test_per_sweep_launches_match_one_launch_per_step(f, prec, tol, tol_oracle, monkeypatch):
    from lsweeps.solver import Solver
    spec, d = _load(f)
    v = torch.from_numpy(d["v"]).cuda()
    monkeypatch.setenv("LSW_SWEEP_LANES", "0")
    S0 = Solver(spec, d["m_grid"], precision=prec)
    S0.factorize()
    y_step = S0.apply_precond(v).cpu().numpy()
    per_step, _ = S0.front_shapes(1)
    S0.close()
    monkeypatch.delenv("LSW_SWEEP_LANES")
    S = Solver(spec, d["m_grid"], precision=prec)
    S.factorize()
    shapes, _ = S.front_shapes(1)
    N = spec.N
    assert len(per_step) == 1 + (N - 1) + (2 * N - 3)
    assert len(shapes) == 1 + 4 * (N - 1) + 4 * (2 * N - 3)
    y_graph = S.apply_precond(v).cpu().numpy()          # captured
    y_replay = S.apply_precond(v).cpu().numpy()         # replayed
    capi.check(capi.lib().lsw_ctx_set_graphs(S.ctx, 0), S.ctx)
    y_eager = S.apply_precond(v).cpu().numpy()          # eager, concurrent streams
    y_prof, prof = S.apply_precond_profiled(v)          # one by one on one stream
    y_prof = y_prof.cpu().numpy()
    S.close()
    assert np.array_equal(y_replay, y_graph)
    assert np.array_equal(y_eager, y_graph)
    assert np.array_equal(y_prof, y_graph)
    assert prof["fronts"] == len(shapes)
    assert rel(y_graph, y_step) <= tol
    assert rel(y_graph, d["Mv"]) <= tol_oracle


def test_per_sweep_solve_matches_one_launch_per_step(monkeypatch):
    """FGMRES with per-sweep applies takes the iterations of one launch per
    step and reaches the same solution (complex64 factors)."""
    from lsweeps.solver import Solver
    spec, d = _load(FIXTURES[-1])
    b = torch.from_numpy(d["b"]).cuda()
    out = []
    for lanes in ("0", "1"):
        monkeypatch.setenv("LSW_SWEEP_LANES", lanes)
        S = Solver(spec, d["m_grid"], precision="c64")
        S.factorize()
        x, rep = S.gmres(b, mode="flexible", tol=1e-8, max_iter=100, restart=30)
        out.append((x.cpu().numpy(), rep))
        S.close()
    (x0, r0), (x1, r1) = out
    assert r0.converged and r1.converged and r1.true_rel_res <= 1e-8
    assert abs(r1.iterations - r0.iterations) <= 1
    assert rel(x1, x0) <= 1e-6


def test_per_sweep_schedule_is_tuned_as_a_whole(monkeypatch):
    """With tuning on, the first single-vector apply times one whole apply per
    assumed sharing of the GPU (2, 4, 8 launches) and keeps the fastest; a
    second context in the process reads the choice from the cache (measures
    nothing) and builds the same launches, and the tuned applies match the
    oracle.  (A cluster cap of 4 CTAs per cell solve gives this test a problem
    shape of its own in the process-wide cache.)"""
    from lsweeps.solver import Solver
    monkeypatch.setenv("LSW_MAX_CLUSTER", "4")
    spec, d = _load(FIXTURES[-1])
    v = torch.from_numpy(d["v"]).cuda()
    runs = []
    for _ in range(2):
        S = Solver(spec, d["m_grid"], precision="c64")
        S.factorize()
        shapes, tune_s = S.front_shapes(1)
        y = S.apply_precond(v).cpu().numpy()
        runs.append((shapes, tune_s, y))
        S.close()
    (sh1, t1, y1), (sh2, t2, y2) = runs
    assert t1 > 0.0 and t2 == 0.0
    key = lambda sh: [(f["items"], f["max_slots"], f["slots_cap"], f["cluster"]) for f in sh]
    assert key(sh1) == key(sh2)
    assert all(f["cluster"] <= 2 for f in sh1)      # 2 x cluster CTAs per cell solve, capped at 4
    assert np.array_equal(y1, y2)
    assert rel(y1, d["Mv"]) <= 2e-4
