"""Sweep-front autotuner: the first apply of a batch size that runs one
launch per sweep step measures every launch shape (slots per item x CTAs per
half chain) on every front and keeps the fastest; the choice is cached per
GPU and problem shape in the process and, with LSW_TUNE_CACHE, in a file that
a later process reads back.

Shapes change only how the cells' right-hand sides are grouped into launches
and how a cell's columns are split over CTAs, so tuned and cost-model
schedules agree with each other and with the oracle within the parity
tolerances (complex128 1e-10, complex64 and bf16 split 2e-4)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps.problems import ProblemSpec  # noqa: E402

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("*.npz"))


def _load(f):
    d = np.load(f)
    N, m, p = (int(v) for v in d["Nmp"])
    spec = ProblemSpec(N=N, m=m, p=p, h=float(d["h"]), omega=float(d["omega"]))
    spec.sources = [tuple(s) for s in d["sources"]]
    return spec, d


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c64", 2e-4), ("bf16x2", 2e-4)])
def test_tuned_schedule_matches_model_and_oracle(prec, tol, monkeypatch):
    from lsweeps.solver import Solver
    # single vectors run one launch per step here: per-sweep launches (the
    # default for one right-hand side) take their shapes from the cost model
    monkeypatch.setenv("LSW_SWEEP_LANES", "0")
    spec, d = _load(FIXTURES[-1])
    v = torch.from_numpy(d["v"]).cuda()
    S0 = Solver(spec, d["m_grid"], precision=prec)
    S0.set_tuning(False)
    S0.factorize()
    y0 = S0.apply_precond(v).cpu().numpy()
    model, _ = S0.front_shapes(1)
    assert all(f["tuned_ms"] < 0 for f in model)
    S0.close()
    S1 = Solver(spec, d["m_grid"], precision=prec)
    S1.set_tuning(True)
    S1.factorize()
    y1 = S1.apply_precond(v).cpu().numpy()
    tuned, _ = S1.front_shapes(1)
    assert len(tuned) == len(model)
    # every front with work was measured, and its shape is one of the candidates
    for f in tuned:
        if f["items"] > 0:
            assert f["tuned_ms"] > 0
            assert f["slots_cap"] in (4, 8, 16) and f["cluster"] in (1, 2, 4)
    assert rel(y1, y0) <= (1e-12 if prec == "c128" else tol)
    assert rel(y1, d["Mv"]) <= tol
    # repeated applies with the tuned schedule are bit-identical
    assert np.array_equal(S1.apply_precond(v).cpu().numpy(), y1)
    S1.close()


def test_tuning_is_cached_in_the_process():
    from lsweeps.solver import Solver
    spec, d = _load(FIXTURES[0])
    S1 = Solver(spec, d["m_grid"], precision="c64")
    S1.factorize()
    shapes1, t1 = S1.front_shapes(2)
    S1.close()
    S2 = Solver(spec, d["m_grid"], precision="c64")
    S2.factorize()
    shapes2, t2 = S2.front_shapes(2)
    S2.close()
    assert t2 == 0.0             # the second context measured nothing
    assert shapes2 == shapes1


_CHILD = r"""
import json, sys
sys.path[:0] = [{root!r}, {pkg!r}]
import numpy as np
from lsweeps.problems import ProblemSpec
from lsweeps.solver import Solver
d = np.load({fixture!r})
N, m, p = (int(v) for v in d["Nmp"])
spec = ProblemSpec(N=N, m=m, p=p, h=float(d["h"]), omega=float(d["omega"]))
S = Solver(spec, d["m_grid"], precision="bf16x2")
S.factorize()
shapes, t = S.front_shapes(3)
print(json.dumps({{"shapes": shapes, "tune_s": t}}))
"""


def test_tuning_file_cache_is_read_by_a_later_process(tmp_path):
    cache = tmp_path / "front_shapes.txt"
    env = dict(os.environ, LSW_TUNE_CACHE=str(cache))
    code = _CHILD.format(root=str(ROOT), pkg=str(ROOT / "l-sweeps-2d_gb300"), fixture=str(FIXTURES[1]))
    out = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        out.append(json.loads(r.stdout.strip().splitlines()[-1]))
    assert cache.exists() and len(cache.read_text().strip().splitlines()) == 1
    assert out[0]["tune_s"] > 0.0
    assert out[1]["tune_s"] == 0.0
    key = lambda sh: [(f["items"], f["max_slots"], f["slots_cap"], f["cluster"]) for f in sh]
    assert key(out[1]["shapes"]) == key(out[0]["shapes"])
    assert np.allclose([f["tuned_ms"] for f in out[1]["shapes"]], [f["tuned_ms"] for f in out[0]["shapes"]],
                       rtol=1e-6)
