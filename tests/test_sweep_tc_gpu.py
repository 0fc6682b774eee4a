"""Complex64 sweep fronts with their line products on the tensor cores
(tcgen05.mma, bf16 x 3 terms, FP32 accumulation in tensor memory): the
opt-in launch variant (LSW_FRONT_SHAPE=RxCt, or LSW_SWEEP_TC=1 for the tuner)
agrees with the oracle at the complex64 tolerance (2e-4) and with the FMA
matvec of the same shape within 2e-5 on the fixtures, every front reports
the variant, and repeated applies are bit-identical."""
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps.problems import ProblemSpec  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("*.npz"))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _apply(monkeypatch, d, spec, shape):
    from lsweeps.solver import Solver
    monkeypatch.setenv("LSW_FRONT_SHAPE", shape)
    S = Solver(spec, d["m_grid"], precision="c64")
    try:
        S.factorize()
        v = torch.from_numpy(d["v"]).cuda()
        y = S.apply_precond(v).cpu().numpy()
        again = S.apply_precond(v).cpu().numpy()
        shapes, _ = S.front_shapes(1)
    finally:
        S.close()
    return y, again, shapes


@pytest.mark.parametrize("fixture", FIXTURES, ids=lambda f: f.stem)
@pytest.mark.parametrize("shape", ["8x1t", "16x2t"])
def test_tensor_core_fronts_match_oracle_and_fma(monkeypatch, fixture, shape):
    d = np.load(fixture)
    N, m, p = (int(x) for x in d["Nmp"])
    spec = ProblemSpec(N=N, m=m, p=p, h=float(d["h"]), omega=float(d["omega"]))
    y_fma, _, shapes_fma = _apply(monkeypatch, d, spec, shape[:-1])
    y_tc, again, shapes_tc = _apply(monkeypatch, d, spec, shape)
    assert all(f["tensor_cores"] == 0 for f in shapes_fma)
    assert all(f["tensor_cores"] == 1 for f in shapes_tc if f["items"] > 0)
    assert rel(y_tc, d["Mv"]) <= 2e-4
    assert rel(y_tc, y_fma) <= 2e-5
    assert np.array_equal(again, y_tc)
