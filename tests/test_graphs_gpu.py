"""CUDA-graph replay of the preconditioner apply, and determinism.

The apply's launches (pool clears, every sweep front, the sum of the four
shifted outputs) are captured once per batch size and replayed; the kernels
read the input and output addresses from a device-side table, so the replay
and the one-by-one launches run the same kernels on the same data.  The
sweep outputs are deterministic (every output value and trace line has one
writer per front), so the two agree bit for bit, repeated applies agree bit
for bit, and so do repeated solves.  A batch of another size reallocates the
sweep pools; the graphs captured against the old pools are captured again."""
import ctypes as C
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
    spec.sources = [tuple(s) for s in d["sources"]]
    return spec, d


def _graphs(S, on):
    capi.check(capi.lib().lsw_ctx_set_graphs(S.ctx, 1 if on else 0), S.ctx)


@pytest.mark.parametrize("prec", ["c128", "c64", "bf16x2"])
def test_graph_replay_equals_eager_bitwise(prec):
    from lsweeps.solver import Solver
    spec, d = _load(FIXTURES[-1])
    S = Solver(spec, d["m_grid"], precision=prec)
    S.factorize()
    rng = np.random.default_rng(31)
    V = torch.from_numpy(rng.standard_normal((3, S.n2)) + 1j * rng.standard_normal((3, S.n2))).cuda()
    v = V[0].contiguous()
    _graphs(S, False)
    y_eager = S.apply_precond(v).cpu().numpy()
    Y3_eager = S.apply_precond(V.reshape(-1)).cpu().numpy()
    _graphs(S, True)
    y_g1 = S.apply_precond(v).cpu().numpy()          # captured
    y_g2 = S.apply_precond(v).cpu().numpy()          # replayed
    assert np.array_equal(y_g1, y_eager) and np.array_equal(y_g2, y_eager)
    Y3 = S.apply_precond(V.reshape(-1)).cpu().numpy()   # a larger batch: pools reallocated
    assert np.array_equal(Y3, Y3_eager)
    y_g3 = S.apply_precond(v).cpu().numpy()          # the batch-1 graph is captured again
    assert np.array_equal(y_g3, y_eager)
    S.release_workspace()                            # pools released: captured again
    y_g4 = S.apply_precond(v).cpu().numpy()
    assert np.array_equal(y_g4, y_eager)
    # a different output buffer and input: the address table follows
    out = torch.empty_like(v)
    w = V[1].contiguous()
    _graphs(S, False)
    yw_eager = S.apply_precond(w).cpu().numpy()
    _graphs(S, True)
    S.apply_precond(w, out=out)
    assert np.array_equal(out.cpu().numpy(), yw_eager)
    S.close()


@pytest.mark.parametrize("prec", ["c128", "c64", "bf16x2"])
def test_repeated_solves_are_bitwise_identical(prec):
    from lsweeps.solver import Solver
    spec, d = _load(FIXTURES[0])
    S = Solver(spec, d["m_grid"], precision=prec)
    S.factorize()
    b = S.assemble_rhs(spec.sources)
    x1, r1 = S.gmres(b, mode="flexible", tol=1e-8, max_iter=100, restart=30)
    x1 = x1.cpu().numpy()
    x2, r2 = S.gmres(b, mode="flexible", tol=1e-8, max_iter=100, restart=30)
    assert r1.iterations == r2.iterations
    assert np.array_equal(x1, x2.cpu().numpy())
    S.close()
