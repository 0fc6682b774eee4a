"""Serving loop on the GPU: every request's solution in the mix (batched with
other requests of its operator, overlapping with other operators' batches,
factors reused from the cache) equals its solution alone, within the solve
tolerance: relative difference <= 1e-5 and true relative residual <= 1e-6."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from lsweeps.problems import small  # noqa: E402
from lsweeps.serving import GpuBackend, Medium, Request, ServeEngine  # noqa: E402

pytestmark = pytest.mark.gpu


def _requests():
    out = []
    rng = np.random.default_rng(7)
    problems = []
    for med_kind, seed in (("lens", 0), ("layered", 2)):
        spec, grid = small(N=3, m=12, p=5, medium=med_kind, seed=seed)
        problems.append((spec, Medium("array", (med_kind, seed), grid)))
    for i in range(10):
        spec, med = problems[i % 2]
        k = int(rng.integers(1, 4))
        srcs = [(float(rng.uniform(0.25, 0.75)) * spec.L, float(rng.uniform(0.25, 0.75)) * spec.L) for _ in range(k)]
        out.append(Request(rid=i, spec=spec, medium=med, sources=srcs, arrival=0.01 * i))
    return out


def _alone(req):
    from lsweeps.solver import Solver
    S = Solver(req.spec, req.medium.build(req.spec), precision="c64")
    S.factorize()
    b = S.assemble_rhs(req.sources)
    x, rep = S.gmres(b, mode="flexible", tol=1e-6, max_iter=200, restart=30)
    out = x.cpu().numpy()
    S.close()
    return out


def test_each_result_is_the_same_alone_and_in_the_mix():
    reqs = _requests()
    ref = {r.rid: _alone(r) for r in reqs}
    eng = ServeEngine(GpuBackend(0), slots=3, max_batch=4, budget=8 << 30)
    st = eng.run(reqs, realtime=False)
    assert st.failures == 0 and st.n == len(reqs), [(r.rid, r.batch_size, r.error) for r in reqs if r.error]
    assert st.factorisations == 2
    assert st.mean_batch > 1.0            # requests of one operator shared sweeps
    for r in reqs:
        d = np.linalg.norm(r.x - ref[r.rid]) / np.linalg.norm(ref[r.rid])
        assert d <= 1e-5, (r.rid, d)
        assert r.true_rel_res <= 1e-6, (r.rid, r.true_rel_res)
    # a second round, arriving over time, is served from the cached factors
    again = _requests()
    st2 = eng.run(again, realtime=True)
    assert st2.failures == 0, [(r.rid, r.error) for r in again if r.error]
    assert st2.factorisations == 0 and st2.cache_hits == len(again)
    for r in again:
        d = np.linalg.norm(r.x - ref[r.rid]) / np.linalg.norm(ref[r.rid])
        assert d <= 1e-5, (r.rid, d)
    eng.close()
