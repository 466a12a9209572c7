"""Serving loop: requests arriving while others run are admitted as the pool frees up,
their work overlaps on the device, and each result equals the same problem run alone."""
import numpy as np
import pytest

from kitgpu import abi, serve
from kitgpu.solver import GpuStep

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [abi.KG_PREC_MIXED, abi.KG_PREC_FP64])
def test_serve_results_equal_alone(prec):
    rng = np.random.default_rng(20261207)
    arrivals = serve.poisson_arrivals(rng, rate=200.0, n=6)
    reqs = [serve.random_request(rng, i, a, small=True) for i, a in enumerate(arrivals)]
    # a pool that holds only part of the requests at once, so admission must wait
    srv = serve.Server(precision=prec, pool_bytes=24 << 20, chunk=10, tol=1e-3, max_steps=60)
    stats = srv.run(reqs, keep_results=True)
    srv.close()
    s = stats.summary()
    assert len(stats.latencies) == len(reqs)
    assert s["p99_ms"] >= s["p50_ms"] > 0
    overlap = [(r.admitted, r.finished) for r in reqs]
    assert any(a2 < f1 for (a1, f1) in overlap for (a2, f2) in overlap if (a1, f1) != (a2, f2)), "no overlap"
    for r in reqs:
        prm = abi.make_params(r.problem, precision=prec, st_check_interval=10)
        g = GpuStep(prm, r.topo)
        g.upload_state(r.state["f"], r.state["w"], r.state["prim"])
        g.step(r.problem.dt(), 0, r.steps)
        alone = g.download_state()
        g.close()
        for key in ("f", "w", "prim"):
            assert np.array_equal(alone[key], r.result[key]), (r.rid, key)
