"""The graph-recorded portfolio batch: every product's value and Greeks equal the single-
product entry points on the same simulation; repeated launches reproduce them; device
completion times are reported per product."""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [F.PRECISION_FP64, F.PRECISION_MIXED])
def test_portfolio_equals_single_products(precision):
    cfg = W.LMM20
    sim = W.build(cfg, paths=5000, precision=precision)
    prods = W.portfolio_products(cfg, n=7, seed=11)
    assert any(b.periodNotionals[0] < 0 for b in prods) and any(b.periodNotionals[0] > 0 for b in prods)
    pf = F.Portfolio(sim, prods, withGreeks=True, checkpointStride=4, concurrency=3, adjointThreads=64)
    out = pf.run()
    for q, b in enumerate(prods):
        g = b.getGradient(sim, checkpointStride=4)
        assert out["values"][q] == pytest.approx(g["value"], rel=1e-12, abs=1e-16)
        assert out["errors"][q] == pytest.approx(g["error"], rel=1e-10, abs=1e-16)
        assert np.allclose(out["deltas"][q], g["deltas"], rtol=1e-12, atol=1e-15)
        assert np.allclose(out["vegas"][q], g["vegas"], rtol=1e-12, atol=1e-15)
    again = pf.run()
    assert np.array_equal(again["values"], out["values"])
    assert np.array_equal(again["vegas"], out["vegas"])
    lat = again["latency_ms"]
    assert np.all(lat > 0) and np.all(lat <= again["total_ms"] + 1e-9)
    pf.close()


def test_portfolio_values_only_and_reseed():
    cfg = W.LMM20
    sim = W.build(cfg, paths=3000)
    prods = W.portfolio_products(cfg, n=4, seed=5)
    pf = F.Portfolio(sim, prods, withGreeks=False, concurrency=2)
    first = pf.run()["values"]
    single = [b.getValue(sim) for b in prods]
    assert np.allclose(first, single, rtol=1e-12, atol=1e-16)
    sim.process.brownianMotion.setSeed(99)   # new increments: the graph re-reads the new simulation
    second = pf.run()["values"]
    assert np.allclose(second, [b.getValue(sim) for b in prods], rtol=1e-12, atol=1e-16)
    assert not np.allclose(first, second)
    pf.close()
