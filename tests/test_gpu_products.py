"""GPU swaption and Bermudan swaption (regression) against the oracle."""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture(scope="module", params=[("lmm20", 5000), ("lmm40", 16384)])
def pair(request):
    name, P = request.param
    cfg = W.WORKLOADS[name]
    m = oracle_model(cfg)
    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    obs = np.zeros(m.T + 1, np.uint8)
    obs[W.tenor_time_indices(cfg)] = 1
    return cfg, po.Simulation(m, dW, observe=obs), W.build(cfg, paths=P)


def test_swaption(pair):
    cfg, osim, sim = pair
    ex, fix, pay, K = W.swaption_schedule(cfg)
    g = F.Swaption(ex, fix, pay, K).getValues(sim)
    v, e = osim.swaption(ex, fix, pay, K)
    assert g["value"] == pytest.approx(v, rel=REL)
    assert g["error"] == pytest.approx(e, rel=1e-10)


@pytest.mark.parametrize("basis", [None, "swaprate"])
def test_bermudan(pair, basis):
    cfg, osim, sim = pair
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    g = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, basis).getValues(sim, per_path=True)
    v, e, pp, _ = osim.bermudan(fix, plen, pay, K, basis_id=1 if basis else 0, per_path=True)
    assert g["value"] == pytest.approx(v, rel=REL)
    assert g["error"] == pytest.approx(e, rel=1e-10)
    assert np.max(np.abs(g["values"] - pp)) <= 1e-12 * np.max(np.abs(pp))


def test_bermudan_variants(pair):
    cfg, osim, sim = pair
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    n = len(fix)
    ex = np.zeros(n, np.uint8)
    ex[::3] = 1                                  # exercisable on every third period
    notional = np.linspace(1.0, 2.0, n)          # amortising notionals
    strikes = K + 0.001 * np.sin(np.arange(n))   # per-period strikes
    for callable_ in (True, False):
        g = F.BermudanSwaption(ex, fix, plen, pay, notional, strikes, callable_, "swaprate").getValues(sim)
        v, e = osim.bermudan(fix, plen, pay, strikes, exercisable=ex, notional=notional, callable_=callable_, basis_id=1)
        assert g["value"] == pytest.approx(v, rel=REL, abs=1e-15)


def test_swaption_strikes_and_partial_schedules(pair):
    cfg, osim, sim = pair
    ex, fix, pay, K = W.swaption_schedule(cfg)
    for k in (0.5 * K, K, 2 * K):
        g = F.Swaption(ex, fix[:3], pay[:3], k).getValue(sim)
        v, _ = osim.swaption(ex, fix[:3], pay[:3], k)
        assert g == pytest.approx(v, rel=REL, abs=1e-16)


def test_invalid_products_raise(pair):
    cfg, osim, sim = pair
    with pytest.raises(ValueError):
        F.Swaption(0.25, [0.25], [0.75], 0.05).getValue(sim)   # off the tenor grid
    with pytest.raises(ValueError):
        F.Swaption(0.0, [0.0], [0.5], 0.05).getValue(sim)      # deterministic first fixing
