"""Analytic formulas of the calibration products and SwaptionSimple's value units, host only."""
import math

import pytest

import finmath_gb300 as F
from finmath_gb300 import analytic as A, workloads as W
from oracle import pyoracle as po


def test_normal_distribution():
    for p in (1e-300, 1e-12, 0.02425, 0.1, 0.3, 0.5, 0.7, 0.97575, 1 - 1e-12):
        x = A.normal_inverse_cdf(p)
        assert x == pytest.approx(po.icdf(p), rel=4e-16, abs=1e-300)  # the oracle's Wichura AS241
    assert A.normal_inverse_cdf(0.0) == 0.0 and A.normal_inverse_cdf(1.0) == 0.0  # the reference's tail value
    for x in (-45.0, -8.0, -1.5, 0.0, 0.3, 2.0, 45.0):
        assert A.normal_cdf(x) == pytest.approx(0.5 * math.erfc(-x / math.sqrt(2.0)), rel=1e-15, abs=0.0)
    assert A.normal_cdf(-41.0) == 0.0 and A.normal_cdf(41.0) == 1.0


@pytest.mark.parametrize("fwd,K,T,vol", [(0.05, 0.05, 1.0, 0.2), (0.05, 0.04, 5.0, 0.15), (0.03, 0.06, 10.0, 0.3),
                                         (0.04, 0.039, 0.5, 0.5)])
def test_black_implied_volatility_round_trip(fwd, K, T, vol):
    annuity = 4.2
    v = A.blackScholesOptionValue(fwd, vol, T, K, annuity)
    assert A.blackScholesOptionImpliedVolatility(fwd, T, K, annuity, v) == pytest.approx(vol, rel=1e-10)
    assert A.blackScholesOptionImpliedVolatility(fwd, T, 0.0, annuity, v) == 0.0  # not an option


@pytest.mark.parametrize("fwd,K,T,vol", [(0.05, 0.05, 1.0, 0.01), (0.05, 0.04, 5.0, 0.008), (0.03, 0.06, 10.0, 0.012)])
def test_bachelier_implied_volatility_round_trip(fwd, K, T, vol):
    annuity = 3.7
    v = A.bachelierOptionValue(fwd, vol, T, K, annuity)
    assert A.bachelierOptionImpliedVolatility(fwd, T, K, annuity, v) == pytest.approx(vol, rel=1e-8)
    # at the money the value is vol sqrt(T / 2 pi) times the annuity
    assert A.bachelierOptionValue(fwd, vol, T, fwd, annuity) == vol * math.sqrt(T / math.pi / 2.0) * annuity


def test_par_swap_rate_and_annuity_on_a_flat_curve():
    f, d = 0.05, 0.5
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", [0.5, 40.0], [f, f], d)
    dc = F.DiscountCurveFromForwardCurve(curve)
    tenor = F.TimeDiscretizationFromArray(2.0, 6, 0.5)
    dfs = [(1 + f * d) ** (-t / d) for t in tenor.getAsDoubleArray()]
    assert [dc.getDiscountFactor(None, t) for t in tenor.getAsDoubleArray()] == pytest.approx(dfs, rel=1e-14)
    assert A.swap_annuity(tenor, dc) == pytest.approx(sum(0.5 * x for x in dfs[1:]), rel=1e-14)
    assert A.swap_annuity(tenor, dc, 2.0) == pytest.approx(sum(0.5 * x for x in dfs[1:]) / dfs[0], rel=1e-14)
    assert A.forward_swap_rate(tenor, curve, dc) == pytest.approx(f, rel=1e-14)  # the par rate of a flat curve


class _PricedSwaption:
    def __init__(self, value):
        self.value = value

    def getValue(self, model):
        return self.value


class _Model:
    def __init__(self, curve):
        self.model = type("M", (), {"forwardRateCurve": curve})()


def test_swaption_simple_value_units():
    # SwaptionSimple.java: the implied volatility of the kernel's price on the curve's par rate and annuity
    cfg = W.LMM20
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])
    dc = F.DiscountCurveFromForwardCurve(curve)
    tenor = F.TimeDiscretizationFromArray(5.0, 10, 0.5)
    par, annuity = A.forward_swap_rate(tenor, curve, dc), A.swap_annuity(tenor, dc)
    K, T = 0.052, 5.0
    model = _Model(curve)
    lognormal = F.SwaptionSimple(K, tenor, "VOLATILITYLOGNORMAL")
    lognormal.swaption = _PricedSwaption(A.blackScholesOptionValue(par, 0.18, T, K, annuity))
    assert lognormal.getValue(model) == pytest.approx(0.18, rel=1e-10)
    normal = F.SwaptionSimple(K, tenor.getAsDoubleArray(), "VOLATILITYNORMAL")
    normal.swaption = _PricedSwaption(A.bachelierOptionValue(par, 0.009, T, K, annuity))
    assert normal.getValue(model) == pytest.approx(0.009, rel=1e-8)
    variance = F.SwaptionSimple(K, tenor, "INTEGRATEDVARIANCELOGNORMAL")
    variance.swaption = lognormal.swaption
    assert variance.getValue(model) == pytest.approx(0.18 * 0.18 * T, rel=1e-9)
    plain = F.SwaptionSimple(K, tenor)
    assert plain.swaption.exerciseDate == 5.0 and list(plain.swaption.fixingDates) == list(tenor.getAsDoubleArray()[:-1])
    with pytest.raises(ValueError):
        F.SwaptionSimple(K, tenor, "PERCENT")
