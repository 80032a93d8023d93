"""Analytic formulas of the calibration products and SwaptionSimple's value units, host only."""
import math

import numpy as np
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


def _lmm_model(cfg):
    td = F.TimeDiscretizationFromArray(0.0, int(round(cfg["T_end"] / cfg["dt"])), cfg["dt"])
    tenor = F.TimeDiscretizationFromArray(0.0, int(round(cfg["tenor_end"] / cfg["period"])), cfg["period"])
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(
        td, tenor, F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *cfg["abcd"]),
        F.LIBORCorrelationModelExponentialDecay(td, tenor, cfg["F"], cfg["corr_decay"]))
    return F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                    cov)


def test_integrated_libor_covariance_matches_the_oracle_loadings():
    # getIntegratedLIBORCovariance (LIBORMarketModelFromCovarianceModel.java:1552-1596)
    from conftest import oracle_model
    cfg = W.LMM40
    model = _lmm_model(cfg)
    m = oracle_model(cfg)
    C = model.getIntegratedLIBORCovariance(model.covarianceModel.timeDiscretization)
    times, tenor = m.times, m.tenor
    acc = np.zeros((len(tenor) - 1, len(tenor) - 1))
    for t in (0, 7, 39, 79):
        acc[:] = 0.0
        for s in range(t + 1):
            alive = tenor[:-1] > times[s]
            lam = m.loadings[s] * alive[:, None]
            acc += (lam @ lam.T) * (times[s + 1] - times[s])
        upper = np.triu_indices(len(tenor) - 1)
        assert np.allclose(C[t][upper], acc[upper], rtol=1e-12, atol=1e-18)


def test_swaption_analytic_approximation():
    # SwaptionAnalyticApproximation (products/SwaptionAnalyticApproximation.java): on a flat curve
    # its log swap-rate derivatives are Rebonato's frozen weights, so it equals that formula
    from conftest import oracle_model
    from test_oracle_lmm import black_swaption_rebonato
    for cfg, cases, tol in ((W.LMM20, ((5.0, 10.0, 0.05), (2.0, 4.0, 0.045), (1.0, 9.5, 0.055)), 1e-12),
                            (W.LMM40, ((10.0, 20.0, 0.04), (2.0, 4.0, 0.035)), 5e-3)):
        model, m = _lmm_model(cfg), oracle_model(cfg)
        for ex, end, K in cases:
            fix = np.arange(ex, end - 1e-12, cfg["period"])
            tenor = list(fix) + [end]
            value = F.SwaptionAnalyticApproximation(K, tenor).getValue(model)
            assert value == pytest.approx(black_swaption_rebonato(m, ex, fix, fix + cfg["period"], K), rel=tol)
            var = F.SwaptionAnalyticApproximation(K, tenor, "INTEGRATEDVARIANCE").getValue(model)
            vol = F.SwaptionAnalyticApproximation(K, tenor, "VOLATILITY").getValue(model)
            assert vol == math.sqrt(var / ex)
            dc = F.DiscountCurveFromForwardCurve(model.forwardRateCurve)
            td = F.TimeDiscretizationFromArray(tenor)
            assert value == A.blackModelSwaptionValue(A.forward_swap_rate(td, model.forwardRateCurve, dc), vol, ex, K,
                                                      A.swap_annuity(td, dc))
    with pytest.raises(ValueError):
        F.SwaptionAnalyticApproximation(0.05, [1.0, 2.0], "VOLATILITYNORMAL")


def test_log_swaprate_derivative_equals_finite_differences():
    # SwaptionAnalyticApproximation.getLogSwaprateDerivative (products/SwaptionAnalyticApproximation.java:188-281)
    # gives d log S / d log L_j of the par swap rate S = float leg / annuity, the discount
    # factors chained from the forward rates; central differences of that S in log L_j,
    # rebuilt here from the rates alone, pin every weight independently of the formula
    for cfg, swapTenor in ((W.LMM40, np.arange(10.0, 20.0 + 1e-9, 0.5)), (W.LMM40, np.arange(2.0, 4.0 + 1e-9, 1.0)),
                           (W.LMM20, np.arange(5.0, 10.0 + 1e-9, 0.5))):
        model = _lmm_model(cfg)
        tenor = model.liborPeriodDiscretization
        w = F.SwaptionAnalyticApproximation(0.04, list(swapTenor)).getLogSwaprateDerivative(
            tenor, model.discountCurve, model.forwardRateCurve)["values"]
        start, end = tenor.getTimeIndex(swapTenor[0]), tenor.getTimeIndex(swapTenor[-1])
        L0 = np.array([model.forwardRateCurve.getForward(None, tenor.getTime(j)) for j in range(start, end)])
        dt = np.array([tenor.getTimeStep(j) for j in range(start, end)])
        pay = np.array([tenor.getTime(j + 1) for j in range(start, end)])

        def log_swaprate(L):
            df = np.cumprod(1.0 / (1.0 + L * dt))  # P(T_{j+1}) / P(T_start)
            floating = np.sum(L * dt * df)
            annuity = sum((swapTenor[k + 1] - swapTenor[k]) * df[np.searchsorted(pay, swapTenor[k + 1] - 1e-9)]
                          for k in range(len(swapTenor) - 1))
            return math.log(floating / annuity)

        h = 1e-6
        for j in range(end - start):
            up, dn = L0.copy(), L0.copy()
            up[j] *= math.exp(h)
            dn[j] *= math.exp(-h)
            fd = (log_swaprate(up) - log_swaprate(dn)) / (2 * h)
            assert w[j] == pytest.approx(fd, rel=1e-6, abs=1e-10)


def test_integrated_libor_covariance_rejects_times_before_the_covariance_grid():
    # AbstractLIBORCovarianceModel.getFactorLoading throws for a time before its grid; the
    # covariance grid here starts at 1.0 while the simulation grid starts at 0.0
    cfg = W.LMM20
    tenor = F.TimeDiscretizationFromArray(0.0, 20, 0.5)
    cov_td = F.TimeDiscretizationFromArray(1.0, 18, 0.5)
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(
        cov_td, tenor, F.LIBORVolatilityModelFourParameterExponentialForm(cov_td, tenor, *cfg["abcd"]),
        F.LIBORCorrelationModelExponentialDecay(cov_td, tenor, cfg["F"], cfg["corr_decay"]))
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     cov)
    with pytest.raises(ValueError):
        model.getIntegratedLIBORCovariance(F.TimeDiscretizationFromArray(0.0, 20, 0.5))
    assert model.getIntegratedLIBORCovariance(F.TimeDiscretizationFromArray(1.0, 18, 0.5)).shape == (18, 20, 20)
