"""The reference's own acceptance tests of the LIBOR Market Model, run on the GPU path.

LIBORMarketModelValuationTest (src/test/java/net/finmath/montecarlo/interestrate/
LIBORMarketModelValuationTest.java) builds one model (:89-161) and checks Monte Carlo values
against analytic ones with fixed tolerances.  The same model is built here through this
library's finmath-style API -- 40 semi-annual forwards on a flat 5 % curve, 0.5y Euler steps
to 20y, volatility (a, b, c, d) = (0.2, 0, 0.25, 0.3), exponential-decay correlation 0.1
reduced to 6 factors, spot measure, lognormal state space, the discount curve derived from
the forward curve, 20,000 paths of MersenneTwister seed 3141, PREDICTOR_CORRECTOR -- and
every check runs with the reference's own loops and tolerances:

  testBond        (:164-200)  zero bonds at maturities 0..20 step 0.125 (off-tenor
                              numeraires included) vs the discount curve, |dev| < 8e-3
  testFRA         (:203-257)  par FRAs starting 0..19.5 step 0.125, |value| < 2e-3
  testSwap        (:260-314)  par 10-period swaps starting 0..14.5, |value| < 2e-3
  testDigitalCaplet (:317-363) vs Black's digital caplet, |dev| < 5e-2
  testSwaption    (:366-428)  5-period swaptions vs SwaptionAnalyticApproximation, < 8e-3
  testCaplet      (:431-493)  one-period swaptions vs the same, < 8e-3
  testCapletSmile (:496-569)  Bachelier implied volatility across moneyness, < 5e-4
  testSwaptionSmile (:572-642) Black implied volatility across moneyness, < 1e-1
  testLIBORInArrearsConvexity (:645-681) the sign of the payment-delay convexity
  testSwaptionCalibration (:685-807) the 5-parameter covariance model calibrated to 36
                              analytic swaption volatilities, RMS < 0.025

The swaptions and caplets run on the fused swaption kernel; bonds, FRAs, swaps, digital
caplets and the convexity check run finmath's product code on device random variables.
"""
import math

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import analytic as A, calibration as C, rvproducts as RP

pytestmark = pytest.mark.gpu

PATHS, FACTORS, SEED = 20000, 6, 3141


def create_libor_market_model(paths=PATHS, factors=FACTORS, correlation_decay=0.1):
    """createLIBORMarketModel (LIBORMarketModelValuationTest.java:89-161)."""
    tenor = F.TimeDiscretizationFromArray(0.0, 40, 0.5)
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards(
        "forwardCurve", [0.5, 1.0, 2.0, 5.0, 40.0], [0.05, 0.05, 0.05, 0.05, 0.05], 0.5)
    td = F.TimeDiscretizationFromArray(0.0, 40, 0.5)
    vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, 0.2, 0.0, 0.25, 0.3, False)
    corr = F.LIBORCorrelationModelExponentialDecay(td, tenor, factors, correlation_decay)
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     cov, [], {"measure": "SPOT", "stateSpace": "LOGNORMAL"})
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, factors, paths, SEED)
    process = F.EulerSchemeFromProcessModel(model, bm, F.EulerSchemeFromProcessModel.PREDICTOR_CORRECTOR)
    return F.LIBORMonteCarloSimulationFromLIBORModel(process)


def par_swaprate(sim, swapTenor):
    """getParSwaprate (:810-812): Swap.getForwardSwapRate on the model's curves."""
    return A.forward_swap_rate(F.TimeDiscretizationFromArray(list(swapTenor)), sim.model.forwardRateCurve,
                               sim.model.discountCurve)


def swap_annuity(sim, swapTenor):
    """getSwapAnnuity (:814-816)."""
    return A.swap_annuity(F.TimeDiscretizationFromArray(list(swapTenor)), sim.model.discountCurve)


def java_range(start, stop, step, inclusive=True):
    """A Java for loop over doubles (x += step), accumulating its rounding the same way."""
    x = start
    while (x <= stop) if inclusive else (x < stop):
        yield x
        x += step


@pytest.fixture(scope="module")
def sim():
    s = create_libor_market_model()
    yield s
    s.process.close()
    s.process.brownianMotion.close()


def _periods(start, n, length=0.5):
    fixing = [start + k * length for k in range(n)]
    payment = [start + (k + 1) * length for k in range(n)]
    return fixing, payment, fixing + [payment[-1]]


def test_bond(sim):
    dc = sim.model.discountCurve
    dev = max(abs(RP.Bond(T).getValue(sim) - dc.getDiscountFactor(None, T)) for T in java_range(0.0, 20.0, 0.125))
    assert dev < 8e-3


def test_fra(sim):
    dev = 0.0
    for start in java_range(0.0, 20.0 - 0.5, 0.125):
        fixing, payment, tenor = _periods(start, 1)
        rate = par_swaprate(sim, tenor)
        dev = max(dev, abs(RP.SimpleSwap(fixing, payment, [rate]).getValue(sim)))
    assert dev < 2e-3


def test_swap(sim):
    dev = 0.0
    for start in java_range(0.0, 15.0, 0.5, inclusive=False):
        fixing, payment, tenor = _periods(start, 10)
        rate = par_swaprate(sim, tenor)
        dev = max(dev, abs(RP.SimpleSwap(fixing, payment, [rate] * 10).getValue(sim)))
    assert dev < 2e-3


def test_digital_caplet(sim):
    covariance = sim.model.getIntegratedLIBORCovariance(sim.getTimeDiscretization())
    dev = 0.0
    for T in java_range(1.0, 19.5, 0.5):
        start, end, strike = T, T + 0.5, 0.02
        value = RP.DigitalCaplet(T, start, end, strike).getValue(sim)
        forward = par_swaprate(sim, [start, end])
        periodLength = end - start
        discountFactor = swap_annuity(sim, [start, end]) / periodLength
        volatility = math.sqrt(covariance[sim.getTimeIndex(T)][sim.getLiborPeriodIndex(start)][
            sim.getLiborPeriodIndex(start)] / T)
        analytic = A.blackModelDigitalCapletValue(forward, volatility, periodLength, discountFactor, T, strike)
        dev = max(dev, abs(value - analytic))
    assert dev < 5e-2


@pytest.mark.parametrize("periods,last", [(5, 17.5), (1, 19.5)], ids=["testSwaption", "testCaplet"])
def test_swaption_and_caplet(sim, periods, last):
    dev = 0.0
    for ex in java_range(1.0, last, 0.5):
        fixing, payment, tenor = _periods(ex, periods)
        rate = par_swaprate(sim, tenor)
        mc = F.Swaption(ex, fixing, payment, [rate] * periods).getValue(sim)
        analytic = F.SwaptionAnalyticApproximation(rate, tenor, "VALUE").getValue(sim)
        dev = max(dev, abs(mc - analytic))
    assert dev < 8e-3


@pytest.mark.parametrize("periods,kind,tol", [(1, "bachelier", 5e-4), (10, "black", 1e-1)],
                         ids=["testCapletSmile", "testSwaptionSmile"])
def test_smiles(sim, periods, kind, tol):
    implied = A.bachelierOptionImpliedVolatility if kind == "bachelier" else A.blackScholesOptionImpliedVolatility
    ex = 5.0
    fixing, payment, tenor = _periods(ex, periods)
    par, annuity = par_swaprate(sim, tenor), swap_annuity(sim, tenor)
    dev = 0.0
    for moneyness in java_range(0.5, 2.0, 0.1, inclusive=False):
        rate = moneyness * par
        mc = F.Swaption(ex, fixing, payment, [rate] * periods).getValue(sim)
        analytic = F.SwaptionAnalyticApproximation(rate, tenor, "VALUE").getValue(sim)
        dev = max(dev, abs(implied(par, ex, rate, annuity, mc) - implied(par, ex, rate, annuity, analytic)))
    assert dev < tol


def test_libor_in_arrears_convexity(sim):
    fixing, periodStart, periodEnd = 5.0, 5.0, 5.5
    for payment in java_range(5.0, 20.0, 0.5, inclusive=False):
        libor = sim.getForwardRate(fixing, periodStart, periodEnd)
        N_pay, N_0 = sim.getNumeraireRandomVariable(payment), sim.getNumeraireRandomVariable(0.0)
        value = libor.div(N_pay).mult(N_0).getAverage()
        rate = value / N_0.div(N_pay).getAverage()
        N_end = sim.getNumeraireRandomVariable(periodEnd)
        forward = libor.div(N_end).mult(N_0).getAverage() / N_0.div(N_end).getAverage()
        if payment < periodEnd:
            assert rate > forward
        if payment > periodEnd:
            assert rate < forward


def calibration_products(sim):
    """The calibration set of testSwaptionCalibration (:690-740): swaptions at every fourth
    tenor index with every fourth length, analytic Black volatilities as products."""
    products = []
    N = sim.model.getNumberOfComponents()
    for exerciseIndex in range(4, N - 5 + 1, 4):
        ex = sim.getLiborPeriod(exerciseIndex)
        numberOfPeriods = 1
        while numberOfPeriods < N - exerciseIndex - 5:
            _, _, tenor = _periods(ex, numberOfPeriods)
            rate = par_swaprate(sim, tenor)
            target = 0.20 + 0.20 * math.exp(-ex / 10.0) + 0.20 * math.exp(-(ex + numberOfPeriods) / 10.0)
            products.append(C.CalibrationProduct(f"{ex}/{numberOfPeriods}", F.SwaptionAnalyticApproximation(
                rate, tenor, "VOLATILITYLOGNORMAL"), target, 1.0))
            numberOfPeriods += 4
    return products


def test_swaption_calibration(sim):
    products = calibration_products(sim)
    assert len(products) == 36
    td = sim.getTimeDiscretization()
    cov = F.LIBORCovarianceModelExponentialForm5Param(td, sim.model.liborPeriodDiscretization,
                                                      sim.getNumberOfFactors())
    properties = {"calibrationParameters": {"accuracy": 1e-6, "numberOfPaths": 20000}}
    calibrated = F.LIBORMarketModelFromCovarianceModel.of(sim.model.liborPeriodDiscretization, None,
                                                          sim.model.forwardRateCurve, None, None, cov, products,
                                                          properties)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, FACTORS, PATHS, SEED)
    process = F.EulerSchemeFromProcessModel(calibrated, bm)
    simulation = F.LIBORMonteCarloSimulationFromLIBORModel(process)
    deviations = [p.getProduct().getValue(simulation) - p.getTargetValue() for p in products]
    rms = math.sqrt(sum(d * d for d in deviations) / len(deviations))
    process.close()
    bm.close()
    assert rms == pytest.approx(0.0, abs=0.025)
