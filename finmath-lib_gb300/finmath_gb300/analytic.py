"""Analytic formulas the calibration products use (host arithmetic, no GPU).

Restated from finmath-lib: the normal distribution (functions/NormalDistribution.java; the
CDF is commons-math's 0.5 erfc(-x / sqrt 2) with its +-40 cut-offs, the inverse Wichura's
AS241, which Python's statistics.NormalDist also implements), Newton's method
(rootfinder/NewtonsMethod.java), the Black implied volatility (functions/AnalyticFormulas.
java:667-716), the Bachelier value and implied volatility (functions/BachelierModel.java:
67-90, 150-179, the latter by golden-section search on the squared error), and the single-
curve swap annuity and par swap rate (marketdata/products/SwapAnnuity.java:83-117,
marketdata/products/Swap.java:146-175) on a forward curve and the discount curve derived
from it.
"""
from __future__ import annotations

import math
import statistics

_STD = statistics.NormalDist()


def normal_cdf(x: float) -> float:
    if x < -40.0:
        return 0.0
    if x > 40.0:
        return 1.0
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


def normal_density(x: float) -> float:
    return math.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def normal_inverse_cdf(p: float) -> float:
    # inverseCumulativeNormalDistributionWichura (functions/NormalDistribution.java:67-162):
    # AS241; outside (0, 1) the reference's tail branch returns 0 (:141-142)
    if p <= 0.0 or p >= 1.0:
        return 0.0
    return _STD.inv_cdf(p)


class NewtonsMethod:
    """Newton iteration remembering the point of smallest |value| seen."""

    def __init__(self, guess: float):
        self.nextPoint = self.bestPoint = float(guess)
        self.accuracy = 1.7976931348623157e308
        self.numberOfIterations = 0

    def setValueAndDerivative(self, value: float, derivative: float):
        if abs(value) < self.accuracy:
            self.accuracy, self.bestPoint = abs(value), self.nextPoint
        self.nextPoint -= value / derivative
        self.numberOfIterations += 1


def blackScholesOptionImpliedVolatility(forward, optionMaturity, optionStrike, payoffUnit, optionValue) -> float:
    """The lognormal volatility that reprices optionValue: Newton from the midpoint of
    analytic bounds, at most 500 steps, to |error| <= 1e-15; 0 for a non-positive strike."""
    maxIterations, maxAccuracy = 500, 1e-15
    if optionStrike <= 0.0:
        return 0.0
    p = normal_inverse_cdf((optionValue / payoffUnit + optionStrike) / (forward + optionStrike)) / math.sqrt(optionMaturity)
    q = 2.0 * abs(math.log(forward / optionStrike)) / optionMaturity
    lower = p + math.sqrt(max(p * p - q, 0.0))
    upper = p + math.sqrt(p * p + q)
    if abs(lower - upper) < maxAccuracy:
        return (lower + upper) / 2.0
    solver = NewtonsMethod(0.5 * (lower + upper))
    sqrtT = math.sqrt(optionMaturity)
    while solver.accuracy > maxAccuracy and solver.numberOfIterations < maxIterations:
        vol = solver.nextPoint
        dPlus = (math.log(forward / optionStrike) + 0.5 * vol * vol * optionMaturity) / (vol * sqrtT)
        dMinus = dPlus - vol * sqrtT
        value = (forward * normal_cdf(dPlus) - optionStrike * normal_cdf(dMinus)) * payoffUnit
        derivative = forward * sqrtT * math.exp(-0.5 * dPlus * dPlus) / math.sqrt(2.0 * math.pi) * payoffUnit
        solver.setValueAndDerivative(value - optionValue, derivative)
    return solver.bestPoint


def blackScholesGeneralizedOptionValue(forward, volatility, optionMaturity, optionStrike, payoffUnit) -> float:
    """The Black value of a call on the forward (functions/AnalyticFormulas.java:54-78): a
    negative forward by put-call parity, the intrinsic value when the forward, strike,
    volatility or maturity leaves nothing to integrate."""
    if optionMaturity < 0:
        return 0.0
    if forward < 0:
        return ((forward - optionStrike) * payoffUnit
                + blackScholesGeneralizedOptionValue(-forward, volatility, optionMaturity, -optionStrike, payoffUnit))
    if forward == 0 or optionStrike <= 0.0 or volatility <= 0.0 or optionMaturity <= 0.0:
        return max(forward - optionStrike, 0.0) * payoffUnit
    dPlus = ((math.log(forward / optionStrike) + 0.5 * volatility * volatility * optionMaturity)
             / (volatility * math.sqrt(optionMaturity)))
    dMinus = dPlus - volatility * math.sqrt(optionMaturity)
    return (forward * normal_cdf(dPlus) - optionStrike * normal_cdf(dMinus)) * payoffUnit


blackScholesOptionValue = blackScholesGeneralizedOptionValue
blackModelSwaptionValue = blackScholesGeneralizedOptionValue  # AnalyticFormulas.java:985-993


def blackScholesDigitalOptionValue(initialStockValue, riskFreeRate, volatility, optionMaturity, optionStrike) -> float:
    """The value of a digital call under Black-Scholes (functions/AnalyticFormulas.java:728-750):
    exp(-r T) N(d-), and 1 for a non-positive strike."""
    if optionStrike <= 0.0:
        return 1.0
    dPlus = ((math.log(initialStockValue / optionStrike) + (riskFreeRate + 0.5 * volatility * volatility) * optionMaturity)
             / (volatility * math.sqrt(optionMaturity)))
    dMinus = dPlus - volatility * math.sqrt(optionMaturity)
    return math.exp(-riskFreeRate * optionMaturity) * normal_cdf(dMinus)


def blackModelDigitalCapletValue(forward, volatility, periodLength, discountFactor, optionMaturity,
                                 optionStrike) -> float:
    """A digital caplet under Black'76 (functions/AnalyticFormulas.java:916-926): the digital
    option on the forward with zero rate, times the period length and the discount factor."""
    return (blackScholesDigitalOptionValue(forward, 0.0, volatility, optionMaturity, optionStrike) * periodLength
            * discountFactor)


def bachelierOptionValue(forward, volatility, optionMaturity, optionStrike, payoffUnit) -> float:
    if optionMaturity < 0:
        return 0.0
    if forward == optionStrike:
        return volatility * math.sqrt(optionMaturity / math.pi / 2.0) * payoffUnit
    s = volatility * math.sqrt(optionMaturity)
    d = (forward - optionStrike) / s
    return ((forward - optionStrike) * normal_cdf(d) + s * normal_density(d)) * payoffUnit


def bachelierOptionImpliedVolatility(forward, optionMaturity, optionStrike, payoffUnit, optionValue) -> float:
    """The normal volatility that reprices optionValue: golden-section search of the squared
    error on [0, sqrt(2 pi e) (value / unit + |F - K|) / sqrt(T)], 100 evaluations."""
    a = 0.0
    b = math.sqrt(2 * math.pi * math.e) * (optionValue / payoffUnit + abs(forward - optionStrike)) / math.sqrt(optionMaturity)
    g = (math.sqrt(5.0) - 1.0) / 2.0
    err = lambda v: (bachelierOptionValue(forward, v, optionMaturity, optionStrike, payoffUnit) - optionValue) ** 2
    x1, x2 = b - g * (b - a), a + g * (b - a)
    f1, f2 = err(x1), err(x2)
    best, fbest = (x1, f1) if f1 <= f2 else (x2, f2)
    for _ in range(98):
        if f1 <= f2:
            b, x2, f2 = x2, x1, f1
            x1 = b - g * (b - a)
            f1 = err(x1)
        else:
            a, x1, f1 = x1, x2, f2
            x2 = a + g * (b - a)
            f2 = err(x2)
        for x, f in ((x1, f1), (x2, f2)):
            if f < fbest:
                best, fbest = x, f
    return best


def swap_annuity(tenor, discountCurve, evaluationTime: float = 0.0) -> float:
    """SwapAnnuity.getSwapAnnuity on the regular schedule of a tenor: the sum over periods paid
    after evaluationTime of periodLength * df(payment), divided by df(evaluationTime)."""
    value = 0.0
    for i in range(tenor.getNumberOfTimeSteps()):
        payment = tenor.getTime(i + 1)
        if payment <= evaluationTime:
            continue
        value += tenor.getTimeStep(i) * discountCurve.getDiscountFactor(None, payment)
    return value / discountCurve.getDiscountFactor(None, evaluationTime)


def forward_swap_rate(tenor, forwardCurve, discountCurve) -> float:
    """Swap.getForwardSwapRate on the regular schedule of a tenor (both legs), valued at the
    first fixing."""
    evaluationTime = tenor.getTime(0)
    annuity = swap_annuity(tenor, discountCurve, evaluationTime)
    floatLeg = 0.0
    for i in range(tenor.getNumberOfTimeSteps()):
        fixing, payment = tenor.getTime(i), tenor.getTime(i + 1)
        forward = forwardCurve.getForward(None, fixing, payment - fixing)
        floatLeg += forward * tenor.getTimeStep(i) * discountCurve.getDiscountFactor(None, payment)
    return floatLeg / discountCurve.getDiscountFactor(None, evaluationTime) / annuity
