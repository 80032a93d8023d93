"""finmath-lib products written against the RandomVariable API, valued on the GPU.

These are finmath's own valuation algorithms, operation for operation, over device random
variables (randomvariable.py): what the Java products do unchanged on a GPU
RandomVariableFactory.  Each operation is one streaming kernel; for the products of the
LMM hot path (Swaption, BermudanSwaption) the fused kernels of lmm.py are the fast path.
"""
from __future__ import annotations

from .randomvariable import RandomVariableGPU


def _weights(model) -> RandomVariableGPU:
    # getMonteCarloWeights: equal weights 1/P
    return RandomVariableGPU.constant(0.0, 1.0 / model.getNumberOfPaths())


class Caplet:
    """Caplet / floorlet (montecarlo/interestrate/products/Caplet.java:60-141): pays
    max(L - K, 0) * daycountFraction (floorlet: -min(L - K, 0) * daycountFraction) at
    maturity + periodLength, L = getForwardRate(maturity, maturity, maturity + periodLength)."""

    def __init__(self, maturity, periodLength, strike, daycountFraction=None, isFloorlet=False):
        self.maturity = float(maturity)
        self.periodLength = float(periodLength)
        self.strike = float(strike)
        self.daycountFraction = self.periodLength if daycountFraction is None else float(daycountFraction)
        self.isFloorlet = bool(isFloorlet)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        paymentDate = self.maturity + self.periodLength
        values = model.getForwardRate(self.maturity, self.maturity, paymentDate)
        numeraire = model.getNumeraireRandomVariable(paymentDate)
        w = _weights(model)
        if not self.isFloorlet:
            values = values.sub(self.strike).floor(0.0).mult(self.daycountFraction)
        else:
            values = values.sub(self.strike).cap(0.0).mult(-1.0 * self.daycountFraction)
        values = values.div(numeraire).mult(w)
        values = values.mult(model.getNumeraireRandomVariable(evaluationTime)).div(_weights(model))
        return values

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


class SimpleSwap:
    """SimpleSwap (montecarlo/interestrate/products/SimpleSwap.java:39-170): the sum over
    periods of (L - swaprate) * periodLength * notional / N(payment), negated for a
    receiver (isPayFix false), skipping periods paid before the evaluation time."""

    def __init__(self, fixingDates, paymentDates, swaprates, isPayFix=True, notional=None):
        self.fixingDates = [float(x) for x in fixingDates]
        self.paymentDates = [float(x) for x in paymentDates]
        self.swaprates = [float(x) for x in swaprates]
        self.isPayFix = bool(isPayFix)
        self.notional = [1.0] * len(self.fixingDates) if notional is None else [float(x) for x in notional]

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        values = RandomVariableGPU.constant(0.0, 0.0)
        for period, (fixingDate, paymentDate) in enumerate(zip(self.fixingDates, self.paymentDates)):
            periodLength = paymentDate - fixingDate
            if paymentDate < evaluationTime:
                continue
            forwardRate = model.getForwardRate(fixingDate, fixingDate, paymentDate)
            payoff = forwardRate.sub(self.swaprates[period]).mult(periodLength).mult(self.notional[period])
            if not self.isPayFix:
                payoff = payoff.mult(-1.0)
            payoff = payoff.div(model.getNumeraireRandomVariable(paymentDate)).mult(_weights(model))
            values = values.add(payoff)
        return values.mult(model.getNumeraireRandomVariable(evaluationTime)).div(_weights(model))

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()
