"""finmath-lib products written against the RandomVariable API, valued on the GPU.

These are finmath's own valuation algorithms, operation for operation, over device random
variables (randomvariable.py): what the Java products do unchanged on a GPU
RandomVariableFactory.  Each operation is one streaming kernel; for the products of the
LMM hot path (Swaption, BermudanSwaption) the fused kernels of lmm.py are the fast path.
"""
from __future__ import annotations

import numpy as np

from .randomvariable import RandomVariableGPU


_NEG_INF = float("-inf")


def _weights(model) -> RandomVariableGPU:
    # getMonteCarloWeights: equal weights 1/P
    return RandomVariableGPU.constant(0.0, 1.0 / model.getNumberOfPaths())


def _constant(value) -> RandomVariableGPU:
    # getRandomVariableForConstant / Scalar: deterministic, measurable at -infinity
    return RandomVariableGPU.constant(_NEG_INF, value)


def _to_evaluation_time(values, evaluationTime, model) -> RandomVariableGPU:
    # the products' common tail: values.mult(N(evaluationTime)).div(weights(evaluationTime))
    return values.mult(model.getNumeraireRandomVariable(evaluationTime)).div(_weights(model))


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

    def getGradient(self, model, checkpointStride: int = 1):
        """Value (this product's own valuation), deltas d V / d L_j(0) and vegas
        d V / d sigma_{i,j} of the caplet by the adjoint kernel: the payoff's pathwise
        derivative (floor(0) differentiates to 1 where its argument is >= 0,
        RandomVariableDifferentiableAAD.java:324-331) through the fixing and the payment
        numeraire, swept back through the Euler scheme.  FP64 processes, caplets only."""
        import ctypes
        from . import _lib
        if self.isFloorlet:
            raise NotImplementedError("the adjoint covers caplets")
        proc = model.process
        T = len(proc._keep["times"]) - 1
        N = len(proc._keep["tenor"]) - 1
        deltas, vegas = np.empty(N), np.empty((T, N))
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        _lib.check(_lib.load().lmm_caplet_get_gradient(proc._h, self.maturity, self.periodLength, self.strike,
                                                        self.daycountFraction, int(checkpointStride), dp(deltas),
                                                        dp(vegas)), "Caplet.getGradient")
        return {"value": self.getValue(model), "deltas": deltas, "vegas": vegas}


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


class SimpleZeroSwap:
    """SimpleZeroSwap (montecarlo/interestrate/products/SimpleZeroSwap.java:94-130): SimpleSwap
    with a notional that compounds by swaprate * periodLength after every period, the LIBOR
    as the float index."""

    def __init__(self, fixingDates, paymentDates, swaprates, isPayFix=True):
        self.fixingDates = [float(x) for x in fixingDates]
        self.paymentDates = [float(x) for x in paymentDates]
        self.swaprates = [float(x) for x in swaprates]
        self.isPayFix = bool(isPayFix)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        values = _constant(0.0)
        notional = _constant(1.0)
        for fixingDate, paymentDate, swaprate in zip(self.fixingDates, self.paymentDates, self.swaprates):
            periodLength = paymentDate - fixingDate
            if paymentDate < evaluationTime:
                continue
            index = model.getForwardRate(fixingDate, fixingDate, paymentDate)
            payoff = index.sub(swaprate).mult(periodLength).mult(notional)
            if not self.isPayFix:
                payoff = payoff.mult(-1.0)
            payoff = payoff.div(model.getNumeraireRandomVariable(paymentDate)).mult(_weights(model))
            values = values.add(payoff)
            notional = notional.mult(swaprate * periodLength)
        return _to_evaluation_time(values, evaluationTime, model)

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


class Bond:
    """Zero-coupon bond (montecarlo/interestrate/products/Bond.java:58-88): 1 / N(T) * N(t),
    zero after maturity (model time offset 0: no reference date)."""

    def __init__(self, maturity):
        self.maturity = float(maturity)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        if evaluationTime > self.maturity:
            return _constant(0.0)
        values = _constant(1.0).div(model.getNumeraireRandomVariable(self.maturity)).mult(_weights(model))
        return _to_evaluation_time(values, evaluationTime, model)

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


class LIBORBond:
    """Bond valued from the forward rate (montecarlo/interestrate/products/LIBORBond.java:43-50):
    1 / (1 + L(t; t, T) (T - t)) at the evaluation time t, not discounted further."""

    def __init__(self, maturity):
        self.maturity = float(maturity)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        if evaluationTime > self.maturity:
            return _constant(0.0)
        return (model.getForwardRate(evaluationTime, evaluationTime, self.maturity)
                .mult(self.maturity - evaluationTime).add(1.0).invert())

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


class DigitalCaplet:
    """Digital caplet (montecarlo/interestrate/products/DigitalCaplet.java:58-85): pays the period
    length at periodEnd when L(optionMaturity; periodStart, periodEnd) - K >= 0 (choose on the
    trigger), discounted by the numeraire."""

    def __init__(self, optionMaturity, periodStart, periodEnd, strike):
        self.optionMaturity = float(optionMaturity)
        self.periodStart = float(periodStart)
        self.periodEnd = float(periodEnd)
        self.strike = float(strike)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        paymentDate = self.periodEnd
        periodLength = self.periodEnd - self.periodStart
        libor = model.getForwardRate(self.optionMaturity, self.periodStart, self.periodEnd)
        values = libor.sub(self.strike).choose(_constant(periodLength), _constant(0.0))
        values = values.div(model.getNumeraireRandomVariable(paymentDate)).mult(_weights(model))
        return _to_evaluation_time(values, evaluationTime, model)

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


class DigitalFloorlet:
    """Digital floorlet (montecarlo/interestrate/products/DigitalFloorlet.java:44-82): the period
    length where L(T; T, T_next) < K, else 0, on the tenor period that contains the maturity.
    The reference discards the results of its numeraire division and weighting (:77-78:
    RandomVariable is immutable), so its value is the undiscounted payoff with filtration
    time paymentDate; that behaviour is kept.  L < K is taken as L - K < 0 (equal for all
    non-NaN rates: a difference of distinct finite doubles is never zero)."""

    def __init__(self, maturity, strike):
        self.maturity = float(maturity)
        self.strike = float(strike)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        liborIndex = model.getLiborPeriodIndex(self.maturity)
        paymentDate = model.getLiborPeriod(liborIndex + 1)
        periodLength = paymentDate - self.maturity
        libor = model.getForwardRate(self.maturity, self.maturity, paymentDate)
        payoff = libor.sub(self.strike).choose(RandomVariableGPU.constant(paymentDate, 0.0),
                                               RandomVariableGPU.constant(paymentDate, periodLength))
        return payoff

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


class MoneyMarketAccount:
    """Money market account (montecarlo/interestrate/products/MoneyMarketAccount.java:70-94):
    initialValue accrued at the forward rate L(t; t, t + accrualPeriod) over accrual periods
    from the inception time to the evaluation time (the last period cut at the evaluation
    time); zero before inception, Double.MAX_VALUE for a non-positive accrual period."""

    def __init__(self, inceptionTime=0.0, initialValue=1.0, accrualPeriod=-1.0):
        self.inceptionTime = float(inceptionTime)
        self.initialValue = float(initialValue)
        self.accrualPeriod = float(accrualPeriod)

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        if self.inceptionTime > evaluationTime:
            return _constant(0.0)
        if self.accrualPeriod <= 0:
            return _constant(1.7976931348623157e308)
        value = _constant(self.initialValue)
        time = self.inceptionTime
        while time < evaluationTime:
            forwardRate = model.getForwardRate(time, time, time + self.accrualPeriod)
            value = value.accrue(forwardRate, min(self.accrualPeriod, evaluationTime - time))
            time += self.accrualPeriod
        return value

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()


# ----------------------------------------------------------------------------- schedule products
def _java_binary_search(a, key) -> int:
    # java.util.Arrays.binarySearch on a sorted double[]: the index, else -(insertion point) - 1
    import bisect
    i = bisect.bisect_left(a, key)
    return i if i < len(a) and a[i] == key else -i - 1


def _model_reference_date(model, fallback):
    ref = model.getReferenceDate() if hasattr(model, "getReferenceDate") else None
    return fallback if ref is None else ref


class SwaptionFromSwapSchedules:
    """European swaption on date schedules (montecarlo/interestrate/products/
    SwaptionFromSwapSchedules.java:67-170): both legs valued analytically at the exercise time
    from forward rates and forward discount bonds (getValueOfLegAnalytic, :184-218), the
    payer or receiver difference floored at zero and discounted by the numeraire at exercise.
    valueUnit VALUE; the implied-volatility units are not part of this path."""

    PAYER, RECEIVER = "PAYER", "RECEIVER"

    def __init__(self, referenceDate, swaptionType, exerciseDate, scheduleFixedLeg, scheduleFloatLeg, swaprate,
                 notional=1.0, valueUnit="VALUE"):
        from .schedule import _as_date
        if str(swaptionType).upper() not in (self.PAYER, self.RECEIVER):
            raise ValueError(f"Unkown swaptionType {swaptionType}")
        if str(valueUnit).upper() != "VALUE":
            raise ValueError(f"value unit {valueUnit} is not supported")
        self.referenceDate = None if referenceDate is None else _as_date(referenceDate)
        self.swaptionType = str(swaptionType).upper()
        self.exerciseDate = _as_date(exerciseDate)
        self.scheduleFixedLeg, self.scheduleFloatLeg = scheduleFixedLeg, scheduleFloatLeg
        self.swaprate, self.notional = float(swaprate), float(notional)

    @staticmethod
    def getValueOfLegAnalytic(evaluationTime, model, schedule, paysFloatingRate, fixRate, notional):
        """The time-t value of a leg: sum over periods, last to first, of the cash flow times
        P(t; payment) (getForwardDiscountBond), forward rates observed at t."""
        from .schedule import FloatingpointDate
        ref = _model_reference_date(model, schedule.getReferenceDate())
        value = _constant(0.0)
        for i in range(schedule.getNumberOfPeriods() - 1, -1, -1):
            period = schedule.getPeriod(i)
            paymentTime = FloatingpointDate.getFloatingPointDateFromDate(ref, period.getPayment())
            fixingTime = FloatingpointDate.getFloatingPointDateFromDate(ref, period.getFixing())
            periodLength = schedule.getPeriodLength(i)
            discountBond = model.getForwardDiscountBond(evaluationTime, paymentTime)
            if paysFloatingRate:
                libor = model.getForwardRate(evaluationTime, fixingTime, paymentTime)
                value = value.add(libor.mult(periodLength).mult(notional).mult(discountBond))
            if fixRate != 0:
                value = value.add(_constant(fixRate * periodLength * notional).mult(discountBond))
        return value

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        from .schedule import FloatingpointDate
        ref = _model_reference_date(model, self.referenceDate)
        exerciseTime = FloatingpointDate.getFloatingPointDateFromDate(ref, self.exerciseDate)
        fixLeg = self.getValueOfLegAnalytic(exerciseTime, model, self.scheduleFixedLeg, False, self.swaprate,
                                            self.notional)
        floatLeg = self.getValueOfLegAnalytic(exerciseTime, model, self.scheduleFloatLeg, True, 0.0, self.notional)
        values = floatLeg.sub(fixLeg) if self.swaptionType == self.PAYER else fixLeg.sub(floatLeg)
        values = values.floor(0.0)
        values = values.div(model.getNumeraireRandomVariable(exerciseTime)).mult(_weights(model))
        return _to_evaluation_time(values, evaluationTime, model)

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()

    def getProcessTimeDiscretization(self, referenceDate):
        """ProcessTimeDiscretizationProvider (SwaptionFromSwapSchedules.java:172-186): the
        exercise time and the payment times of both legs."""
        from .lmm import TimeDiscretizationFromArray
        from .schedule import FloatingpointDate
        f = lambda d: FloatingpointDate.getFloatingPointDateFromDate(referenceDate, d)
        times = {f(self.exerciseDate)}
        for s in (self.scheduleFixedLeg, self.scheduleFloatLeg):
            times.update(f(p.getPayment()) for p in s.getPeriods())
        return TimeDiscretizationFromArray(sorted(times))


class BermudanSwaptionFromSwapSchedules:
    """Bermudan swaption on date schedules (montecarlo/interestrate/products/
    BermudanSwaptionFromSwapSchedules.java:77-92 constructor, :191-254 getValues, :316-349
    the analytic underlying, :361-428 the basis): backward induction over the exercise dates;
    at each, the underlying swap of that date valued analytically at its first fixing and
    made numeraire-relative, the continuation estimated by MonteCarloConditionalExpectation-
    Regression on the product's own basis (constant, 1/N(t), the discounted swap rates of the
    remaining underlyings and their squares, the discounted short rate to the next date and
    its square), and the exercise taken where the estimate is negative.  Schedules are given
    explicitly (the reference's ScheduleGenerator constructors, with business-day calendars,
    are not part of this path)."""

    PAYER, RECEIVER = "PAYER", "RECEIVER"

    def __init__(self, referenceDate, swaptionType, exerciseDates, swapEndDate, swaprates, notionals, fixSchedules,
                 floatSchedules, conditionalExpectationRegressionFactory=None, regressionBasisFunctionProvider=None):
        from .schedule import _as_date
        if str(swaptionType).upper() not in (self.PAYER, self.RECEIVER):
            raise ValueError(f"Unkown swaptionType {swaptionType}")
        n = len(exerciseDates)
        if not (len(swaprates) == len(notionals) == len(fixSchedules) == len(floatSchedules) == n):
            raise ValueError("one swaprate, notional and pair of schedules per exercise date")
        self.referenceDate = None if referenceDate is None else _as_date(referenceDate)
        self.swaptionType = str(swaptionType).upper()
        self.exerciseDates = [_as_date(d) for d in exerciseDates]
        self.swapEndDate = _as_date(swapEndDate)
        self.swaprates = [float(x) for x in swaprates]
        self.notionals = [float(x) for x in notionals]
        self.fixSchedules, self.floatSchedules = list(fixSchedules), list(floatSchedules)
        self.regressionBasisFunctionProvider = regressionBasisFunctionProvider or self
        self.conditionalExpectationRegressionFactory = conditionalExpectationRegressionFactory

    def _reference_date(self, model):
        ref = model.getReferenceDate() if hasattr(model, "getReferenceDate") else None
        if ref is None:
            raise ValueError("the model needs a reference date (its forward curve's) for date schedules")
        return ref

    def _underlying(self, model, legSchedule, paysFloat, swaprate, notional):
        # getValueUnderlyingNumeraireRelative with isUseAnalyticSwapValuationAtExercise (:316-328)
        from .schedule import FloatingpointDate
        valuationTime = FloatingpointDate.getFloatingPointDateFromDate(self._reference_date(model),
                                                                        legSchedule.getPeriod(0).getFixing())
        value = SwaptionFromSwapSchedules.getValueOfLegAnalytic(valuationTime, model, legSchedule, paysFloat, swaprate,
                                                                notional)
        return value.div(model.getNumeraireRandomVariable(valuationTime)).mult(_weights(model))

    def getBasisFunctions(self, evaluationTime, model):
        """The product's own regression basis at an exercise time (:361-428)."""
        from .schedule import FloatingpointDate
        ref = self._reference_date(model)
        times = sorted([FloatingpointDate.getFloatingPointDateFromDate(ref, d) for d in self.exerciseDates]
                       + [FloatingpointDate.getFloatingPointDateFromDate(ref, self.swapEndDate)])
        exerciseTime = evaluationTime
        exerciseIndex = _java_binary_search(times, exerciseTime)
        if exerciseIndex < 0:
            exerciseIndex = -exerciseIndex  # as the reference: one past the insertion point
        if exerciseIndex >= len(self.exerciseDates):
            exerciseIndex = len(self.exerciseDates) - 1
        basis = [_constant(1.0)]
        discountFactor = model.getNumeraireRandomVariable(exerciseTime).invert()
        basis.append(discountFactor)
        for u in range(exerciseIndex, len(self.exerciseDates)):
            floatLeg = SwaptionFromSwapSchedules.getValueOfLegAnalytic(exerciseTime, model, self.floatSchedules[u], True,
                                                                       0.0, 1.0)
            annuity = SwaptionFromSwapSchedules.getValueOfLegAnalytic(exerciseTime, model, self.fixSchedules[u], False,
                                                                      1.0, 1.0)
            basisFunction = floatLeg.div(annuity).mult(discountFactor)
            basis.append(basisFunction)
            basis.append(basisFunction.squared())
        rateShort = model.getForwardRate(exerciseTime, exerciseTime, times[exerciseIndex + 1])
        basis.append(rateShort.mult(discountFactor))
        basis.append(rateShort.mult(discountFactor).pow(2.0))
        return basis

    def getValues(self, evaluationTime, model):
        from .randomvariable import MonteCarloConditionalExpectationRegression
        from .schedule import FloatingpointDate
        ref = self._reference_date(model)
        values = _constant(0.0)
        exerciseTimes = _constant(float("inf"))
        for k in range(len(self.exerciseDates) - 1, -1, -1):
            exerciseTime = FloatingpointDate.getFloatingPointDateFromDate(ref, self.exerciseDates[k])
            fixLeg = self._underlying(model, self.fixSchedules[k], False, self.swaprates[k], self.notionals[k])
            floatLeg = self._underlying(model, self.floatSchedules[k], True, 0.0, self.notionals[k])
            underlying = floatLeg.sub(fixLeg) if self.swaptionType == self.PAYER else fixLeg.sub(floatLeg)
            basis = self.regressionBasisFunctionProvider.getBasisFunctions(exerciseTime, model)
            factory = self.conditionalExpectationRegressionFactory or MonteCarloConditionalExpectationRegression
            estimator = factory(basis, basis)
            trigger = values.sub(underlying).getConditionalExpectation(estimator)
            values = trigger.choose(values, underlying)
            exerciseTimes = trigger.choose(exerciseTimes, _constant(exerciseTime))
        values = _to_evaluation_time(values, evaluationTime, model)
        return {"values": values, "exerciseTimes": exerciseTimes}

    def getValueRandomVariable(self, evaluationTime, model) -> RandomVariableGPU:
        return self.getValues(evaluationTime, model)["values"]

    def getValue(self, model, evaluationTime: float = 0.0) -> float:
        return self.getValueRandomVariable(evaluationTime, model).getAverage()

    def getProcessTimeDiscretization(self, referenceDate):
        """ProcessTimeDiscretizationProvider (BermudanSwaptionFromSwapSchedules.java:286-304): the
        exercise times and the payment times of every underlying's legs."""
        from .lmm import TimeDiscretizationFromArray
        from .schedule import FloatingpointDate
        f = lambda d: FloatingpointDate.getFloatingPointDateFromDate(referenceDate, d)
        times = set()
        for k, d in enumerate(self.exerciseDates):
            times.add(f(d))
            for s in (self.fixSchedules[k], self.floatSchedules[k]):
                times.update(f(p.getPayment()) for p in s.getPeriods())
        return TimeDiscretizationFromArray(sorted(times))

    def getExerciseProbabilitiesFromTimes(self, referenceDate, exerciseTimes):
        """:268-283: the probability of exercise at each date (after the previous ones) and,
        last, of no exercise, from the exerciseTimes random variable."""
        from .schedule import FloatingpointDate
        probabilities = []
        toExercise = 1.0
        for d in self.exerciseDates:
            t = FloatingpointDate.getFloatingPointDateFromDate(referenceDate, d)
            after = exerciseTimes.sub(t + 1.0 / 365.0).choose(_constant(1.0), _constant(0.0)).getAverage()
            probabilities.append(toExercise - after)
            toExercise = after
        probabilities.append(toExercise)
        return probabilities
