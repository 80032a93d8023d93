"""Date schedules for the schedule-based products (net.finmath.time).

Period, ScheduleFromPeriods, the ACT/365 and ACT/360 day counts and FloatingpointDate's
date-to-time conversion, as the reference defines them, on Python dates.  Host-only: a
schedule becomes fixing, payment and period-length doubles before any valuation.
"""
from __future__ import annotations

import datetime as _dt


def _as_date(d) -> _dt.date:
    if isinstance(d, _dt.datetime):
        if d.time() != _dt.time(0, 0):
            raise ValueError("only dates at the start of the day are supported")
        return d.date()
    if isinstance(d, _dt.date):
        return d
    raise TypeError("a datetime.date is required")


def _days_between(start, end) -> float:
    # DayCountConvention_ACT.daysBetween (time/daycount/DayCountConvention_ACT.java:54-56)
    return float(_as_date(end).toordinal() - _as_date(start).toordinal())


class DayCountConvention_ACT_365:
    """ACT/365 (time/daycount/DayCountConvention_ACT_365.java:42-50): days / 365."""

    def getDaycount(self, startDate, endDate) -> float:
        return _days_between(startDate, endDate)

    def getDaycountFraction(self, startDate, endDate) -> float:
        if _as_date(startDate) > _as_date(endDate):
            return -self.getDaycountFraction(endDate, startDate)
        return self.getDaycount(startDate, endDate) / 365.0


class DayCountConvention_ACT_360(DayCountConvention_ACT_365):
    """ACT/360 (time/daycount/DayCountConvention_ACT_360.java:45-53): days / 360."""

    def getDaycountFraction(self, startDate, endDate) -> float:
        if _as_date(startDate) > _as_date(endDate):
            return -self.getDaycountFraction(endDate, startDate)
        return self.getDaycount(startDate, endDate) / 360.0


class FloatingpointDate:
    """time/FloatingpointDate.java:83-116: a date as a double, its ACT/365 year fraction from a
    reference date (the LocalDateTime form, seconds / (365 * 86400), gives the same doubles
    for dates at the start of the day)."""

    _internal = DayCountConvention_ACT_365()

    @staticmethod
    def getFloatingPointDateFromDate(referenceDate, date) -> float:
        return FloatingpointDate._internal.getDaycountFraction(referenceDate, date)


class Period:
    """time/Period.java:36-59: fixing, payment, period start and period end dates."""

    def __init__(self, fixing, payment, periodStart, periodEnd):
        self._fixing, self._payment = _as_date(fixing), _as_date(payment)
        self._start, self._end = _as_date(periodStart), _as_date(periodEnd)

    def getFixing(self):
        return self._fixing

    def getPayment(self):
        return self._payment

    def getPeriodStart(self):
        return self._start

    def getPeriodEnd(self):
        return self._end


class ScheduleFromPeriods:
    """time/ScheduleFromPeriods.java:45-147: periods with their dates as doubles relative to the
    reference date (FloatingpointDate) and period lengths by the day count convention."""

    def __init__(self, referenceDate, periods, daycountconvention):
        if referenceDate is None:
            raise ValueError("referenceDate must not be null.")
        self.referenceDate = _as_date(referenceDate)
        self.periods = list(periods)
        self.daycountconvention = daycountconvention
        f = lambda d: FloatingpointDate.getFloatingPointDateFromDate(self.referenceDate, d)
        self._fixing = [f(p.getFixing()) for p in self.periods]
        self._payment = [f(p.getPayment()) for p in self.periods]
        self._start = [f(p.getPeriodStart()) for p in self.periods]
        self._end = [f(p.getPeriodEnd()) for p in self.periods]
        self._length = [daycountconvention.getDaycountFraction(p.getPeriodStart(), p.getPeriodEnd())
                        for p in self.periods]

    def getReferenceDate(self):
        return self.referenceDate

    def getPeriods(self):
        return list(self.periods)

    def getDaycountconvention(self):
        return self.daycountconvention

    def getNumberOfPeriods(self) -> int:
        return len(self.periods)

    def getPeriod(self, periodIndex) -> Period:
        return self.periods[periodIndex]

    def getFixing(self, periodIndex) -> float:
        return self._fixing[periodIndex]

    def getPayment(self, periodIndex) -> float:
        return self._payment[periodIndex]

    def getPeriodStart(self, periodIndex) -> float:
        return self._start[periodIndex]

    def getPeriodEnd(self, periodIndex) -> float:
        return self._end[periodIndex]

    def getPeriodLength(self, periodIndex) -> float:
        return self._length[periodIndex]

    def getPeriodIndex(self, time) -> int:
        if isinstance(time, _dt.date):
            time = FloatingpointDate.getFloatingPointDateFromDate(self.referenceDate, time)
        if time < self.getPeriodStart(0) or time >= self.getPeriodEnd(self.getNumberOfPeriods() - 1):
            raise ValueError("Time point not included")
        for i in range(self.getNumberOfPeriods() - 1):
            if time <= self.getPeriodEnd(i):
                return i
        return self.getNumberOfPeriods() - 1
