"""Date schedules and day counts of the schedule products (net.finmath.time), host only."""
import datetime as dt

import pytest

import finmath_gb300 as F
from finmath_gb300.rvproducts import _java_binary_search


def test_day_counts_and_floating_point_dates():
    a, b = dt.date(2026, 1, 5), dt.date(2028, 1, 5)  # 730 days across a leap day
    act365, act360 = F.DayCountConvention_ACT_365(), F.DayCountConvention_ACT_360()
    assert act365.getDaycount(a, b) == 730.0
    assert act365.getDaycountFraction(a, b) == 730 / 365.0 and act360.getDaycountFraction(a, b) == 730 / 360.0
    assert act365.getDaycountFraction(b, a) == -(730 / 365.0)  # reversed dates: negative fraction
    assert F.FloatingpointDate.getFloatingPointDateFromDate(a, b) == 730 / 365.0
    # a LocalDateTime at the start of the day is the same date; other times of day are not part of this path
    assert F.FloatingpointDate.getFloatingPointDateFromDate(dt.datetime(2026, 1, 5), b) == 730 / 365.0
    with pytest.raises(ValueError):
        F.FloatingpointDate.getFloatingPointDateFromDate(dt.datetime(2026, 1, 5, 12), b)


def test_schedule_from_periods():
    ref = dt.date(2026, 1, 5)
    d = [dt.date(2026, 1, 5), dt.date(2026, 7, 6), dt.date(2027, 1, 5)]
    periods = [F.Period(d[i] - dt.timedelta(days=2), d[i + 1], d[i], d[i + 1]) for i in range(2)]
    s = F.ScheduleFromPeriods(ref, periods, F.DayCountConvention_ACT_360())
    assert s.getNumberOfPeriods() == 2 and s.getReferenceDate() == ref
    assert s.getFixing(0) == -2 / 365.0 and s.getPeriodStart(0) == 0.0  # fixing two days before the start
    assert s.getPayment(1) == 365 / 365.0 and s.getPeriodEnd(0) == 182 / 365.0
    assert s.getPeriodLength(0) == 182 / 360.0 and s.getPeriodLength(1) == 183 / 360.0
    assert s.getPeriod(1).getPeriodStart() == d[1]
    # getPeriodIndex (ScheduleFromPeriods.java:130-147): the first period whose end is at or after t
    assert s.getPeriodIndex(0.0) == 0 and s.getPeriodIndex(182 / 365.0) == 0 and s.getPeriodIndex(0.6) == 1
    assert s.getPeriodIndex(dt.date(2026, 9, 1)) == 1
    for t in (-0.01, 1.0):
        with pytest.raises(ValueError):
            s.getPeriodIndex(t)
    with pytest.raises(ValueError):
        F.ScheduleFromPeriods(None, periods, F.DayCountConvention_ACT_365())


def test_java_binary_search_semantics():
    a = [0.5, 1.0, 2.0]
    assert _java_binary_search(a, 1.0) == 1
    assert _java_binary_search(a, 0.1) == -1 and _java_binary_search(a, 1.5) == -3 and _java_binary_search(a, 9.0) == -4


def test_process_time_discretizations_of_the_schedule_products():
    # ProcessTimeDiscretizationProvider: exercise and payment times, as the model grid for the products
    ref = dt.date(2026, 1, 5)
    d = [dt.date(2026 + (i // 2), 1 + 6 * (i % 2), 5) for i in range(7)]
    leg = lambda first, dc: F.ScheduleFromPeriods(ref, [F.Period(d[i], d[i + 1], d[i], d[i + 1])
                                                        for i in range(first, 6)], dc)
    fd = lambda x: F.FloatingpointDate.getFloatingPointDateFromDate(ref, x)
    euro = F.SwaptionFromSwapSchedules(ref, "PAYER", d[2], leg(2, F.DayCountConvention_ACT_360()),
                                       leg(2, F.DayCountConvention_ACT_365()), 0.04)
    assert list(euro.getProcessTimeDiscretization(ref).getAsDoubleArray()) == \
        list(F.TimeDiscretizationFromArray([fd(x) for x in d[2:7]]).getAsDoubleArray())
    berm = F.BermudanSwaptionFromSwapSchedules(ref, "RECEIVER", d[1:3], d[6], [0.04] * 2, [1.0] * 2,
                                               [leg(1, F.DayCountConvention_ACT_360()), leg(2, F.DayCountConvention_ACT_360())],
                                               [leg(1, F.DayCountConvention_ACT_365()), leg(2, F.DayCountConvention_ACT_365())])
    assert list(berm.getProcessTimeDiscretization(ref).getAsDoubleArray()) == \
        list(F.TimeDiscretizationFromArray([fd(x) for x in d[1:7]]).getAsDoubleArray())
    with pytest.raises(ValueError):
        F.BermudanSwaptionFromSwapSchedules(ref, "PAYER", d[1:3], d[6], [0.04], [1.0] * 2, [], [])
