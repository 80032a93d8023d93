"""Host-side compositions over random variables, checked without a GPU.

getForwardRate (all three interpolation methods, LOG_LINEAR_CORRECTED's drift adjustment
included) and the products of finmath_gb300.rvproducts choose time indices, tenor periods
and operation order on the host and issue device random-variable operations.  Here a test
double with the same methods, each a single numpy IEEE operation, stands in for the device
layer (monkeypatched for the duration of each test only), so the host logic is checked on
CPU against the same numpy restatements the GPU tests use.  The device operations
themselves, and these compositions on the GPU, are tested in test_gpu_randomvariable.py.
"""
import math
import types

import numpy as np
import pytest

import finmath_gb300
from finmath_gb300 import lmm as LM, randomvariable as R, rvproducts as RP, workloads as W
from oracle import pyoracle as po
from conftest import oracle_model
import test_gpu_randomvariable as TG


class NumpyRV:
    """Test double of RandomVariableGPU: deterministic float or numpy realizations."""

    def __init__(self, t, v):
        self.t, self.v = t, v

    @classmethod
    def constant(cls, t, v):
        return cls(t, float(v))

    @staticmethod
    def _operand(y):
        return (y.t, y.v) if isinstance(y, NumpyRV) else (-math.inf, float(y))

    def isDeterministic(self):
        return np.ndim(self.v) == 0

    def getFiltrationTime(self):
        return self.t

    def getRealizations(self):
        return np.atleast_1d(np.asarray(self.v, dtype=np.float64)).copy()

    def getAverage(self):
        return float(self.v) if self.isDeterministic() else po.kahan_average(self.v)

    def getStandardError(self):
        return 0.0 if self.isDeterministic() else po.standard_error(self.v)

    def _bin(self, y, f):
        t, v = self._operand(y)
        return NumpyRV(max(self.t, t), f(self.v, v))

    def add(self, y): return self._bin(y, lambda a, b: a + b)
    def sub(self, y): return self._bin(y, lambda a, b: a - b)
    def mult(self, y): return self._bin(y, lambda a, b: a * b)
    def div(self, y): return self._bin(y, lambda a, b: a / b)
    def floor(self, y): return self._bin(y, np.maximum)
    def cap(self, y): return self._bin(y, np.minimum)
    def squared(self): return NumpyRV(self.t, self.v * self.v)
    def log(self): return NumpyRV(self.t, np.log(self.v))
    def exp(self): return NumpyRV(self.t, np.exp(self.v))
    def invert(self): return NumpyRV(self.t, 1.0 / np.asarray(self.v))

    def discount(self, rate, periodLength):
        t, v = self._operand(rate)
        return NumpyRV(max(self.t, t), self.v / (1 + v * periodLength))

    def accrue(self, rate, periodLength):
        t, v = self._operand(rate)
        return NumpyRV(max(self.t, t), self.v * (1 + v * periodLength))

    def addRatio(self, numerator, denominator):
        (tn, vn), (td, vd) = self._operand(numerator), self._operand(denominator)
        return NumpyRV(max(self.t, tn, td), self.v + vn / vd)

    def pow(self, e):
        return NumpyRV(self.t, np.power(self.v, float(e)))

    def addProduct(self, factor1, factor2):
        (t1, v1), (t2, v2) = self._operand(factor1), self._operand(factor2)
        return NumpyRV(max(self.t, t1, t2), self.v + v1 * v2)

    def getConditionalExpectation(self, estimator):
        return estimator.getConditionalExpectation(self)

    def close(self):
        pass

    def choose(self, a, b):
        (ta, va), (tb, vb) = self._operand(a), self._operand(b)
        return NumpyRV(max(self.t, ta, tb), np.where(np.asarray(self.v) >= 0, va, vb))


@pytest.fixture
def lmm20_host(monkeypatch):
    monkeypatch.setattr(R, "RandomVariableGPU", NumpyRV)
    monkeypatch.setattr(RP, "RandomVariableGPU", NumpyRV)
    monkeypatch.setattr(finmath_gb300, "RandomVariableGPU", NumpyRV)
    cfg = W.LMM20
    m = oracle_model(cfg)
    P = 2000
    osim = po.Simulation(m, po.brownian_increments(m.times, m.F, P, cfg["seed"]))
    td = LM.TimeDiscretizationFromArray(0.0, int(round(cfg["T_end"] / cfg["dt"])), cfg["dt"])
    tenor = LM.TimeDiscretizationFromArray(0.0, int(round(cfg["tenor_end"] / cfg["period"])), cfg["period"])
    curve = LM.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                        cfg["curve_values"], cfg["period"])
    vol = LM.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *cfg["abcd"], False)
    corr = LM.LIBORCorrelationModelExponentialDecay(td, tenor, cfg["F"], cfg["corr_decay"])
    cov = LM.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)
    model = LM.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, LM.DiscountCurveFromForwardCurve(curve),
                                                      None, cov, None, {})

    class HostSimulation(LM.LIBORMonteCarloSimulationFromLIBORModel):
        # the simulation's own getForwardRate and helpers over the oracle's paths
        def __init__(self):
            self.model = model
            self.process = types.SimpleNamespace(getTimeDiscretization=lambda: td, numberOfPaths=P)

        def getLIBORRandomVariable(self, timeIndex, liborIndex):
            return NumpyRV(td.getTime(timeIndex), osim.process_value(timeIndex, liborIndex))

        def getNumeraireRandomVariable(self, time):
            return NumpyRV(time, osim.numeraire(time))

        def getLIBOR(self, timeIndex, liborIndex):
            return osim.process_value(timeIndex, liborIndex)

    return cfg, m, osim, HostSimulation()


@pytest.mark.parametrize("method", ["LOG_LINEAR_UNCORRECTED", "LINEAR", "LOG_LINEAR_CORRECTED"])
def test_forward_rate_composition(lmm20_host, method):
    TG.test_forward_rates_primitive_accrued_and_interpolated(lmm20_host, method)


def test_log_linear_corrected_moves_interpolated_rates_only(lmm20_host):
    _, _, _, sim = lmm20_host
    sim.model.interpolationMethod = "LOG_LINEAR_CORRECTED"
    corrected = [sim.getForwardRate(*a).getRealizations() for a in ((1.25, 1.25, 1.5), (2.0, 2.0, 3.0))]
    sim.model.interpolationMethod = "LOG_LINEAR_UNCORRECTED"
    plain = [sim.getForwardRate(*a).getRealizations() for a in ((1.25, 1.25, 1.5), (2.0, 2.0, 3.0))]
    rel = np.max(np.abs(corrected[0] - plain[0]) / plain[0])
    assert 1e-5 < rel < 1e-2  # the convexity drift adjustment: small but present
    assert np.array_equal(corrected[1], plain[1])  # tenor-aligned periods need no interpolation


def test_product_compositions(lmm20_host):
    TG.test_bonds_digitals_zero_swap_and_money_market_account(lmm20_host)
    TG.test_caplets_and_swap_through_the_random_variable_api(lmm20_host)


@pytest.fixture
def dated_host(monkeypatch):
    monkeypatch.setattr(R, "RandomVariableGPU", NumpyRV)
    monkeypatch.setattr(RP, "RandomVariableGPU", NumpyRV)
    monkeypatch.setattr(finmath_gb300, "RandomVariableGPU", NumpyRV)
    P = 1000
    td, tenor, model = TG.dated_model()
    m, osim = TG.dated_oracle(td, tenor, P)

    class HostSimulation(LM.LIBORMonteCarloSimulationFromLIBORModel):
        def __init__(self):
            self.model = model
            self.process = types.SimpleNamespace(getTimeDiscretization=lambda: td, numberOfPaths=P)

        def getLIBORRandomVariable(self, timeIndex, liborIndex):
            return NumpyRV(td.getTime(timeIndex), osim.process_value(timeIndex, liborIndex))

        def getNumeraireRandomVariable(self, time):
            return NumpyRV(time, osim.numeraire(time))

    return TG.DATED, m, osim, HostSimulation()


def test_schedule_swaption_compositions(dated_host):
    TG.test_swaptions_on_date_schedules(dated_host)


def test_simulation_facade(lmm20_host):
    # LIBORMonteCarloSimulationFromLIBORModel.java:53-165 over the host double
    cfg, m, osim, sim = lmm20_host
    w = sim.getMonteCarloWeights(1.2)  # a time between simulation times: the index before it
    assert w.isDeterministic() and w.getAverage() == 1.0 / sim.getNumberOfPaths() and w.getFiltrationTime() == 1.0
    assert sim.getMonteCarloWeights(3).getFiltrationTime() == 1.5
    assert sim.getTimeIndex(2.0) == 4 and sim.getTime(4) == 2.0 and sim.getTimeIndex(2.1) < 0
    assert sim.getNumberOfComponents() == sim.getNumberOfLibors() == 20
    libors = sim.getLIBORs(4)
    assert len(libors) == 20 and np.array_equal(libors[7].getRealizations(), osim.process_value(4, 7))
    assert sim.getLiborPeriod(3) == 1.5 and sim.getLiborPeriodIndex(1.5) == 3 and sim.getLiborPeriodIndex(1.6) < 0


def test_bermudan_with_a_user_basis_provider(lmm20_host):
    # BermudanSwaption.getValues (BermudanSwaption.java:91-157) with a user
    # RegressionBasisFunctionsProvider: a provider returning the built-in basis (:215-252)
    # reprices the oracle's Bermudan with that basis, path by path
    cfg, m, osim, sim = lmm20_host
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    builtin = finmath_gb300.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, None)

    class Provider:
        def getBasisFunctions(self, fixingDate, model):
            return builtin.getBasisFunctions(fixingDate, model)

    custom = finmath_gb300.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, Provider())
    r = custom.getValues(sim, per_path=True)
    v, e, pp, et = osim.bermudan(fix, plen, pay, K, basis_id=0, per_path=True)  # 0: the built-in basis
    assert r["value"] == pytest.approx(v, rel=1e-10) and r["error"] == pytest.approx(e, rel=1e-8)
    assert np.mean(np.abs(r["values"] - pp) <= 1e-10 * np.max(np.abs(pp))) >= 0.999
    assert custom.getExerciseTimes() == list(fix)
    with pytest.raises(ValueError):
        custom._desc()  # the fused gradient and portfolio kernels take the built-in bases only


def test_numeraire_between_tenor_times(lmm20_host):
    # getNumeraire off the tenor grid (LIBORMarketModelFromCovarianceModel.java:860-876,
    # :883-943, :968-1015) over the oracle's paths: the next tenor time's unadjusted numeraire
    # discounted with L(t; t, T_next) over T_next - t, times mean(N(0) / N(t)) and divided by
    # the geometric interpolation of the discount-curve chain
    cfg, m, osim, sim = lmm20_host
    sim._unadjustedNumeraire = lambda T: NumpyRV(T, osim.numeraire_unadjusted(T))
    base = LM.LIBORMonteCarloSimulationFromLIBORModel.getNumeraireRandomVariable
    tenor = sim.model.liborPeriodDiscretization
    for t in (0.125, 1.3, 4.75, 9.9):
        got = base(sim, t).getRealizations()
        up = tenor.getTime(-tenor.getTimeIndex(t) - 1)
        lo = up - cfg["period"]
        fwd = sim.getForwardRate(t, t, up).getRealizations()
        nu = osim.numeraire_unadjusted(up) / (1.0 + fwd * (up - t))
        a0, a1 = m.discount_chain[int(round(lo / cfg["period"]))], m.discount_chain[int(round(up / cfg["period"]))]
        pd = a0 * (a1 / a0) ** ((t - lo) / (up - lo))
        expected = nu * po.kahan_average(osim.numeraire_unadjusted(0.0) / nu) / pd
        assert np.allclose(got, expected, rtol=1e-13, atol=0.0)
    with pytest.raises(ValueError):
        base(sim, 10.25)  # beyond the last tenor time
