"""The Levenberg-Marquardt optimizer and the calibration loop, host only.

The optimizer is checked on the reference's own example and against scipy's least squares;
the calibration loop (clone the covariance model with trial parameters, build the model and
process on one Brownian motion, reprice, step) runs with the oracle's swaption pricer on the
oracle's paths standing in for the GPU process and fused kernel (monkeypatched for the test
only), so the whole loop is exercised without a GPU.
"""
import math

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import lmm as LM, workloads as W
from oracle import pyoracle as po


def test_levenberg_marquardt_reference_example():
    # optimizer/LevenbergMarquardt.java:190-215: values (p1, 2 p0 + p1) to targets (5, 10)
    opt = F.LevenbergMarquardt([0.0, 0.0], [5.0, 10.0], 100, lambda p: [p[0] * 0.0 + p[1], p[0] * 2.0 + p[1]])
    opt.setWeights([1.0, 1.0]).run()
    best = opt.getBestFitParameters()
    assert best == pytest.approx([2.5, 5.0], abs=1e-9)
    assert opt.getRootMeanSquaredError() <= 1e-9
    assert 2 <= opt.getIterations() <= 101


def test_levenberg_marquardt_matches_scipy_least_squares():
    scipy_opt = pytest.importorskip("scipy.optimize")
    rng = np.random.default_rng(11)
    x = np.linspace(0.0, 4.0, 25)
    y = 2.0 * np.exp(-1.3 * x) + 0.5 + rng.normal(0.0, 0.01, x.size)
    f = lambda p: list(p[0] * np.exp(-p[1] * x) + p[2])
    opt = F.OptimizerFactoryLevenbergMarquardt(200, 0.0).getOptimizer(f, [1.0, 1.0, 0.0], None, None, None, list(y))
    opt.run()
    ref = scipy_opt.least_squares(lambda p: np.asarray(f(p)) - y, [1.0, 1.0, 0.0], xtol=1e-15, ftol=1e-15, gtol=1e-15)
    assert opt.getBestFitParameters() == pytest.approx(list(ref.x), rel=1e-6)
    assert opt.getRootMeanSquaredError() == pytest.approx(math.sqrt(np.mean(ref.fun ** 2)), rel=1e-6)


def test_levenberg_marquardt_batch_objective_gives_the_same_fit():
    # the Jacobian's columns evaluated together take the same path as one at a time
    rng = np.random.default_rng(5)
    x = np.linspace(0.0, 4.0, 25)
    y = 2.0 * np.exp(-1.3 * x) + 0.5 + rng.normal(0.0, 0.01, x.size)
    f = lambda p: list(p[0] * np.exp(-p[1] * x) + p[2])  # noqa: E731
    calls = []

    def batch(ps):
        calls.append(len(ps))
        return [f(p) for p in ps]

    a = F.OptimizerFactoryLevenbergMarquardt(100, 0.0).getOptimizer(f, [1.0, 1.0, 0.0], None, None, None, list(y))
    a.run()
    b = F.OptimizerFactoryLevenbergMarquardt(100, 0.0).getOptimizer(f, [1.0, 1.0, 0.0], None, None, None, list(y))
    b.setBatchObjective(batch).run()
    assert b.getBestFitParameters() == a.getBestFitParameters()
    assert b.getIterations() == a.getIterations() and b.evaluations == a.evaluations
    assert calls and all(n == 3 for n in calls)


def test_levenberg_marquardt_rejects_nan_points():
    # a NaN error compares false: the point is rejected and lambda grows (:662-676)
    def f(p):
        if p[0] > 1.5:
            return [math.nan]
        return [(p[0] - 1.0) ** 2 + 1.0]
    opt = F.LevenbergMarquardt([3.0 - 2.0], [1.0], 50, f).setParameterSteps([1e-6])
    opt.run()
    assert opt.getBestFitParameters()[0] == pytest.approx(1.0, abs=1e-3)


def _covariance(cfg, vol_cal=True, corr_cal=True, abcd=None, decay=None):
    td = F.TimeDiscretizationFromArray(0.0, int(round(cfg["T_end"] / cfg["dt"])), cfg["dt"])
    tenor = F.TimeDiscretizationFromArray(0.0, int(round(cfg["tenor_end"] / cfg["period"])), cfg["period"])
    vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *(abcd or cfg["abcd"]), vol_cal)
    corr = F.LIBORCorrelationModelExponentialDecay(td, tenor, cfg["F"], cfg["corr_decay"] if decay is None else decay,
                                                   corr_cal)
    return td, tenor, F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)


def test_covariance_parameters_and_clones():
    cfg = W.LMM20
    _, _, cov = _covariance(cfg)
    assert list(cov.getParameterAsDouble()) == list(cfg["abcd"]) + [cfg["corr_decay"]]
    new = [0.25, 0.05, 0.3, 0.12, 0.08]
    clone = cov.getCloneWithModifiedParameters(new)
    _, _, fresh = _covariance(cfg, abcd=new[:4], decay=new[4])
    assert np.array_equal(clone.factorLoadings, fresh.factorLoadings) and np.array_equal(clone.variance, fresh.variance)
    # the reference's correlation clone uses its non-calibrateable constructor (LIBORCorrelationModelExponentialDecay.java:79)
    assert clone.getParameter() == new[:4]
    same_corr = cov.getCloneWithModifiedParameters(new[:4] + [cfg["corr_decay"]])
    assert same_corr.getCorrelationModel() is cov.getCorrelationModel()
    _, _, fixed = _covariance(cfg, vol_cal=False, corr_cal=False)
    assert fixed.getParameter() == []


class _HostBrownian:
    def __init__(self, times, F_, P, seed):
        self.dW = po.brownian_increments(times, F_, P, seed)

    def close(self):
        pass


class _HostProcess:
    def __init__(self, model, brownianMotion):
        self.model, self.bm = model, brownianMotion

    def close(self):
        pass


class _HostSimulation:
    """The simulation of a model on the oracle: the model's own host tables, the oracle's paths."""

    def __init__(self, process):
        self.model, self._bm, self._osim = process.model, process.bm, None

    def oracle(self):
        if self._osim is None:
            m, cov = self.model, self.model.covarianceModel
            corr = cov.getCorrelationModel()
            om = po.Model(cov.timeDiscretization.getAsDoubleArray(),
                          m.liborPeriodDiscretization.getAsDoubleArray(), corr.factorMatrix, corr.correlationMatrix,
                          cov.volatility, cov.factorLoadings, cov.variance, m.initialForwards, m.discountChain)
            self._osim = po.Simulation(om, self._bm.dW)
        return self._osim


class _OracleSwaption:
    def __init__(self, ex, fix, pay, K):
        self.args = (ex, fix, pay, K)

    def getValue(self, sim):
        return sim.oracle().swaption(*self.args)[0]


def test_calibration_loop_recovers_a_consistent_surface(monkeypatch):
    monkeypatch.setattr(LM, "EulerSchemeFromProcessModel", _HostProcess)
    monkeypatch.setattr(LM, "LIBORMonteCarloSimulationFromLIBORModel", _HostSimulation)
    cfg = W.LMM20
    td, tenor, truth = _covariance(cfg, corr_cal=False)
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     truth, None, {})
    bm = _HostBrownian(td.getAsDoubleArray(), cfg["F"], 400, 7)
    swaptions = []
    for ex, n in ((1.0, 4), (2.0, 6), (3.0, 4), (5.0, 8), (7.0, 4), (2.0, 12)):
        fix = [ex + 0.5 * i for i in range(n)]
        swaptions.append(_OracleSwaption(ex, fix, [x + 0.5 for x in fix], 0.05))
    base = _HostSimulation(_HostProcess(model, bm))
    targets = [s.getValue(base) for s in swaptions]
    items = [F.CalibrationProduct(f"swaption{i}", s, t, 1.0) for i, (s, t) in enumerate(zip(swaptions, targets))]
    _, _, start = _covariance(cfg, corr_cal=False, abcd=(0.25, 0.15, 0.2, 0.12))
    params = {"brownianMotion": bm, "maxIterations": 60, "accuracy": 0.0}
    calibrated = start.getCloneCalibrated(model, items, params)
    opt = params["optimizer"]
    assert opt.getRootMeanSquaredError() <= 1e-10 * max(targets)  # common random numbers: exact fit exists
    assert calibrated.getParameter() == pytest.approx(list(cfg["abcd"]), rel=1e-8)  # and it is the truth
    refit = _HostSimulation(_HostProcess(model.getCloneWithModifiedCovarianceModel(calibrated), bm))
    assert [s.getValue(refit) for s in swaptions] == pytest.approx(targets, rel=1e-8)
    # the model-level entry point calibrates the same way
    params2 = {"brownianMotion": bm, "maxIterations": 60, "accuracy": 0.0}
    m2 = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                  start, items, {"calibrationParameters": params2})
    assert m2.getCovarianceModel().getParameter() == pytest.approx(calibrated.getParameter(), rel=1e-12)


def test_reference_swaption_calibration_on_the_host(monkeypatch):
    # testSwaptionCalibration (LIBORMarketModelValuationTest.java:685-807) with its analytic
    # calibration products: the 5-parameter covariance model calibrated to 36 swaption
    # volatilities, RMS below the reference's 0.025.  The products need no simulation, so
    # a process test double stands in for the GPU process the calibration loop builds.
    import test_gpu_reference_acceptance as RA

    class Process:
        def __init__(self, model, brownianMotion, *args, **kwargs):
            self.model, self.brownianMotion, self.numberOfPaths = model, brownianMotion, RA.PATHS

        def getTimeDiscretization(self):
            return self.brownianMotion.timeDiscretization

        def close(self):
            pass

    class BrownianMotion:
        def __init__(self, timeDiscretization, *args):
            self.timeDiscretization = timeDiscretization

        def close(self):
            pass

    monkeypatch.setattr(LM, "EulerSchemeFromProcessModel", Process)
    monkeypatch.setattr(LM, "BrownianMotionFromMersenneRandomNumbers", BrownianMotion)
    td = F.TimeDiscretizationFromArray(0.0, 40, 0.5)
    tenor = F.TimeDiscretizationFromArray(0.0, 40, 0.5)
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards(
        "forwardCurve", [0.5, 1.0, 2.0, 5.0, 40.0], [0.05] * 5, 0.5)
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     F.LIBORCovarianceModelExponentialForm5Param(td, tenor, 6), [], {})
    sim = F.LIBORMonteCarloSimulationFromLIBORModel(Process(model, BrownianMotion(td)))
    products = RA.calibration_products(sim)
    assert len(products) == 36
    params = {"accuracy": 1e-6, "numberOfPaths": RA.PATHS}
    calibrated = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, None, None,
                                                          F.LIBORCovarianceModelExponentialForm5Param(td, tenor, 6),
                                                          products, {"calibrationParameters": params})
    simulation = F.LIBORMonteCarloSimulationFromLIBORModel(Process(calibrated, BrownianMotion(td)))
    deviations = [p.getProduct().getValue(simulation) - p.getTargetValue() for p in products]
    rms = math.sqrt(sum(d * d for d in deviations) / len(deviations))
    assert rms < 0.025
    assert params["optimizer"].getIterations() > 1  # the parameters moved
    assert list(calibrated.covarianceModel.getParameterAsDouble()) != [0.20, 0.05, 0.10, 0.20, 0.10]
