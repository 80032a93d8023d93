"""Monte Carlo calibration on the GPU: the covariance model's abcd parameters fitted to
swaption prices by Levenberg-Marquardt, every objective evaluation a new Euler process on
one resident Brownian motion and the fused swaption kernel."""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_calibration_recovers_the_generating_volatility_parameters():
    cfg = W.LMM20
    td = F.TimeDiscretizationFromArray(0.0, int(round(cfg["T_end"] / cfg["dt"])), cfg["dt"])
    tenor = F.TimeDiscretizationFromArray(0.0, int(round(cfg["tenor_end"] / cfg["period"])), cfg["period"])
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])

    def covariance(abcd):
        vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *abcd, True)
        corr = F.LIBORCorrelationModelExponentialDecay(td, tenor, cfg["F"], cfg["corr_decay"], False)
        return F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)

    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     covariance(cfg["abcd"]), None, {})
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, cfg["F"], 2000, 31415)
    swaptions = []
    for ex, n in ((1.0, 4), (2.0, 6), (3.0, 4), (5.0, 8), (7.0, 4), (2.0, 12)):
        fix = [ex + 0.5 * i for i in range(n)]
        swaptions.append(F.Swaption(ex, fix, [x + 0.5 for x in fix], 0.05))
    process = F.EulerSchemeFromProcessModel(model, bm)
    targets = [s.getValue(F.LIBORMonteCarloSimulationFromLIBORModel(process)) for s in swaptions]
    process.close()
    items = [F.CalibrationProduct(f"swaption{i}", s, t) for i, (s, t) in enumerate(zip(swaptions, targets))]
    params = {"brownianMotion": bm, "maxIterations": 60, "accuracy": 0.0}
    calibrated = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve),
                                                          None, covariance((0.25, 0.15, 0.2, 0.12)), items,
                                                          {"calibrationParameters": params})
    opt = params["optimizer"]
    # the same random numbers for every evaluation: the generating parameters fit exactly
    assert opt.getRootMeanSquaredError() <= 1e-10 * max(targets)
    assert np.allclose(calibrated.getCovarianceModel().getParameter(), cfg["abcd"], rtol=1e-7)
    bm.close()


def test_calibration_matches_the_oracle_calibration():
    # the same Levenberg-Marquardt calibration to targets no parameter set fits exactly (the
    # prices of another volatility surface, moved by up to 3 %), once with the GPU process and
    # fused swaption kernel and once with the oracle pricing the same paths: the iterations see
    # the same objective values to rounding, so they end at the same parameters and error
    import test_host_calibration as HC
    from finmath_gb300 import lmm as LM
    cfg = W.LMM20
    td, tenor, truth = HC._covariance(cfg, corr_cal=False)
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     truth, None, {})
    P, seed = 2000, 31415
    specs = []
    for ex, n in ((1.0, 4), (2.0, 6), (3.0, 4), (5.0, 8), (7.0, 4), (2.0, 12), (4.0, 10)):
        fix = [ex + 0.5 * i for i in range(n)]
        specs.append((ex, fix, [x + 0.5 for x in fix], 0.05))
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, cfg["F"], P, seed)
    process = F.EulerSchemeFromProcessModel(model, bm)
    sim = F.LIBORMonteCarloSimulationFromLIBORModel(process)
    targets = [F.Swaption(*sp).getValue(sim) * (1.0 + 0.03 * np.sin(3.0 * i)) for i, sp in enumerate(specs)]
    process.close()
    _, _, start = HC._covariance(cfg, corr_cal=False, abcd=(0.25, 0.15, 0.2, 0.12))

    gpu_items = [F.CalibrationProduct(f"s{i}", F.Swaption(*sp), t) for i, (sp, t) in enumerate(zip(specs, targets))]
    gp = {"brownianMotion": bm, "maxIterations": 40, "accuracy": 0.0}
    gpu = start.getCloneCalibrated(model, gpu_items, gp)

    saved = (LM.EulerSchemeFromProcessModel, LM.LIBORMonteCarloSimulationFromLIBORModel)
    LM.EulerSchemeFromProcessModel, LM.LIBORMonteCarloSimulationFromLIBORModel = HC._HostProcess, HC._HostSimulation
    try:
        hbm = HC._HostBrownian(td.getAsDoubleArray(), cfg["F"], P, seed)
        host_items = [F.CalibrationProduct(f"s{i}", HC._OracleSwaption(*sp), t)
                      for i, (sp, t) in enumerate(zip(specs, targets))]
        hp = {"brownianMotion": hbm, "maxIterations": 40, "accuracy": 0.0}
        host = start.getCloneCalibrated(model, host_items, hp)
    finally:
        LM.EulerSchemeFromProcessModel, LM.LIBORMonteCarloSimulationFromLIBORModel = saved
    bm.close()
    assert gp["optimizer"].getRootMeanSquaredError() > 1e-4 * max(targets)  # no exact fit exists
    assert gpu.getParameter() == pytest.approx(host.getParameter(), rel=1e-6)
    assert gp["optimizer"].getRootMeanSquaredError() == pytest.approx(hp["optimizer"].getRootMeanSquaredError(),
                                                                      rel=1e-6)
    assert gp["optimizer"].getIterations() == hp["optimizer"].getIterations()


def test_batched_swaption_values_equal_single_valuations():
    """lmm_swaption_values_batch: the same kernels and reductions as Swaption.getValues, queued
    for several trial models at once: equal values and errors."""
    cfg = W.LMM20
    sims = [W.build(cfg, paths=3000, seed=11) for _ in range(3)]
    fix = [2.0 + 0.5 * i for i in range(6)]
    swaptions = [F.Swaption(2.0, fix, [x + 0.5 for x in fix], K) for K in (0.04, 0.05, 0.06)]
    values, errors = F.swaptionValuesBatch(sims, swaptions)
    for i, sim in enumerate(sims):
        for k, s in enumerate(swaptions):
            r = s.getValues(sim)
            assert values[i, k] == r["value"] and errors[i, k] == r["error"]
    for sim in sims:
        sim.process.close()
        sim.process.brownianMotion.close()
