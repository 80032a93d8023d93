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
