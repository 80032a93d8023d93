"""The GPU adjoint against the reference's own AAD gradient, restated (lmm20, 5,000 paths).

finmath-lib's RandomVariableDifferentiableAAD differentiates BermudanSwaption.getValues with
three rules that a frozen-exercise adjoint does not state by itself: the numeraire
adjustment's getAverage is a constant (RandomVariableDifferentiableAAD.java:771), the
conditional expectation re-projects the adjoint through the regression (:188-192), and the
exercise choice passes a DISCRETE_DELTA term to its trigger by default (:409-429, width 0.05
standard deviations) or nothing under diracDeltaApproximationMethod ZERO.  oracle/
aad_reference.py restates that sweep (the backward induction's adjoint weights in C, the
Euler scheme's by central differences of the weighted cash flows, per path).

* ZERO: the GPU adjoint with the numeraire adjustment frozen is the same pathwise
  derivative, so every delta and vega agrees to 1e-6 of the largest Greek.
* DISCRETE_DELTA (the reference's default): the GPU runs the same sweep over its backward
  induction (lmm_bermudan_get_gradient_aad) and its Greeks agree with the restatement's to
  1e-6 of the largest Greek; the boundary term itself, measured in standard errors of the
  per-path gradient, is reported; with an empty window (width 0) both reduce to ZERO.
"""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from oracle import pyoracle as po, aad_reference as AR
from conftest import oracle_model

pytestmark = pytest.mark.gpu

P = 5000
DELTAS = [0, 3, 9, 15, 19]
VEGAS = [(0, 1), (2, 5), (4, 10), (9, 12), (15, 19)]


@pytest.fixture(scope="module")
def setup():
    cfg = W.LMM20
    m = oracle_model(cfg)
    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    sim = W.build(cfg, paths=P)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    g = berm.getGradient(sim, checkpointStride=4, freezeNumeraireAdjustment=True)
    build = lambda vol: oracle_model(cfg, vol_matrix=vol)  # noqa: E731
    refs = {meth: AR.bermudan_gradient(m, dW, fix, plen, pay, K, method=meth, deltas=DELTAS, vegas=VEGAS,
                                       build_model=build)
            for meth in ("ZERO", "DISCRETE_DELTA")}
    empty = AR.bermudan_gradient(m, dW, fix, plen, pay, K, method="DISCRETE_DELTA", width=0.0, deltas=DELTAS[:2],
                                 build_model=build)
    gdd = berm.getGradient(sim, checkpointStride=4, freezeNumeraireAdjustment=True,
                           diracDeltaApproximationMethod="DISCRETE_DELTA")
    gdd0 = berm.getGradient(sim, checkpointStride=4, freezeNumeraireAdjustment=True,
                            diracDeltaApproximationMethod="DISCRETE_DELTA", diracDeltaApproximationWidthPerStdDev=0.0)
    yield dict(g=g, refs=refs, empty=empty, gdd=gdd, gdd0=gdd0)
    sim.process.close()
    sim.process.brownianMotion.close()


def test_value_equals_the_plain_value(setup):
    # the reference's invariant: the AAD valuation's value is the plain valuation's
    # (LIBORMarketModelNormalAADSensitivitiesTest.java:552, 710, 905)
    value_zero, _ = setup["refs"]["ZERO"]
    value_dd, _ = setup["refs"]["DISCRETE_DELTA"]
    assert setup["g"]["value"] == pytest.approx(value_zero, rel=1e-12)
    assert value_dd == value_zero


def test_zero_method_equals_the_gpu_adjoint(setup):
    g = setup["g"]
    _, ref = setup["refs"]["ZERO"]
    scale_d, scale_v = np.max(np.abs(g["deltas"])), np.max(np.abs(g["vegas"]))
    for j, (mean, se) in ref["deltas"].items():
        assert g["deltas"][j] == pytest.approx(mean, abs=1e-6 * scale_d)
    for (i, j), (mean, se) in ref["vegas"].items():
        assert g["vegas"][i, j] == pytest.approx(mean, abs=1e-6 * scale_v)


def test_discrete_delta_term(setup, record_property):
    g = setup["g"]
    _, dd = setup["refs"]["DISCRETE_DELTA"]
    _, zero = setup["refs"]["ZERO"]
    report = []
    for j, (mean, se) in dd["deltas"].items():
        report.append(("delta", j, g["deltas"][j], mean, (mean - g["deltas"][j]) / se))
    for (i, j), (mean, se) in dd["vegas"].items():
        report.append(("vega", (i, j), g["vegas"][i, j], mean, (mean - g["vegas"][i, j]) / se))
    record_property("discrete_delta_minus_gpu_in_se", [(k, idx, round(z, 2)) for k, idx, _, _, z in report])
    assert all(np.isfinite(z) for *_, z in report)
    # an empty window (width 0) leaves only the frozen-exercise term
    _, empty = setup["empty"]
    for j, (mean, se) in empty["deltas"].items():
        assert mean == pytest.approx(zero["deltas"][j][0], rel=1e-12, abs=1e-15)


def test_discrete_delta_method_equals_the_restated_reference(setup):
    g, gdd = setup["g"], setup["gdd"]
    _, ref = setup["refs"]["DISCRETE_DELTA"]
    assert gdd["value"] == g["value"]  # the AAD valuation's value is the plain value
    scale_d, scale_v = np.max(np.abs(gdd["deltas"])), np.max(np.abs(gdd["vegas"]))
    for j, (mean, se) in ref["deltas"].items():
        assert gdd["deltas"][j] == pytest.approx(mean, abs=1e-6 * scale_d)
    for (i, j), (mean, se) in ref["vegas"].items():
        assert gdd["vegas"][i, j] == pytest.approx(mean, abs=1e-6 * scale_v)
    # the boundary term is present, and an empty window gives back the frozen-exercise Greeks
    assert np.max(np.abs(gdd["deltas"] - g["deltas"])) > 1e-4 * scale_d
    assert np.allclose(setup["gdd0"]["deltas"], g["deltas"], rtol=1e-12, atol=1e-15)
    assert np.allclose(setup["gdd0"]["vegas"], g["vegas"], rtol=1e-12, atol=1e-15)


def test_mixed_precision_discrete_delta_close_to_fp64(setup):
    """The mixed form runs the same DISCRETE_DELTA sweep (FP64 sweep over its FP32 backward
    induction): its Greeks agree with the FP64 form's to 2e-3 of the largest Greek (paths whose
    trigger sits at the window's edge may fall on either side in FP32)."""
    cfg = W.LMM20
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    sim32 = W.build(cfg, paths=P, precision=F.PRECISION_MIXED)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    g32 = berm.getGradient(sim32, checkpointStride=4, freezeNumeraireAdjustment=True,
                           diracDeltaApproximationMethod="DISCRETE_DELTA")
    g64 = setup["gdd"]
    assert abs(g32["value"] - g64["value"]) <= 1e-5
    assert np.max(np.abs(g32["deltas"] - g64["deltas"])) <= 2e-3 * np.max(np.abs(g64["deltas"]))
    assert np.max(np.abs(g32["vegas"] - g64["vegas"])) <= 2e-3 * np.max(np.abs(g64["vegas"]))
    # and the boundary term is there: it moves the deltas away from the frozen-exercise ones
    g32z = berm.getGradient(sim32, checkpointStride=4, freezeNumeraireAdjustment=True)
    assert np.max(np.abs(g32["deltas"] - g32z["deltas"])) > 1e-4 * np.max(np.abs(g64["deltas"]))
    sim32.process.close()
    sim32.process.brownianMotion.close()
