"""Adjoint Greeks (deltas to the initial forwards, vegas to the volatility matrix) of the
Bermudan swaption against finite differences.

1. Exact check: the FP64 adjoint equals central finite differences (bump 1e-5, common
   random numbers) of the oracle's frozen-exercise Bermudan value -- the pathwise
   derivative the adjoint computes -- to 1e-6.
2. The checkpoint stride does not change the result, not by one bit.
3. The mixed-precision adjoint agrees with the FP64 adjoint.
4. Statistical check: full central finite differences on the GPU (regression re-run in
   every bumped valuation, common random numbers) agree with the adjoint within 2 % or
   3 standard errors of the difference, as the target of the differentiation form says.
"""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

pytestmark = pytest.mark.gpu

H = 1e-5


@pytest.fixture(scope="module")
def lmm20():
    cfg = W.LMM20
    P = 5000
    m = oracle_model(cfg)
    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    base = po.Simulation(m, dW)
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    v, e, pp, et = base.bermudan(fix, plen, pay, K, basis_id=1, per_path=True)
    sim = W.build(cfg, paths=P)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    g = berm.getGradient(sim, checkpointStride=8)
    return dict(cfg=cfg, m=m, dW=dW, v=v, et=et, g=g, sched=(fix, plen, pay, K), sim=sim, berm=berm, P=P)


def _frozen_value(d, m):
    fix, plen, pay, K = d["sched"]
    return po.Simulation(m, d["dW"]).bermudan_frozen(fix, plen, pay, K, d["et"])


def _bumped_forward(m, j, h):
    m2 = po.Model(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in m.__dict__.items()})
    m2.initial_forwards[j] += h
    return m2


def _bumped_vol(cfg, m, i, j, h):
    vol = m.vol.copy()
    vol[i, j] += h
    return oracle_model(cfg, vol_matrix=vol)


def test_value_is_the_forward_value(lmm20):
    assert lmm20["g"]["value"] == pytest.approx(lmm20["v"], rel=1e-12)


@pytest.mark.parametrize("j", [0, 1, 2, 7, 12, 19])
def test_deltas_equal_frozen_exercise_finite_differences(lmm20, j):
    m = lmm20["m"]
    fd = (_frozen_value(lmm20, _bumped_forward(m, j, H)) - _frozen_value(lmm20, _bumped_forward(m, j, -H))) / (2 * H)
    ad = lmm20["g"]["deltas"][j]
    assert ad == pytest.approx(fd, rel=1e-6, abs=1e-9)


@pytest.mark.parametrize("i,j", [(0, 1), (0, 19), (1, 2), (3, 10), (9, 12), (15, 19), (18, 19)])
def test_vegas_equal_frozen_exercise_finite_differences(lmm20, i, j):
    cfg, m = lmm20["cfg"], lmm20["m"]
    fd = (_frozen_value(lmm20, _bumped_vol(cfg, m, i, j, H)) - _frozen_value(lmm20, _bumped_vol(cfg, m, i, j, -H))) / (2 * H)
    ad = lmm20["g"]["vegas"][i, j]
    assert ad == pytest.approx(fd, rel=1e-6, abs=1e-9)


def test_vegas_vanish_where_volatility_does_not_enter(lmm20):
    m = lmm20["m"]
    vg = lmm20["g"]["vegas"]
    for i in range(m.T):
        for j in range(m.N):
            if not (m.tenor[j] > m.times[i]):
                assert vg[i, j] == 0.0


def test_checkpoint_stride_invariance(lmm20):
    """The FP64 replay between checkpoints runs the path kernel's own step (its double-float
    sums and exponential), so every stride gives the stride-8 Greeks bit for bit."""
    for stride in (1, 3, 16):
        g = lmm20["berm"].getGradient(lmm20["sim"], checkpointStride=stride)
        assert np.array_equal(g["deltas"], lmm20["g"]["deltas"])
        assert np.array_equal(g["vegas"], lmm20["g"]["vegas"])


def test_mixed_precision_checkpoint_stride_is_exact(lmm20):
    """The mixed form replays the steps between checkpoints with the FP32 path kernel's own
    component step on its own tables, so the replayed forward rates are the stored ones bit
    for bit; the reverse sweep's partition and order of sums do not depend on the stride, so
    the Greeks at strides 3 and 8 equal those at stride 1 exactly."""
    sim = W.build(lmm20["cfg"], paths=lmm20["P"], precision=F.PRECISION_MIXED)
    g1 = lmm20["berm"].getGradient(sim, checkpointStride=1)
    for stride in (3, 8):
        g = lmm20["berm"].getGradient(sim, checkpointStride=stride)
        assert g["value"] == g1["value"]
        assert np.array_equal(g["deltas"], g1["deltas"])
        assert np.array_equal(g["vegas"], g1["vegas"])
    sim.process.close()
    sim.process.brownianMotion.close()


def test_mixed_precision_adjoint_close_to_fp64(lmm20):
    cfg = lmm20["cfg"]
    sim = W.build(cfg, paths=lmm20["P"], precision=F.PRECISION_MIXED)
    g = lmm20["berm"].getGradient(sim, checkpointStride=8)
    g64 = lmm20["g"]
    scale_d = np.max(np.abs(g64["deltas"]))
    scale_v = np.max(np.abs(g64["vegas"]))
    # the form's target: 0.1 bp (1e-5 absolute on the unit notional) on the price and on
    # every delta and vega, and small against the largest Greek
    assert abs(g["value"] - g64["value"]) <= 1e-5
    assert np.max(np.abs(g["deltas"] - g64["deltas"])) <= 1e-5
    assert np.max(np.abs(g["vegas"] - g64["vegas"])) <= 1e-5
    assert np.max(np.abs(g["deltas"] - g64["deltas"])) <= 2e-4 * scale_d
    assert np.max(np.abs(g["vegas"] - g64["vegas"])) <= 2e-4 * scale_v


def test_full_finite_differences_statistically(lmm20):
    """Bump-and-revalue on the GPU (FP64, regression re-run, common random numbers)."""
    cfg = W.LMM20
    P = 1 << 15
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    g = berm.getGradient(W.build(cfg, paths=P), checkpointStride=8)

    def value(bump_fwd=None, bump_vol=None, h=0.0):
        sim = W.build(cfg, paths=P)
        model = sim.process.model
        cov = model.covarianceModel
        if bump_fwd is not None:
            model.initialForwards[bump_fwd] += h
        if bump_vol is not None:
            i, j = bump_vol
            s = cov.volatility[i, j]
            cov.volatility[i, j] = s + h
            cov.factorLoadings[i, j] *= (s + h) / s
            cov.variance[i, j] = (s + h) * (s + h)
        proc = F.EulerSchemeFromProcessModel(model, sim.process.brownianMotion,
                                             observedTimeIndices=W.tenor_time_indices(cfg))
        return berm.getValues(F.LIBORMonteCarloSimulationFromLIBORModel(proc), per_path=True)

    h = 1e-4
    for kind, arg, ad in (("fwd", 9, g["deltas"][9]), ("fwd", 15, g["deltas"][15]), ("vol", (4, 10), g["vegas"][4, 10])):
        up = value(bump_fwd=arg, h=h) if kind == "fwd" else value(bump_vol=arg, h=h)
        dn = value(bump_fwd=arg, h=-h) if kind == "fwd" else value(bump_vol=arg, h=-h)
        diff = (up["values"] - dn["values"]) / (2 * h)
        fd = diff.mean()
        se = diff.std() / np.sqrt(P)
        assert abs(ad - fd) <= max(0.02 * abs(fd), 3 * se), (kind, arg, ad, fd, se)
