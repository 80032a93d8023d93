"""GPU Euler-log path kernel and numeraire against the oracle (FP64 form)."""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

pytestmark = pytest.mark.gpu

REL = 1e-12  # FP64 form: within 1e-12 relative of the oracle


def _pair(cfg, P, scheme=1, cap=1e5, seed=None, observe_tenor_only=False):
    seed = cfg["seed"] if seed is None else seed
    m = oracle_model(cfg, scheme=scheme, libor_cap=cap)
    dW = po.brownian_increments(m.times, m.F, P, seed)
    obs = None
    if observe_tenor_only:
        obs = np.zeros(m.T + 1, np.uint8)
        obs[W.tenor_time_indices(cfg)] = 1
    osim = po.Simulation(m, dW, observe=obs)
    td = F.TimeDiscretizationFromArray(0.0, m.T, cfg["dt"])
    tn = F.TimeDiscretizationFromArray(0.0, m.N, cfg["period"])
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("f", cfg["curve_nodes"], cfg["curve_values"], cfg["period"])
    vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tn, *cfg["abcd"])
    corr = F.LIBORCorrelationModelExponentialDecay(td, tn, cfg["F"], cfg["corr_decay"])
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tn, vol, corr)
    model = F.LIBORMarketModelFromCovarianceModel.of(tn, None, curve, F.DiscountCurveFromForwardCurve(curve), None, cov,
                                                     None, {"liborCap": cap})
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, cfg["F"], P, seed)
    proc = F.EulerSchemeFromProcessModel(model, bm, scheme, observedTimeIndices=W.tenor_time_indices(cfg) if observe_tenor_only else None)
    return m, osim, F.LIBORMonteCarloSimulationFromLIBORModel(proc)


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


@pytest.mark.parametrize("scheme", [1, 0])
def test_lmm20_all_states(scheme):
    m, osim, sim = _pair(W.LMM20, 5000, scheme=scheme)
    worst = 0.0
    for t in range(m.T + 1):
        for j in range(m.N):
            worst = max(worst, _rel(sim.getLIBOR(t, j), osim.process_value(t, j)))
    assert worst <= REL


@pytest.mark.parametrize("P", [1, 37, 1000])
def test_ragged_path_counts(P):
    m, osim, sim = _pair(W.LMM20, P)
    for t in (0, 1, 11, 20):
        for j in (0, 7, 19):
            assert _rel(sim.getLIBOR(t, j), osim.process_value(t, j)) <= REL


def test_cap_is_applied():
    cap = 0.06
    m, osim, sim = _pair(W.LMM20, 2000, cap=cap)
    got = sim.getLIBOR(20, 19)
    assert got.max() <= cap and np.any(got == cap)
    assert _rel(got, osim.process_value(20, 19)) <= REL


def test_numeraire_and_adjustment():
    m, osim, sim = _pair(W.LMM20, 5000)
    for T in (0.5, 1.0, 3.5, 10.0):
        g, o = sim.getNumeraire(T), osim.numeraire(T)
        assert _rel(g, o) <= REL
        i = int(round(T / 0.5))
        assert np.mean(1.0 / g) == pytest.approx(m.discount_chain[i], rel=1e-12)


def test_lmm40_tenor_observation_subset():
    m, osim, sim = _pair(W.LMM40, 4096, observe_tenor_only=True)
    for t in (2, 40, 78, 80):
        for j in (0, 5, 39):
            assert _rel(sim.getLIBOR(t, j), osim.process_value(t, j)) <= REL
    with pytest.raises(F.CalculationException):
        sim.getLIBOR(3, 5)  # not observed


def test_single_forward_single_factor():
    cfg = dict(W.LMM20, tenor_end=0.5, T_end=0.5, F=1)
    m, osim, sim = _pair(cfg, 100)
    assert _rel(sim.getLIBOR(1, 0), osim.process_value(1, 0)) <= REL


def test_repeatable_bitwise():
    a = W.build(W.LMM20, paths=3000)
    b = W.build(W.LMM20, paths=3000)
    assert np.array_equal(a.getLIBOR(20, 19), b.getLIBOR(20, 19))


def test_fp64_small_exp_and_newton_reciprocal():
    # the FP64 path kernel's exp(d) of the step increment (table-driven, |d| <= 1) and its
    # Newton reciprocal against CUDA's exp and correctly rounded division
    import ctypes
    e, r = ctypes.c_double(), ctypes.c_double()
    assert F.load().lmm_fp64_math_check(1 << 20, ctypes.byref(e), ctypes.byref(r)) == 0
    assert e.value <= 4.0, e.value
    assert r.value <= 1.0, r.value
