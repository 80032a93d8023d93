"""The oracle's LMM valuation: snapshot, structural properties and statistical checks (CPU)."""
import json
import os

import numpy as np
import pytest
from scipy.stats import norm

from finmath_gb300 import workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def lmm20():
    cfg = W.LMM20
    m = oracle_model(cfg)
    dW = po.brownian_increments(m.times, m.F, cfg["paths"], cfg["seed"])
    return cfg, m, dW, po.Simulation(m, dW)


def test_snapshot(lmm20):
    cfg, m, dW, sim = lmm20
    g = json.load(open(os.path.join(GOLD, "oracle_lmm20.json")))
    ex, fix, pay, K = W.swaption_schedule(cfg)
    assert sim.swaption(ex, fix, pay, K) == pytest.approx(tuple(g["swaption"]), rel=1e-12)
    bf, bl, bp, bK = W.bermudan_schedule(cfg)
    assert sim.bermudan(bf, bl, bp, bK, basis_id=0) == pytest.approx(tuple(g["bermudan_reference_basis"]), rel=1e-12)
    assert sim.bermudan(bf, bl, bp, bK, basis_id=1) == pytest.approx(tuple(g["bermudan_swaprate_basis"]), rel=1e-12)
    assert np.allclose(sim.process_value(10, 19)[:8], g["L_10_19_first8"], rtol=1e-13, atol=0)
    assert np.allclose(dW[3, 1, :8], g["dW_t3_f1_first8"], rtol=1e-14, atol=0)


def test_numeraire_adjustment_reprices_discount_bonds(lmm20):
    # getNumeraire rescales so that E[N(0)/N(T)] equals the discount curve P^d(T) (:869-874)
    cfg, m, dW, sim = lmm20
    for i in (1, 2, 7, 20):
        T = m.tenor[i]
        assert po.kahan_average(1.0 / sim.numeraire(T)) == pytest.approx(m.discount_chain[i], rel=1e-13)


def test_frozen_forwards_after_fixing(lmm20):
    cfg, m, dW, sim = lmm20
    # L_j stops evolving at T_j (EulerSchemeFromProcessModel copies components whose drift is null)
    for j in (2, 9):
        tj = int(round(m.tenor[j] / cfg["dt"]))
        assert np.array_equal(sim.process_value(tj, j), sim.process_value(m.T, j))


def black_swaption_rebonato(m, ex, fix, pay, K):
    """Black price of a payer swaption with Rebonato's frozen-weight swap-rate volatility."""
    tenor = m.tenor
    idx = [int(np.searchsorted(tenor, f)) for f in fix]
    L0 = m.initial_forwards
    df = np.cumprod(1.0 / (1.0 + L0 * np.diff(tenor)))
    df = np.concatenate([[1.0], df])
    ann = sum((pay[q] - fix[q]) * df[idx[q] + 1] for q in range(len(fix)))
    S0 = (df[idx[0]] - df[idx[-1] + 1]) / ann
    w = np.array([(pay[q] - fix[q]) * df[idx[q] + 1] / ann for q in range(len(fix))])
    var = 0.0
    for i in range(len(m.times) - 1):
        if m.times[i] >= ex:
            break
        dt = m.times[i + 1] - m.times[i]
        lam = m.loadings[i][idx]
        cov = lam @ lam.T
        wl = w * L0[idx]
        var += wl @ cov @ wl * dt
    sig = np.sqrt(var) / S0
    d1 = (np.log(S0 / K) + 0.5 * sig * sig) / sig
    return df[0] * ann * (S0 * norm.cdf(d1) - K * norm.cdf(d1 - sig))


def test_swaption_close_to_rebonato_approximation(lmm20):
    cfg, m, dW, sim = lmm20
    ex, fix, pay, K = W.swaption_schedule(cfg)
    v, se = sim.swaption(ex, fix, pay, K)
    approx = black_swaption_rebonato(m, ex, fix, pay, np.full(len(fix), K)[0])
    # same tolerance idea as LIBORMarketModelValuationTest.testSwaption (:366-428): statistical + approximation error
    assert abs(v - approx) < 3 * se + 0.03 * approx


def test_bermudan_dominates_european_swaptions(lmm20):
    cfg, m, dW, sim = lmm20
    bf, bl, bp, K = W.bermudan_schedule(cfg)
    berm, se = sim.bermudan(bf, bl, bp, K, basis_id=1)
    for ex in (2.0, 5.0):
        fix = bf[bf >= ex]
        v, _ = sim.swaption(ex, fix, fix + 0.5, K)
        assert berm > v - 3 * se


def test_euler_and_functional_schemes_agree_to_rounding():
    cfg = W.LMM20
    P = 500
    mf = oracle_model(cfg, scheme=1)
    me = oracle_model(cfg, scheme=0)
    dW = po.brownian_increments(mf.times, mf.F, P, cfg["seed"])
    a = po.Simulation(mf, dW).process_value(20, 19)
    b = po.Simulation(me, dW).process_value(20, 19)
    assert np.allclose(a, b, rtol=1e-12, atol=0)


# --------------------------------------------------------------------------- variants
@pytest.mark.parametrize("measure,state_space,scheme", [(0, 0, 3), (0, 0, 2), (1, 0, 1), (0, 1, 1), (1, 1, 2)])
def test_oracle_variants_reprice_zero_bonds(measure, state_space, scheme):
    """Every scheme / measure / state space: the adjusted numeraire reprices the discount
    curve's zero bonds, N(0) E[1/N(T_l)] = P^d(T_l), to rounding."""
    cfg = dict(W.LMM20)
    if state_space == 1:
        a, b, c, d = cfg["abcd"]
        cfg["abcd"] = (a * 0.05, b * 0.05, c, d * 0.05)
    m = oracle_model(cfg, measure=measure, state_space=state_space, scheme=scheme)
    P = 2000
    sim = po.Simulation(m, po.brownian_increments(m.times, m.F, P, cfg["seed"]))
    n0 = sim.numeraire(0.0)[0]
    if measure == 0:
        assert n0 == 1.0
    for l in range(1, m.N + 1):
        zb = n0 * np.mean(1.0 / sim.numeraire(m.tenor[l]))
        assert zb == pytest.approx(m.discount_chain[l], rel=1e-13)


def test_oracle_terminal_and_spot_agree_statistically():
    cfg = W.LMM20
    P = 20000
    ex, fix, pay, K = W.swaption_schedule(cfg)
    out = []
    for measure in (0, 1):
        m = oracle_model(cfg, measure=measure)
        sim = po.Simulation(m, po.brownian_increments(m.times, m.F, P, cfg["seed"]))
        out.append(sim.swaption(ex, fix, pay, K))
    (vs, es), (vt, et) = out
    assert abs(vs - vt) < 4.0 * np.hypot(es, et)


def test_oracle_euler_and_functional_agree_to_rounding():
    """EULER keeps the log state, EULER_FUNCTIONAL re-takes log(L) every step: without a cap
    they differ only by the rounding of log(exp(y))."""
    cfg = W.LMM20
    P = 500
    m1 = oracle_model(cfg, scheme=1)
    m0 = oracle_model(cfg, scheme=0)
    dW = po.brownian_increments(m1.times, m1.F, P, cfg["seed"])
    a = po.Simulation(m1, dW).process_value(m1.T, m1.N - 1)
    b = po.Simulation(m0, dW).process_value(m0.T, m0.N - 1)
    np.testing.assert_allclose(a, b, rtol=1e-12)


def test_reference_aad_weights_of_the_bermudan():
    # orc_bermudan_aad (the reverse sweep of RandomVariableDifferentiableAAD over
    # BermudanSwaption.getValues): under ZERO the weights are the frozen exercise decisions,
    # so the weighted discounted cash flows rebuild the value; DISCRETE_DELTA with an empty
    # window reduces to ZERO; with the default window the boundary term, projected through
    # the regression, moves the weights of every path
    cfg = W.LMM20
    P = 2000
    m = oracle_model(cfg)
    sim = po.Simulation(m, po.brownian_increments(m.times, m.F, P, cfg["seed"]))
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    v, e, pp, et = sim.bermudan(fix, plen, pay, K, basis_id=1, per_path=True)
    v0, w0 = sim.bermudan_aad(fix, plen, pay, K, method="ZERO")
    assert v0 == v
    paid = (np.asarray(fix)[:, None] >= et[None, :]).astype(float)
    assert np.array_equal(w0, paid)
    cash = np.array([((sim.process_value(int(round(f / cfg["dt"])), int(round(f / cfg["period"]))) - K) * d)
                     / sim.numeraire(t) for f, d, t in zip(fix, plen, pay)])
    assert np.allclose(np.sum(w0 * cash, axis=0), pp, rtol=1e-12, atol=1e-15)
    _, we = sim.bermudan_aad(fix, plen, pay, K, method="DISCRETE_DELTA", width=0.0)
    assert np.array_equal(we, w0)
    _, wd = sim.bermudan_aad(fix, plen, pay, K, method="DISCRETE_DELTA")
    assert np.all(np.isfinite(wd)) and np.any(wd != w0)
