"""Scheme, measure and state-space variants of the FP64 path against the oracle.

The reference's own LMM tests run the PREDICTOR_CORRECTOR scheme, the TERMINAL measure and
the NORMAL state space (LIBORMarketModelValuationTest.java:158,
LIBORMarketModelNormalAADSensitivitiesTest.java:382,399).  Each variant of the general FP64
path kernel must reproduce the oracle's restatement (the same operation order) to 1e-12
relative on paths, numeraires and prices, like the default form.
"""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

pytestmark = pytest.mark.gpu

SCHEMES = {"EULER": 0, "EULER_FUNCTIONAL": 1, "PREDICTOR_CORRECTOR": 2, "PREDICTOR_CORRECTOR_FUNCTIONAL": 3}
NORMAL_VOL_SCALE = 0.05  # normal volatilities: the lognormal abcd levels times a 5 % rate


def _cfg(state_space):
    cfg = dict(W.LMM20)
    if state_space == "NORMAL":
        a, b, c, d = cfg["abcd"]
        s = NORMAL_VOL_SCALE
        cfg["abcd"] = (a * s, b * s, c, d * s)
    return cfg


CASES = [
    ("SPOT", "LOGNORMAL", "PREDICTOR_CORRECTOR_FUNCTIONAL"),
    ("SPOT", "LOGNORMAL", "PREDICTOR_CORRECTOR"),
    ("TERMINAL", "LOGNORMAL", "EULER_FUNCTIONAL"),
    ("SPOT", "NORMAL", "EULER_FUNCTIONAL"),
    ("TERMINAL", "NORMAL", "PREDICTOR_CORRECTOR"),
]


@pytest.mark.parametrize("measure,state_space,scheme", CASES)
def test_variant_paths_numeraires_and_prices(measure, state_space, scheme):
    cfg = _cfg(state_space)
    P = 3000
    m = oracle_model(cfg, measure={"SPOT": 0, "TERMINAL": 1}[measure],
                     state_space={"LOGNORMAL": 0, "NORMAL": 1}[state_space], scheme=SCHEMES[scheme])
    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    ref = po.Simulation(m, dW)
    sim = W.build(cfg, paths=P, observe_tenor_only=False, measure=measure, state_space=state_space,
                  scheme=SCHEMES[scheme])
    proc = sim.process
    for ti in (1, m.T // 2, m.T):
        for j in (0, m.N // 2, m.N - 1):
            g = proc.getProcessValue(ti, j)
            o = ref.process_value(ti, j)
            np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-15)
    for t in (0.0, m.tenor[1], m.tenor[m.N // 2], m.tenor[m.N]):
        np.testing.assert_allclose(sim.getNumeraire(t), ref.numeraire(t), rtol=1e-12, atol=0)
    ex, fix, pay, K = W.swaption_schedule(cfg)
    v_ref, _ = ref.swaption(ex, fix, pay, K)
    sw = F.Swaption(ex, fix, pay, K)
    assert sw.getValue(sim) == pytest.approx(v_ref, rel=1e-12, abs=1e-15)
    bfix, plen, bpay, bK = W.bermudan_schedule(cfg)
    b_ref, _ = ref.bermudan(bfix, plen, bpay, bK, basis_id=1)
    berm = F.BermudanSwaption(np.ones(len(bfix)), bfix, plen, bpay, 1.0, bK, True, "swaprate")
    assert berm.getValue(sim) == pytest.approx(b_ref, rel=1e-12, abs=1e-15)
    proc.close()
    proc.brownianMotion.close()


def test_terminal_and_spot_swaption_agree_statistically():
    """The same model priced under both measures: equal within the Monte Carlo errors."""
    cfg = W.LMM20
    P = 1 << 15
    ex, fix, pay, K = W.swaption_schedule(cfg)
    vals = {}
    for measure in ("SPOT", "TERMINAL"):
        sim = W.build(cfg, paths=P, measure=measure)
        r = F.Swaption(ex, fix, pay, K).getValues(sim)
        vals[measure] = (r["value"], r["error"])
        sim.process.close()
        sim.process.brownianMotion.close()
    (vs, es), (vt, et) = vals["SPOT"], vals["TERMINAL"]
    assert abs(vs - vt) < 4.0 * np.hypot(es, et)


def test_mixed_form_and_adjoint_reject_variants():
    with pytest.raises(ValueError):  # invalid arguments (LMM_ERR_INVALID) raise ValueError
        W.build(W.LMM20, paths=1024, precision=F.PRECISION_MIXED, measure="TERMINAL")
    sim = W.build(W.LMM20, paths=1024, measure="TERMINAL")
    fix, plen, pay, K = W.bermudan_schedule(W.LMM20)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    with pytest.raises(ValueError):
        berm.getGradient(sim)
    sim.process.close()
    sim.process.brownianMotion.close()
