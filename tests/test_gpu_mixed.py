"""The mixed-precision form against the FP64 form on the same Brownian increments.

The mixed form has no bit-parity target: its FP32 path state, FP32 basis and FP32 payoffs
(with the regression sums carried in twice FP32 precision) move prices by amounts far
below the Monte Carlo error.  The Bermudan bound is the form's target, 0.1 bp of the unit
notional (1e-5 absolute), and a small share of the FP64 standard error; the European
swaption's is relative to its price."""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W

pytestmark = pytest.mark.gpu

P = 65536
BERMUDAN_TOL_ABS = 1e-5    # |mixed - FP64|: 0.1 bp of the unit notional
BERMUDAN_TOL_SE = 0.05     # |mixed - FP64| in FP64 standard errors
SWAPTION_TOL_REL = 2e-5    # |mixed - FP64| / FP64
FLIP_FRACTION = 2e-3       # share of paths whose exercise date differs


@pytest.fixture(scope="module", params=["lmm20", "lmm40"])
def sims(request):
    cfg = W.WORKLOADS[request.param]
    s64 = W.build(cfg, paths=P, precision=F.PRECISION_FP64)
    s32 = W.build(cfg, paths=P, precision=F.PRECISION_MIXED)
    yield cfg, s64, s32
    for s in (s64, s32):
        s.process.close()
        s.process.brownianMotion.close()


def test_swaption_mixed_vs_fp64(sims):
    cfg, s64, s32 = sims
    ex, fix, pay, K = W.swaption_schedule(cfg)
    for k in (0.5 * K, K, 2 * K):
        a = F.Swaption(ex, fix, pay, k).getValue(s64)
        b = F.Swaption(ex, fix, pay, k).getValue(s32)
        assert abs(b - a) <= SWAPTION_TOL_REL * abs(a) + 1e-12


@pytest.mark.parametrize("basis", [None, "swaprate"])
def test_bermudan_mixed_vs_fp64(sims, basis):
    cfg, s64, s32 = sims
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    prod = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, basis)
    a = prod.getValues(s64, per_path=True)
    b = prod.getValues(s32, per_path=True)
    assert abs(b["value"] - a["value"]) <= BERMUDAN_TOL_ABS
    assert abs(b["value"] - a["value"]) <= BERMUDAN_TOL_SE * a["error"]
    assert b["error"] == pytest.approx(a["error"], rel=1e-2)
    # the per-path values agree wherever the exercise decisions agree
    same = np.abs(b["values"] - a["values"]) <= 1e-4 * np.max(np.abs(a["values"]))
    assert np.mean(~same) <= FLIP_FRACTION


def test_bermudan_variants_mixed_vs_fp64(sims):
    cfg, s64, s32 = sims
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    n = len(fix)
    ex = np.zeros(n, np.uint8)
    ex[::3] = 1
    notional = np.linspace(1.0, 2.0, n)
    strikes = K + 0.001 * np.sin(np.arange(n))
    for callable_ in (True, False):
        prod = F.BermudanSwaption(ex, fix, plen, pay, notional, strikes, callable_, "swaprate")
        a = prod.getValues(s64)
        b = prod.getValues(s32)
        assert abs(b["value"] - a["value"]) <= BERMUDAN_TOL_ABS * np.max(notional)
        assert abs(b["value"] - a["value"]) <= BERMUDAN_TOL_SE * a["error"]
