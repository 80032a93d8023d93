"""Parity at the benchmark's own size: the lmm40 workload at 2^20 paths, seed 7.

The GPU's FP64 valuation (MT19937 increments, the path kernel, the numeraire adjustment,
the Bermudan by regression and the European swaption) against the oracle run on the host
cores over the same 2^20 paths: prices and standard errors to 1e-12 / 1e-10 relative,
every per-path Bermudan value within 1e-12 of the largest, and forward rates and
numeraires at the first, middle and last tenor times to 1e-12.  The oracle needs about
20 GB of host memory and 20-40 s on 16 cores for this size.

Beside the stated 1e-12, a guard on the arithmetic itself: the path kernel carries its sums
and its exponential step on float pairs (about 2^-47 per step), which keeps the forward
rates and numeraires within about 1.2e-13 of the oracle here and the per-path values within
about 1.3e-14 of the largest; the guard asserts 5e-13 and 1e-13, so that a loss of a few
bits per step fails a test although it would stay inside 1e-12.
"""
import os

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

pytestmark = pytest.mark.gpu

P = 1 << 20


def test_lmm40_full_size_matches_the_oracle():
    cfg = W.LMM40
    m = oracle_model(cfg)
    tidx = W.tenor_time_indices(cfg)
    obs = np.zeros(m.T + 1, np.uint8)
    obs[tidx] = 1
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    ex, sfix, spay, sK = W.swaption_schedule(cfg)

    sim = W.build(cfg, paths=P)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    gb = berm.getValues(sim, per_path=True)
    gs = F.Swaption(ex, sfix, spay, sK).getValues(sim)

    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    osim = po.Simulation(m, dW, observe=obs, threads=os.cpu_count() or 1)
    del dW
    ov, oe, opp, _ = osim.bermudan(fix, plen, pay, K, basis_id=1, per_path=True)
    sv, se = osim.swaption(ex, sfix, spay, sK)

    assert gb["value"] == pytest.approx(ov, rel=1e-12)
    assert gb["error"] == pytest.approx(oe, rel=1e-10)
    assert gs["value"] == pytest.approx(sv, rel=1e-12)
    assert gs["error"] == pytest.approx(se, rel=1e-10)
    scale = np.max(np.abs(opp))
    assert np.max(np.abs(gb["values"] - opp)) <= 1e-12 * scale
    assert np.max(np.abs(gb["values"] - opp)) <= 1e-13 * scale  # guard
    for t in (tidx[1], tidx[20], tidx[-1]):
        for j in (10, 39):
            o = osim.process_value(int(t), j)
            rel = np.max(np.abs(sim.process.getProcessValue(int(t), j) - o) / np.abs(o))
            assert rel <= 1e-12
            assert rel <= 5e-13  # guard
    for T in (0.5, 10.0, 20.0):
        o = osim.numeraire(T)
        rel = np.max(np.abs(sim.process.getNumeraire(T) - o) / np.abs(o))
        assert rel <= 1e-12
        assert rel <= 5e-13  # guard
    sim.process.close()
    sim.process.brownianMotion.close()
