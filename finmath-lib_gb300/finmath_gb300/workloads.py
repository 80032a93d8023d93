"""The benchmark workloads: the LMM configurations the reference's path is measured on.

Each workload is a plain parameter dict (the same numbers feed the GPU library and the
oracle in the tests) plus a builder that assembles the finmath-style objects.
  lmm20: 20 semi-annual forwards on 0-10y, 0.5y Euler steps, flat 5 %, abcd
         (0.2, 0.1, 0.25, 0.1), rho = exp(-0.05|dT|) reduced to 3 factors, 5,000 paths,
         seed 3141; 5y-into-5y payer swaption and 1y-9.5y payer Bermudan at K = 5 %.
  lmm40: 40 semi-annual forwards on 0-20y, 0.25y Euler steps (80 steps),
         f(T) = 0.02 + 0.02 (1 - exp(-T/5)), abcd (0.15, 0.1, 0.3, 0.08),
         rho = exp(-0.03|dT|) reduced to 10 factors, 2^20 paths, seed 7; payer Bermudan
         1y-19.5y at K = 4 % and a 10y-into-10y payer swaption.
"""
from __future__ import annotations

import math

import numpy as np

LMM20 = dict(name="lmm20", dt=0.5, T_end=10.0, period=0.5, tenor_end=10.0, F=3, corr_decay=0.05,
             abcd=(0.2, 0.1, 0.25, 0.1), curve_nodes=[0.5, 1.0, 2.0, 5.0, 40.0], curve_values=[0.05] * 5,
             paths=5000, seed=3141, swaption=(5.0, 10.0, 0.05), bermudan=(1.0, 10.0, 0.05))


def _lmm40_curve():
    nodes = [0.5 * i for i in range(41)]
    return nodes, [0.02 + 0.02 * (1.0 - math.exp(-t / 5.0)) for t in nodes]


_n40, _v40 = _lmm40_curve()
LMM40 = dict(name="lmm40", dt=0.25, T_end=20.0, period=0.5, tenor_end=20.0, F=10, corr_decay=0.03,
             abcd=(0.15, 0.1, 0.3, 0.08), curve_nodes=_n40, curve_values=_v40,
             paths=1 << 20, seed=7, swaption=(10.0, 20.0, 0.04), bermudan=(1.0, 20.0, 0.04))

WORKLOADS = {"lmm20": LMM20, "lmm40": LMM40}


def swaption_schedule(cfg):
    ex, end, K = cfg["swaption"]
    fix = np.arange(ex, end - 1e-12, cfg["period"])
    return ex, fix, fix + cfg["period"], K


def bermudan_schedule(cfg):
    first, end, K = cfg["bermudan"]
    fix = np.arange(first, end - 1e-12, cfg["period"])
    return fix, np.full(len(fix), cfg["period"]), fix + cfg["period"], K


def tenor_time_indices(cfg):
    """Process time indices of the tenor times (what the products read)."""
    step = int(round(cfg["period"] / cfg["dt"]))
    T = int(round(cfg["T_end"] / cfg["dt"]))
    return list(range(0, T + 1, step))


def build(cfg, paths=None, precision=0, observe_tenor_only=True, seed=None, measure="SPOT", state_space="LOGNORMAL",
          scheme=None):
    """Assemble the finmath-style simulation of a workload on the GPU library (default: the
    reference's SPOT measure, LOGNORMAL state space and EULER_FUNCTIONAL scheme)."""
    from . import lmm as F
    td = F.TimeDiscretizationFromArray(0.0, int(round(cfg["T_end"] / cfg["dt"])), cfg["dt"])
    tenor = F.TimeDiscretizationFromArray(0.0, int(round(cfg["tenor_end"] / cfg["period"])), cfg["period"])
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])
    vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *cfg["abcd"], False)
    corr = F.LIBORCorrelationModelExponentialDecay(td, tenor, cfg["F"], cfg["corr_decay"])
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None, cov,
                                                     None, {"measure": measure, "stateSpace": state_space})
    P = cfg["paths"] if paths is None else paths
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, cfg["F"], P, cfg["seed"] if seed is None else seed, precision)
    obs = tenor_time_indices(cfg) if observe_tenor_only else None
    process = F.EulerSchemeFromProcessModel(model, bm, scheme=scheme, observedTimeIndices=obs)
    return F.LIBORMonteCarloSimulationFromLIBORModel(process)


def portfolio_products(cfg=LMM40, n=256, seed=20261203, basis="swaprate"):
    """The batching workload: n Bermudan swaptions on the shared model, drawn from a seed.

    First exercise: uniform integer 1-10y; swap end: first exercise plus a uniform integer
    tenor of 1-10y; strike: the ATM par swap rate of the initial curve plus a uniform
    -100..+100 bp; payer or receiver (notional +1 / -1) with probability 1/2; exercisable
    on every semi-annual period start.  Generator: numpy.random.default_rng(seed).
    """
    from .lmm import BermudanSwaption, ForwardCurveInterpolation
    rng = np.random.default_rng(seed)
    period = cfg["period"]
    tenor = np.arange(0.0, cfg["tenor_end"] + 1e-9, period)
    curve = ForwardCurveInterpolation.createForwardCurveFromForwards("f", cfg["curve_nodes"], cfg["curve_values"], period)
    L0 = np.array([curve.getForward(None, t, period) for t in tenor[:-1]])
    df = np.concatenate([[1.0], np.cumprod(1.0 / (1.0 + L0 * period))])
    out = []
    horizon = cfg["tenor_end"]
    for _ in range(n):
        first = int(rng.integers(1, min(10, int(horizon) - 1) + 1))
        end = min(first + int(rng.integers(1, 11)), int(horizon))
        i0, i1 = int(round(first / period)), int(round(end / period))
        ann = sum(period * df[k + 1] for k in range(i0, i1))
        atm = (df[i0] - df[i1]) / ann
        strike = atm + rng.uniform(-0.01, 0.01)
        notional = 1.0 if rng.random() < 0.5 else -1.0
        fix = tenor[i0:i1]
        out.append(BermudanSwaption(np.ones(len(fix)), fix, np.full(len(fix), period), fix + period, notional, strike,
                                    True, basis))
    return out
