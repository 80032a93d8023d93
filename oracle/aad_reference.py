"""The reference's AAD gradient of a Bermudan swaption, restated (test infrastructure).

finmath-lib differentiates BermudanSwaption.getValues with RandomVariableDifferentiableAAD:
a tape of the random-variable operations, swept backward.  For this product the sweep has
three special rules (RandomVariableDifferentiableAAD.java): the conditional expectation's
argument receives the conditional expectation of the adjoint (:188-192), the exercise
choice passes a DISCRETE_DELTA term to its trigger by default (:409-429, width 0.05
standard deviations, RandomVariableDifferentiableAADFactory.java:67-68) or nothing under
ZERO, and getAverage returns a double, so the numeraire adjustment is a constant (:771).

The sweep over the backward induction is restated in C (orc_bermudan_aad in
lmm_oracle.c): it yields, per path, the adjoint weight omega[k][p] of each discounted cash
flow c[k][p] = ((L_k(T_k) - K_k) d_k) n_k / N(T_pay).  The rest of the tape -- the cash
flows' dependence on the initial forwards and on the volatility matrix through the Euler
scheme -- is differentiated here by central finite differences with common random numbers
of the weighted cash-flow sum, the weights and the numeraire adjustment held fixed: the
exact pathwise derivative of the swept cash flows, per path, so its standard error comes
with it.  Only the tests and the benchmark's checking legs call this module.
"""
from __future__ import annotations

import numpy as np

from . import pyoracle as po


def _cashflows(sim, m, fixing, period_length, payment, strike, notional, adj_ratio):
    """c[k][p] with the base simulation's numeraire adjustment (adj_ratio = adjusted over
    unadjusted numeraire at each payment time, a deterministic factor)."""
    out = np.empty((len(fixing), sim.P))
    for k, (fix, dl, pay) in enumerate(zip(fixing, period_length, payment)):
        ti = int(np.searchsorted(m.times, fix - 1e-12))
        j = int(np.searchsorted(m.tenor, fix - 1e-12))
        L = sim.process_value(ti, j)
        N = sim.numeraire_unadjusted(pay) * adj_ratio[k]
        out[k] = ((L - strike[k]) * dl) * notional[k] / N
    return out


def bermudan_gradient(model, dW, fixing, period_length, payment, strike, method="DISCRETE_DELTA", width=0.05,
                      notional=None, deltas=None, vegas=None, h=1e-5, build_model=None, threads=0):
    """The reference AAD gradient of the Bermudan's value (mean over paths):
    returns (value, {"deltas": {j: (mean, se)}, "vegas": {(i, j): (mean, se)}}).

    model: the oracle's base model; dW: its Brownian increments [T][F][P];
    deltas: tenor indices j (d value / d L_j(0)); vegas: (time index i, tenor index j) of
    volatility entries, for which build_model(vol_matrix) rebuilds the model."""
    fixing, period_length, payment = (np.asarray(x, dtype=np.float64) for x in (fixing, period_length, payment))
    n = len(fixing)
    strike = np.broadcast_to(np.asarray(strike, dtype=np.float64), (n,))
    notional = np.ones(n) if notional is None else np.broadcast_to(np.asarray(notional, dtype=np.float64), (n,))
    base = po.Simulation(model, dW, threads=threads)
    value, omega = base.bermudan_aad(fixing, period_length, payment, strike, method=method, width=width,
                                     notional=notional)
    adj_ratio = [base.numeraire(pay)[0] / base.numeraire_unadjusted(pay)[0] for pay in payment]

    def weighted(m):
        sim = po.Simulation(m, dW, threads=threads)
        return np.sum(omega * _cashflows(sim, m, fixing, period_length, payment, strike, notional, adj_ratio), axis=0)

    def central(m_up, m_dn):
        d = (weighted(m_up) - weighted(m_dn)) / (2.0 * h)
        return float(np.mean(d)), float(np.std(d) / np.sqrt(d.size))

    out = {"deltas": {}, "vegas": {}}
    for j in deltas or []:
        up = po.Model(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in model.__dict__.items()})
        dn = po.Model(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in model.__dict__.items()})
        up.initial_forwards[j] += h
        dn.initial_forwards[j] -= h
        out["deltas"][j] = central(up, dn)
    for (i, j) in vegas or []:
        vu, vd = model.vol.copy(), model.vol.copy()
        vu[i, j] += h
        vd[i, j] -= h
        out["vegas"][(i, j)] = central(build_model(vu), build_model(vd))
    return value, out
