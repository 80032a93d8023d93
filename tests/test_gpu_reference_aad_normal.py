"""The reference's own AAD sensitivity test configuration, on the GPU adjoint (NORMAL state space).

LIBORMarketModelNormalAADSensitivitiesTest (src/test/java8/net/finmath/montecarlo/interestrate/
LIBORMarketModelNormalAADSensitivitiesTest.java:288-401) builds 80 semi-annual forwards on
0-40y at a flat 5 %, Euler steps of 0.125y to 40y, a 4 x 4 normal volatility matrix
d = 0.3 / 20 / 2 on the grid {0, 10, 20, 30, 40} for both times and forwards (read at the
floor indices of t_i and T_j), one factor with correlation decay 0, the SPOT measure, the
NORMAL state space, no LIBOR cap, no discount curve, 5,000 paths of MersenneTwister seed
1352 and the EULER scheme.  Its Bermudan case exercises every six months from 30y into a swap
to 40y at the par swap rate (:98-165).  The checks, with the reference's tolerances:

  testVega  (:411-553)  the AAD vega to the matrix entry (2, 2) against central differences
                        with a 1e-8 shift of that entry, |FD - AD| <= 1.3e-2;
  testDelta (:563-711)  the AAD delta to L_60(0) (DISCRETE_DELTA, width 0.05) against central
                        differences with a 1e-2 bump of that forward, |FD - AD| <= 1.3e-2;
  both                  the AAD run's value equals the plain valuation's exactly.

Tighter than the reference: the GPU paths and Bermudan value equal the oracle's on the same
tables, and the frozen-exercise (ZERO) adjoint equals central differences of the oracle's
frozen-exercise value to 1e-6 for deltas and for vegas of the simulation grid.
"""
import math

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import analytic as A
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

PATHS, FACTORS, SEED = 5000, 1, 1352
D = 0.3 / 20.0 / 2.0
EXERCISE, PERIODS = 30.0, 20


def _swaption_schedule():
    fixing = [EXERCISE + k * 0.5 for k in range(PERIODS)]
    payment = [EXERCISE + (k + 1) * 0.5 for k in range(PERIODS)]
    return fixing, payment, fixing + [payment[-1]]


def par_swaprate():
    """Swap.getForwardSwapRate on the data() curve (:83-106): flat 5 % on {0.5, 1, 2, 5, 40}."""
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards(
        "forwardCurve", [0.5, 1.0, 2.0, 5.0, 40.0], [0.05] * 5, 0.5)
    _, _, tenor = _swaption_schedule()
    return A.forward_swap_rate(F.TimeDiscretizationFromArray(tenor), curve, F.DiscountCurveFromForwardCurve(curve))


def create_libor_market_model(delta_bucket=None, delta_shift=0.0, vol_bucket=(0, 0), vol_shift=0.0):
    """createLIBORMarketModel (:288-401) with its bumps: one forward (delta_bucket) or all of
    them shifted by delta_shift, and one entry of the volatility matrix shifted by vol_shift."""
    tenor = F.TimeDiscretizationFromArray(0.0, 80, 0.5)
    times = tenor.getAsDoubleArray()
    rates = np.full(len(times), 0.05)
    if delta_bucket is not None:
        rates[delta_bucket] += delta_shift
    else:
        rates += delta_shift
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", list(times), list(rates), 0.5)
    td = F.TimeDiscretizationFromArray(0.0, 320, 0.125)
    tdv = F.TimeDiscretizationFromArray(0.0, 4, 10.0)
    vol = np.full((4, 4), D)
    vol[vol_bucket] += vol_shift
    vm = F.LIBORVolatilityModelFromGivenMatrix(tdv, tdv, vol)
    corr = F.LIBORCorrelationModelExponentialDecay(tdv, tdv, FACTORS, 0.0)
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(tdv, tdv, vm, corr)
    model = F.LIBORMarketModelFromCovarianceModel.of(
        tenor, None, curve, None, None, cov, [], {"measure": "SPOT", "stateSpace": "NORMAL", "liborCap": math.inf})
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, FACTORS, PATHS, SEED)
    process = F.EulerSchemeFromProcessModel(model, bm, F.EulerSchemeFromProcessModel.EULER)
    return F.LIBORMonteCarloSimulationFromLIBORModel(process)


def _close(sim):
    sim.process.close()
    sim.process.brownianMotion.close()


def bermudan(K):
    fixing, payment, _ = _swaption_schedule()
    return F.BermudanSwaption(np.ones(PERIODS), fixing, np.full(PERIODS, 0.5), payment, np.ones(PERIODS),
                              np.full(PERIODS, K))


def _value(product, **bumps):
    sim = create_libor_market_model(**bumps)
    v = product.getValue(sim)
    _close(sim)
    return v


@pytest.fixture(scope="module")
def case():
    K = par_swaprate()
    berm = bermudan(K)
    sim = create_libor_market_model()
    plain = berm.getValue(sim)
    g_dd = berm.getGradient(sim, diracDeltaApproximationMethod="DISCRETE_DELTA",
                            diracDeltaApproximationWidthPerStdDev=0.05)
    g_zero = berm.getGradient(sim, checkpointStride=1)
    g_zero8 = berm.getGradient(sim, checkpointStride=8)
    yield dict(K=K, berm=berm, sim=sim, plain=plain, g_dd=g_dd, g_zero=g_zero, g_zero8=g_zero8)
    _close(sim)


def _coarse_vega(sim, vegas, ic, jc):
    """d V / d sigma_coarse(ic, jc): the simulation-grid vegas of the times and forwards read
    from that entry of the 4 x 4 matrix (the floor indices of t_i and T_j in {0, 10, ..., 40})."""
    t = sim.process._keep["times"][:-1]
    tn = sim.process._keep["tenor"][:-1]
    rows = (np.floor(t / 10.0 + 1e-12).astype(int) == ic)
    cols = (np.floor(tn / 10.0 + 1e-12).astype(int) == jc)
    return float(vegas[np.ix_(rows, cols)].sum())


def test_aad_value_equals_the_plain_value(case):
    # Assert.assertEquals("Valuation", valueSimulation2, valueSimulation, 0.0) (:552, :710)
    assert case["g_dd"]["value"] == case["plain"]
    assert case["g_zero"]["value"] == case["plain"]


def test_delta(case):
    bucket, shift = int(round(EXERCISE * 2)), 1e-2
    fd = (_value(case["berm"], delta_bucket=bucket, delta_shift=shift)
          - _value(case["berm"], delta_bucket=bucket, delta_shift=-shift)) / shift / 2
    ad = case["g_dd"]["deltas"][bucket]
    assert ad == pytest.approx(fd, abs=1.3e-2)


def test_vega(case):
    ic, jc, shift = 2, 2, 1e-8
    fd = (_value(case["berm"], vol_bucket=(ic, jc), vol_shift=shift)
          - _value(case["berm"], vol_bucket=(ic, jc), vol_shift=-shift)) / shift / 2
    ad = _coarse_vega(case["sim"], case["g_dd"]["vegas"], ic, jc)
    assert ad == pytest.approx(fd, abs=1.3e-2)


# ---------------------------------------------------------------- against the oracle
def _oracle_model(sim, loadings=None, init=None):
    k = sim.process._keep
    lam = k["lam"] if loadings is None else loadings
    T, N, Fk = lam.shape
    return po.Model(times=k["times"].copy(), tenor=k["tenor"].copy(), factor=np.ones((N, Fk)), corr=np.ones((N, N)),
                    vol=np.zeros((T, N)), loadings=np.ascontiguousarray(lam), variance=k["var"].copy(),
                    initial_forwards=(k["init"] if init is None else init).copy(), discount_chain=None,
                    libor_cap=math.inf, scheme=0, measure=0, state_space=1)


@pytest.fixture(scope="module")
def oracle(case):
    sim = case["sim"]
    m = _oracle_model(sim)
    dW = po.brownian_increments(m.times, m.F, PATHS, SEED)
    base = po.Simulation(m, dW)
    fixing, payment, _ = _swaption_schedule()
    v, e, pp, et = base.bermudan(fixing, np.full(PERIODS, 0.5), payment, case["K"], basis_id=0, per_path=True)
    return dict(m=m, dW=dW, base=base, v=v, et=et)


def test_paths_and_value_equal_the_oracle(case, oracle):
    sim, base = case["sim"], oracle["base"]
    for t_index, j in ((8, 1), (160, 40), (240, 60), (320, 79)):
        g = sim.process.getProcessValue(t_index, j)
        o = base.process_value(t_index, j)
        assert np.allclose(g, o, rtol=1e-12, atol=1e-15)
    for t in (10.0, 30.0, 40.0):
        assert np.allclose(sim.process.getNumeraire(t), base.numeraire(t), rtol=1e-12)
    assert case["plain"] == pytest.approx(oracle["v"], rel=1e-12)


def _frozen(oracle, m, K):
    fixing, payment, _ = _swaption_schedule()
    return po.Simulation(m, oracle["dW"]).bermudan_frozen(fixing, np.full(PERIODS, 0.5), payment, K, oracle["et"])


@pytest.mark.parametrize("j", [0, 30, 60, 70, 79])
def test_frozen_exercise_deltas_equal_oracle_differences(case, oracle, j):
    h = 1e-5
    m = oracle["m"]
    up, dn = m.initial_forwards.copy(), m.initial_forwards.copy()
    up[j] += h
    dn[j] -= h
    fd = (_frozen(oracle, _oracle_model(case["sim"], init=up), case["K"])
          - _frozen(oracle, _oracle_model(case["sim"], init=dn), case["K"])) / (2 * h)
    scale = np.max(np.abs(case["g_zero"]["deltas"]))
    assert case["g_zero"]["deltas"][j] == pytest.approx(fd, abs=1e-6 * scale)


@pytest.mark.parametrize("i,j", [(0, 1), (100, 45), (200, 62), (239, 66), (300, 79)])
def test_frozen_exercise_vegas_equal_oracle_differences(case, oracle, i, j):
    h = 1e-7
    lam = case["sim"].process._keep["lam"]
    sigma = np.sqrt(np.sum(lam[i, j] ** 2))
    up, dn = lam.copy(), lam.copy()
    up[i, j] *= (sigma + h) / sigma
    dn[i, j] *= (sigma - h) / sigma
    fd = (_frozen(oracle, _oracle_model(case["sim"], loadings=up), case["K"])
          - _frozen(oracle, _oracle_model(case["sim"], loadings=dn), case["K"])) / (2 * h)
    scale = np.max(np.abs(case["g_zero"]["vegas"]))
    assert case["g_zero"]["vegas"][i, j] == pytest.approx(fd, abs=1e-6 * scale)


def test_checkpoint_stride_invariance(case):
    assert np.allclose(case["g_zero8"]["deltas"], case["g_zero"]["deltas"], rtol=1e-12, atol=1e-15)
    assert np.allclose(case["g_zero8"]["vegas"], case["g_zero"]["vegas"], rtol=1e-12, atol=1e-15)
