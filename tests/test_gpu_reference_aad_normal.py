"""The reference's own AAD sensitivity test configuration, on the GPU adjoint (NORMAL state space).

LIBORMarketModelNormalAADSensitivitiesTest (src/test/java8/net/finmath/montecarlo/interestrate/
LIBORMarketModelNormalAADSensitivitiesTest.java:288-401) builds 80 semi-annual forwards on
0-40y at a flat 5 %, Euler steps of 0.125y to 40y, a 4 x 4 normal volatility matrix
d = 0.3 / 20 / 2 on the grid {0, 10, 20, 30, 40} for both times and forwards (read at the
floor indices of t_i and T_j), one factor with correlation decay 0, the SPOT measure, the
NORMAL state space, no LIBOR cap, no discount curve, 5,000 paths of MersenneTwister seed
1352 and the EULER scheme.  Its five cases (:127-165, the bucket of each delta in brackets):
caplets at 5y [10], 10y [20] and 30y [60] struck at the par rate of the 30y-into-10y swap,
that swaption [60], and the Bermudan exercisable every six months from 30y into the same
swap [60].  The checks, with the reference's tolerances:

  testVega  (:411-553)  the AAD vega to the matrix entry (2, 2) against central differences
                        with a 1e-8 shift of that entry, |FD - AD| <= 1.3e-2;
  testDelta (:563-711)  the AAD delta to the bucket's initial forward (the Bermudan:
                        DISCRETE_DELTA, width 0.05) against central differences with a 1e-2
                        bump of that forward, |FD - AD| <= 1.3e-2;
  both                  the AAD run's value equals the plain valuation's exactly.

Tighter than the reference: the GPU paths and the Bermudan and swaption values equal the
oracle's on the same tables; the frozen-exercise (ZERO) Bermudan adjoint and the swaption's
adjoint equal central differences of the oracle's values to 1e-6 for deltas and for vegas of
the simulation grid; the caplets' deltas equal small-bump GPU differences to 1e-6.
"""
import math

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import analytic as A
from finmath_gb300 import rvproducts as RP
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


def swaption(K):
    fixing, payment, _ = _swaption_schedule()
    return F.Swaption(EXERCISE, fixing, payment, np.full(PERIODS, 0.5), np.full(PERIODS, K))


def products(K):
    """data() (:127-165): name -> (product, delta bucket, its AAD gradient on a simulation)"""
    def dd(p):
        return lambda sim: p.getGradient(sim, diracDeltaApproximationMethod="DISCRETE_DELTA",
                                         diracDeltaApproximationWidthPerStdDev=0.05)
    out = {}
    for T in (5.0, 10.0, EXERCISE):
        c = RP.Caplet(T, 0.5, K)
        out[f"caplet{T:g}"] = (c, int(round(T * 2)), c.getGradient)
    sw = swaption(K)
    out["swaption"] = (sw, int(round(EXERCISE * 2)), sw.getGradient)
    b = bermudan(K)
    out["bermudan"] = (b, int(round(EXERCISE * 2)), dd(b))
    return out


BUMPS = {"delta10+": dict(delta_bucket=10, delta_shift=1e-2), "delta10-": dict(delta_bucket=10, delta_shift=-1e-2),
         "delta20+": dict(delta_bucket=20, delta_shift=1e-2), "delta20-": dict(delta_bucket=20, delta_shift=-1e-2),
         "delta60+": dict(delta_bucket=60, delta_shift=1e-2), "delta60-": dict(delta_bucket=60, delta_shift=-1e-2),
         "vega+": dict(vol_bucket=(2, 2), vol_shift=1e-8), "vega-": dict(vol_bucket=(2, 2), vol_shift=-1e-8)}


@pytest.fixture(scope="module")
def case():
    K = par_swaprate()
    prods = products(K)
    sim = create_libor_market_model()
    plain = {name: p.getValue(sim) for name, (p, _, _) in prods.items()}
    grads = {name: grad(sim) for name, (_, _, grad) in prods.items()}
    g_zero = prods["bermudan"][0].getGradient(sim, checkpointStride=1)
    g_zero8 = prods["bermudan"][0].getGradient(sim, checkpointStride=8)
    g_sw8 = prods["swaption"][0].getGradient(sim, checkpointStride=8)
    bumped = {}
    for key, kw in BUMPS.items():
        b = create_libor_market_model(**kw)
        bumped[key] = {name: p.getValue(b) for name, (p, _, _) in prods.items()}
        _close(b)
    yield dict(K=K, prods=prods, sim=sim, plain=plain, grads=grads, g_zero=g_zero, g_zero8=g_zero8, g_sw8=g_sw8,
               bumped=bumped, berm=prods["bermudan"][0], g_dd=grads["bermudan"])
    _close(sim)


def _coarse_vega(sim, vegas, ic, jc):
    """d V / d sigma_coarse(ic, jc): the simulation-grid vegas of the times and forwards read
    from that entry of the 4 x 4 matrix (the floor indices of t_i and T_j in {0, 10, ..., 40})."""
    t = sim.process._keep["times"][:-1]
    tn = sim.process._keep["tenor"][:-1]
    rows = (np.floor(t / 10.0 + 1e-12).astype(int) == ic)
    cols = (np.floor(tn / 10.0 + 1e-12).astype(int) == jc)
    return float(vegas[np.ix_(rows, cols)].sum())


NAMES = ["caplet5", "caplet10", "caplet30", "swaption", "bermudan"]


@pytest.mark.parametrize("name", NAMES)
def test_aad_value_equals_the_plain_value(case, name):
    # Assert.assertEquals("Valuation", valueSimulation2, valueSimulation, 0.0) (:552, :710)
    assert case["grads"][name]["value"] == case["plain"][name]


@pytest.mark.parametrize("name", NAMES)
def test_delta(case, name):
    bucket, shift = case["prods"][name][1], 1e-2
    up, dn = case["bumped"][f"delta{bucket}+"][name], case["bumped"][f"delta{bucket}-"][name]
    fd = (up - dn) / shift / 2
    ad = case["grads"][name]["deltas"][bucket]
    assert ad == pytest.approx(fd, abs=1.3e-2)


@pytest.mark.parametrize("name", NAMES)
def test_vega(case, name):
    ic, jc, shift = 2, 2, 1e-8
    fd = (case["bumped"]["vega+"][name] - case["bumped"]["vega-"][name]) / shift / 2
    ad = _coarse_vega(case["sim"], case["grads"][name]["vegas"], ic, jc)
    assert ad == pytest.approx(fd, abs=1.3e-2)


def test_bermudan_value_equals_zero_method_value(case):
    assert case["g_zero"]["value"] == case["plain"]["bermudan"]


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
    sv, _ = base.swaption(EXERCISE, fixing, payment, case["K"])
    return dict(m=m, dW=dW, base=base, v=v, et=et, sv=sv)


def test_paths_and_value_equal_the_oracle(case, oracle):
    sim, base = case["sim"], oracle["base"]
    for t_index, j in ((8, 1), (160, 40), (240, 60), (320, 79)):
        g = sim.process.getProcessValue(t_index, j)
        o = base.process_value(t_index, j)
        assert np.allclose(g, o, rtol=1e-12, atol=1e-15)
    for t in (10.0, 30.0, 40.0):
        assert np.allclose(sim.process.getNumeraire(t), base.numeraire(t), rtol=1e-12)
    assert case["plain"]["bermudan"] == pytest.approx(oracle["v"], rel=1e-12)
    assert case["plain"]["swaption"] == pytest.approx(oracle["sv"], rel=1e-12)


def _frozen(oracle, m, K):
    fixing, payment, _ = _swaption_schedule()
    return po.Simulation(m, oracle["dW"]).bermudan_frozen(fixing, np.full(PERIODS, 0.5), payment, K, oracle["et"])


def _swaption_value(oracle, m, K):
    fixing, payment, _ = _swaption_schedule()
    return po.Simulation(m, oracle["dW"]).swaption(EXERCISE, fixing, payment, K)[0]


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


@pytest.mark.parametrize("j", [0, 30, 59, 60, 79])
def test_swaption_deltas_equal_oracle_differences(case, oracle, j):
    h = 1e-6
    m = oracle["m"]
    up, dn = m.initial_forwards.copy(), m.initial_forwards.copy()
    up[j] += h
    dn[j] -= h
    fd = (_swaption_value(oracle, _oracle_model(case["sim"], init=up), case["K"])
          - _swaption_value(oracle, _oracle_model(case["sim"], init=dn), case["K"])) / (2 * h)
    g = case["grads"]["swaption"]["deltas"]
    assert g[j] == pytest.approx(fd, abs=1e-6 * np.max(np.abs(g)))


@pytest.mark.parametrize("i,j", [(0, 1), (100, 45), (200, 62), (239, 70)])
def test_swaption_vegas_equal_oracle_differences(case, oracle, i, j):
    h = 1e-8
    lam = case["sim"].process._keep["lam"]
    sigma = np.sqrt(np.sum(lam[i, j] ** 2))
    up, dn = lam.copy(), lam.copy()
    up[i, j] *= (sigma + h) / sigma
    dn[i, j] *= (sigma - h) / sigma
    fd = (_swaption_value(oracle, _oracle_model(case["sim"], loadings=up), case["K"])
          - _swaption_value(oracle, _oracle_model(case["sim"], loadings=dn), case["K"])) / (2 * h)
    g = case["grads"]["swaption"]["vegas"]
    assert g[i, j] == pytest.approx(fd, abs=1e-6 * np.max(np.abs(g)))


@pytest.mark.parametrize("T,j", [(5.0, 10), (5.0, 3), (30.0, 60), (30.0, 41)])
def test_caplet_deltas_equal_small_bump_differences(case, T, j):
    h = 1e-6
    c = RP.Caplet(T, 0.5, case["K"])
    up = create_libor_market_model(delta_bucket=j, delta_shift=h)
    dn = create_libor_market_model(delta_bucket=j, delta_shift=-h)
    fd = (c.getValue(up) - c.getValue(dn)) / (2 * h)
    _close(up)
    _close(dn)
    g = case["grads"][f"caplet{T:g}"]["deltas"]
    assert g[j] == pytest.approx(fd, abs=1e-6 * np.max(np.abs(g)))


def test_swaption_checkpoint_stride_invariance(case):
    g1, g8 = case["grads"]["swaption"], case["g_sw8"]
    assert np.allclose(g8["deltas"], g1["deltas"], rtol=1e-12, atol=1e-15)
    assert np.allclose(g8["vegas"], g1["vegas"], rtol=1e-12, atol=1e-15)
