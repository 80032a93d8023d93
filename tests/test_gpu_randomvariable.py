"""Device random variables (include/lmm_rv.h) against the reference's semantics.

The elementwise operations of RandomVariableFromDoubleArray round every + - * / separately,
so on the same inputs the GPU equals numpy's IEEE arithmetic bit for bit; Math.min/max
rules (NaN wins, -0.0 < +0.0) are checked on special values; exp/log/pow/sin/cos are
CUDA's (within 2 ulp).  Averages are compensated sums (as the reference's Kahan sums).
Finmath products written against the random-variable API (caplets, swaps, bonds, digitals,
money market account) reprice against the same operations in numpy on the oracle's paths
to 1e-12."""
import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W
from finmath_gb300.randomvariable import RandomVariableGPU as RV
from oracle import pyoracle as po
from conftest import oracle_model

pytestmark = pytest.mark.gpu

N = 100_003  # ragged: not a multiple of the launch geometry


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


@pytest.fixture(scope="module")
def xy():
    rng = np.random.default_rng(20261204)
    x = rng.normal(0.03, 0.02, N)
    y = rng.normal(0.5, 0.3, N)
    z = rng.normal(1.0, 0.1, N)
    return x, y, z


def test_binary_operations_bit_exact(xy):
    x, y, _ = xy
    X, Y = RV.from_array(1.0, x), RV.from_array(2.0, y)
    cases = {"add": x + y, "sub": x - y, "bus": y - x, "mult": x * y, "div": x / y, "vid": y / x}
    for name, ref in cases.items():
        r = getattr(X, name)(Y)
        assert np.array_equal(bits(r.getRealizations()), bits(ref)), name
        assert r.getFiltrationTime() == 2.0  # the later filtration time
    for name, ref in {"add": x + 0.7, "sub": x - 0.7, "bus": 0.7 - x, "mult": x * 0.7, "div": x / 0.7,
                      "vid": 0.7 / x}.items():
        assert np.array_equal(bits(getattr(X, name)(0.7).getRealizations()), bits(ref)), name


def test_three_argument_operations_bit_exact(xy):
    x, y, z = xy
    X, Y, Z = RV.from_array(0.0, x), RV.from_array(0.0, y), RV.from_array(0.0, z)
    assert np.array_equal(bits(Z.accrue(X, 0.5).getRealizations()), bits(z * (1 + x * 0.5)))
    assert np.array_equal(bits(Z.discount(X, 0.5).getRealizations()), bits(z / (1.0 + x * 0.5)))
    assert np.array_equal(bits(X.addProduct(Y, Z).getRealizations()), bits(x + y * z))
    assert np.array_equal(bits(X.addProduct(Y, 0.25).getRealizations()), bits(x + y * 0.25))
    assert np.array_equal(bits(X.addRatio(Y, Z).getRealizations()), bits(x + y / z))
    assert np.array_equal(bits(X.subRatio(Y, Z).getRealizations()), bits(x - y / z))
    assert np.array_equal(bits(X.choose(Y, Z).getRealizations()), bits(np.where(x >= 0.0, y, z)))
    # deterministic rate: x (1 + r c) with the same rounding
    assert np.array_equal(bits(Z.accrue(0.04, 0.5).getRealizations()), bits(z * (1 + 0.04 * 0.5)))


def test_unary_operations(xy):
    x, y, z = xy
    Z = RV.from_array(0.0, z)
    assert np.array_equal(bits(Z.squared().getRealizations()), bits(z * z))
    assert np.array_equal(bits(Z.sqrt().getRealizations()), bits(np.sqrt(z)))  # correctly rounded
    assert np.array_equal(bits(Z.invert().getRealizations()), bits(1.0 / z))
    assert np.array_equal(bits(RV.from_array(0.0, x).abs().getRealizations()), bits(np.abs(x)))
    for name, ref in {"exp": np.exp(z), "log": np.log(z), "sin": np.sin(z), "cos": np.cos(z), "expm1": np.expm1(x)}.items():
        src = RV.from_array(0.0, x if name == "expm1" else z)
        got = getattr(src, name)().getRealizations()
        assert np.max(np.abs(got - ref) / np.abs(ref)) <= 4.5e-16, name
    got = Z.pow(1.7).getRealizations()
    assert np.max(np.abs(got - z ** 1.7) / z ** 1.7) <= 4.5e-16


def test_min_max_nan_and_signed_zero():
    x = np.array([1.0, np.nan, -0.0, 0.0, 2.0, -3.0, 0.0, -0.0])
    y = np.array([2.0, 1.0, 0.0, -0.0, np.nan, -3.0, 0.0, -0.0])
    X, Y = RV.from_array(0.0, x), RV.from_array(0.0, y)

    def jmin(a, b):
        if a != a or b != b:
            return np.nan
        if a < b:
            return a
        if b < a:
            return b
        return a if np.signbit(a) else b

    def jmax(a, b):
        if a != a or b != b:
            return np.nan
        if a > b:
            return a
        if b > a:
            return b
        return b if np.signbit(a) else a

    cap = X.cap(Y).getRealizations()
    flo = X.floor(Y).getRealizations()
    for i in range(len(x)):
        for got, ref in ((cap[i], jmin(x[i], y[i])), (flo[i], jmax(x[i], y[i]))):
            assert (np.isnan(got) and np.isnan(ref)) or (got == ref and np.signbit(got) == np.signbit(ref)), (i, got, ref)
    assert np.array_equal(X.isNaN().getRealizations(), np.isnan(x).astype(float))
    mn, mx = X.getMin(), X.getMax()
    assert np.isnan(mn) and np.isnan(mx)  # a NaN realization makes Math.min/max NaN
    Zs = RV.from_array(0.0, np.array([0.0, -0.0, 3.0]))
    assert Zs.getMin() == 0.0 and np.signbit(Zs.getMin()) and Zs.getMax() == 3.0


def test_deterministic_and_broadcast(xy):
    x, _, _ = xy
    a, b = RV.constant(0.5, 0.04), RV.constant(1.5, 0.5)
    c = a.mult(b).add(1.0)
    assert c.isDeterministic() and c.doubleValue() == 0.04 * 0.5 + 1.0 and c.getFiltrationTime() == 1.5
    assert c.getAverage() == c.doubleValue() and c.getStandardError() == 0.0 and c.getVariance() == 0.0
    X = RV.from_array(1.0, x)
    assert np.array_equal(bits(X.add(a).getRealizations()), bits(x + 0.04))
    assert np.array_equal(bits(a.sub(X).getRealizations()), bits(0.04 - x))
    with pytest.raises(ValueError):
        X.add(RV.from_array(0.0, np.ones(7)))


def test_reference_random_variable_kats():
    # montecarlo/RandomVariableTest.java:72-137 on device random variables: exact averages and
    # variances of small integer samples, pow(0.5) == sqrt and pow(2) == squared bit for bit
    r2 = RV.from_array(0.0, [-4.0, -2.0, 0.0, 2.0, 4.0]).add(4.0).div(2.0)
    assert r2.getAverage() == 2.0
    assert r2.getVariance() == pytest.approx(2.0, abs=1e-12)
    r = RV.constant(float("-inf"), 3.0).mult(r2)
    assert r.getAverage() == 6.0 and r.getVariance() == 2.0 * 9.0
    x = RV.from_array(0.0, [3.0, 1.0, 0.0, 2.0, 4.0, 1.0 / 3.0])
    for check in (x.sqrt().sub(x.pow(0.5)), x.squared().sub(x.pow(2.0))):
        assert check.getAverage() == 0.0 and check.getVariance() == 0.0
    assert x.getStandardDeviation() - np.sqrt(x.getVariance()) == 0.0
    # testAdd, testCap, testFloor (:175-231)
    a = RV.from_array(0.0, [-4.0, -2.0, 0.0, 2.0, 4.0])
    s = a.add(RV.from_array(0.0, [4.0, 2.0, 0.0, -2.0, -4.0]))
    assert abs(s.getAverage()) <= 1e-15 and abs(s.getVariance()) <= 1e-15
    var = (1.0 / 5.0) ** 2 * 4.0 / 5.0 + (1.0 - 1.0 / 5 - 0) ** 2 * 1.0 / 5.0
    capped = a.cap(RV.from_array(0.0, [-3.0] * 5))
    assert capped.getAverage() == pytest.approx(-3.0 - 1.0 / 5, abs=1e-15)
    assert capped.getVariance() == pytest.approx(var, abs=1e-15)
    floored = a.floor(RV.from_array(0.0, [3.0] * 5))
    assert floored.getAverage() == pytest.approx(3.0 + 1.0 / 5, abs=1e-15)
    assert floored.getVariance() == pytest.approx(var, abs=1e-15)
    # testApply: apply(DoubleUnaryOperator) is allowed to be unsupported (:233-251)
    with pytest.raises(NotImplementedError):
        a.apply(lambda v: np.exp(v * 2.0))


def test_reductions(xy):
    x, _, _ = xy
    X = RV.from_array(0.0, x)
    assert X.getAverage() == pytest.approx(po.kahan_average(x), rel=1e-15, abs=1e-18)
    m = po.kahan_average(x)
    var = po.kahan_average((x - m) * (x - m))
    assert X.getVariance() == pytest.approx(var, rel=1e-14)
    assert X.getStandardError() == pytest.approx(np.sqrt(var) / np.sqrt(N), rel=1e-14)
    assert X.getMin() == np.min(x) and X.getMax() == np.max(x)


@pytest.fixture(scope="module")
def lmm20():
    cfg = W.LMM20
    m = oracle_model(cfg)
    P = 5000
    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    obs = np.zeros(m.T + 1, np.uint8)
    obs[W.tenor_time_indices(cfg)] = 1
    return cfg, m, po.Simulation(m, dW, observe=obs), W.build(cfg, paths=P)


def test_caplets_and_swap_through_the_random_variable_api(lmm20):
    # Caplet.getValue (montecarlo/interestrate/products/Caplet.java:115-141) as a user writes
    # it against RandomVariable, on the GPU simulation, against the same operations in numpy
    # on the oracle's paths
    cfg, m, osim, sim = lmm20
    P = sim.getNumberOfPaths()
    w = 1.0 / P
    N0g, N0o = sim.getNumeraireRandomVariable(0.0), osim.numeraire(0.0)
    dt, period = cfg["dt"], cfg["period"]
    for j, K in ((2, 0.04), (9, 0.05), (15, 0.06)):
        T_fix, T_pay = j * period, (j + 1) * period
        t = int(round(T_fix / dt))
        g = sim.getLIBORRandomVariable(t, j).sub(K).floor(0.0).mult(period)
        g = g.div(sim.getNumeraireRandomVariable(T_pay)).mult(w).mult(N0g).div(w)
        o = np.maximum(osim.process_value(t, j) - K, 0.0) * period
        o = o / osim.numeraire(T_pay) * w * N0o / w
        assert g.getAverage() == pytest.approx(po.kahan_average(o), rel=1e-12)
        assert g.getStandardError() == pytest.approx(po.standard_error(o), rel=1e-10)
    # the library's Caplet (Caplet.java's operations) is the same computation
    j, K = 9, 0.05
    t = int(round(j * period / dt))
    o = np.maximum(osim.process_value(t, j) - K, 0.0) * period / osim.numeraire((j + 1) * period) * w * N0o / w
    assert F.Caplet(j * period, period, K).getValue(sim) == pytest.approx(po.kahan_average(o), rel=1e-12)
    of = -np.minimum(osim.process_value(t, j) - K, 0.0) * period / osim.numeraire((j + 1) * period) * w * N0o / w
    assert F.Caplet(j * period, period, K, isFloorlet=True).getValue(sim) == pytest.approx(po.kahan_average(of), rel=1e-12)
    # a payer swap: sum over periods of (L_j(T_j) - K) delta / N(T_{j+1})
    K = 0.05
    g = F.RandomVariableGPU.constant(0.0, 0.0)
    o = np.zeros(P)
    for j in range(2, 12):
        t = int(round(j * period / dt))
        N = sim.getNumeraireRandomVariable((j + 1) * period)
        g = g.addRatio(sim.getLIBORRandomVariable(t, j).sub(K).mult(period), N)
        o = o + (osim.process_value(t, j) - K) * period / osim.numeraire((j + 1) * period)
    assert g.getAverage() == pytest.approx(po.kahan_average(o), rel=1e-12)
    fixes = [j * period for j in range(2, 12)]
    swap = F.SimpleSwap(fixes, [x + period for x in fixes], [K] * len(fixes))
    ref = po.kahan_average(o * N0o)  # the same sum, times N(0), as SimpleSwap.java values it
    scale = po.kahan_average(np.abs(o * N0o))  # an at-the-money swap: cancellation in the sum
    assert swap.getValue(sim) == pytest.approx(ref, rel=1e-12, abs=1e-13 * scale)
    receiver = F.SimpleSwap(fixes, [x + period for x in fixes], [K] * len(fixes), isPayFix=False)
    assert receiver.getValue(sim) == pytest.approx(-ref, rel=1e-12, abs=1e-13 * scale)


def test_process_values_as_random_variables_match_host_copies():
    cfg = W.LMM20
    for prec in (F.PRECISION_FP64, F.PRECISION_MIXED):
        sim = W.build(cfg, paths=3001, precision=prec)
        t = W.tenor_time_indices(cfg)[5]
        assert np.array_equal(sim.getLIBORRandomVariable(t, 7).getRealizations(), sim.getLIBOR(t, 7))
        assert np.array_equal(sim.getNumeraireRandomVariable(3.0).getRealizations(), sim.getNumeraire(3.0))
        # between tenor times the numeraire is composed from the next tenor time's unadjusted
        # numeraire and the short forward rate (LIBORMarketModelFromCovarianceModel.java:968-1015)
        n = sim.getNumeraireRandomVariable(0.25).getRealizations()
        nu = sim._unadjustedNumeraire(0.5).getRealizations() / (
            1.0 + sim.getForwardRate(0.25, 0.25, 0.5).getRealizations() * 0.25)
        a = po.kahan_average(sim._unadjustedNumeraire(0.0).getRealizations() / nu)
        assert np.allclose(n, nu * a / sim.model.getNumeraireDefaultableZeroBondAsOfTimeZero(0.25), rtol=1e-13, atol=0)
        with pytest.raises(ValueError):
            sim.getNumeraireRandomVariable(10.25)  # beyond the last tenor time
        sim.process.close()
        sim.process.brownianMotion.close()


def _forward_rate_numpy(osim, m, cfg, method, time, ps, pe):
    """The same getForwardRate (LIBORMarketModelFromCovarianceModel.java:1238-1497) in numpy on
    the oracle's paths and factor loadings, with the forward curve interpolated linearly on
    values."""
    tenor = np.asarray(m.tenor)
    times = np.asarray(m.times)
    nodes, values = np.asarray(cfg["curve_nodes"]), np.asarray(cfg["curve_values"])
    po_off = cfg["period"]

    def fwd(t, dt):  # ForwardCurveInterpolation.getForward with a payment offset dt
        f = float(np.interp(t, nodes, values))
        return f if dt == po_off else (np.exp(np.log(1 + f * po_off) * dt / po_off) - 1.0) / dt

    def idx(grid, t):  # TimeDiscretizationFromArray.getTimeIndex: the time rounded to the 1-hour tick
        tick = 1.0 / (365.0 * 24.0)
        key = np.rint(t / tick) * tick
        i = int(np.searchsorted(grid, key))
        return i if i < len(grid) and grid[i] == key else -(i + 1)

    def drift_adjustment(ti, j):
        # getInterpolationDriftAdjustmentEvaluated (:1433-1497): trapezoid rule over 0..ti of
        # |lambda_j|^2 / (1 + L_j dT)^2 * L_j^2, L_j at min(s, index of T_j)
        tdt = tenor[j + 1] - tenor[j]
        start = idx(times, tenor[j])

        def integrand(s, k):
            sq = 0.0
            for lam in m.loadings[s, j]:
                sq = sq + lam * lam
            L = osim.process_value(k, j)
            x = L * tdt + 1.0
            return sq / (x * x) * (L * L)

        prev, acc = integrand(0, 0), 0.0
        for s in range(1, ti + 1):
            k = min(s, start)
            cur = integrand(s, k if k >= 0 else -k - 2)
            acc = acc + (cur + prev) * (0.5 * (times[s] - times[s - 1]))
            prev = cur
        return acc

    def one_plus(ti, pst, k):
        ts, te = tenor[k], tenor[k + 1]
        tdt = te - ts
        if ts < times[ti]:
            ti = min(ti, idx(times, ts))
        lg = osim.process_value(ti, k) * tdt + 1.0
        small = te - pst
        alpha = small / tdt
        if method == "LINEAR":
            interp = lg * alpha + (1 - alpha)
        elif method == "LOG_LINEAR_CORRECTED":
            interp = np.exp(np.log(lg) * alpha - drift_adjustment(ti, k) * (0.5 * small * (ts - pst)))
        else:
            interp = np.exp(np.log(lg) * alpha)
        a_long = 1 + fwd(ts, tdt) * tdt
        a_short = 1 + fwd(pst, small) * small
        a_int = a_long * alpha + (1 - alpha) if method == "LINEAR" else np.exp(np.log(a_long) * alpha)
        return interp * (a_short / a_int)

    def fr(time, ps, pe):
        psi, pei = idx(tenor, ps), idx(tenor, pe)
        time = min(time, ps)
        ti = idx(times, time)
        if ti < 0:
            ti = -ti - 2
            if time - times[ti] > times[ti + 1] - time:
                ti += 1
        if pei < 0:
            prev = -pei - 2
            ne = tenor[prev + 1]
            return ((fr(time, ps, ne) * (ne - ps) + 1.0) / one_plus(ti, pe, prev) - 1.0) / (pe - ps)
        if psi < 0:
            prev = -psi - 2
            ns = tenor[prev + 1]
            if ns == pe:
                return (one_plus(ti, ps, prev) - 1.0) / (pe - ps)
            return ((fr(time, ns, pe) * (pe - ns) + 1.0) * one_plus(ti, ps, prev) - 1.0) / (pe - ps)
        if psi + 1 == pei:
            return osim.process_value(ti, psi)
        acc = None
        for k in range(psi, pei):
            sub = tenor[k + 1] - tenor[k]
            L = osim.process_value(ti, k)
            acc = L * sub + 1.0 if acc is None else acc * (1 + L * sub)
        return (acc - 1.0) / (pe - ps)

    return fr(time, ps, pe)


@pytest.mark.parametrize("method", ["LOG_LINEAR_UNCORRECTED", "LINEAR", "LOG_LINEAR_CORRECTED"])
def test_forward_rates_primitive_accrued_and_interpolated(lmm20, method):
    cfg, m, osim, sim = lmm20
    old = sim.model.interpolationMethod
    sim.model.interpolationMethod = method
    try:
        for (t, ps, pe) in ((2.0, 2.0, 2.5), (1.0, 1.0, 3.0), (1.0, 1.0, 1.75), (1.25, 1.25, 2.0), (1.25, 1.25, 1.5),
                            (0.9, 1.2, 3.3), (5.0, 3.0, 3.5)):
            g = sim.getForwardRate(t, ps, pe).getRealizations()
            o = _forward_rate_numpy(osim, m, cfg, method, t, ps, pe)
            assert np.max(np.abs(g - o) / np.abs(o)) <= 1e-12, (t, ps, pe)
        # the model primitive is getLIBOR itself
        assert np.array_equal(sim.getForwardRate(2.0, 2.0, 2.5).getRealizations(), sim.getLIBOR(4, 4))
    finally:
        sim.model.interpolationMethod = old
    with pytest.raises(ValueError):
        sim.model.interpolationMethod = "CUBIC"
        try:
            sim.getForwardRate(1.0, 1.0, 1.75)
        finally:
            sim.model.interpolationMethod = old


def test_conditional_expectation_regression():
    # MonteCarloConditionalExpectationRegression on device random variables against the same
    # scalar products (Kahan averages of IEEE products) and the oracle's pseudo-inverse
    rng = np.random.default_rng(3)
    n = 50_001
    s = rng.normal(0.05, 0.01, n)
    y = np.maximum(s - 0.05, 0.0) + rng.normal(0.0, 0.002, n)
    X = [np.ones(n), s, s * s, s * s * s]
    basis = [F.RandomVariableGPU.constant(1.0, 1.0), RV.from_array(1.0, s), RV.from_array(1.0, s * s),
             RV.from_array(1.0, s * s * s)]
    est = F.MonteCarloConditionalExpectationRegression(basis)
    Y = RV.from_array(2.0, y)
    beta = est.getLinearRegressionParameters(Y)
    xtx = np.array([[po.kahan_average(X[i] * X[j]) for j in range(4)] for i in range(4)])
    xty = np.array([po.kahan_average(y * X[i]) for i in range(4)])
    ref = po.lstsq_pinv(xtx, xty)
    fit_ref = ref[0] * X[0]
    for i in range(1, 4):
        fit_ref = fit_ref + X[i] * ref[i]
    fit = Y.getConditionalExpectation(est).getRealizations()
    assert np.max(np.abs(fit - fit_ref)) <= 1e-9 * np.max(np.abs(fit_ref))
    assert np.max(np.abs(beta - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-6  # beta is ill-determined, the fit is not


def test_bermudan_written_against_the_random_variable_api_equals_the_fused_kernel(lmm20):
    # BermudanSwaption.getValues (montecarlo/interestrate/products/BermudanSwaption.java:91-157)
    # with its built-in basis (:215-252), written only against getForwardRate / getNumeraire
    # random variables and the regression estimator, against the fused Bermudan kernel on the
    # same simulation
    cfg, m, osim, sim = lmm20
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    P = sim.getNumberOfPaths()
    w = 1.0 / P
    values = F.RandomVariableGPU.constant(0.0, 0.0)
    under = F.RandomVariableGPU.constant(0.0, 0.0)
    for period in range(len(fix) - 1, -1, -1):
        f, dt, p = fix[period], plen[period], pay[period]
        libor = sim.getForwardRate(f, f, f + dt)
        payoff = libor.sub(K).mult(dt).mult(1.0).div(sim.getNumeraireRandomVariable(p)).mult(w)
        under = under.add(payoff)  # callable
        # the built-in basis at the exercise date (the fixing date)
        i = int(np.searchsorted(fix, f))
        ds = sim.getForwardRate(f, f, pay[i]).mult(pay[i] - f).add(1.0).invert()
        dl = sim.getForwardRate(f, fix[i], pay[-1]).mult(pay[-1] - fix[i]).add(1.0).invert()
        basis = [F.RandomVariableGPU.constant(0.0, 1.0), ds, ds.pow(2.0), dl, dl.pow(2.0),
                 sim.getNumeraireRandomVariable(f).invert()]
        trigger = values.sub(under).getConditionalExpectation(F.MonteCarloConditionalExpectationRegression(basis))
        values = trigger.choose(values, under)
    values = values.mult(sim.getNumeraireRandomVariable(0.0)).div(w)
    fused = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, None).getValues(sim, per_path=True)
    assert values.getAverage() == pytest.approx(fused["value"], rel=1e-12)
    assert values.getStandardError() == pytest.approx(fused["error"], rel=1e-10)
    got = values.getRealizations()
    assert np.max(np.abs(got - fused["values"])) <= 1e-12 * np.max(np.abs(fused["values"]))


def test_bonds_digitals_zero_swap_and_money_market_account(lmm20):
    # Bond, LIBORBond, DigitalCaplet, DigitalFloorlet, SimpleZeroSwap and MoneyMarketAccount
    # (montecarlo/interestrate/products/) on the GPU simulation against their operations in
    # numpy on the oracle's paths
    cfg, m, osim, sim = lmm20
    P = sim.getNumberOfPaths()
    w = 1.0 / P
    N0 = osim.numeraire(0.0)
    fr = lambda t, ps, pe: _forward_rate_numpy(osim, m, cfg, "LOG_LINEAR_UNCORRECTED", t, ps, pe)
    avg = po.kahan_average

    # zero-coupon bonds: 1 / N(T), and zero once the evaluation time is past maturity
    for T in (0.5, 3.0, 10.0):
        assert F.Bond(T).getValue(sim) == pytest.approx(avg(1.0 / osim.numeraire(T) * w * N0 / w), rel=1e-12)
    assert F.Bond(3.0).getValue(sim, evaluationTime=3.5) == 0.0
    assert F.Bond(3.0).getValueRandomVariable(3.5, sim).isDeterministic()

    # LIBORBond: 1 / (1 + L(t; t, T) (T - t)) at t
    for t, T in ((0.0, 4.0), (1.0, 3.0), (1.25, 2.75)):
        o = 1.0 / (fr(t, t, T) * (T - t) + 1.0)
        assert F.LIBORBond(T).getValue(sim, evaluationTime=t) == pytest.approx(avg(o), rel=1e-12)

    # digital caplets on and off the tenor grid
    for (tm, ps, pe, K) in ((2.0, 2.0, 2.5, 0.05), (4.5, 4.5, 5.0, 0.055), (1.25, 1.25, 2.0, 0.05)):
        L = fr(tm, ps, pe)
        o = np.where(L - K >= 0, pe - ps, 0.0) / osim.numeraire(pe) * w * N0 / w
        g = F.DigitalCaplet(tm, ps, pe, K).getValueRandomVariable(0.0, sim)
        assert g.getAverage() == pytest.approx(avg(o), rel=1e-12)
        assert np.count_nonzero(g.getRealizations()) == np.count_nonzero(o)  # the same exercise set

    # digital floorlet: the reference's undiscounted payoff (its discounting results are discarded)
    L = osim.process_value(6, 6)
    o = np.where(L < 0.05, 0.5, 0.0)
    g = F.DigitalFloorlet(3.0, 0.05).getValueRandomVariable(0.0, sim)
    assert np.array_equal(g.getRealizations(), o) and g.getFiltrationTime() == 3.5
    with pytest.raises(IndexError):  # an off-tenor maturity has no period index, as in the reference
        F.DigitalFloorlet(3.2, 0.05).getValue(sim)

    # zero swap: the notional compounds by swaprate * periodLength after each period
    fixes = [2.0, 2.5, 3.0, 3.5, 4.0]
    pays = [x + 0.5 for x in fixes]
    rates = [0.05, 0.045, 0.05, 0.055, 0.05]
    for payFix in (True, False):
        o, notional = np.zeros(P), 1.0
        for fx, pm, r in zip(fixes, pays, rates):
            payoff = (fr(fx, fx, pm) - r) * (pm - fx) * notional
            if not payFix:
                payoff = payoff * -1.0
            o = o + payoff / osim.numeraire(pm) * w
            notional = notional * (r * (pm - fx))
        o = o * N0 / w
        v = F.SimpleZeroSwap(fixes, pays, rates, isPayFix=payFix).getValue(sim)
        assert v == pytest.approx(avg(o), rel=1e-12, abs=1e-13 * avg(np.abs(o)))

    # money market account: tenor-aligned accrual, and 0.75y periods whose forwards are
    # interpolated (off-tenor starts and ends, the last period cut at the evaluation time)
    for (accrual, t_eval) in ((0.5, 3.0), (0.75, 2.0)):
        o, time = np.ones(P), 0.0
        while time < t_eval:
            o = o * (1 + fr(time, time, time + accrual) * min(accrual, t_eval - time))
            time += accrual
        g = F.MoneyMarketAccount(0.0, 1.0, accrual).getValueRandomVariable(t_eval, sim).getRealizations()
        assert np.max(np.abs(g - o) / o) <= 1e-12
    assert F.MoneyMarketAccount(1.0, 1.0, 0.5).getValue(sim, evaluationTime=0.5) == 0.0
    assert F.MoneyMarketAccount().getValue(sim, evaluationTime=1.0) == 1.7976931348623157e308


# ----------------------------------------------------------------------------- date schedules
import datetime as _dt  # noqa: E402

REF_DATE = _dt.date(2026, 1, 5)
DATED = dict(curve_nodes=[0.5, 1.0, 2.0, 5.0, 40.0], curve_values=[0.03, 0.035, 0.04, 0.045, 0.045], period=0.5,
             F=3, corr_decay=0.04, abcd=(0.2, 0.1, 0.25, 0.1), seed=2718)


def dated_dates():
    """Semi-annual dates over 5 years from 2026-01-05: 181- to 184-day periods."""
    def add_months(d, k):
        y, m = divmod(d.month - 1 + k, 12)
        return d.replace(year=d.year + y, month=m + 1)
    return [add_months(REF_DATE, 6 * i) for i in range(11)]


def dated_model():
    """An LMM whose tenor and simulation times are the ACT/365 times of the dates, and whose
    forward curve carries the reference date (finmath_gb300 classes; host tables only)."""
    D = dated_dates()
    times = [F.FloatingpointDate.getFloatingPointDateFromDate(REF_DATE, d) for d in D]
    td = F.TimeDiscretizationFromArray(times)
    tenor = F.TimeDiscretizationFromArray(times)
    c = DATED
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", c["curve_nodes"],
                                                                       c["curve_values"], c["period"], REF_DATE)
    vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *c["abcd"], False)
    corr = F.LIBORCorrelationModelExponentialDecay(td, tenor, c["F"], c["corr_decay"])
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)
    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     cov, None, {})
    return td, tenor, model


def dated_oracle(td, tenor, P):
    c = DATED
    m = po.build_model(dt=0.5, T_end=5.0, period=c["period"], tenor_end=5.0, F=c["F"], corr_decay=c["corr_decay"],
                       abcd=c["abcd"], curve_nodes=c["curve_nodes"], curve_values=c["curve_values"],
                       times=td.getAsDoubleArray(), tenor=tenor.getAsDoubleArray())
    return m, po.Simulation(m, po.brownian_increments(m.times, m.F, P, c["seed"]))


@pytest.fixture(scope="module")
def dated():
    P = 2000
    td, tenor, model = dated_model()
    m, osim = dated_oracle(td, tenor, P)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, DATED["F"], P, DATED["seed"])
    sim = F.LIBORMonteCarloSimulationFromLIBORModel(F.EulerSchemeFromProcessModel(model, bm))
    return DATED, m, osim, sim


def _schedule(D, first, last, daycount):
    periods = [F.Period(D[i], D[i + 1], D[i], D[i + 1]) for i in range(first, last)]
    return F.ScheduleFromPeriods(REF_DATE, periods, daycount)


def _schedule_numpy(osim, m, cfg):
    """Forward discount bonds and analytic legs (LIBORMarketModelFromCovarianceModel.java:947-952,
    SwaptionFromSwapSchedules.java:184-218) in numpy on the oracle's paths."""
    fr = lambda t, ps, pe: _forward_rate_numpy(osim, m, cfg, "LOG_LINEAR_UNCORRECTED", t, ps, pe)
    tenor, chain = np.asarray(m.tenor), np.asarray(m.discount_chain)
    tick = 1.0 / (365.0 * 24.0)

    def zb(t):
        key = np.rint(t / tick) * tick
        i = int(np.searchsorted(tenor, key))
        if i < len(tenor) and tenor[i] == key:
            return chain[i]
        p = min(i - 1, len(tenor) - 2)
        return chain[p] * ((chain[p + 1] / chain[p]) ** ((t - tenor[p]) / (tenor[p + 1] - tenor[p])))

    def bond(t, T):
        return (zb(T) / zb(t)) * (fr(0.0, t, T) * (T - t) + 1.0) / (fr(t, t, T) * (T - t) + 1.0)

    def leg(t, sched, pays_float, fix_rate, notional):
        acc = 0.0
        for i in range(sched.getNumberOfPeriods() - 1, -1, -1):
            per = sched.getPeriod(i)
            pt = F.FloatingpointDate.getFloatingPointDateFromDate(REF_DATE, per.getPayment())
            ft = F.FloatingpointDate.getFloatingPointDateFromDate(REF_DATE, per.getFixing())
            pl = sched.getPeriodLength(i)
            pb = bond(t, pt)
            if pays_float:
                acc = acc + fr(t, ft, pt) * pl * notional * pb
            if fix_rate != 0:
                acc = acc + (fix_rate * pl * notional) * pb
        return acc

    return fr, leg


def test_swaptions_on_date_schedules(dated):
    # SwaptionFromSwapSchedules and BermudanSwaptionFromSwapSchedules on an LMM built on the
    # schedule's dates, against their operations in numpy (the regression by the oracle's
    # pinned pseudo-inverse of the same Kahan scalar products)
    cfg, m, osim, sim = dated
    D = dated_dates()
    P = sim.getNumberOfPaths()
    w = 1.0 / P
    N0 = osim.numeraire(0.0)
    fd = lambda d: F.FloatingpointDate.getFloatingPointDateFromDate(REF_DATE, d)
    fr, leg = _schedule_numpy(osim, m, cfg)
    act360, act365 = F.DayCountConvention_ACT_360(), F.DayCountConvention_ACT_365()
    assert sim.getReferenceDate() == REF_DATE
    assert act360.getDaycountFraction(D[0], D[1]) == 181 / 360.0 and act365.getDaycountFraction(D[1], D[0]) == -181 / 365.0

    # forward discount bonds P(t; T)
    for (t, T) in ((fd(D[2]), fd(D[6])), (fd(D[4]), fd(D[5])), (0.0, fd(D[3]))):
        g = sim.getForwardDiscountBond(t, T).getRealizations()
        o = (np.ones(P) * (m.discount_chain[int(np.argmin(np.abs(m.tenor - T)))] /
                           m.discount_chain[int(np.argmin(np.abs(m.tenor - t)))]))
        o = o * (fr(0.0, t, T) * (T - t) + 1.0) / (fr(t, t, T) * (T - t) + 1.0)
        assert np.max(np.abs(g - o) / o) <= 1e-12

    # European: exercise 1y into a 4y swap, fixed leg ACT/360, float leg ACT/365
    fixS, floatS = _schedule(D, 2, 10, act360), _schedule(D, 2, 10, act365)
    te = fd(D[2])
    for K, kind in ((0.04, "PAYER"), (0.045, "RECEIVER")):
        fixl, flol = leg(te, fixS, False, K, 1.0), leg(te, floatS, True, 0.0, 1.0)
        o = flol - fixl if kind == "PAYER" else fixl - flol
        o = np.maximum(o, 0.0) / osim.numeraire(te) * w * N0 / w
        g = F.SwaptionFromSwapSchedules(REF_DATE, kind, D[2], fixS, floatS, K, 1.0).getValue(sim)
        assert g == pytest.approx(po.kahan_average(o), rel=1e-12)
    with pytest.raises(ValueError):
        F.SwaptionFromSwapSchedules(REF_DATE, "STRADDLE", D[2], fixS, floatS, 0.04)

    # Bermudan: exercise at 1y, 1.5y, 2y, 2.5y into swaps ending at 5y
    ex = D[2:6]
    fixes = [_schedule(D, 2 + k, 10, act360) for k in range(4)]
    floats = [_schedule(D, 2 + k, 10, act365) for k in range(4)]
    K = 0.042
    berm = F.BermudanSwaptionFromSwapSchedules(REF_DATE, "PAYER", ex, D[10], [K] * 4, [1.0] * 4, fixes, floats)
    res = berm.getValues(0.0, sim)
    times = sorted([fd(d) for d in ex] + [fd(D[10])])
    values, ex_time = np.zeros(P), np.full(P, np.inf)
    for k in range(3, -1, -1):
        t = fd(ex[k])

        def underlying(s, pays_float, rate):
            vt = fd(s.getPeriod(0).getFixing())
            return leg(vt, s, pays_float, rate, 1.0) / osim.numeraire(vt) * w

        u = underlying(floats[k], True, 0.0) - underlying(fixes[k], False, K)
        i = times.index(t)
        df = 1.0 / osim.numeraire(t)
        X = [np.ones(P), df]
        for j in range(i, 4):
            b = leg(t, floats[j], True, 0.0, 1.0) / leg(t, fixes[j], False, 1.0, 1.0) * df
            X += [b, b * b]
        rs = fr(t, t, times[i + 1]) * df
        X += [rs, rs ** 2.0]
        y = values - u
        n = len(X)
        xtx = np.array([[po.kahan_average(X[a] * X[b]) for b in range(n)] for a in range(n)])
        beta = po.lstsq_pinv(xtx, np.array([po.kahan_average(y * X[a]) for a in range(n)]))
        ce = X[0] * beta[0]
        for a in range(1, n):
            ce = ce + X[a] * beta[a]
        values = np.where(ce >= 0, values, u)
        ex_time = np.where(ce >= 0, ex_time, t)
    values = values * N0 / w
    g_ex = res["exerciseTimes"].getRealizations()
    flips = g_ex != ex_time  # exercise decisions on regression estimates within rounding of zero
    assert flips.sum() <= 2
    g = res["values"].getRealizations()
    assert np.max(np.abs(g - values)[~flips]) <= 1e-10 * np.max(np.abs(values))
    probs = berm.getExerciseProbabilitiesFromTimes(REF_DATE, res["exerciseTimes"])
    assert sum(probs) == pytest.approx(1.0, abs=1e-15) and len(probs) == 5
    assert probs[0] == pytest.approx(np.mean(ex_time == fd(ex[0])), abs=2.0 / P)
