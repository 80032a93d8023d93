"""The C ABI library on the CPU: loads, exports every declared symbol, host-side model
setup is identical to the oracle's, the MT19937 jump polynomials are right, and GPU
entry points fail loudly (no CPU fallback) when no GPU is present."""
import ctypes
import os
import re

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import _lib, workloads as W
from oracle import pyoracle as po
from conftest import oracle_model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include"))) if h.endswith(".h")]


def declared_functions():
    src = "".join(open(h).read() for h in HEADERS)
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(lmm_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    lib = F.load()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_lib.SIGNATURES), "every declared entry point has a ctypes signature"


def test_time_discretization_matches_oracle():
    for n, dt in ((20, 0.5), (80, 0.25), (7, 1.0 / 3.0)):
        assert np.array_equal(F.TimeDiscretizationFromArray(0.0, n, dt).getAsDoubleArray(), po.time_discretization(0.0, n, dt))


@pytest.mark.parametrize("name", ["lmm20", "lmm40"])
def test_model_tables_match_oracle_bitwise(name):
    cfg = W.WORKLOADS[name]
    m = oracle_model(cfg)
    td = F.TimeDiscretizationFromArray(0.0, m.T, cfg["dt"])
    tn = F.TimeDiscretizationFromArray(0.0, m.N, cfg["period"])
    corr = F.LIBORCorrelationModelExponentialDecay(td, tn, cfg["F"], cfg["corr_decay"])
    vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tn, *cfg["abcd"])
    cov = F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tn, vol, corr)
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("f", cfg["curve_nodes"], cfg["curve_values"], cfg["period"])
    model = F.LIBORMarketModelFromCovarianceModel.of(tn, None, curve, F.DiscountCurveFromForwardCurve(curve), None, cov)
    assert np.array_equal(corr.factorMatrix, m.factor)
    assert np.array_equal(corr.correlationMatrix, m.corr)
    assert np.array_equal(vol.volatility, m.vol)
    assert np.array_equal(cov.factorLoadings, m.loadings)
    assert np.array_equal(cov.variance, m.variance)
    assert np.array_equal(model.initialForwards, m.initial_forwards)
    assert np.array_equal(model.discountChain, m.discount_chain)


def test_factor_reduction_reproduces_pca_of_numpy():
    tn = np.arange(0, 20.5, 0.5)[:-1]
    corr = np.exp(-0.03 * np.abs(tn[:, None] - tn[None, :]))
    out = np.empty((40, 10))
    _lib.check(F.load().lmm_factor_reduction(corr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 40, 10,
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    # rows have unit length after the reduction; F F^T is the best rank-10 correlation
    assert np.allclose(np.sum(out * out, axis=1), 1.0, atol=1e-12)
    ev, V = np.linalg.eigh(corr)
    top = V[:, -10:] * np.sqrt(ev[-10:])
    top = top / np.linalg.norm(top, axis=1, keepdims=True)
    assert np.allclose(out @ out.T, top @ top.T, atol=1e-10)


@pytest.mark.parametrize("seed,skip", [(3141, 0), (3141, 1), (3141, 623), (3141, 624), (7, 99991), (7, 5_000_001),
                                       (1352, 1 << 21)])
def test_mt19937_jump_polynomials_host(seed, skip):
    out = np.empty(40, dtype=np.uint32)
    rc = F.load().lmm_mt19937_words_host(seed, skip, 40, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    assert rc == 0
    assert np.array_equal(out, po.mt_words(seed, 40, skip=skip))


@pytest.mark.parametrize("chunk", [0, 1, 7, 8, 9, 63, 64, 303, 511, 512, 777])
def test_mt19937_chunk_jumps_host(chunk):
    # the generator's chunk starts, reached by one jump per nonzero base-8 digit of the chunk
    seed, stride = 3141, 2 * 27_594
    out = np.empty(24, dtype=np.uint32)
    rc = F.load().lmm_mt19937_chunk_words_host(seed, stride, chunk, 24,
                                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    assert rc == 0
    assert np.array_equal(out, po.mt_words(seed, 24, skip=chunk * stride))


def test_invalid_arguments_are_rejected_with_messages():
    lib = F.load()
    out = np.empty(4)
    rc = lib.lmm_factor_reduction(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2, 3,
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == _lib.LMM_ERR_INVALID
    assert b"F <= n" in lib.lmm_last_error()
    h = ctypes.c_void_p()
    t = np.array([0.0, 0.5, 0.5])
    rc = lib.lmm_brownian_create(t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 3, 1, 10, 1, 0, ctypes.byref(h))
    assert rc == _lib.LMM_ERR_INVALID and b"increasing" in lib.lmm_last_error()


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_have_gpu(), reason="checks the behaviour without a GPU")
def test_gpu_entry_points_fail_loudly_without_gpu():
    with pytest.raises(F.CalculationException):
        F.mersenne_twister_uniforms(3141, 10)
    from finmath_gb300.randomvariable import RandomVariableGPU
    with pytest.raises(F.CalculationException):
        RandomVariableGPU.from_array(0.0, np.ones(8))  # realizations live in GPU memory


def test_deterministic_random_variables_on_the_host():
    # operations on deterministic random variables run on the host with the reference's
    # formulas (RandomVariableFromDoubleArray.java:743-1486): no GPU involved
    from finmath_gb300.randomvariable import RandomVariableGPU as RV
    a = RV.constant(0.5, 0.04)
    assert a.mult(0.5).add(1.0).doubleValue() == 0.04 * 0.5 + 1.0
    assert a.isDeterministic() and a.size() == 1
    assert a.getAverage() == 0.04 and a.getVariance() == 0.0 and a.getStandardError() == 0.0
    assert a.mult(RV.constant(2.0, 1.0)).getFiltrationTime() == 2.0  # the later filtration time
    # Math.min / Math.max: NaN wins, -0.0 < +0.0
    z, nz = RV.constant(0.0, 0.0), RV.constant(0.0, -0.0)
    m = z.cap(nz).doubleValue()
    assert m == 0.0 and np.signbit(m)
    M = nz.floor(z).doubleValue()
    assert M == 0.0 and not np.signbit(M)
    assert np.isnan(RV.constant(0.0, float("nan")).cap(1.0).doubleValue())
    # Math.pow's special cases where C's pow differs
    assert np.isnan(RV.constant(0.0, 1.0).pow(float("nan")).doubleValue())
    assert np.isnan(RV.constant(0.0, -1.0).pow(float("inf")).doubleValue())
    assert RV.constant(0.0, 2.0).pow(10.0).doubleValue() == 1024.0
    # ... and its exact exponents (fdlibm e_pow): +-1, 2, and 0.5 for x >= +0
    for x in (3.0, 1.0 / 3.0, 0.1, 7.25e-300, 1e300):
        r = RV.constant(0.0, x)
        assert r.pow(2.0).doubleValue() == r.squared().doubleValue() == x * x
        assert r.pow(0.5).doubleValue() == r.sqrt().doubleValue() == np.sqrt(x)
        assert r.pow(1.0).doubleValue() == x and r.pow(-1.0).doubleValue() == 1.0 / x
    p = RV.constant(0.0, -0.0).pow(0.5).doubleValue()
    assert p == 0.0 and not np.signbit(p)  # pow(-0, 0.5) = +0 where sqrt(-0) = -0
    assert np.isnan(RV.constant(0.0, -4.0).pow(0.5).doubleValue())
    assert a.accrue(RV.constant(0.0, 0.03), 0.5).doubleValue() == 0.04 * (1 + 0.03 * 0.5)
    assert a.discount(RV.constant(0.0, 0.03), 0.5).doubleValue() == 0.04 / (1.0 + 0.03 * 0.5)
    assert a.choose(RV.constant(0.0, 1.0), RV.constant(0.0, 2.0)).doubleValue() == 1.0
    assert a.addRatio(RV.constant(0.0, 1.0), RV.constant(0.0, 3.0)).doubleValue() == 0.04 + 1.0 / 3.0
    assert RV.constant(0.0, float("nan")).isNaN().doubleValue() == 1.0
    with pytest.raises(ValueError):
        a._scalar(99)  # unknown operation


def test_reference_random_variable_kats_on_deterministic_values():
    # montecarlo/RandomVariableTest.java:52-70: ((2 * 2 + 1)^2 - 4) / 7 = 3 on a deterministic value
    from finmath_gb300.randomvariable import RandomVariableGPU as RV
    r = F.RandomVariableGPUFactory().createRandomVariable(2.0)
    r = r.mult(2.0).add(1.0).squared().sub(4.0).div(7.0)
    assert r.getAverage() == 3.0 and r.getVariance() == 0.0 and r.isDeterministic()
    assert r.getFiltrationTime() == float("-inf")  # createRandomVariable(value): measurable at -infinity
    assert RV.constant(0.0, 3.0).getStandardDeviation() == 0.0


@pytest.mark.parametrize("n,rank", [(1, 1), (4, 4), (6, 6), (6, 4), (12, 9)])
def test_svd_solve_matches_the_pinned_pseudo_inverse(n, rank):
    # lmm_solve_svd: the regression's SVD solver (cutoff max(n s_max 2^-52, sqrt(2^-1022)))
    # against the oracle's pseudo-inverse, pinned by finmath's LinearAlgebraTest KATs
    rng = np.random.default_rng(n * 100 + rank)
    B = rng.normal(size=(n, rank))
    A = np.ascontiguousarray(B @ B.T + (0.0 if rank < n else 0.05) * np.eye(n))
    b = rng.normal(size=n)
    x = np.empty(n)
    dp = ctypes.POINTER(ctypes.c_double)
    assert F.load().lmm_solve_svd(n, A.ctypes.data_as(dp), b.ctypes.data_as(dp), x.ctypes.data_as(dp)) == 0
    ref = po.lstsq_pinv(A, b)
    assert np.max(np.abs(x - ref)) <= 1e-10 * max(1.0, np.max(np.abs(ref)))


def test_swaption_constructors_follow_the_reference_overloads():
    # Swaption.java:58-127: (fix, pay, periodLengths, swaprates[, notional]), (fix, pay, swaprates)
    # and (exerciseDate, swapTenor, swaprate); no GPU call
    fix, pay = [5.0, 5.5, 6.0], [5.5, 6.0, 6.5]
    a = F.Swaption(5.0, fix, pay, [0.5, 0.5, 0.5], [0.04, 0.05, 0.06], 2.0)
    assert list(a.periodLengths) == [0.5] * 3 and list(a.swaprates) == [0.04, 0.05, 0.06] and a.notional == 2.0
    b = F.Swaption(5.0, fix, pay, [0.5, 0.5, 0.5], 0.05)
    assert list(b.swaprates) == [0.05] * 3 and b.notional == 1.0
    c = F.Swaption(5.0, fix, pay, 0.05)
    assert c.periodLengths is None and list(c.swaprates) == [0.05] * 3
    d = F.Swaption(5.0, F.TimeDiscretizationFromArray(5.0, 3, 0.5), 0.05)
    assert list(d.fixingDates) == fix and list(d.paymentDates) == pay and d.periodLengths is None
    with pytest.raises(TypeError):
        F.Swaption(5.0, fix)
    with pytest.raises(ValueError):
        F.Swaption(5.0, fix, pay[:2], 0.05)


def test_unsupported_random_variable_operations_raise():
    # apply(operator) and the weighted quantile: UnsupportedOperationException / "Method not
    # implemented." in the reference's terms
    from finmath_gb300.randomvariable import RandomVariableGPU as RV
    r = RV.constant(0.0, 1.0)
    for call in (lambda: r.apply(abs), lambda: r.getQuantile(0.5, r)):
        with pytest.raises(NotImplementedError):
            call()


def test_deterministic_quantiles_and_histogram():
    # RandomVariableFromDoubleArray.java:446-553 for a deterministic value: the value itself,
    # and the reference's histogram of a 1 at the first interval point the value exceeds and a
    # 1 in the last entry (no device work)
    from finmath_gb300.randomvariable import RandomVariableGPU as RV
    r = RV.constant(0.0, 1.0)
    assert r.getQuantile(0.3) == 1.0 and r.getQuantileExpectation(0.9, 0.1) == 1.0
    assert list(r.getHistogram([2.0, 0.5, 0.0])) == [0.0, 1.0, 0.0, 1.0]
    assert list(r.getHistogram([])) == [1.0]
    f = RV.constant_float(0.0, 2.5)
    assert f.isFloat() and f.isDeterministic() and f.getQuantile(0.5) == 2.5
