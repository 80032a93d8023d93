"""The float class (RandomVariableFromFloatArray) and the quantiles, on the GPU.

Expected values are restated in numpy from the reference's own loops
(montecarlo/RandomVariableFromFloatArray.java:755-1486): numpy's float32 operations are IEEE
single-precision operations rounded once each, as Java's float arithmetic, so + - * / and
everything built from them must agree bit for bit.  Square root and the transcendental
functions are FP64 functions rounded to FP32 ((float) Math.f): the GPU's and the host's FP64
libraries agree to an ulp of FP64, which after rounding to FP32 changes at most an ulp of
FP32 on a rare value.  Quantiles (RandomVariableFromDoubleArray.java:446-553) are elements of
the sorted realizations, so they must be equal exactly, on ragged sizes.
"""
import math

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300.randomvariable import RandomVariableGPU as RV
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

N = 100_003
f32 = np.float32


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(17)
    x = (rng.standard_normal(N) * 3.0).astype(f32)
    y = (rng.standard_normal(N) * 2.0 + 0.5).astype(f32)
    z = (rng.random(N) * 0.1).astype(f32)
    return x, y, z


def _eq(rv, expected):
    got = rv.getFloatRealizations()
    assert rv.isFloat()
    assert np.array_equal(got.view(np.uint32), np.asarray(expected, dtype=f32).view(np.uint32))


def test_arithmetic_is_fp32(data):
    x, y, z = data
    X, Y = RV.from_float_array(0.0, x), RV.from_float_array(0.0, y)
    with np.errstate(all="ignore"):
        _eq(X.add(Y), x + y)
        _eq(X.sub(Y), x - y)
        _eq(X.bus(Y), y - x)
        _eq(X.mult(Y), x * y)
        _eq(X.div(Y), x / y)
        _eq(X.vid(Y), y / x)
        _eq(X.add(0.1), x + f32(0.1))            # realizations[i] + (float) value (:791)
        _eq(X.mult(1.0 / 3.0), x * f32(1.0 / 3.0))
        _eq(X.squared(), x * x)
        _eq(X.invert(), f32(1.0) / x)
        _eq(X.abs(), np.abs(x))
        _eq(X.cap(Y), np.minimum(x, y))
        _eq(X.floor(0.25), np.maximum(x, f32(0.25)))
        _eq(X.accrue(RV.from_float_array(0.0, z), 0.5), x * (f32(1.0) + z * f32(0.5)))
        _eq(X.discount(RV.from_float_array(0.0, z), 0.5), x / (f32(1.0) + z * f32(0.5)))
        # a deterministic rate: mult / div by (1 + r dt) formed in double (:1277, :1305)
        _eq(X.accrue(RV.constant(0.0, 0.03), 0.5), x * f32(1.0 + 0.03 * 0.5))
        _eq(X.discount(RV.constant(0.0, 0.03), 0.5), x / f32(1.0 + 0.03 * 0.5))
        _eq(X.choose(Y, RV.from_float_array(0.0, z)), np.where(x >= 0, y, z))
        _eq(X.addProduct(Y, 0.7), x + y * f32(0.7))
        _eq(X.addProduct(Y, RV.from_float_array(0.0, z)), x + y * z)
        _eq(X.addProduct(RV.constant(0.0, 0.2), 0.7), x + f32(0.2 * 0.7))  # this.add(f1 * f2) (:1361)
        _eq(X.addRatio(Y, RV.from_float_array(0.0, z + f32(1))), x + y / (z + f32(1)))
        _eq(X.subRatio(Y, RV.from_float_array(0.0, z + f32(1))), x - y / (z + f32(1)))
        _eq(X.isNaN(), np.zeros(N, dtype=f32))


def test_functions_are_fp64_rounded_to_fp32(data):
    x, y, z = data
    X = RV.from_float_array(0.0, x)
    A = RV.from_float_array(0.0, np.abs(x) + f32(0.01))
    xd = x.astype(np.float64)
    ad = (np.abs(x) + f32(0.01)).astype(np.float64)
    for rv, ref in ((X.exp(), np.exp(xd)), (A.log(), np.log(ad)), (X.sin(), np.sin(xd)), (X.cos(), np.cos(xd)),
                    (A.sqrt(), np.sqrt(ad)), (A.pow(1.7), np.power(ad, float(f32(1.7))))):
        got = rv.getFloatRealizations().view(np.int32).astype(np.int64)
        exp = ref.astype(f32).view(np.int32).astype(np.int64)
        diff = np.abs(got - exp)
        assert np.max(diff) <= 1 and np.count_nonzero(diff) <= 1e-4 * N
    # sqrt is correctly rounded in both steps: exact
    _eq(A.sqrt(), np.sqrt(ad).astype(f32))


def test_classes_and_type_priority(data):
    x, y, _ = data
    X = RV.from_float_array(0.0, x)
    D = RV.from_array(0.0, y.astype(np.float64) * 1.1)
    # the receiver decides: a double-class receiver computes in FP64 with the floats widened
    r = D.mult(X)
    assert not r.isFloat()
    assert np.array_equal(r.getRealizations(), y.astype(np.float64) * 1.1 * x.astype(np.float64))
    # a float-class receiver reads a double operand as (float) get(i)
    _eq(X.mult(D), x * (y.astype(np.float64) * 1.1).astype(f32))
    # a deterministic double-class receiver (Scalar) hands the operation to the float class
    _eq(RV.constant(0.0, 2.0).sub(X), f32(2.0) - x)
    # floor of a deterministic float-class value: Math.max in double, then rounded (:1249)
    c = RV.constant_float(0.0, 0.1)
    _eq(c.floor(X), np.maximum(0.1, x.astype(np.float64)).astype(f32))
    _eq(c.cap(X), np.minimum(f32(0.1), x))
    # RandomVariableFromFloatArray(RandomVariable) and getRealizations (:214-228)
    _eq(D.toFloat(), (y.astype(np.float64) * 1.1).astype(f32))
    assert np.array_equal(X.getRealizations(), x.astype(np.float64))
    assert RV.constant_float(0.0, 0.5).add(0.25).isFloat()


def test_reductions_read_floats_as_doubles(data):
    x, _, _ = data
    X = RV.from_float_array(0.0, x)
    xd = x.astype(np.float64)
    assert X.getAverage() == pytest.approx(po.kahan_average(xd), rel=1e-15, abs=1e-18)
    assert X.getStandardError() == pytest.approx(po.standard_error(xd), rel=1e-12)
    assert (X.getMin(), X.getMax()) == (float(xd.min()), float(xd.max()))


def _java_round(v):
    r = math.floor(v)
    return int(r + 1 if v - r >= 0.5 else r)


def _index(n, q):
    return min(max(_java_round((n + 1) * q - 1), 0), n - 1)


def _histogram(sorted_values, points):
    out, i = [], 0
    for p in points:
        c = 0
        while i < len(sorted_values) and sorted_values[i] <= p:
            i += 1
            c += 1
        out.append(c)
    out.append(len(sorted_values) - i)
    return np.array(out, dtype=np.float64) / len(sorted_values)


@pytest.mark.parametrize("n", [1, 2, 7, 1000, N])
@pytest.mark.parametrize("cls", ["double", "float"])
def test_quantiles_and_histograms(n, cls):
    rng = np.random.default_rng(n)
    v = rng.standard_normal(n)
    if n > 10:
        v[3] = np.nan  # Arrays.sort puts NaN last
        v[5] = -0.0
    if cls == "float":
        v = v.astype(f32)
        X = RV.from_float_array(0.0, v)
    else:
        X = RV.from_array(0.0, v)
    s = np.sort(v).astype(np.float64)
    for q in (0.0, 0.1, 0.25, 1.0 / 3.0, 0.5, 0.9, 0.99, 1.0):
        got, exp = X.getQuantile(q), s[_index(n, q)]
        assert got == exp or (math.isnan(got) and math.isnan(exp))
    for qs, qe in ((0.1, 0.5), (0.9, 0.2), (0.0, 1.0 if n < 10 else 0.95)):
        a, b = sorted((qs, qe))
        i0, i1 = _index(n, a), _index(n, b)
        total = 0.0
        for k in range(i0, i1 + 1):
            total += float(s[k])
        exp = total / (i1 - i0 + 1)
        got = X.getQuantileExpectation(qs, qe)
        assert got == exp or (math.isnan(got) and math.isnan(exp))
    points = [-1.5, -0.2, 0.0, 0.3, 0.1, 2.0]
    assert np.array_equal(X.getHistogram(points), _histogram(s, points))
    anchors, hist = X.getHistogram(5, 2.0)
    assert len(anchors) == 6 and len(hist) == 6 and hist.sum() == pytest.approx(1.0)


def test_factory_makes_the_float_class():
    fac = F.RandomVariableGPUFactory(False)
    r = fac.createRandomVariable(0.0, [1.0, 2.0, 3.0])
    assert r.isFloat() and list(r.getFloatRealizations()) == [1.0, 2.0, 3.0]
    assert fac.createRandomVariable(0.25).isFloat()
    assert not F.RandomVariableGPUFactory().createRandomVariable(0.0, [1.0]).isFloat()
