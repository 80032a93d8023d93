"""Device random variables with finmath-lib's RandomVariable API (include/lmm_rv.h).

RandomVariableGPU mirrors net.finmath.stochastic.RandomVariable as implemented by
RandomVariableFromDoubleArray (montecarlo/RandomVariableFromDoubleArray.java): immutable,
deterministic or with n FP64 realizations (here in GPU memory), a filtration time, and
operations that return new random variables.  RandomVariableGPUFactory mirrors
RandomVariableFactory.createRandomVariable (RandomVariableFactory.java:56-94).  Every
operation runs in liblmm_gb300.so; realizations reach the host only through
getRealizations() and the reductions.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, load

ADD, SUB, BUS, MULT, DIV, VID, CAP, FLOOR, POW = 0, 1, 2, 3, 4, 5, 6, 7, 8
SQUARED, SQRT, EXP, LOG, SIN, COS, INVERT, ABS, ISNAN, EXPM1 = 16, 17, 18, 19, 20, 21, 22, 23, 24, 25
ACCRUE, DISCOUNT, CHOOSE, ADD_PRODUCT, ADD_RATIO, SUB_RATIO = 32, 33, 34, 35, 36, 37


class RandomVariableGPU:
    """One deterministic value or n realizations in GPU memory (owned; freed on close)."""

    def __init__(self, handle):
        self._L = load()
        self._h = handle

    # -- construction
    @classmethod
    def constant(cls, time: float, value: float) -> "RandomVariableGPU":
        h = ctypes.c_void_p()
        check(load().lmm_rv_create_constant(float(time), float(value), ctypes.byref(h)), "createRandomVariable")
        return cls(h)

    @classmethod
    def from_array(cls, time: float, values) -> "RandomVariableGPU":
        a = np.ascontiguousarray(values, dtype=np.float64)
        h = ctypes.c_void_p()
        check(load().lmm_rv_create(float(time), a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size,
                                   ctypes.byref(h)), "createRandomVariable")
        return cls(h)

    @classmethod
    def from_float_array(cls, time: float, values) -> "RandomVariableGPU":
        """RandomVariableFromFloatArray(time, float[]): FP32 realizations of the float class."""
        a = np.ascontiguousarray(values, dtype=np.float32)
        h = ctypes.c_void_p()
        check(load().lmm_rv_create_float(float(time), a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.size,
                                         ctypes.byref(h)), "createRandomVariable")
        return cls(h)

    @classmethod
    def constant_float(cls, time: float, value: float) -> "RandomVariableGPU":
        """RandomVariableFromFloatArray(time, value): a deterministic value of the float class."""
        h = ctypes.c_void_p()
        check(load().lmm_rv_create_constant_float(float(time), float(value), ctypes.byref(h)), "createRandomVariable")
        return cls(h)

    def toFloat(self) -> "RandomVariableGPU":
        """RandomVariableFromFloatArray(RandomVariable): the realizations rounded to FP32."""
        h = ctypes.c_void_p()
        check(self._L.lmm_rv_to_float(self._h, ctypes.byref(h)), "RandomVariableFromFloatArray")
        return RandomVariableGPU(h)

    def isFloat(self) -> bool:
        out = ctypes.c_int()
        check(self._L.lmm_rv_is_float(self._h, ctypes.byref(out)), "isFloat")
        return bool(out.value)

    def getFloatRealizations(self) -> np.ndarray:
        t, n, det, v = self._describe()
        out = np.empty(n, dtype=np.float32)
        check(self._L.lmm_rv_get_float(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
              "getRealizations")
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._L.lmm_rv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown: the library may already be unloaded
            pass

    # -- description
    def _describe(self):
        t, n, det, v = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_double()
        check(self._L.lmm_rv_describe(self._h, ctypes.byref(t), ctypes.byref(n), ctypes.byref(det), ctypes.byref(v)),
              "describe")
        return t.value, n.value, bool(det.value), v.value

    def getFiltrationTime(self) -> float:
        return self._describe()[0]

    def isDeterministic(self) -> bool:
        return self._describe()[2]

    def size(self) -> int:
        t, n, det, v = self._describe()
        return 1 if det else n

    def doubleValue(self) -> float:
        t, n, det, v = self._describe()
        if not det:
            raise RuntimeError("doubleValue of a stochastic random variable")
        return v

    def getRealizations(self) -> np.ndarray:
        t, n, det, v = self._describe()
        out = np.empty(1 if det else n)
        check(self._L.lmm_rv_get(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "getRealizations")
        return out

    def get(self, i: int) -> float:
        return float(self.getRealizations()[0 if self.isDeterministic() else i])

    # -- reductions
    def _reduce(self, fn) -> float:
        out = ctypes.c_double()
        check(fn(self._h, ctypes.byref(out)), "reduction")
        return out.value

    def getAverage(self) -> float:
        return self._reduce(self._L.lmm_rv_average)

    def getVariance(self) -> float:
        return self._reduce(self._L.lmm_rv_variance)

    def getStandardDeviation(self) -> float:
        return float(np.sqrt(self.getVariance()))

    def getStandardError(self) -> float:
        return self._reduce(self._L.lmm_rv_standard_error)

    def _minmax(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        check(self._L.lmm_rv_min_max(self._h, ctypes.byref(a), ctypes.byref(b)), "getMin/getMax")
        return a.value, b.value

    def getMin(self) -> float:
        return self._minmax()[0]

    def getMax(self) -> float:
        return self._minmax()[1]

    def average(self) -> "RandomVariableGPU":
        return RandomVariableGPU.constant(0.0, self.getAverage())

    def apply(self, operator, *arguments):
        """apply(DoubleUnaryOperator / DoubleBinaryOperator / DoubleTernaryOperator): a host
        function cannot run on the device; unsupported, as the reference's own tests allow
        (RandomVariableTest.java:233-272 accept UnsupportedOperationException)."""
        raise NotImplementedError("apply(operator) is not supported on device random variables")

    def getQuantile(self, quantile, probabilities=None) -> float:
        """getQuantile (RandomVariableFromDoubleArray.java:446-460): the sorted realizations'
        element at (int) Math.round((n + 1) quantile - 1), clamped; sorted on the device.
        The weighted form is not implemented in the reference either (:463-472)."""
        if probabilities is not None:
            raise NotImplementedError("Method not implemented.")
        return self._reduce(lambda h, out: self._L.lmm_rv_quantile(h, float(quantile), out))

    def getQuantileExpectation(self, quantileStart, quantileEnd) -> float:
        """getQuantileExpectation (:475-499): the mean of the sorted realizations between the
        two quantiles' indices."""
        return self._reduce(lambda h, out: self._L.lmm_rv_quantile_expectation(h, float(quantileStart),
                                                                                float(quantileEnd), out))

    def getHistogram(self, intervalPoints, standardDeviations=None):
        """getHistogram(double[] intervalPoints) (:502-553): the share of realizations in each
        interval, numberOfPoints + 1 entries; getHistogram(int numberOfPoints, double
        standardDeviations) (:556-575): interval points spread standardDeviations standard
        deviations around the mean, returned with their anchor points as [anchors, histogram]."""
        if standardDeviations is not None:
            numberOfPoints = int(intervalPoints)
            center, radius = self.getAverage(), standardDeviations * self.getStandardDeviation()
            stepSize = (numberOfPoints - 1) / 2.0
            points, anchors = np.empty(numberOfPoints), np.empty(numberOfPoints + 1)
            for i in range(numberOfPoints):
                alpha = (-float(numberOfPoints - 1) / 2.0 + i) / stepSize
                points[i] = center + alpha * radius
                anchors[i] = center + alpha * radius - radius / (2 * stepSize)
            anchors[numberOfPoints] = center + 1 * radius + radius / (2 * stepSize)
            return [anchors, self.getHistogram(points)]
        p = np.ascontiguousarray(intervalPoints, dtype=np.float64)
        out = np.empty(p.size + 1)
        dp = ctypes.POINTER(ctypes.c_double)
        check(self._L.lmm_rv_histogram(self._h, p.ctypes.data_as(dp), p.size, out.ctypes.data_as(dp)), "getHistogram")
        return out

    def getConditionalExpectation(self, conditionalExpectationOperator):
        """RandomVariableFromDoubleArray.getConditionalExpectation: the estimator's estimate of this."""
        return conditionalExpectationOperator.getConditionalExpectation(self)

    # -- operations
    def _scalar(self, op, y=0.0) -> "RandomVariableGPU":
        h = ctypes.c_void_p()
        check(self._L.lmm_rv_apply_scalar(self._h, op, float(y), ctypes.byref(h)), "operation")
        return RandomVariableGPU(h)

    def _binary(self, op, y) -> "RandomVariableGPU":
        if not isinstance(y, RandomVariableGPU):
            return self._scalar(op, y)
        h = ctypes.c_void_p()
        check(self._L.lmm_rv_apply(self._h, op, y._h, ctypes.byref(h)), "operation")
        return RandomVariableGPU(h)

    def _ternary(self, op, a, b=None, c=0.0) -> "RandomVariableGPU":
        a = _as_rv(a)
        b = None if b is None else _as_rv(b)
        h = ctypes.c_void_p()
        check(self._L.lmm_rv_apply3(self._h, op, a._h, None if b is None else b._h, float(c), ctypes.byref(h)),
              "operation")
        return RandomVariableGPU(h)

    def add(self, y): return self._binary(ADD, y)
    def sub(self, y): return self._binary(SUB, y)
    def bus(self, y): return self._binary(BUS, y)
    def mult(self, y): return self._binary(MULT, y)
    def div(self, y): return self._binary(DIV, y)
    def vid(self, y): return self._binary(VID, y)
    def cap(self, y): return self._binary(CAP, y)
    def floor(self, y): return self._binary(FLOOR, y)
    def pow(self, exponent: float): return self._scalar(POW, exponent)
    def squared(self): return self._scalar(SQUARED)
    def sqrt(self): return self._scalar(SQRT)
    def exp(self): return self._scalar(EXP)
    def expm1(self): return self._scalar(EXPM1)
    def log(self): return self._scalar(LOG)
    def sin(self): return self._scalar(SIN)
    def cos(self): return self._scalar(COS)
    def invert(self): return self._scalar(INVERT)
    def abs(self): return self._scalar(ABS)
    def isNaN(self): return self._scalar(ISNAN)
    def accrue(self, rate, periodLength: float): return self._ternary(ACCRUE, rate, None, periodLength)
    def discount(self, rate, periodLength: float): return self._ternary(DISCOUNT, rate, None, periodLength)

    def choose(self, valueIfTriggerNonNegative, valueIfTriggerNegative):
        return self._ternary(CHOOSE, valueIfTriggerNonNegative, valueIfTriggerNegative)

    def addProduct(self, factor1, factor2):
        if isinstance(factor2, RandomVariableGPU):
            return self._ternary(ADD_PRODUCT, factor1, factor2)
        return self._ternary(ADD_PRODUCT, factor1, None, factor2)

    def addRatio(self, numerator, denominator): return self._ternary(ADD_RATIO, numerator, denominator)
    def subRatio(self, numerator, denominator): return self._ternary(SUB_RATIO, numerator, denominator)

    # Python operators (the same operations)
    __add__ = add
    __sub__ = sub
    __mul__ = mult
    __truediv__ = div
    def __radd__(self, y): return self.add(y)
    def __rsub__(self, y): return self.bus(y)
    def __rmul__(self, y): return self.mult(y)
    def __rtruediv__(self, y): return self.vid(y)
    def __neg__(self): return self.mult(-1.0)


def _as_rv(x) -> RandomVariableGPU:
    return x if isinstance(x, RandomVariableGPU) else RandomVariableGPU.constant(0.0, float(x))


class RandomVariableGPUFactory:
    """RandomVariableFactory.createRandomVariable (RandomVariableFactory.java:56-94) on the GPU;
    like RandomVariableFromArrayFactory(isUseDoublePrecisionFloatingPointImplementation)
    (RandomVariableFromArrayFactory.java:37-60) it makes double-class random variables, or
    float-class ones (RandomVariableFromFloatArray) when that flag is False."""

    def __init__(self, isUseDoublePrecisionFloatingPointImplementation: bool = True):
        self.isUseDoublePrecisionFloatingPointImplementation = bool(isUseDoublePrecisionFloatingPointImplementation)

    def createRandomVariable(self, *args) -> RandomVariableGPU:
        if len(args) == 1:  # AbstractRandomVariableFactory.java:22-24: measurable at -infinity
            time, value = float("-inf"), args[0]
        else:
            time, value = args
        double = self.isUseDoublePrecisionFloatingPointImplementation
        if np.ndim(value) == 0:
            return RandomVariableGPU.constant(time, value) if double else RandomVariableGPU.constant_float(time, value)
        return RandomVariableGPU.from_array(time, value) if double else RandomVariableGPU.from_float_array(time, value)


class MonteCarloConditionalExpectationRegression:
    """MonteCarloConditionalExpectationRegression (montecarlo/conditionalexpectation/
    MonteCarloConditionalExpectationRegression.java:79-150) over device random variables: the
    scalar products X^T X and X^T y as compensated averages of products on the GPU, the
    small system solved by the library's SVD pseudo-inverse (lmm_solve_svd, the reference's
    commons-math solver and cutoff), and the estimate X beta as the reference builds it
    (mult, then addProduct per basis function)."""

    def __init__(self, basisFunctions, basisFunctionsPredictor=None):
        self._est = [b for b in basisFunctions if b is not None]
        self._pred = self._est if basisFunctionsPredictor is None else [b for b in basisFunctionsPredictor if b is not None]
        self._xtx = None

    def getLinearRegressionParameters(self, dependents: "RandomVariableGPU") -> np.ndarray:
        b = self._est
        n = len(b)
        if self._xtx is None:  # the reference caches its solver per estimator
            xtx = np.empty((n, n))
            for i in range(n):
                for j in range(i, n):
                    prod = b[i].mult(b[j])
                    xtx[i, j] = xtx[j, i] = prod.getAverage()
                    prod.close()
            self._xtx = np.ascontiguousarray(xtx)
        xty = np.empty(n)
        for i in range(n):
            prod = dependents.mult(b[i])
            xty[i] = prod.getAverage()
            prod.close()
        x = np.empty(n)
        dp = ctypes.POINTER(ctypes.c_double)
        check(load().lmm_solve_svd(n, self._xtx.ctypes.data_as(dp), xty.ctypes.data_as(dp), x.ctypes.data_as(dp)),
              "getLinearRegressionParameters")
        return x

    def getConditionalExpectation(self, randomVariable: "RandomVariableGPU") -> "RandomVariableGPU":
        beta = self.getLinearRegressionParameters(randomVariable)
        ce = self._pred[0].mult(float(beta[0]))
        for i in range(1, len(self._pred)):
            ce = ce.addProduct(self._pred[i], float(beta[i]))
        return ce
