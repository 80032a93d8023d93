"""Host-side mirror of finmath-lib's API for the LIBOR Market Model Monte Carlo path.

Class and method names follow finmath-lib (src/main/java/net/finmath/...), so code and
tests read like the reference's: build a TimeDiscretizationFromArray, a covariance model,
LIBORMarketModelFromCovarianceModel.of(...), a BrownianMotionFromMersenneRandomNumbers,
an EulerSchemeFromProcessModel, wrap it in LIBORMonteCarloSimulationFromLIBORModel and
ask products for getValue(model).  Every numeric step runs in liblmm_gb300.so: host
setup in its C++ part, simulation and valuation in its CUDA kernels.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import check

_D = ctypes.POINTER(ctypes.c_double)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return None if a is None else a.ctypes.data_as(_D)


# --------------------------------------------------------------------------- time
class TimeDiscretizationFromArray:
    """net.finmath.time.TimeDiscretizationFromArray (tick-rounded, sorted)."""

    def __init__(self, initial_or_times, numberOfTimeSteps: int | None = None, deltaT: float | None = None):
        L = _lib.load()
        if numberOfTimeSteps is None:
            t = np.unique(np.asarray([np.rint(x / (1.0 / (365.0 * 24.0))) * (1.0 / (365.0 * 24.0))
                                      for x in initial_or_times], dtype=np.float64))
            self._t = t
        else:
            out = np.empty(numberOfTimeSteps + 1)
            check(L.lmm_time_discretization(float(initial_or_times), int(numberOfTimeSteps), float(deltaT), _p(out)),
                  "TimeDiscretizationFromArray")
            self._t = out

    def getNumberOfTimes(self):
        return len(self._t)

    def getNumberOfTimeSteps(self):
        return len(self._t) - 1

    def getTime(self, i):
        if i < 0:  # Java arrays do not wrap
            raise IndexError(f"time index {i} out of range")
        return float(self._t[i])

    def getTimeStep(self, i):
        return float(self._t[i + 1] - self._t[i])

    def getTimeIndex(self, time: float) -> int:
        key = np.rint(time / (1.0 / (365.0 * 24.0))) * (1.0 / (365.0 * 24.0))
        i = int(np.searchsorted(self._t, key))
        if i < len(self._t) and self._t[i] == key:
            return i
        return -(i + 1)

    def getAsDoubleArray(self):
        return self._t.copy()


# --------------------------------------------------------------------------- curves
class ForwardCurveInterpolation:
    """ForwardCurveInterpolation with LINEAR interpolation on values, CONSTANT extrapolation."""

    def __init__(self, name, times, forwards, paymentOffset, referenceDate=None):
        self.name = name
        self.times = _f64(times)
        self.forwards = _f64(forwards)
        self.paymentOffset = float(paymentOffset)
        self.referenceDate = referenceDate  # a datetime.date, or None

    @staticmethod
    def createForwardCurveFromForwards(name, times, givenForwards, paymentOffset, referenceDate=None):
        return ForwardCurveInterpolation(name, times, givenForwards, paymentOffset, referenceDate)

    def getReferenceDate(self):
        return self.referenceDate

    def getPaymentOffset(self, fixingTime=None):
        return self.paymentOffset

    def getForward(self, model, fixingTime, paymentOffset=None):
        out = ctypes.c_double()
        check(_lib.load().lmm_forward_curve_value(_p(self.times), _p(self.forwards), len(self.times), float(fixingTime),
                                                  ctypes.byref(out)), "getForward")
        f = out.value
        if paymentOffset is not None and paymentOffset != self.paymentOffset:
            po = self.paymentOffset
            f = (np.exp(np.log(1 + f * po) * paymentOffset / po) - 1.0) / paymentOffset
        return f


class DiscountCurveFromForwardCurve:
    def __init__(self, forwardCurve: ForwardCurveInterpolation):
        self.forwardCurve = forwardCurve

    def getDiscountFactor(self, model, maturity=None):
        if maturity is None:
            maturity = model
        c = self.forwardCurve
        out = ctypes.c_double()
        check(_lib.load().lmm_discount_factor_from_forward_curve(_p(c.times), _p(c.forwards), len(c.times),
                                                                  c.paymentOffset, float(maturity), ctypes.byref(out)),
              "getDiscountFactor")
        return out.value


# --------------------------------------------------------------------------- covariance
class LIBORCorrelationModelExponentialDecay:
    def __init__(self, timeDiscretization, liborPeriodDiscretization, numberOfFactors, a, isCalibrateable=False):
        self.timeDiscretization, self.liborPeriodDiscretization = timeDiscretization, liborPeriodDiscretization
        self.numberOfFactors, self.a, self.isCalibrateable = int(numberOfFactors), float(a), bool(isCalibrateable)
        tenor = liborPeriodDiscretization.getAsDoubleArray()
        N = len(tenor) - 1
        self.factorMatrix = np.empty((N, numberOfFactors))
        self.correlationMatrix = np.empty((N, N))
        check(_lib.load().lmm_correlation_exponential_decay(_p(_f64(tenor)), N, int(numberOfFactors), float(a),
                                                           _p(self.factorMatrix), _p(self.correlationMatrix)),
              "LIBORCorrelationModelExponentialDecay")

    def getNumberOfFactors(self):
        return self.factorMatrix.shape[1]

    def getFactorLoading(self, timeIndex, factor, component):
        return float(self.factorMatrix[component, factor])

    def getCorrelation(self, timeIndex, component1, component2):
        return float(self.correlationMatrix[component1, component2])

    def getParameter(self):
        """LIBORCorrelationModelExponentialDecay.java:137-147: [a] when calibrateable, else None."""
        return [self.a] if self.isCalibrateable else None

    def getCloneWithModifiedParameter(self, parameter):
        """:74-80: the same model for an unchanged a; else a new, non-calibrateable one (the
        reference's four-argument constructor)."""
        if not self.isCalibrateable or self.a == float(parameter[0]):
            return self
        return LIBORCorrelationModelExponentialDecay(self.timeDiscretization, self.liborPeriodDiscretization,
                                                     self.numberOfFactors, float(parameter[0]), False)


class LIBORVolatilityModelFourParameterExponentialForm:
    def __init__(self, timeDiscretization, liborPeriodDiscretization, a, b, c, d, isCalibrateable=False):
        self.timeDiscretization, self.liborPeriodDiscretization = timeDiscretization, liborPeriodDiscretization
        self.a, self.b, self.c, self.d = float(a), float(b), float(c), float(d)
        self.isCalibrateable = bool(isCalibrateable)
        t = _f64(timeDiscretization.getAsDoubleArray())
        tn = _f64(liborPeriodDiscretization.getAsDoubleArray())
        T, N = len(t) - 1, len(tn) - 1
        self.volatility = np.empty((T, N))
        check(_lib.load().lmm_volatility_four_parameter(_p(t), T, _p(tn), N, float(a), float(b), float(c), float(d),
                                                       _p(self.volatility)), "LIBORVolatilityModelFourParameterExponentialForm")

    def getVolatility(self, timeIndex, liborIndex):
        return float(self.volatility[timeIndex, liborIndex])

    def getParameter(self):
        """LIBORVolatilityModelFourParameterExponentialForm.java:135-147: [a, b, c, d] when calibrateable."""
        return [self.a, self.b, self.c, self.d] if self.isCalibrateable else None

    def getCloneWithModifiedParameter(self, parameter):
        """:150-162: a calibrateable clone with the new a, b, c, d."""
        if not self.isCalibrateable:
            return self
        return LIBORVolatilityModelFourParameterExponentialForm(self.timeDiscretization, self.liborPeriodDiscretization,
                                                                *[float(x) for x in parameter[:4]], True)


class LIBORVolatilityModelFromGivenMatrix:
    def __init__(self, timeDiscretization, liborPeriodDiscretization, volatility):
        self.volatility = _f64(volatility)

    def getParameter(self):
        return None  # a given matrix is not calibrated on this path

    def getVolatility(self, timeIndex, liborIndex):
        return float(self.volatility[timeIndex, liborIndex])


class LIBORCovarianceModelFromVolatilityAndCorrelation:
    def __init__(self, timeDiscretization, liborPeriodDiscretization, volatilityModel, correlationModel):
        vol = _f64(volatilityModel.volatility)
        fm = _f64(correlationModel.factorMatrix)
        corr = _f64(correlationModel.correlationMatrix)
        T, N = vol.shape
        F = fm.shape[1]
        self.factorLoadings = np.empty((T, N, F))
        self.variance = np.empty((T, N))
        check(_lib.load().lmm_covariance_tables(T, N, F, _p(vol), _p(fm), _p(corr), _p(self.factorLoadings),
                                               _p(self.variance)), "LIBORCovarianceModelFromVolatilityAndCorrelation")
        self.timeDiscretization = timeDiscretization
        self.liborPeriodDiscretization = liborPeriodDiscretization
        self.volatility = vol
        self.volatilityModel, self.correlationModel = volatilityModel, correlationModel

    def getNumberOfFactors(self):
        return self.factorLoadings.shape[2]

    def getVolatilityModel(self):
        return self.volatilityModel

    def getCorrelationModel(self):
        return self.correlationModel

    def getParameter(self):
        """LIBORCovarianceModelFromVolatilityAndCorrelation.java:96-117: the volatility model's
        parameters followed by the correlation model's (each only when calibrateable)."""
        out = []
        for m in (self.volatilityModel, self.correlationModel):
            p = m.getParameter() if hasattr(m, "getParameter") else None
            out += list(p or [])
        return out

    def getParameterAsDouble(self):
        return np.asarray(self.getParameter(), dtype=np.float64)

    def getCloneWithModifiedParameters(self, parameters):
        """:143-169: the parameters split between the volatility and correlation models; a model
        whose parameters did not change is kept."""
        parameters = [float(x) for x in parameters]
        vol, corr, i = self.volatilityModel, self.correlationModel, 0
        vp = vol.getParameter() if hasattr(vol, "getParameter") else None
        cp = corr.getParameter() if hasattr(corr, "getParameter") else None
        if vp is not None:
            new = parameters[i:i + len(vp)]
            i += len(vp)
            if new != list(vp):
                vol = vol.getCloneWithModifiedParameter(new)
        if cp is not None:
            new = parameters[i:i + len(cp)]
            i += len(cp)
            if new != list(cp):
                corr = corr.getCloneWithModifiedParameter(new)
        return LIBORCovarianceModelFromVolatilityAndCorrelation(self.timeDiscretization, self.liborPeriodDiscretization,
                                                                vol, corr)

    def getCloneCalibrated(self, calibrationModel, calibrationProducts, calibrationParameters=None):
        """AbstractLIBORCovarianceModelParametric.getCloneCalibrated (:150-315, its Levenberg-Marquardt
        branch :333-460): see finmath_gb300.calibration."""
        from .calibration import calibrate_covariance_model
        return calibrate_covariance_model(self, calibrationModel, calibrationProducts, calibrationParameters)

    def getFactorLoading(self, timeIndex, component):
        return self.factorLoadings[timeIndex, component].copy()

    def getCovariance(self, timeIndex, component1, component2):
        if component1 != component2:
            return float(np.dot(self.factorLoadings[timeIndex, component1], self.factorLoadings[timeIndex, component2]))
        return float(self.variance[timeIndex, component1])


class LIBORCovarianceModelExponentialForm5Param(LIBORCovarianceModelFromVolatilityAndCorrelation):
    """covariance/LIBORCovarianceModelExponentialForm5Param.java: the four-parameter
    exponential volatility (a, b, c, d) on the simulation and tenor grids and the
    exponential-decay correlation (decay e) on the tenor grid, reduced to numberOfFactors;
    all five parameters calibrateable (default 0.20, 0.05, 0.10, 0.20, 0.10)."""

    def __init__(self, timeDiscretization, liborPeriodDiscretization, numberOfFactors,
                 parameters=(0.20, 0.05, 0.10, 0.20, 0.10)):
        p = [float(x) for x in parameters]
        if len(p) != 5:
            raise ValueError("LIBORCovarianceModelExponentialForm5Param takes five parameters")
        vol = LIBORVolatilityModelFourParameterExponentialForm(timeDiscretization, liborPeriodDiscretization, *p[:4],
                                                               False)
        corr = LIBORCorrelationModelExponentialDecay(liborPeriodDiscretization, liborPeriodDiscretization,
                                                     int(numberOfFactors), p[4], False)
        super().__init__(timeDiscretization, liborPeriodDiscretization, vol, corr)
        self.parameter = p
        self.numberOfFactors = int(numberOfFactors)

    def getParameter(self):
        return list(self.parameter)

    def getParameterAsDouble(self):
        return np.asarray(self.parameter, dtype=np.float64)

    def getCloneWithModifiedParameters(self, parameters):
        return LIBORCovarianceModelExponentialForm5Param(self.timeDiscretization, self.liborPeriodDiscretization,
                                                         self.numberOfFactors, parameters)


# --------------------------------------------------------------------------- model
class LIBORMarketModelFromCovarianceModel:
    """The model's tables as finmath-lib evaluates them (LIBORMarketModelFromCovarianceModel.java:388-444)."""

    MEASURE_SPOT = "SPOT"
    MEASURE_TERMINAL = "TERMINAL"
    STATE_LOGNORMAL = "LOGNORMAL"
    STATE_NORMAL = "NORMAL"

    def __init__(self, liborPeriodDiscretization, analyticModel, forwardRateCurve, discountCurve, randomVariableFactory,
                 covarianceModel, calibrationItems=None, properties=None):
        props = dict(properties or {})
        measures = {"SPOT": _lib.MEASURE_SPOT, "TERMINAL": _lib.MEASURE_TERMINAL}
        spaces = {"LOGNORMAL": _lib.STATE_SPACE_LOGNORMAL, "NORMAL": _lib.STATE_SPACE_NORMAL}
        m, sp = str(props.get("measure", "SPOT")).upper(), str(props.get("stateSpace", "LOGNORMAL")).upper()
        if m not in measures:
            raise ValueError(f"measure {m} is not implemented on this path")
        if sp not in spaces:
            raise ValueError(f"state space {sp} is not implemented on this path")
        self.measure, self.stateSpace = measures[m], spaces[sp]
        if calibrationItems:
            raise ValueError("calibrating models are built by LIBORMarketModelFromCovarianceModel.of(...)")
        self._args = (liborPeriodDiscretization, analyticModel, forwardRateCurve, discountCurve, randomVariableFactory)
        self.properties = props
        self.liborPeriodDiscretization = liborPeriodDiscretization
        self.forwardRateCurve = forwardRateCurve
        self.discountCurve = discountCurve
        self.covarianceModel = covarianceModel
        self.liborCap = float(props.get("liborCap", 1e5))
        # getForwardRate's tenor interpolation and simulation-time rounding (:191-192, :407-410)
        self.interpolationMethod = str(props.get("interpolationMethod", "LOG_LINEAR_UNCORRECTED")).upper()
        self.simulationTimeInterpolationMethod = str(props.get("simulationTimeInterpolationMethod",
                                                               "ROUND_NEAREST")).upper()
        tenor = liborPeriodDiscretization.getAsDoubleArray()
        N = len(tenor) - 1
        # getInitialState (:1081-1093): forward over [T_j, T_j + delta_j]
        self.initialForwards = np.array([forwardRateCurve.getForward(None, tenor[j], tenor[j + 1] - tenor[j])
                                         for j in range(N)])
        self.discountChain = None
        if discountCurve is not None:
            df = _f64([discountCurve.getDiscountFactor(None, t) for t in tenor])
            self.discountChain = np.empty(N + 1)
            check(_lib.load().lmm_numeraire_discount_chain(_p(_f64(tenor)), N, _p(df), _p(self.discountChain)),
                  "numeraire adjustment")

    @staticmethod
    def of(liborPeriodDiscretization, analyticModel, forwardRateCurve, discountCurve, randomVariableFactory,
           covarianceModel, calibrationItems=None, properties=None):
        """:270-322: the model, calibrated first when calibration products are given (the
        covariance model must be calibrateable; properties["calibrationParameters"] as in the
        reference: numberOfPaths, seed, maxIterations, accuracy, parameterStep, brownianMotion)."""
        model = LIBORMarketModelFromCovarianceModel(liborPeriodDiscretization, analyticModel, forwardRateCurve,
                                                    discountCurve, randomVariableFactory, covarianceModel, None,
                                                    properties)
        if not calibrationItems:
            return model
        if not hasattr(covarianceModel, "getCloneCalibrated"):
            raise TypeError("Calibration restricted to covariance models implementing LIBORCovarianceModelCalibrateable.")
        calibrationParameters = (properties or {}).get("calibrationParameters")
        calibrated = covarianceModel.getCloneCalibrated(model, calibrationItems, calibrationParameters)
        return model.getCloneWithModifiedCovarianceModel(calibrated)

    def getCovarianceModel(self):
        return self.covarianceModel

    def getIntegratedLIBORCovariance(self, simulationTimeDiscretization):
        """LIBORMarketModelFromCovarianceModel.getIntegratedLIBORCovariance (:1552-1596):
        [t][i][j] = the sum over simulation steps up to t of lambda_i . lambda_j dt, each step
        counting only components not yet fixed (T_i above the step's start); the upper
        triangle of step 0 and both triangles after it, as the reference fills them.  The
        reference caches the result in the model; so does this class, per simulation grid.
        Each step's sums run over the factors in the reference's order ((l_ik l_jk) dt added
        factor by factor), vectorised over the component pairs."""
        key = tuple(float(x) for x in simulationTimeDiscretization.getAsDoubleArray())
        cache = self.__dict__.setdefault("_integratedLIBORCovariance", {})
        if key in cache:
            return cache[key]
        cov = self.covarianceModel
        tenor = self.liborPeriodDiscretization
        n, N = simulationTimeDiscretization.getNumberOfTimeSteps(), tenor.getNumberOfTimeSteps()
        tenorTimes = np.array([tenor.getTime(i) for i in range(N)])
        upper = np.triu(np.ones((N, N), dtype=bool))
        out = np.zeros((n, N, N))
        for t in range(n):
            time = simulationTimeDiscretization.getTime(t)
            dt = simulationTimeDiscretization.getTime(t + 1) - time
            ct = cov.timeDiscretization.getTimeIndex(time)
            ct = ct if ct >= 0 else -ct - 2
            if ct < 0 or ct >= cov.factorLoadings.shape[0]:
                # the reference's factor-loading lookup throws outside the covariance grid
                raise ValueError(f"simulation time {time} outside the covariance model's time discretization")
            loadings = np.asarray(cov.factorLoadings[ct], dtype=np.float64)
            acc = np.zeros((N, N))
            for k in range(loadings.shape[1]):
                acc = acc + (loadings[:, None, k] * loadings[None, :, k]) * dt
            alive = (tenorTimes > time)[:, None] & upper
            out[t] = np.where(alive, acc, 0.0)
        for t in range(1, n):
            u = out[t - 1] + out[t]
            out[t] = np.where(upper, u, u.T)
        cache[key] = out
        return out

    def getCloneWithModifiedCovarianceModel(self, covarianceModel):
        """:1646-1650: the same model with another covariance model."""
        clone = LIBORMarketModelFromCovarianceModel(*self._args, covarianceModel, None, self.properties)
        clone.interpolationMethod = self.interpolationMethod
        clone.simulationTimeInterpolationMethod = self.simulationTimeInterpolationMethod
        return clone

    def getNumberOfComponents(self):
        return self.liborPeriodDiscretization.getNumberOfTimeSteps()

    def getReferenceDate(self):
        """The forward curve's reference date (LIBORMarketModelFromCovarianceModel.java:844-846)."""
        return self.forwardRateCurve.getReferenceDate() if self.forwardRateCurve is not None else None

    def getNumeraireDefaultableZeroBondAsOfTimeZero(self, time):
        """The deterministic numeraire adjustment at time (:883-943): the discount-curve chain at
        a tenor date, interpolated geometrically between tenor dates."""
        if self.discountChain is None:
            raise ValueError("the numeraire adjustment needs the model's discount curve")
        tenor = self.liborPeriodDiscretization
        i = tenor.getTimeIndex(time)
        if i >= 0:
            return float(self.discountChain[i])
        prev = min(-i - 2, tenor.getNumberOfTimes() - 2)
        t0, t1 = tenor.getTime(prev), tenor.getTime(prev + 1)
        a0, a1 = float(self.discountChain[prev]), float(self.discountChain[prev + 1])
        return a0 * ((a1 / a0) ** ((time - t0) / (t1 - t0)))


# --------------------------------------------------------------------------- Brownian motion
class BrownianMotionFromMersenneRandomNumbers:
    """GPU-resident BrownianMotionFromMersenneRandomNumbers (bit-exact MT19937 uniforms)."""

    def __init__(self, timeDiscretization, numberOfFactors, numberOfPaths, seed, precision=_lib.PRECISION_FP64):
        self._L = _lib.load()
        self.timeDiscretization = timeDiscretization
        self.numberOfFactors = int(numberOfFactors)
        self.numberOfPaths = int(numberOfPaths)
        self.seed = int(seed)
        self.precision = precision
        self._times = _f64(timeDiscretization.getAsDoubleArray())
        h = ctypes.c_void_p()
        check(self._L.lmm_brownian_create(_p(self._times), len(self._times), self.numberOfFactors, self.numberOfPaths,
                                          self.seed, int(precision), ctypes.byref(h)), "BrownianMotionFromMersenneRandomNumbers")
        self._h = h

    def getBrownianIncrement(self, timeIndex, factor) -> np.ndarray:
        out = np.empty(self.numberOfPaths)
        check(self._L.lmm_brownian_get_increment(self._h, int(timeIndex), int(factor), _p(out)), "getBrownianIncrement")
        return out

    getIncrement = getBrownianIncrement

    def setSeed(self, seed):
        """getCloneWithModifiedSeed, in place (keeps the device allocation)."""
        self.seed = int(seed)
        check(self._L.lmm_brownian_set_seed(self._h, self.seed), "setSeed")

    def getTimeDiscretization(self):
        return self.timeDiscretization

    def getNumberOfFactors(self):
        return self.numberOfFactors

    def getNumberOfPaths(self):
        return self.numberOfPaths

    def close(self):
        if getattr(self, "_h", None):
            self._L.lmm_brownian_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mersenne_twister_uniforms(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """The first values of MersenneTwister(seed).nextDouble(), generated on the GPU."""
    out = np.empty(count)
    check(_lib.load().lmm_mt19937_uniforms(int(seed), int(offset), int(count), _p(out)), "lmm_mt19937_uniforms")
    return out


# --------------------------------------------------------------------------- process
def _covariance_on_process_grid(cov, times, tenor, state_space):
    """The covariance model's factor loadings, variances and volatilities at the process's
    simulation times t_i and forward rates j.  A model on its own (coarser) time and tenor
    grids is read as the reference reads it: the loading of (t_i, j) is the model's loading
    at the floor indices of t_i and of T_j in its grids
    (AbstractLIBORCovarianceModel.java:45-60, called from
    LIBORMarketModelFromCovarianceModel.java:1198); the LOGNORMAL drift's variance term is
    getCovariance(time, j, j) (:1188), whose component j is the model's own index, not mapped
    (AbstractLIBORCovarianceModel.java:69-75)."""
    lam = _f64(cov.factorLoadings)
    T, N = len(times) - 1, len(tenor) - 1
    vol = getattr(cov, "volatility", None)
    if lam.shape[:2] == (T, N):
        return lam, _f64(cov.variance), None if vol is None else _f64(vol)
    ct = np.asarray(cov.timeDiscretization.getAsDoubleArray(), dtype=np.float64)
    cc = np.asarray(cov.liborPeriodDiscretization.getAsDoubleArray(), dtype=np.float64)
    ti = np.searchsorted(ct, times[:-1], side="right") - 1
    tj = np.searchsorted(cc, tenor[:-1], side="right") - 1
    if ti.min() < 0 or tj.min() < 0 or ti.max() >= lam.shape[0] or tj.max() >= lam.shape[1]:
        raise ValueError("the covariance model's grids do not cover the process's times and forward rates")
    mapped = np.ascontiguousarray(lam[ti][:, tj, :])
    if state_space == _lib.STATE_SPACE_LOGNORMAL:
        if N > lam.shape[1]:
            raise ValueError("LOGNORMAL drift: getCovariance(time, j, j) reads the covariance model's component j, "
                             "which this model does not have")
        var = np.ascontiguousarray(np.einsum("ijk,ijk->ij", lam[ti][:, :N, :], lam[ti][:, :N, :]))
    else:
        var = np.ascontiguousarray(np.einsum("ijk,ijk->ij", mapped, mapped))  # not read by the NORMAL drift
    vm = None if vol is None else np.ascontiguousarray(_f64(vol)[ti][:, tj])
    return mapped, var, vm


class EulerSchemeFromProcessModel:
    EULER = _lib.SCHEME_EULER
    EULER_FUNCTIONAL = _lib.SCHEME_EULER_FUNCTIONAL
    PREDICTOR_CORRECTOR = _lib.SCHEME_PREDICTOR_CORRECTOR
    PREDICTOR_CORRECTOR_FUNCTIONAL = _lib.SCHEME_PREDICTOR_CORRECTOR_FUNCTIONAL

    def __init__(self, model: LIBORMarketModelFromCovarianceModel, brownianMotion: BrownianMotionFromMersenneRandomNumbers,
                 scheme=None, observedTimeIndices=None):
        self._L = _lib.load()
        self.model = model
        self.brownianMotion = brownianMotion
        self.scheme = _lib.SCHEME_EULER_FUNCTIONAL if scheme is None else scheme
        cov = model.covarianceModel
        times = _f64(brownianMotion._times)
        tenor = _f64(model.liborPeriodDiscretization.getAsDoubleArray())
        lam, var, vol = _covariance_on_process_grid(cov, times, tenor, model.stateSpace)
        self._keep = dict(times=times, tenor=tenor, lam=lam, var=var, init=_f64(model.initialForwards),
                          chain=None if model.discountChain is None else _f64(model.discountChain), vol=vol)
        k = self._keep
        T = len(k["times"]) - 1
        N = len(k["tenor"]) - 1
        desc = _lib.LmmModelDesc(T, _p(k["times"]), N, _p(k["tenor"]), cov.getNumberOfFactors(), _p(k["lam"]),
                                 _p(k["var"]), _p(k["init"]), _p(k["chain"]), model.liborCap, int(self.scheme),
                                 int(model.measure), int(model.stateSpace), _p(k["vol"]))
        h = ctypes.c_void_p()
        check(self._L.lmm_process_create(ctypes.byref(desc), brownianMotion._h, ctypes.byref(h)), "EulerSchemeFromProcessModel")
        self._h = h
        self.numberOfPaths = brownianMotion.numberOfPaths
        if observedTimeIndices is not None:
            mask = np.zeros(T + 1, dtype=np.uint8)
            mask[np.asarray(list(observedTimeIndices), dtype=np.int64)] = 1
            check(self._L.lmm_process_set_observed_times(self._h, mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
                  "observed times")

    def getProcessValue(self, timeIndex, componentIndex) -> np.ndarray:
        out = np.empty(self.numberOfPaths)
        check(self._L.lmm_process_get_value(self._h, int(timeIndex), int(componentIndex), _p(out)), "getProcessValue")
        return out

    def simulate(self):
        check(self._L.lmm_process_simulate(self._h), "doPrecalculateProcess")

    def getNumeraire(self, time) -> np.ndarray:
        out = np.empty(self.numberOfPaths)
        check(self._L.lmm_process_get_numeraire(self._h, float(time), _p(out)), "getNumeraire")
        return out

    def getTimeDiscretization(self):
        return self.brownianMotion.timeDiscretization

    def close(self):
        if getattr(self, "_h", None):
            self._L.lmm_process_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LIBORMonteCarloSimulationFromLIBORModel:
    def __init__(self, process: EulerSchemeFromProcessModel):
        self.process = process
        self.model = process.model

    def getLIBOR(self, timeIndex, liborIndex):
        return self.process.getProcessValue(timeIndex, liborIndex)

    def getNumeraire(self, time):
        return self.process.getNumeraire(time)

    def getLIBORRandomVariable(self, timeIndex, liborIndex):
        """getLIBOR as a device random variable (no host copy), LIBORMonteCarloSimulationFromLIBORModel.java:123-126."""
        from .randomvariable import RandomVariableGPU
        h = ctypes.c_void_p()
        check(_lib.load().lmm_process_get_value_rv(self.process._h, int(timeIndex), int(liborIndex), ctypes.byref(h)),
              "getLIBOR")
        return RandomVariableGPU(h)

    def getNumeraireRandomVariable(self, time):
        """getNumeraire as a device random variable (adjusted, as getNumeraire), :153-155.

        At a tenor time the library serves it directly.  Between tenor times it is composed as
        LIBORMarketModelFromCovarianceModel.getNumeraire does (:860-876, :968-1015): under SPOT
        the unadjusted numeraire of the next tenor time discounted with the forward rate
        L(t; t, T_next) over T_next - t; under TERMINAL the product of the discount factors of
        the periods from T_next on with the rates read at min(t, T_l); then, with a discount
        curve, times mean(N(0) / N(t)) and divided by the geometrically interpolated
        discount-curve chain (:883-943).  Before time 0 it is the discount curve's factor."""
        from .randomvariable import RandomVariableGPU
        time = float(time)
        m = self.model
        tenor = m.liborPeriodDiscretization
        if time < 0:
            return RandomVariableGPU.constant(float("-inf"), m.discountCurve.getDiscountFactor(None, time))
        L = _lib.load()
        if tenor.getTimeIndex(time) >= 0:
            h = ctypes.c_void_p()
            check(L.lmm_process_get_numeraire_rv(self.process._h, time, ctypes.byref(h)), "getNumeraire")
            return RandomVariableGPU(h)
        upperIndex = -tenor.getTimeIndex(time) - 1
        if upperIndex - 1 < 0 or upperIndex > tenor.getNumberOfTimeSteps():
            raise ValueError(f"Numeraire requested for time {time}. Unsupported")
        upper = tenor.getTime(upperIndex)
        if m.measure == _lib.MEASURE_TERMINAL:
            numeraire = RandomVariableGPU.constant(float("-inf"), 1.0)
            for liborIndex in range(upperIndex, tenor.getNumberOfTimeSteps()):
                libor = self.getLIBORRandomVariable(self.getTimeIndex(min(time, tenor.getTime(liborIndex))), liborIndex)
                numeraire = numeraire.discount(libor, tenor.getTimeStep(liborIndex))
        else:
            numeraire = self._unadjustedNumeraire(upper)
        numeraire = numeraire.discount(self.getForwardRate(time, time, upper), upper - time)
        if m.discountCurve is not None:
            zeroBond = m.getNumeraireDefaultableZeroBondAsOfTimeZero(time)
            nonDefaultableZeroBond = numeraire.invert().mult(self._unadjustedNumeraire(0.0)).getAverage()
            numeraire = numeraire.mult(nonDefaultableZeroBond).div(zeroBond)
        return numeraire

    def _unadjustedNumeraire(self, tenorTime):
        """getNumerairetUnAdjusted at a tenor time (:1017-1074), from the simulated paths."""
        from .randomvariable import RandomVariableGPU
        h = ctypes.c_void_p()
        check(_lib.load().lmm_process_get_numeraire_unadjusted_rv(self.process._h, float(tenorTime), ctypes.byref(h)),
              "getNumerairetUnAdjusted")
        return RandomVariableGPU(h)

    def getForwardRate(self, time, periodStart, periodEnd):
        """LIBORMarketModelFromCovarianceModel.getForwardRate (…/models/LIBORMarketModelFromCovarianceModel.java:1238-1305)
        as device random variables: the model primitive L_j(t), the accrual over several tenor
        periods, or an off-tenor period by the model's interpolationMethod (:1318-1381; LINEAR,
        LOG_LINEAR_UNCORRECTED and LOG_LINEAR_CORRECTED, each with the analytic forward-curve
        adjustment)."""
        m = self.model
        tenor, td = m.liborPeriodDiscretization, self.process.getTimeDiscretization()
        ps_i, pe_i = tenor.getTimeIndex(periodStart), tenor.getTimeIndex(periodEnd)
        time = min(time, periodStart)  # beyond the fixing: the fixing time
        ti = td.getTimeIndex(time)
        if ti < 0:
            ti = -ti - 2
            if m.simulationTimeInterpolationMethod == "ROUND_NEAREST" and time - td.getTime(ti) > td.getTime(ti + 1) - time:
                ti += 1
        if pe_i < 0:
            prev = (-pe_i - 1) - 1
            next_end = tenor.getTime(prev + 1)
            long_ = self.getForwardRate(time, periodStart, next_end).mult(next_end - periodStart).add(1.0)
            interp = self._onePlusInterpolatedLIBORDt(ti, periodEnd, prev)
            return long_.div(interp).sub(1.0).div(periodEnd - periodStart)
        if ps_i < 0:
            prev = (-ps_i - 1) - 1
            next_start = tenor.getTime(prev + 1)
            if next_start > periodEnd:
                raise ValueError("Interpolation not possible.")
            if next_start == periodEnd:
                return self._onePlusInterpolatedLIBORDt(ti, periodStart, prev).sub(1.0).div(periodEnd - periodStart)
            long_ = self.getForwardRate(time, next_start, periodEnd).mult(periodEnd - next_start).add(1.0)
            interp = self._onePlusInterpolatedLIBORDt(ti, periodStart, prev)
            return long_.mult(interp).sub(1.0).div(periodEnd - periodStart)
        if ps_i + 1 == pe_i:
            return self.getLIBORRandomVariable(ti, ps_i)
        acc = None
        for k in range(ps_i, pe_i):
            sub = tenor.getTime(k + 1) - tenor.getTime(k)
            L = self.getLIBORRandomVariable(ti, k)
            acc = L.mult(sub).add(1.0) if acc is None else acc.accrue(L, sub)
        return acc.sub(1.0).div(periodEnd - periodStart)

    def _onePlusInterpolatedLIBORDt(self, ti, periodStartTime, idx):
        """getOnePlusInterpolatedLIBORDt (:1318-1381)."""
        m = self.model
        tenor, td = m.liborPeriodDiscretization, self.process.getTimeDiscretization()
        ts, te = tenor.getTime(idx), tenor.getTime(idx + 1)
        tdt = te - ts
        if ts < td.getTime(ti):
            ti = min(ti, td.getTimeIndex(ts))  # fixed at the long period's start
            if ti < 0:
                raise ValueError("Tenor discretization not part of time discretization.")
        long_ = self.getLIBORRandomVariable(ti, idx).mult(tdt).add(1.0)
        small = te - periodStartTime
        alpha = small / tdt
        if m.interpolationMethod == "LINEAR":
            interp = long_.mult(alpha).add(1 - alpha)
        elif m.interpolationMethod == "LOG_LINEAR_UNCORRECTED":
            interp = long_.log().mult(alpha).exp()
        elif m.interpolationMethod == "LOG_LINEAR_CORRECTED":
            adjustmentCoefficient = 0.5 * small * (ts - periodStartTime)
            adjustment = self._interpolationDriftAdjustment(ti, idx).mult(adjustmentCoefficient)
            interp = long_.log().mult(alpha).sub(adjustment).exp()
        else:
            raise ValueError(f"interpolation method {m.interpolationMethod} is not supported")
        fc = m.forwardRateCurve
        a_long = 1 + fc.getForward(None, ts, tdt) * tdt
        a_short = 1 + fc.getForward(None, periodStartTime, small) * small
        a_interp = a_long * alpha + (1 - alpha) if m.interpolationMethod == "LINEAR" else np.exp(np.log(a_long) * alpha)
        return interp.mult(a_short / a_interp)

    def _interpolationDriftAdjustment(self, evaluationTimeIndex, liborIndex):
        """getInterpolationDriftAdjustmentEvaluated (:1433-1497): the trapezoid integral over the
        simulation times 0..evaluationTimeIndex of |lambda_j(t)|^2 / (1 + L_j(t) dT_j)^2 (times
        L_j(t)^2 in the lognormal state space), with L_j read at min(t, T_j) (the simulation
        time at or before T_j when T_j is off the simulation grid).  The factor
        loadings are the covariance model's deterministic ones, summed on the host in the
        reference's order; the L-dependent part runs as device random-variable operations.
        The reference caches the value per LIBOR index when evaluated at the period start
        (:1405-1422); every evaluation gives the same numbers, so none is cached here."""
        from .randomvariable import RandomVariableGPU
        m = self.model
        tenor, td = m.liborPeriodDiscretization, self.process.getTimeDiscretization()
        cov = m.covarianceModel
        tenorDt = tenor.getTime(liborIndex + 1) - tenor.getTime(liborIndex)
        lognormal = m.stateSpace == _lib.STATE_SPACE_LOGNORMAL
        start = td.getTimeIndex(tenor.getTime(liborIndex))  # raw: negative off the simulation grid

        def integrand(sumTimeIndex, realizationIndex):
            ct = cov.timeDiscretization.getTimeIndex(td.getTime(sumTimeIndex))
            if ct < 0:
                ct = -ct - 2
            if ct < 0 or ct >= cov.factorLoadings.shape[0]:
                raise ValueError("factor loading beyond the covariance model's time discretization")
            squares = 0.0  # getRandomVariableForConstant(0.0).add(oneFactor.squared()) per factor
            for loading in cov.getFactorLoading(ct, liborIndex):
                squares = squares + float(loading) * float(loading)
            libor = self.getLIBORRandomVariable(realizationIndex, liborIndex)
            value = RandomVariableGPU.constant(float("-inf"), squares).div(libor.mult(tenorDt).add(1.0).squared())
            return value.mult(libor.squared()) if lognormal else value

        previous = integrand(0, 0)
        adjustment = RandomVariableGPU.constant(float("-inf"), 0.0)
        for sumTimeIndex in range(1, evaluationTimeIndex + 1):
            k = min(sumTimeIndex, start)  # :1473-1478, the minimum taken before the off-grid mapping
            current = integrand(sumTimeIndex, k if k >= 0 else -k - 2)
            integralDt = 0.5 * (td.getTime(sumTimeIndex) - td.getTime(sumTimeIndex - 1))
            adjustment = adjustment.add(current.add(previous).mult(integralDt))
            previous = current
        return adjustment

    def getNumberOfPaths(self):
        return self.process.numberOfPaths

    def getTimeDiscretization(self):
        return self.process.getTimeDiscretization()

    def getLiborPeriodDiscretization(self):
        return self.model.liborPeriodDiscretization

    def getLiborPeriod(self, timeIndex):
        return self.model.liborPeriodDiscretization.getTime(timeIndex)

    def getLiborPeriodIndex(self, time):
        """LIBORMarketModelFromCovarianceModel.getLiborPeriodIndex (:1528-1530): the tenor index of
        time, negative (-insertion point - 1) off the tenor grid."""
        return self.model.liborPeriodDiscretization.getTimeIndex(time)

    def getRandomVariableForConstant(self, value):
        from .randomvariable import RandomVariableGPU
        return RandomVariableGPU.constant(float("-inf"), value)

    # -- the rest of the facade (LIBORMonteCarloSimulationFromLIBORModel.java:53-165)
    def getMonteCarloWeights(self, timeOrIndex):
        """Equal weights 1/P (MonteCarloProcessFromProcessModel's weights), as a deterministic
        random variable; a time is mapped to the index at or before it (:58-64)."""
        from .randomvariable import RandomVariableGPU
        if isinstance(timeOrIndex, float):
            i = self.getTimeIndex(timeOrIndex)
            timeOrIndex = i if i >= 0 else (-i - 1) - 1
        return RandomVariableGPU.constant(self.getTime(int(timeOrIndex)), 1.0 / self.getNumberOfPaths())

    def getNumberOfFactors(self):
        return self.process.brownianMotion.getNumberOfFactors()

    def getTime(self, timeIndex):
        return self.process.getTimeDiscretization().getTime(timeIndex)

    def getTimeIndex(self, time):
        return self.process.getTimeDiscretization().getTimeIndex(time)

    def getBrownianMotion(self):
        return self.process.brownianMotion

    def getNumberOfComponents(self):
        return self.model.getNumberOfComponents()

    getNumberOfLibors = getNumberOfComponents

    def getProcess(self):
        return self.process

    def getLIBORs(self, timeIndex):
        """getLIBORs (:113-121): every component at a time index, as device random variables."""
        return [self.getLIBORRandomVariable(timeIndex, j) for j in range(self.getNumberOfComponents())]

    def getReferenceDate(self):
        return self.model.getReferenceDate()

    def getModel(self):
        return self.model

    def getForwardDiscountBond(self, time, maturity):
        """LIBORMarketModelFromCovarianceModel.getForwardDiscountBond (:947-952): P(time; maturity)
        from the forward rates as of time and as of zero and the deterministic numeraire
        adjustment, as device random variables."""
        from .randomvariable import RandomVariableGPU
        asOfTime = self.getForwardRate(time, time, maturity).mult(maturity - time).add(1.0)
        asOfZero = self.getForwardRate(0.0, time, maturity).mult(maturity - time).add(1.0)
        m = self.model
        zb = (RandomVariableGPU.constant(float("-inf"), m.getNumeraireDefaultableZeroBondAsOfTimeZero(maturity))
              .div(RandomVariableGPU.constant(float("-inf"), m.getNumeraireDefaultableZeroBondAsOfTimeZero(time))))
        return zb.mult(asOfZero).div(asOfTime)


# --------------------------------------------------------------------------- products
class Swaption:
    """net.finmath.montecarlo.interestrate.products.Swaption, with the reference's constructors
    (Swaption.java:58-127), told apart by their arguments after exerciseDate:
      (fixingDates, paymentDates, periodLengths, swaprates, notional)
      (fixingDates, paymentDates, periodLengths, swaprates)   notional 1
      (fixingDates, paymentDates, swaprates)                  period lengths from the dates
      (swapTenor: TimeDiscretizationFromArray, swaprate)      one period per tenor step
    periodLengths=None means payment - fixing, as the reference's null.  A scalar swaprate is
    used for every period."""

    def __init__(self, exerciseDate, *args, periodLengths=None, notional=1.0):
        if len(args) == 2 and isinstance(args[0], TimeDiscretizationFromArray):
            t = args[0].getAsDoubleArray()
            fixingDates, paymentDates, swaprates = t[:-1], t[1:], args[1]
        elif len(args) == 3:
            fixingDates, paymentDates, swaprates = args
        elif len(args) == 4:
            fixingDates, paymentDates, periodLengths, swaprates = args
        elif len(args) == 5:
            fixingDates, paymentDates, periodLengths, swaprates, notional = args
        else:
            raise TypeError("Swaption(exerciseDate, fixingDates, paymentDates[, periodLengths], swaprates[, notional]) "
                            "or Swaption(exerciseDate, swapTenor, swaprate)")
        self.exerciseDate = float(exerciseDate)
        self.fixingDates = _f64(fixingDates)
        self.paymentDates = _f64(paymentDates)
        if self.paymentDates.shape != self.fixingDates.shape:
            raise ValueError("paymentDates must have the length of fixingDates")
        self.swaprates = _f64(np.broadcast_to(swaprates, self.fixingDates.shape))
        self.periodLengths = None if periodLengths is None else _f64(np.broadcast_to(periodLengths,
                                                                                     self.fixingDates.shape))
        self.notional = float(notional)

    def getValues(self, model: LIBORMonteCarloSimulationFromLIBORModel):
        d = _lib.LmmSwaptionDesc(self.exerciseDate, len(self.fixingDates), _p(self.fixingDates), _p(self.paymentDates),
                                 _p(self.periodLengths), _p(self.swaprates), self.notional)
        v, e = ctypes.c_double(), ctypes.c_double()
        check(_lib.load().lmm_swaption_get_value(model.process._h, ctypes.byref(d), ctypes.byref(v), ctypes.byref(e)),
              "Swaption.getValue")
        return {"value": v.value, "error": e.value}

    def getValue(self, model):
        return self.getValues(model)["value"]

    def getGradient(self, model: LIBORMonteCarloSimulationFromLIBORModel, checkpointStride: int = 1):
        """Value, deltas d V / d L_j(0) and vegas d V / d sigma_{i,j}: the payoff's pathwise
        derivative (floor(0) differentiates to 1 where its argument is >= 0, as the reference's
        AAD does; RandomVariableDifferentiableAAD.java:324-331) swept back through the Euler
        scheme by the adjoint kernel.  FP64 processes; the value is the plain valuation's."""
        proc = model.process
        T = len(proc._keep["times"]) - 1
        N = len(proc._keep["tenor"]) - 1
        d = _lib.LmmSwaptionDesc(self.exerciseDate, len(self.fixingDates), _p(self.fixingDates), _p(self.paymentDates),
                                 _p(self.periodLengths), _p(self.swaprates), self.notional)
        v, e = ctypes.c_double(), ctypes.c_double()
        deltas, vegas = np.empty(N), np.empty((T, N))
        check(_lib.load().lmm_swaption_get_gradient(proc._h, ctypes.byref(d), int(checkpointStride), ctypes.byref(v),
                                                     ctypes.byref(e), _p(deltas), _p(vegas)), "Swaption.getGradient")
        return {"value": v.value, "error": e.value, "deltas": deltas, "vegas": vegas}


def swaptionValuesBatch(simulations, swaptions):
    """Values and standard errors of every swaption on every simulation (a calibration's trial
    models on one Brownian motion): the simulations, the fused swaption kernels and the
    reductions are queued without a host round trip, one copy back per simulation
    (lmm_swaption_values_batch).  Returns (values, errors), arrays [simulations][swaptions]."""
    sims, prods = list(simulations), list(swaptions)
    descs = (_lib.LmmSwaptionDesc * len(prods))(*[
        _lib.LmmSwaptionDesc(s.exerciseDate, len(s.fixingDates), _p(s.fixingDates), _p(s.paymentDates),
                             _p(s.periodLengths), _p(s.swaprates), s.notional) for s in prods])
    handles = (ctypes.c_void_p * len(sims))(*[m.process._h for m in sims])
    values, errors = np.empty((len(sims), len(prods))), np.empty((len(sims), len(prods)))
    check(_lib.load().lmm_swaption_values_batch(len(sims), handles, len(prods), descs, _p(values), _p(errors)),
          "swaptionValuesBatch")
    return values, errors


class SwaptionSimple:
    """net.finmath.montecarlo.interestrate.products.SwaptionSimple (SwaptionSimple.java): the
    swaption on a swap tenor, exercised at its first date, valued by the fused swaption
    kernel; the value unit VALUE returns the price, VOLATILITY / VOLATILITYLOGNORMAL and
    VOLATILITYNORMAL the Black and Bachelier volatilities implied from it on the par swap
    rate and annuity of the model's forward curve (single curve: the model carries no
    analytic model), INTEGRATEDVARIANCE* their variance times maturity."""

    _UNITS = ("VALUE", "VOLATILITY", "VOLATILITYLOGNORMAL", "VOLATILITYNORMAL", "INTEGRATEDVARIANCE",
              "INTEGRATEDVARIANCELOGNORMAL", "INTEGRATEDLOGNORMALVARIANCE", "INTEGRATEDVARIANCENORMAL",
              "INTEGRATEDNORMALVARIANCE")

    def __init__(self, swaprate, swapTenor, valueUnit="VALUE"):
        t = swapTenor.getAsDoubleArray() if isinstance(swapTenor, TimeDiscretizationFromArray) else _f64(swapTenor)
        self.tenor = TimeDiscretizationFromArray(list(t))
        self.swaprate = float(swaprate)
        self.valueUnit = str(valueUnit).upper()
        if self.valueUnit not in self._UNITS:
            raise ValueError("Provided valueUnit not implemented.")
        self.swaption = Swaption(float(t[0]), self.tenor, self.swaprate)

    def getValue(self, model):
        from . import analytic as A
        value = self.swaption.getValue(model)
        if self.valueUnit == "VALUE":
            return value
        forwardCurve = model.model.forwardRateCurve
        discountCurve = DiscountCurveFromForwardCurve(forwardCurve)
        parSwaprate = A.forward_swap_rate(self.tenor, forwardCurve, discountCurve)
        optionMaturity = self.tenor.getTime(0)
        annuity = A.swap_annuity(self.tenor, discountCurve)
        if self.valueUnit in ("VOLATILITY", "VOLATILITYLOGNORMAL"):
            return A.blackScholesOptionImpliedVolatility(parSwaprate, optionMaturity, self.swaprate, annuity, value)
        if self.valueUnit == "VOLATILITYNORMAL":
            return A.bachelierOptionImpliedVolatility(parSwaprate, optionMaturity, self.swaprate, annuity, value)
        if self.valueUnit in ("INTEGRATEDVARIANCE", "INTEGRATEDVARIANCELOGNORMAL", "INTEGRATEDLOGNORMALVARIANCE"):
            v = A.blackScholesOptionImpliedVolatility(parSwaprate, optionMaturity, self.swaprate, annuity, value)
        else:
            v = A.bachelierOptionImpliedVolatility(parSwaprate, optionMaturity, self.swaprate, annuity, value)
        return v * v * optionMaturity


class SwaptionAnalyticApproximation:
    """net.finmath.montecarlo.interestrate.products.SwaptionAnalyticApproximation (host
    arithmetic on the model's tables, no simulation): Rebonato's frozen-weight swap-rate
    variance  sum_ij w_i w_j C_ij(T0)  from the log swap-rate derivatives w (:188-281) and
    the integrated LIBOR covariance C up to the option maturity, returned as the integrated
    variance, the Black volatility, or the Black price on the par swap rate and annuity
    (:125-172)."""

    def __init__(self, swaprate, swapTenor, valueUnit="VALUE"):
        t = swapTenor.getAsDoubleArray() if isinstance(swapTenor, TimeDiscretizationFromArray) else _f64(swapTenor)
        self.swapTenor = [float(x) for x in t]
        self.swaprate = float(swaprate)
        self.valueUnit = str(valueUnit).upper()
        if self.valueUnit not in ("VALUE", "VOLATILITY", "VOLATILITYLOGNORMAL", "INTEGRATEDVARIANCE",
                                  "INTEGRATEDVARIANCELOGNORMAL"):
            raise ValueError(f"Unknown valueUnit: {valueUnit}")

    def getLogSwaprateDerivative(self, liborPeriodDiscretization, discountCurve, forwardCurve):
        if discountCurve is None:
            discountCurve = DiscountCurveFromForwardCurve(forwardCurve)
        tenor, swapTenor = liborPeriodDiscretization, self.swapTenor
        start, end = tenor.getTimeIndex(swapTenor[0]), tenor.getTimeIndex(swapTenor[-1])
        forwardRates = [0.0] * (end - start + 1)
        discountFactors = [0.0] * (end - start + 1)
        discountFactors[0] = discountCurve.getDiscountFactor(None, swapTenor[0])
        for j in range(start, end):
            forwardRates[j - start] = forwardCurve.getForward(None, tenor.getTime(j))
            discountFactors[j - start + 1] = discountCurve.getDiscountFactor(None, tenor.getTime(j + 1))
        swapAnnuities = [0.0] * (len(swapTenor) - 1)
        swapAnnuity = 0.0
        for k in range(len(swapTenor) - 2, -1, -1):
            periodEnd = tenor.getTimeIndex(swapTenor[k + 1])
            swapAnnuity += discountFactors[periodEnd - start] * (swapTenor[k + 1] - swapTenor[k])
            swapAnnuities[k] = swapAnnuity
        valueFloatLeg = 0.0
        for j in range(start, end):
            valueFloatLeg += forwardRates[j - start] * discountFactors[j - start + 1] * tenor.getTimeStep(j)
        weights = [0.0] * (end - start)
        k, upToStart = 0, 0.0
        for j in range(start, end):
            if tenor.getTime(j) >= swapTenor[k + 1]:
                k += 1
            libor, length = forwardRates[j - start], tenor.getTimeStep(j)
            upToStart += forwardRates[j - start] * discountFactors[j - start + 1] * length
            dfEnd = discountCurve.getDiscountFactor(None, tenor.getTime(j + 1))
            dFloat = (dfEnd + upToStart - valueFloatLeg) * length / (1.0 + libor * length) / valueFloatLeg
            dFix = -swapAnnuities[k] / swapAnnuity * length / (1.0 + libor * length)
            weights[j - start] = (dFloat - dFix) * libor
        return {"values": weights, "discountFactors": discountFactors, "swapAnnuities": swapAnnuities}

    def getValue(self, model, evaluationTime: float = 0.0):
        from . import analytic as A
        if evaluationTime > 0:
            raise ValueError("Forward start evaluation currently not supported.")
        m = model.model if hasattr(model, "model") and hasattr(model, "process") else model
        td = model.getTimeDiscretization() if m is not model else m.covarianceModel.timeDiscretization
        swapStart, swapEnd = self.swapTenor[0], self.swapTenor[-1]
        tenor = m.liborPeriodDiscretization
        start, end = tenor.getTimeIndex(swapStart), tenor.getTimeIndex(swapEnd)
        maturityIndex = m.covarianceModel.timeDiscretization.getTimeIndex(swapStart) - 1
        w = self.getLogSwaprateDerivative(tenor, m.discountCurve, m.forwardRateCurve)["values"]
        C = m.getIntegratedLIBORCovariance(td)[maturityIndex]
        variance = 0.0
        for i in range(start, end):
            for j in range(i + 1, end):
                variance += 2.0 * w[i - start] * w[j - start] * C[i, j]
            variance += w[i - start] * w[i - start] * C[i, i]
        if self.valueUnit in ("INTEGRATEDVARIANCELOGNORMAL", "INTEGRATEDVARIANCE"):
            return variance
        volatility = math.sqrt(variance / swapStart)
        if self.valueUnit in ("VOLATILITYLOGNORMAL", "VOLATILITY"):
            return volatility
        dc = m.discountCurve if m.discountCurve is not None else DiscountCurveFromForwardCurve(m.forwardRateCurve)
        tenorSwap = TimeDiscretizationFromArray(self.swapTenor)
        par = A.forward_swap_rate(tenorSwap, m.forwardRateCurve, dc)
        annuity = A.swap_annuity(tenorSwap, dc)
        return A.blackModelSwaptionValue(par, volatility, swapStart, self.swaprate, annuity)


class BermudanSwaption:
    """net.finmath.montecarlo.interestrate.products.BermudanSwaption.

    regressionBasisFunctionsProvider: None for the reference's built-in basis, or
    "swaprate" for the {1, S, S^2, N, N^2, S*N} provider (both fused into the library's
    Bermudan kernels); or any object with getBasisFunctions(fixingDate, model) returning
    random variables (RegressionBasisFunctionsProvider.java:28), which runs the reference's
    getValues (BermudanSwaption.java:91-157) on device random variables with that basis.
    """

    def __init__(self, isPeriodStartDateExerciseDate, fixingDates, periodLength, paymentDates, periodNotionals, swaprates,
                 isCallable=True, regressionBasisFunctionsProvider=None):
        self.isPeriodStartDateExerciseDate = np.ascontiguousarray(isPeriodStartDateExerciseDate, dtype=np.uint8)
        n = len(self.isPeriodStartDateExerciseDate)
        self.fixingDates = _f64(fixingDates)
        self.periodLengths = _f64(np.broadcast_to(periodLength, (n,)))
        self.paymentDates = _f64(paymentDates)
        self.periodNotionals = _f64(np.broadcast_to(periodNotionals, (n,)))
        self.swaprates = _f64(np.broadcast_to(swaprates, (n,)))
        self.isCallable = bool(isCallable)
        self.provider = None
        if regressionBasisFunctionsProvider is None or (isinstance(regressionBasisFunctionsProvider, str)
                                                        and regressionBasisFunctionsProvider == "reference"):
            self.basis = _lib.BASIS_REFERENCE
        elif isinstance(regressionBasisFunctionsProvider, str) and regressionBasisFunctionsProvider == "swaprate":
            self.basis = _lib.BASIS_SWAPRATE
        elif hasattr(regressionBasisFunctionsProvider, "getBasisFunctions"):
            self.basis, self.provider = None, regressionBasisFunctionsProvider
        else:
            raise ValueError("unknown regression basis provider")

    def getExerciseTimes(self):
        """BermudanSwaption.getExerciseTimes (:254-262): the exercisable fixing dates."""
        return [float(f) for f, e in zip(self.fixingDates, self.isPeriodStartDateExerciseDate) if e]

    def getBasisFunctions(self, fixingDate, model):
        """The built-in basis (:215-252) as device random variables: 1, the discount factor to the
        next payment and to the end and their squares, and 1/N(fixingDate)."""
        from .randomvariable import RandomVariableGPU
        fix, pay = list(self.fixingDates), list(self.paymentDates)
        import bisect
        i = bisect.bisect_left(fix, fixingDate)
        if not (i < len(fix) and fix[i] == fixingDate):
            i = i + 1  # the reference's -(-(insertion) - 1)
        i = min(i, len(fix) - 1)
        rateShort = model.getForwardRate(fixingDate, fixingDate, pay[i])
        discountShort = rateShort.mult(pay[i] - fixingDate).add(1.0).invert()
        rateLong = model.getForwardRate(fixingDate, fix[i], pay[-1])
        discountLong = rateLong.mult(pay[-1] - fix[i]).add(1.0).invert()
        return [RandomVariableGPU.constant(float("-inf"), 1.0), discountShort, discountShort.pow(2.0), discountLong,
                discountLong.pow(2.0), model.getNumeraireRandomVariable(fixingDate).invert()]

    def _getValuesRandomVariable(self, model, evaluationTime=0.0):
        # BermudanSwaption.getValues (:91-157) on device random variables
        from .randomvariable import MonteCarloConditionalExpectationRegression, RandomVariableGPU
        const = lambda v: RandomVariableGPU.constant(float("-inf"), v)
        values, underlying, exerciseTime = const(0.0), const(0.0), const(float("inf"))
        for period in range(len(self.fixingDates) - 1, -1, -1):
            fixingDate, periodLength = float(self.fixingDates[period]), float(self.periodLengths[period])
            paymentDate, notional = float(self.paymentDates[period]), float(self.periodNotionals[period])
            libor = model.getForwardRate(fixingDate, fixingDate, fixingDate + periodLength)
            payoff = libor.sub(float(self.swaprates[period])).mult(periodLength).mult(notional)
            payoff = payoff.div(model.getNumeraireRandomVariable(paymentDate)).mult(model.getMonteCarloWeights(paymentDate))
            if self.isCallable:
                underlying = underlying.add(payoff)
            else:
                values = values.add(payoff)
            if self.isPeriodStartDateExerciseDate[period]:
                estimator = MonteCarloConditionalExpectationRegression(self.provider.getBasisFunctions(fixingDate, model))
                trigger = values.sub(underlying).getConditionalExpectation(estimator)
                values = trigger.choose(values, underlying)
                exerciseTime = trigger.choose(exerciseTime, const(fixingDate))
        values = values.mult(model.getNumeraireRandomVariable(evaluationTime)).div(
            model.getMonteCarloWeights(evaluationTime))
        return values, exerciseTime

    def getValues(self, model: LIBORMonteCarloSimulationFromLIBORModel, per_path: bool = False):
        if self.provider is not None:
            values, exerciseTime = self._getValuesRandomVariable(model)
            out = {"value": values.getAverage(), "error": values.getStandardError(), "exerciseTime": exerciseTime}
            if per_path:
                out["values"] = values.getRealizations()
            return out
        d = _lib.LmmBermudanDesc(len(self.fixingDates),
                                 self.isPeriodStartDateExerciseDate.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                 _p(self.fixingDates), _p(self.periodLengths), _p(self.paymentDates),
                                 _p(self.periodNotionals), _p(self.swaprates), int(self.isCallable), self.basis)
        v, e = ctypes.c_double(), ctypes.c_double()
        pp = np.empty(model.getNumberOfPaths()) if per_path else None
        check(_lib.load().lmm_bermudan_get_value(model.process._h, ctypes.byref(d), ctypes.byref(v), ctypes.byref(e),
                                                 _p(pp)), "BermudanSwaption.getValues")
        out = {"value": v.value, "error": e.value}
        if per_path:
            out["values"] = pp
        return out

    def getValue(self, model):
        return self.getValues(model)["value"]

    def _desc(self):
        if self.provider is not None:
            raise ValueError("the fused Bermudan kernels (gradient, portfolio) take the built-in or swap-rate basis")
        return _lib.LmmBermudanDesc(len(self.fixingDates),
                                    self.isPeriodStartDateExerciseDate.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                    _p(self.fixingDates), _p(self.periodLengths), _p(self.paymentDates),
                                    _p(self.periodNotionals), _p(self.swaprates), int(self.isCallable), self.basis)

    def getGradient(self, model: LIBORMonteCarloSimulationFromLIBORModel, checkpointStride: int = 1,
                    freezeNumeraireAdjustment: bool = False, diracDeltaApproximationMethod: str = "ZERO",
                    diracDeltaApproximationWidthPerStdDev: float = 0.05):
        """Value, deltas d V / d L_j(0) and vegas d V / d sigma_{i,j} by the adjoint kernel
        (the role of RandomVariableDifferentiable.getGradient with these leaves).  The
        exercise decisions are frozen (diracDeltaApproximationMethod "ZERO"), or the reference
        AAD's default "DISCRETE_DELTA" sweep weights the cash flows
        (RandomVariableDifferentiableAADFactory.java:60-72; an FP64 sweep in both precision
        forms)."""
        proc = model.process
        T = len(proc._keep["times"]) - 1
        N = len(proc._keep["tenor"]) - 1
        d = self._desc()
        v, e = ctypes.c_double(), ctypes.c_double()
        deltas, vegas = np.empty(N), np.empty((T, N))
        methods = {"ZERO": _lib.LMM_DIRAC_ZERO, "DISCRETE_DELTA": _lib.LMM_DIRAC_DISCRETE_DELTA}
        if diracDeltaApproximationMethod not in methods:
            raise ValueError(f"diracDeltaApproximationMethod {diracDeltaApproximationMethod} is not supported")
        check(_lib.load().lmm_bermudan_get_gradient_aad(proc._h, ctypes.byref(d), int(checkpointStride),
                                                        int(freezeNumeraireAdjustment),
                                                        methods[diracDeltaApproximationMethod],
                                                        float(diracDeltaApproximationWidthPerStdDev),
                                                        ctypes.byref(v), ctypes.byref(e), _p(deltas), _p(vegas)),
              "BermudanSwaption.getGradient")
        return {"value": v.value, "error": e.value, "deltas": deltas, "vegas": vegas}


class Portfolio:
    """Bermudan swaptions valued together (with deltas and vegas) on one shared simulation:
    the per-product kernels are recorded once into a CUDA graph; run() launches it."""

    def __init__(self, model: LIBORMonteCarloSimulationFromLIBORModel, products, withGreeks=True, checkpointStride=1,
                 concurrency=4, adjointThreads=128, gramBlocks=0):
        self._L = _lib.load()
        self.model = model
        self.products = list(products)
        self._descs = (_lib.LmmBermudanDesc * len(self.products))(*[b._desc() for b in self.products])
        d = _lib.LmmPortfolioDesc(len(self.products), ctypes.cast(self._descs, ctypes.c_void_p), int(withGreeks),
                                  int(checkpointStride), int(concurrency), int(adjointThreads), int(gramBlocks))
        h = ctypes.c_void_p()
        check(self._L.lmm_portfolio_create(model.process._h, ctypes.byref(d), ctypes.byref(h)), "Portfolio")
        self._h = h
        self.withGreeks = bool(withGreeks)
        proc = model.process
        self.T = len(proc._keep["times"]) - 1
        self.N = len(proc._keep["tenor"]) - 1

    def run(self):
        n = len(self.products)
        v, e, lat, tot = np.empty(n), np.empty(n), np.empty(n), ctypes.c_double()
        dl = np.empty((n, self.N)) if self.withGreeks else None
        vg = np.empty((n, self.T, self.N)) if self.withGreeks else None
        check(self._L.lmm_portfolio_run(self._h, _p(v), _p(e), _p(dl), _p(vg), _p(lat), ctypes.byref(tot)),
              "Portfolio.run")
        return {"values": v, "errors": e, "deltas": dl, "vegas": vg, "latency_ms": lat, "total_ms": tot.value}

    def close(self):
        if getattr(self, "_h", None):
            self._L.lmm_portfolio_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------- instrumentation
def kernel_stats():
    L = _lib.load()
    n = 16
    names = (ctypes.c_char_p * n)()
    launches = (ctypes.c_int64 * n)()
    ms = (ctypes.c_double * n)()
    k = L.lmm_stats_get(n, names, launches, ms)
    return {names[i].decode(): (int(launches[i]), float(ms[i])) for i in range(k)}
