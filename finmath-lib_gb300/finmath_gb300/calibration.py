"""Monte Carlo calibration of the LIBOR market model's covariance parameters.

LevenbergMarquardt restates net.finmath.optimizer.LevenbergMarquardt (optimizer/
LevenbergMarquardt.java: run :640-700, the step :749-816, forward-difference derivatives,
done() :623-637), with its defaults (lambda 0.001, divided by 3 after an accepted step,
multiplied by 2 after a rejected one, by 16 when the normal equations cannot be solved;
the normal equations solved by the commons-math SVD solver the library restates in
lmm_solve_svd).  calibrate_covariance_model is AbstractLIBORCovarianceModelParametric.
getCloneCalibrated's Levenberg-Marquardt branch (models/covariance/
AbstractLIBORCovarianceModelParametric.java:333-460): every objective evaluation clones
the covariance model with the trial parameters, builds the LMM and its Euler process on
one shared Brownian motion (common random numbers, resident on the GPU) and reprices the
calibration products with the library's fused kernels; a product that fails contributes 0.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib


class LevenbergMarquardt:
    """The reference's optimizer: minimise sum_k w_k (f_k(p) - target_k)^2 / n over p."""

    LEVENBERG, LEVENBERG_MARQUARDT = "LEVENBERG", "LEVENBERG_MARQUARDT"

    def __init__(self, initialParameters, targetValues, maxIteration=100, objective=None,
                 regularizationMethod=LEVENBERG_MARQUARDT, weights=None):
        self.regularizationMethod = regularizationMethod
        self.initialParameters = [float(x) for x in initialParameters]
        self.targetValues = [float(x) for x in targetValues]
        self.maxIteration = int(maxIteration)
        self.weights = [1.0] * len(self.targetValues) if weights is None else [float(x) for x in weights]
        self.parameterSteps = None
        self.lambda_ = 0.001
        self.lambdaDivisor, self.lambdaMultiplicator = 3.0, 2.0
        self.errorRootMeanSquaredTolerance = 0.0
        self._objective = objective
        self._batch_objective = None  # f over several parameter vectors at once (the Jacobian's columns)
        self.evaluations = 0          # parameter vectors evaluated
        self.iteration = 0
        self.parameterCurrent = None
        self.errorMeanSquaredCurrent = math.inf

    # -- configuration (the reference's fluent setters)
    def setLambda(self, lambda_):
        self.lambda_ = float(lambda_)
        return self

    def setErrorTolerance(self, errorTolerance):
        self.errorRootMeanSquaredTolerance = float(errorTolerance)
        return self

    def setParameterSteps(self, parameterSteps):
        self.parameterSteps = None if parameterSteps is None else [float(x) for x in parameterSteps]
        return self

    def setWeights(self, weights):
        self.weights = [float(x) for x in weights]
        return self

    # -- the objective
    def setValues(self, parameters, values):
        """Write f(parameters) into values (a list of floats); override or pass objective."""
        if self._objective is None:
            raise NotImplementedError("setValues must be overridden or an objective given")
        out = self._objective(list(parameters))
        self.evaluations += 1
        for k in range(len(values)):
            values[k] = float(out[k])

    def getMeanSquaredError(self, value):
        error = 0.0
        for k in range(len(value)):
            deviation = value[k] - self.targetValues[k]
            error += self.weights[k] * deviation * deviation
        return error / len(value)

    def setBatchObjective(self, batchObjective):
        """f over a list of parameter vectors at once: the derivative's columns are then
        evaluated together, as the reference evaluates them in parallel threads
        (LevenbergMarquardt.java's executor; AbstractLIBORCovarianceModelParametric.java:177-178)."""
        self._batch_objective = batchObjective
        return self

    def setDerivatives(self, parameters, derivatives):
        # forward differences, one parameter at a time; a failed or NaN valuation gives 0
        steps, columns = [], []
        for i in range(len(parameters)):
            shifted = list(parameters)
            h = self.parameterSteps[i] if self.parameterSteps is not None else (abs(shifted[i]) + 1) * 1e-8
            shifted[i] += h
            steps.append(h)
            columns.append(shifted)
        batch = None
        if self._batch_objective is not None:
            try:
                batch = [[float(x) for x in out] for out in self._batch_objective(columns)]
                self.evaluations += len(columns)
            except Exception:
                batch = None
        for i in range(len(parameters)):
            h = steps[i]
            if batch is not None:
                d = list(batch[i])
            else:
                d = [0.0] * len(self.valueCurrent)
                try:
                    self.setValues(columns[i], d)
                except Exception:
                    d = [math.nan] * len(self.valueCurrent)
            for k in range(len(d)):
                d[k] -= self.valueCurrent[k]
                d[k] /= h
                if math.isnan(d[k]):
                    d[k] = 0.0
            derivatives[i] = d

    def done(self):
        return (self.iteration > self.maxIteration or self.errorRootMeanSquaredChange <= self.errorRootMeanSquaredTolerance
                or math.isinf(self.lambda_))

    def _solve(self, hessian, beta):
        n = len(beta)
        a = np.ascontiguousarray(hessian, dtype=np.float64)
        b = np.ascontiguousarray(beta, dtype=np.float64)
        x = np.empty(n)
        dp = ctypes.POINTER(ctypes.c_double)
        if not (np.all(np.isfinite(a)) and np.all(np.isfinite(b))):
            return None
        rc = _lib.load().lmm_solve_svd(n, a.ctypes.data_as(dp), b.ctypes.data_as(dp), x.ctypes.data_as(dp))
        return None if rc != 0 else list(x)

    def _updateParameterTest(self):
        n = len(self.parameterCurrent)
        if not self._derivativeValid:
            self.setDerivatives(self.parameterCurrent, self.derivativeCurrent)
            self._derivativeValid = True
        increment = None
        while increment is None and math.isfinite(self.lambda_):
            hessian = [[0.0] * n for _ in range(n)]
            for i in range(n):
                for j in range(i, n):
                    h = 0.0
                    for k in range(len(self.valueCurrent)):
                        h += self.weights[k] * self.derivativeCurrent[i][k] * self.derivativeCurrent[j][k]
                    if i == j:
                        if self.regularizationMethod == self.LEVENBERG:
                            h += self.lambda_
                        elif h == 0.0:
                            h = self.lambda_
                        else:
                            h *= 1 + self.lambda_
                    hessian[i][j] = hessian[j][i] = h
            beta = [0.0] * n
            for i in range(n):
                b = 0.0
                for k in range(len(self.valueCurrent)):
                    b += self.weights[k] * (self.targetValues[k] - self.valueCurrent[k]) * self.derivativeCurrent[i][k]
                beta[i] = b
            increment = self._solve(hessian, beta)
            if increment is None:
                self.lambda_ *= 16
        if increment is None:
            increment = [0.0] * n
        self.parameterTest = [self.parameterCurrent[i] + increment[i] for i in range(n)]

    def run(self):
        n, m = len(self.initialParameters), len(self.targetValues)
        self.parameterTest = list(self.initialParameters)
        self.parameterCurrent = [0.0] * n
        self.valueCurrent = [0.0] * m
        self.derivativeCurrent = [[0.0] * m for _ in range(n)]
        self.errorMeanSquaredCurrent = math.inf
        self.errorRootMeanSquaredChange = math.inf
        self._derivativeValid = False
        self.iteration = 0
        while True:
            self.iteration += 1
            valueTest = [0.0] * m
            self.setValues(self.parameterTest, valueTest)
            errorTest = self.getMeanSquaredError(valueTest)
            if errorTest < self.errorMeanSquaredCurrent:  # False for NaN: a rejected point
                self.errorRootMeanSquaredChange = math.sqrt(self.errorMeanSquaredCurrent) - math.sqrt(errorTest)
                self.parameterCurrent = list(self.parameterTest)
                self.valueCurrent = list(valueTest)
                self.errorMeanSquaredCurrent = errorTest
                self._derivativeValid = False
                self.lambda_ /= self.lambdaDivisor
            else:
                self.errorRootMeanSquaredChange = math.sqrt(errorTest) - math.sqrt(self.errorMeanSquaredCurrent)
                self.lambda_ *= self.lambdaMultiplicator
            if self.done():
                break
            self._updateParameterTest()
        return self

    def getBestFitParameters(self):
        return list(self.parameterCurrent)

    def getRootMeanSquaredError(self):
        return math.sqrt(self.errorMeanSquaredCurrent)

    def getIterations(self):
        return self.iteration


class OptimizerFactoryLevenbergMarquardt:
    """optimizer/OptimizerFactoryLevenbergMarquardt.java:23-73."""

    def __init__(self, maxIterations, errorTolerance=0.0, maxThreads=1,
                 regularizationMethod=LevenbergMarquardt.LEVENBERG_MARQUARDT, lambda_=0.001):
        self.maxIterations, self.errorTolerance = int(maxIterations), float(errorTolerance)
        self.regularizationMethod, self.lambda_ = regularizationMethod, float(lambda_)

    def getOptimizer(self, objectiveFunction, initialParameters, lowerBound=None, upperBound=None, parameterSteps=None,
                     targetValues=None):
        # the reference's Levenberg-Marquardt ignores the bounds
        return (LevenbergMarquardt(initialParameters, targetValues, self.maxIterations, objectiveFunction,
                                   self.regularizationMethod)
                .setLambda(self.lambda_).setErrorTolerance(self.errorTolerance).setParameterSteps(parameterSteps))


class CalibrationProduct:
    """net.finmath.montecarlo.interestrate.CalibrationProduct: a product, its target value and weight."""

    def __init__(self, name, product, targetValue, weight=1.0, priority=0):
        self.name, self.product = name, product
        self.targetValue, self.weight, self.priority = float(targetValue), float(weight), int(priority)

    def getName(self):
        return self.name

    def getProduct(self):
        return self.product

    def getTargetValue(self):
        return self.targetValue

    def getWeight(self):
        return self.weight


def _calibration_error(product: CalibrationProduct, simulation) -> float:
    """(value - target) * weight of one product; 0 when its valuation fails (:392-399, :416)."""
    try:
        value = product.getProduct().getValue(simulation)
        if hasattr(value, "getAverage"):  # a random variable, as the reference's products return
            return value.sub(product.getTargetValue()).mult(product.getWeight()).getAverage()
        return (float(value) - product.getTargetValue()) * product.getWeight()
    except Exception:
        return 0.0


def calibrate_covariance_model(covarianceModel, calibrationModel, calibrationProducts, calibrationParameters=None):
    """getCloneCalibrated: returns the covariance model at the best-fit parameters.

    calibrationParameters (the reference's keys and defaults): numberOfPaths 2000, seed 31415,
    maxIterations 400, accuracy 1e-7, parameterStep 1e-4, brownianMotion (else a new
    BrownianMotionFromMersenneRandomNumbers on the covariance model's time discretization),
    optimizerFactory (else OptimizerFactoryLevenbergMarquardt(maxIterations, accuracy)).
    The optimizer is kept in calibrationParameters["optimizer"] after the run when the caller
    passes a dict, for its iteration count and error."""
    from .lmm import BrownianMotionFromMersenneRandomNumbers, EulerSchemeFromProcessModel, \
        LIBORMonteCarloSimulationFromLIBORModel, Swaption, swaptionValuesBatch
    params = {} if calibrationParameters is None else calibrationParameters
    numberOfPaths = int(params.get("numberOfPaths", 2000))
    seed = int(params.get("seed", 31415))
    maxIterations = int(params.get("maxIterations", 400))
    accuracy = float(params.get("accuracy", 1e-7))
    step = float(params.get("parameterStep", 1e-4))
    bm = params.get("brownianMotion")
    own_bm = bm is None
    if own_bm:
        bm = BrownianMotionFromMersenneRandomNumbers(covarianceModel.timeDiscretization,
                                                     covarianceModel.getNumberOfFactors(), numberOfPaths, seed)
    initial = covarianceModel.getParameterAsDouble()
    if len(initial) == 0:
        raise ValueError("the covariance model has no calibrateable parameters")
    products = list(calibrationProducts)

    def batch_objective(parameter_list):
        # every calibration product a fused swaption: the trial models' processes are simulated
        # and priced in one batch (lmm_swaption_values_batch)
        processes = []
        try:
            for parameters in parameter_list:
                cov = covarianceModel.getCloneWithModifiedParameters(parameters)
                model = calibrationModel.getCloneWithModifiedCovarianceModel(cov)
                processes.append(EulerSchemeFromProcessModel(model, bm))
            sims = [LIBORMonteCarloSimulationFromLIBORModel(pr) for pr in processes]
            values, _ = swaptionValuesBatch(sims, [p.getProduct() for p in products])
            return [[(float(values[i, k]) - p.getTargetValue()) * p.getWeight() for k, p in enumerate(products)]
                    for i in range(len(parameter_list))]
        finally:
            for pr in processes:
                pr.close()

    batched = all(isinstance(p.getProduct(), Swaption) for p in products)

    def objective(parameters):
        if batched:
            try:
                return batch_objective([parameters])[0]
            except Exception:
                pass  # a failing batch falls back to the product-by-product valuation
        cov = covarianceModel.getCloneWithModifiedParameters(parameters)
        model = calibrationModel.getCloneWithModifiedCovarianceModel(cov)
        process = EulerSchemeFromProcessModel(model, bm)
        try:
            sim = LIBORMonteCarloSimulationFromLIBORModel(process)
            return [_calibration_error(p, sim) for p in products]
        finally:
            process.close()

    factory = params.get("optimizerFactory") or OptimizerFactoryLevenbergMarquardt(maxIterations, accuracy)
    optimizer = factory.getOptimizer(objective, initial, [-math.inf] * len(initial), [math.inf] * len(initial),
                                     [step] * len(initial), [0.0] * len(products))
    if batched and hasattr(optimizer, "setBatchObjective"):
        optimizer.setBatchObjective(batch_objective)
    try:
        optimizer.run()
    finally:
        if own_bm:
            bm.close()
    if calibrationParameters is not None:
        calibrationParameters["optimizer"] = optimizer
    return covarianceModel.getCloneWithModifiedParameters(optimizer.getBestFitParameters())
