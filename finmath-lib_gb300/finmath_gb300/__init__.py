"""GB300-native LIBOR Market Model Monte Carlo path with finmath-lib's API surface.

The numeric work runs in liblmm_gb300.so (CUDA kernels for sm_103a behind the C ABI of
include/lmm_gb300.h and include/lmm_rv.h).  Importing this package does not touch the GPU; the first call
that needs the library loads it (and builds it from source if it is not built yet).
"""
from ._lib import (CalculationException, PRECISION_FP64, PRECISION_MIXED, SCHEME_EULER, SCHEME_EULER_FUNCTIONAL,
                   BASIS_REFERENCE, BASIS_SWAPRATE, load, library_path)
from .lmm import (TimeDiscretizationFromArray, ForwardCurveInterpolation, DiscountCurveFromForwardCurve,
                  LIBORCorrelationModelExponentialDecay, LIBORVolatilityModelFourParameterExponentialForm,
                  LIBORVolatilityModelFromGivenMatrix, LIBORCovarianceModelFromVolatilityAndCorrelation,
                  LIBORCovarianceModelExponentialForm5Param,
                  LIBORMarketModelFromCovarianceModel, BrownianMotionFromMersenneRandomNumbers,
                  EulerSchemeFromProcessModel, LIBORMonteCarloSimulationFromLIBORModel, Swaption, SwaptionSimple,
                  swaptionValuesBatch,
                  SwaptionAnalyticApproximation, BermudanSwaption, Portfolio,
                  mersenne_twister_uniforms, kernel_stats)
from .randomvariable import RandomVariableGPU, RandomVariableGPUFactory, MonteCarloConditionalExpectationRegression
from .rvproducts import (Bond, BermudanSwaptionFromSwapSchedules, Caplet, DigitalCaplet, DigitalFloorlet, LIBORBond,
                         MoneyMarketAccount, SimpleSwap, SimpleZeroSwap, SwaptionFromSwapSchedules)
from .calibration import CalibrationProduct, LevenbergMarquardt, OptimizerFactoryLevenbergMarquardt
from .schedule import (DayCountConvention_ACT_360, DayCountConvention_ACT_365, FloatingpointDate, Period,
                       ScheduleFromPeriods)
from . import analytic, workloads, autotune

__all__ = [n for n in dir() if not n.startswith("_")]
