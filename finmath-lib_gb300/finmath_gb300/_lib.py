"""ctypes binding of liblmm_gb300.so (the C ABI declared in include/lmm_gb300.h and lmm_rv.h).

The library is the product: every call below runs the CUDA implementation.  There is
no CPU fallback; if the library or a GPU is missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

_D = ctypes.POINTER(ctypes.c_double)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_I64 = ctypes.POINTER(ctypes.c_int64)
_VP = ctypes.c_void_p

LMM_OK = 0
LMM_ERR_INVALID = -1
LMM_ERR_NOMEM = -2
LMM_ERR_CUDA = -3
LMM_ERR_TIMEOUT = -4
LMM_ERR_STATE = -5
PRECISION_FP64 = 0
PRECISION_MIXED = 1
SCHEME_EULER = 0
SCHEME_EULER_FUNCTIONAL = 1
SCHEME_PREDICTOR_CORRECTOR = 2
SCHEME_PREDICTOR_CORRECTOR_FUNCTIONAL = 3
MEASURE_SPOT = 0
MEASURE_TERMINAL = 1
STATE_SPACE_LOGNORMAL = 0
STATE_SPACE_NORMAL = 1
BASIS_REFERENCE = 0
BASIS_SWAPRATE = 1
LMM_DIRAC_ZERO = 0
LMM_DIRAC_DISCRETE_DELTA = 1


class LmmModelDesc(ctypes.Structure):
    _fields_ = [("num_steps", ctypes.c_int), ("times", _D), ("num_periods", ctypes.c_int), ("tenor", _D),
                ("num_factors", ctypes.c_int), ("factor_loadings", _D), ("variance", _D),
                ("initial_forwards", _D), ("discount_chain", _D), ("libor_cap", ctypes.c_double),
                ("scheme", ctypes.c_int), ("measure", ctypes.c_int), ("state_space", ctypes.c_int),
                ("volatility", _D)]


class LmmSwaptionDesc(ctypes.Structure):
    _fields_ = [("exercise_date", ctypes.c_double), ("num_periods", ctypes.c_int), ("fixing_dates", _D),
                ("payment_dates", _D), ("period_lengths", _D), ("swaprates", _D), ("notional", ctypes.c_double)]


class LmmBermudanDesc(ctypes.Structure):
    _fields_ = [("num_periods", ctypes.c_int), ("is_exercise_date", _U8), ("fixing_dates", _D),
                ("period_lengths", _D), ("payment_dates", _D), ("notionals", _D), ("swaprates", _D),
                ("is_callable", ctypes.c_int), ("basis", ctypes.c_int)]


class LmmPortfolioDesc(ctypes.Structure):
    _fields_ = [("num_products", ctypes.c_int), ("products", ctypes.c_void_p), ("with_greeks", ctypes.c_int),
                ("checkpoint_stride", ctypes.c_int), ("concurrency", ctypes.c_int), ("adjoint_threads", ctypes.c_int),
                ("gram_blocks", ctypes.c_int)]


# name -> (restype, argtypes); every exported symbol of include/lmm_gb300.h
SIGNATURES = {
    "lmm_last_error": (ctypes.c_char_p, []),
    "lmm_version": (ctypes.c_int, []),
    "lmm_time_discretization": (ctypes.c_int, [ctypes.c_double, ctypes.c_int, ctypes.c_double, _D]),
    "lmm_factor_reduction": (ctypes.c_int, [_D, ctypes.c_int, ctypes.c_int, _D]),
    "lmm_correlation_exponential_decay": (ctypes.c_int, [_D, ctypes.c_int, ctypes.c_int, ctypes.c_double, _D, _D]),
    "lmm_volatility_four_parameter": (ctypes.c_int, [_D, ctypes.c_int, _D, ctypes.c_int] + [ctypes.c_double] * 4 + [_D]),
    "lmm_covariance_tables": (ctypes.c_int, [ctypes.c_int] * 3 + [_D] * 5),
    "lmm_forward_curve_value": (ctypes.c_int, [_D, _D, ctypes.c_int, ctypes.c_double, _D]),
    "lmm_discount_factor_from_forward_curve": (ctypes.c_int, [_D, _D, ctypes.c_int, ctypes.c_double, ctypes.c_double, _D]),
    "lmm_numeraire_discount_chain": (ctypes.c_int, [_D, ctypes.c_int, _D, _D]),
    "lmm_solve_svd": (ctypes.c_int, [ctypes.c_int, _D, _D, _D]),
    "lmm_brownian_create": (ctypes.c_int, [_D, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(_VP)]),
    "lmm_brownian_get_increment": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, _D]),
    "lmm_brownian_generate": (ctypes.c_int, [_VP]),
    "lmm_brownian_set_seed": (ctypes.c_int, [_VP, ctypes.c_int]),
    "lmm_brownian_destroy": (ctypes.c_int, [_VP]),
    "lmm_mt19937_uniforms": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _D]),
    "lmm_mt19937_words_host": (ctypes.c_int, [ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64,
                                              ctypes.POINTER(ctypes.c_uint32)]),
    "lmm_mt19937_chunk_words_host": (ctypes.c_int, [ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64,
                                                    ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32)]),
    "lmm_process_create": (ctypes.c_int, [ctypes.POINTER(LmmModelDesc), _VP, ctypes.POINTER(_VP)]),
    "lmm_process_set_observed_times": (ctypes.c_int, [_VP, _U8]),
    "lmm_process_simulate": (ctypes.c_int, [_VP]),
    "lmm_process_get_value": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, _D]),
    "lmm_process_get_numeraire": (ctypes.c_int, [_VP, ctypes.c_double, _D]),
    "lmm_process_get_value_rv": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_VP)]),
    "lmm_process_get_numeraire_rv": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.POINTER(_VP)]),
    "lmm_process_get_numeraire_unadjusted_rv": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.POINTER(_VP)]),
    "lmm_rv_create_constant": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.POINTER(_VP)]),
    "lmm_rv_create": (ctypes.c_int, [ctypes.c_double, _D, ctypes.c_int64, ctypes.POINTER(_VP)]),
    "lmm_rv_create_float": (ctypes.c_int, [ctypes.c_double, ctypes.POINTER(ctypes.c_float), ctypes.c_int64,
                                           ctypes.POINTER(_VP)]),
    "lmm_rv_create_constant_float": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.POINTER(_VP)]),
    "lmm_rv_to_float": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "lmm_rv_is_float": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_int)]),
    "lmm_rv_get_float": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_float)]),
    "lmm_rv_quantile": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "lmm_rv_quantile_expectation": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.c_double,
                                                   ctypes.POINTER(ctypes.c_double)]),
    "lmm_rv_histogram": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double)]),
    "lmm_rv_destroy": (ctypes.c_int, [_VP]),
    "lmm_rv_stream": (ctypes.c_int, [ctypes.POINTER(_VP)]),
    "lmm_rv_describe": (ctypes.c_int, [_VP, _D, _I64, ctypes.POINTER(ctypes.c_int), _D]),
    "lmm_rv_get": (ctypes.c_int, [_VP, _D]),
    "lmm_rv_apply_scalar": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_VP)]),
    "lmm_rv_apply": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.POINTER(_VP)]),
    "lmm_rv_apply3": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, ctypes.c_double, ctypes.POINTER(_VP)]),
    "lmm_rv_average": (ctypes.c_int, [_VP, _D]),
    "lmm_rv_variance": (ctypes.c_int, [_VP, _D]),
    "lmm_rv_standard_error": (ctypes.c_int, [_VP, _D]),
    "lmm_rv_min_max": (ctypes.c_int, [_VP, _D, _D]),
    "lmm_process_destroy": (ctypes.c_int, [_VP]),
    "lmm_swaption_get_value": (ctypes.c_int, [_VP, ctypes.POINTER(LmmSwaptionDesc), _D, _D]),
    "lmm_bermudan_get_value": (ctypes.c_int, [_VP, ctypes.POINTER(LmmBermudanDesc), _D, _D, _D]),
    "lmm_bermudan_get_gradient": (ctypes.c_int, [_VP, ctypes.POINTER(LmmBermudanDesc), ctypes.c_int, ctypes.c_int,
                                                 _D, _D, _D, _D]),
    "lmm_bermudan_get_gradient_aad": (ctypes.c_int, [_VP, ctypes.POINTER(LmmBermudanDesc), ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_double, _D, _D, _D, _D]),
    "lmm_swaption_values_batch": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_VP), ctypes.c_int,
                                                 ctypes.POINTER(LmmSwaptionDesc), _D, _D]),
    "lmm_swaption_get_gradient": (ctypes.c_int, [_VP, ctypes.POINTER(LmmSwaptionDesc), ctypes.c_int, _D, _D, _D, _D]),
    "lmm_caplet_get_gradient": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_int, _D, _D]),
    "lmm_portfolio_create": (ctypes.c_int, [_VP, ctypes.POINTER(LmmPortfolioDesc), ctypes.POINTER(_VP)]),
    "lmm_portfolio_run": (ctypes.c_int, [_VP, _D, _D, _D, _D, _D, _D]),
    "lmm_portfolio_destroy": (ctypes.c_int, [_VP]),
    "lmm_values_mean_stderr_noalloc": (ctypes.c_int, [_VP, ctypes.c_int64, _VP, _D, _D]),
    "lmm_stats_enable_timing": (ctypes.c_int, [ctypes.c_int]),
    "lmm_stats_reset": (ctypes.c_int, []),
    "lmm_stats_h2d_bytes": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    "lmm_stats_pool_bytes": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "lmm_stats_get": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), _I64, _D]),
    "lmm_process_stream": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "lmm_probe_fp64_fma_rate": (ctypes.c_int, [_D]),
    "lmm_fp64_math_check": (ctypes.c_int, [ctypes.c_int64, _D, _D]),
}


class CalculationException(RuntimeError):
    """Raised for a failed valuation (the role of net.finmath.exception.CalculationException)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the native library and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"native library {path} is missing; run the build")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = ""):
    if rc != LMM_OK:
        msg = load().lmm_last_error().decode(errors="replace")
        if rc == LMM_ERR_INVALID:
            raise ValueError(f"{what}: {msg}")
        raise CalculationException(rc, f"{what}: {msg}")
    return rc
