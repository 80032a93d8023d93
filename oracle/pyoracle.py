"""ctypes binding of the C oracle (oracle/lmm_oracle.c).

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module; it checks the CUDA library and never stands
in for it.

The helpers below assemble a LIBOR market model from the same parametric inputs the
reference's tests use (tick-rounded time grids, an exponential-decay correlation
reduced to F factors, a four-parameter volatility, a forward curve given by nodes and
the discount curve derived from it), using only the oracle's own restatement of
finmath-lib's setup code.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "lmm_oracle.c")
_LIB = os.path.join(_HERE, "_build", "liblmm_oracle.so")

_D = ctypes.POINTER(ctypes.c_double)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_U8 = ctypes.POINTER(ctypes.c_uint8)


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, OpenMP over paths)."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < max(
            os.path.getmtime(_SRC), os.path.getmtime(os.path.join(_HERE, "lmm_oracle.h"))):
        tmp = _LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


class _OrcLmm(ctypes.Structure):
    _fields_ = [("T", ctypes.c_int), ("times", _D), ("N", ctypes.c_int), ("tenor", _D),
                ("F", ctypes.c_int), ("loadings", _D), ("variance", _D),
                ("initial_forwards", _D), ("discount_chain", _D), ("libor_cap", ctypes.c_double),
                ("scheme", ctypes.c_int), ("measure", ctypes.c_int), ("state_space", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        L.orc_mt_words.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _U32]
        L.orc_mt_doubles.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _D]
        L.orc_mt_seeded_state.argtypes = [ctypes.c_int64, _U32]
        L.orc_icdf_wichura.argtypes = [ctypes.c_double]
        L.orc_icdf_wichura.restype = ctypes.c_double
        L.orc_round_to_tick.argtypes = [ctypes.c_double]
        L.orc_round_to_tick.restype = ctypes.c_double
        L.orc_time_discretization.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_double, _D]
        L.orc_brownian_increments.argtypes = [_D, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D]
        L.orc_factor_reduction.argtypes = [_D, ctypes.c_int, ctypes.c_int, _D]
        L.orc_lstsq_pinv.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D, _D]
        L.orc_exp_decay_correlation.argtypes = [_D, ctypes.c_int, ctypes.c_int, ctypes.c_double, _D, _D]
        L.orc_vol_abcd.argtypes = [_D, ctypes.c_int, _D, ctypes.c_int] + [ctypes.c_double] * 4 + [_D]
        L.orc_covariance_tables.argtypes = [ctypes.c_int] * 3 + [_D] * 5
        L.orc_curve_forward.argtypes = [_D, _D, ctypes.c_int, ctypes.c_double]
        L.orc_curve_forward.restype = ctypes.c_double
        L.orc_discount_factor_from_forward_curve.argtypes = [_D, _D, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_discount_factor_from_forward_curve.restype = ctypes.c_double
        L.orc_numeraire_discount_chain.argtypes = [_D, ctypes.c_int, _D, _D]
        L.orc_simulate.argtypes = [ctypes.POINTER(_OrcLmm), ctypes.c_int, _D, _U8, ctypes.c_int]
        L.orc_simulate.restype = ctypes.c_void_p
        L.orc_sim_free.argtypes = [ctypes.c_void_p]
        L.orc_sim_process_value.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _D]
        L.orc_sim_numeraire.argtypes = [ctypes.c_void_p, ctypes.c_double, _D]
        L.orc_sim_numeraire_unadjusted.argtypes = [ctypes.c_void_p, ctypes.c_double, _D]
        L.orc_kahan_average.argtypes = [_D, ctypes.c_int64]
        L.orc_kahan_average.restype = ctypes.c_double
        L.orc_standard_error.argtypes = [_D, ctypes.c_int64]
        L.orc_standard_error.restype = ctypes.c_double
        L.orc_swaption.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _D, _D, _D, _D,
                                   ctypes.c_double, _D, _D, _D]
        L.orc_bermudan.argtypes = [ctypes.c_void_p, ctypes.c_int, _U8, _D, _D, _D, _D, _D, ctypes.c_int,
                                   ctypes.c_int, _D, _D, _D, _D]
        L.orc_bermudan_frozen.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, _D, _D, _D, _D, ctypes.c_int, _D, _D]
        L.orc_bermudan_aad.argtypes = [ctypes.c_void_p, ctypes.c_int, _U8, _D, _D, _D, _D, _D, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_double, _D, _D]
        _lib = L
    return _lib


def _p(a, t=_D):
    return a.ctypes.data_as(t) if a is not None else None


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# --------------------------------------------------------------------------- RNG
def mt_words(seed: int, count: int, skip: int = 0) -> np.ndarray:
    out = np.empty(count, dtype=np.uint32)
    lib().orc_mt_words(seed, skip, count, _p(out, _U32))
    return out


def mt_doubles(seed: int, count: int, skip: int = 0) -> np.ndarray:
    out = np.empty(count, dtype=np.float64)
    lib().orc_mt_doubles(seed, skip, count, _p(out))
    return out


def mt_seeded_state(seed: int) -> np.ndarray:
    out = np.empty(624, dtype=np.uint32)
    lib().orc_mt_seeded_state(seed, _p(out, _U32))
    return out


def icdf(p: float) -> float:
    return lib().orc_icdf_wichura(float(p))


def brownian_increments(times, F: int, P: int, seed: int) -> np.ndarray:
    times = f64(times)
    T = len(times) - 1
    out = np.empty((T, F, P), dtype=np.float64)
    lib().orc_brownian_increments(_p(times), T, F, P, seed, _p(out))
    return out


# --------------------------------------------------------------------------- setup
def time_discretization(initial: float, n: int, dt: float) -> np.ndarray:
    out = np.empty(n + 1, dtype=np.float64)
    lib().orc_time_discretization(initial, n, dt, _p(out))
    return out


def factor_reduction(corr, F: int) -> np.ndarray:
    corr = f64(corr)
    n = corr.shape[0]
    out = np.empty((n, F), dtype=np.float64)
    lib().orc_factor_reduction(_p(corr), n, F, _p(out))
    return out


def lstsq_pinv(A, B) -> np.ndarray:
    A = f64(np.atleast_2d(A))
    B = f64(B)
    vec = B.ndim == 1
    B2 = B.reshape(A.shape[0], -1)
    X = np.empty((A.shape[1], B2.shape[1]), dtype=np.float64)
    lib().orc_lstsq_pinv(A.shape[0], A.shape[1], B2.shape[1], _p(A), _p(f64(B2)), _p(X))
    return X[:, 0] if vec else X


@dataclass
class Model:
    """Tables of a LIBOR market model, evaluated the way finmath-lib evaluates them."""
    times: np.ndarray          # T+1
    tenor: np.ndarray          # N+1
    factor: np.ndarray         # [N][F]
    corr: np.ndarray           # [N][N] reduced correlation
    vol: np.ndarray            # [T][N]
    loadings: np.ndarray       # [T][N][F]
    variance: np.ndarray       # [T][N]
    initial_forwards: np.ndarray  # [N]
    discount_chain: np.ndarray | None  # [N+1]
    libor_cap: float = 1e5
    scheme: int = 1            # EULER_FUNCTIONAL (0 EULER, 2 PREDICTOR_CORRECTOR, 3 ..._FUNCTIONAL)
    measure: int = 0           # SPOT (1 TERMINAL)
    state_space: int = 0       # LOGNORMAL (1 NORMAL)

    @property
    def T(self):
        return len(self.times) - 1

    @property
    def N(self):
        return len(self.tenor) - 1

    @property
    def F(self):
        return self.factor.shape[1]


def build_model(*, dt: float, T_end: float, period: float, tenor_end: float, F: int,
                corr_decay: float, abcd, curve_nodes, curve_values, payment_offset=None,
                discount_curve: bool = True, libor_cap: float = 1e5, scheme: int = 1,
                vol_matrix=None, measure: int = 0, state_space: int = 0, times=None, tenor=None) -> Model:
    """times / tenor, when given, replace the uniform grids of dt / T_end and period / tenor_end
    (date-derived grids, already tick-rounded as TimeDiscretizationFromArray rounds them)."""
    L = lib()
    times = time_discretization(0.0, int(round(T_end / dt)), dt) if times is None else f64(times)
    tenor = time_discretization(0.0, int(round(tenor_end / period)), period) if tenor is None else f64(tenor)
    T, N = len(times) - 1, len(tenor) - 1
    factor = np.empty((N, F)); corr = np.empty((N, N))
    L.orc_exp_decay_correlation(_p(tenor), N, F, corr_decay, _p(factor), _p(corr))
    if vol_matrix is None:
        vol = np.empty((T, N))
        a, b, c, d = abcd
        L.orc_vol_abcd(_p(times), T, _p(tenor), N, a, b, c, d, _p(vol))
    else:
        vol = f64(vol_matrix)
    loadings = np.empty((T, N, F)); variance = np.empty((T, N))
    L.orc_covariance_tables(T, N, F, _p(vol), _p(factor), _p(corr), _p(loadings), _p(variance))
    cx, cy = f64(curve_nodes), f64(curve_values)
    po = period if payment_offset is None else payment_offset
    fwd = np.empty(N)
    for j in range(N):
        f = L.orc_curve_forward(_p(cx), _p(cy), len(cx), tenor[j])
        plen = tenor[j + 1] - tenor[j]
        if plen != po:  # ForwardCurveInterpolation.getForward(model, t, paymentOffset) :338-346
            f = (np.exp(np.log(1 + f * po) * plen / po) - 1.0) / plen
        fwd[j] = f
    chain = None
    if discount_curve:
        df = np.array([L.orc_discount_factor_from_forward_curve(_p(cx), _p(cy), len(cx), po, t) for t in tenor])
        chain = np.empty(N + 1)
        L.orc_numeraire_discount_chain(_p(tenor), N, _p(df), _p(chain))
    return Model(times, tenor, factor, corr, vol, loadings, variance, fwd, chain, libor_cap, scheme, measure,
                 state_space)


class Simulation:
    """Euler process + numeraire over given Brownian increments (oracle side)."""

    def __init__(self, model: Model, dW: np.ndarray, observe=None, threads: int = 0):
        self.model = model
        self._keep = [f64(model.times), f64(model.tenor), f64(model.loadings), f64(model.variance),
                      f64(model.initial_forwards),
                      None if model.discount_chain is None else f64(model.discount_chain)]
        t, tn, ld, var, fw, ch = self._keep
        self._s = _OrcLmm(model.T, _p(t), model.N, _p(tn), model.F, _p(ld), _p(var), _p(fw), _p(ch),
                          model.libor_cap, model.scheme, model.measure, model.state_space)
        self.P = dW.shape[2]
        dW = f64(dW)
        obs = None if observe is None else np.ascontiguousarray(observe, dtype=np.uint8)
        self._h = lib().orc_simulate(ctypes.byref(self._s), self.P, _p(dW), _p(obs, _U8), threads)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_sim_free(self._h)
            self._h = None

    def process_value(self, time_index: int, component: int) -> np.ndarray:
        out = np.empty(self.P)
        rc = lib().orc_sim_process_value(self._h, time_index, component, _p(out))
        if rc != 0:
            raise ValueError(f"process value not available (rc={rc})")
        return out

    def numeraire(self, time: float) -> np.ndarray:
        out = np.empty(self.P)
        rc = lib().orc_sim_numeraire(self._h, time, _p(out))
        if rc < 0:
            raise ValueError("numeraire off the tenor grid")
        return out

    def numeraire_unadjusted(self, time: float) -> np.ndarray:
        out = np.empty(self.P)
        if lib().orc_sim_numeraire_unadjusted(self._h, time, _p(out)) < 0:
            raise ValueError("numeraire off the tenor grid")
        return out

    def swaption(self, exercise, fixing, payment, strike, notional=1.0, per_path=False):
        fixing, payment = f64(fixing), f64(payment)
        strike = f64(np.broadcast_to(strike, fixing.shape))
        v, e = ctypes.c_double(), ctypes.c_double()
        pp = np.empty(self.P) if per_path else None
        rc = lib().orc_swaption(self._h, exercise, len(fixing), _p(fixing), _p(payment), None, _p(strike),
                                notional, ctypes.byref(v), ctypes.byref(e), _p(pp))
        if rc != 0:
            raise ValueError(f"swaption failed rc={rc}")
        return (v.value, e.value, pp) if per_path else (v.value, e.value)

    def bermudan(self, fixing, period_length, payment, strike, exercisable=None, notional=None,
                 callable_=True, basis_id=1, per_path=False):
        fixing, period_length, payment = f64(fixing), f64(period_length), f64(payment)
        n = len(fixing)
        strike = f64(np.broadcast_to(strike, (n,)))
        notional = f64(np.ones(n) if notional is None else np.broadcast_to(notional, (n,)))
        ex = np.ascontiguousarray(np.ones(n) if exercisable is None else exercisable, dtype=np.uint8)
        v, e = ctypes.c_double(), ctypes.c_double()
        pp = np.empty(self.P) if per_path else None
        et = np.empty(self.P) if per_path else None
        rc = lib().orc_bermudan(self._h, n, _p(ex, _U8), _p(fixing), _p(period_length), _p(payment),
                                _p(notional), _p(strike), int(callable_), basis_id, ctypes.byref(v),
                                ctypes.byref(e), _p(pp), _p(et))
        if rc != 0:
            raise ValueError(f"bermudan failed rc={rc}")
        return (v.value, e.value, pp, et) if per_path else (v.value, e.value)


def _bermudan_aad(self, fixing, period_length, payment, strike, method="ZERO", width=0.05, exercisable=None,
                  notional=None, callable_=True, basis_id=1):
    """The reference AAD's adjoint weights omega[k][p] of the discounted cash flows (see
    orc_bermudan_aad) and the forward value."""
    fixing, period_length, payment = f64(fixing), f64(period_length), f64(payment)
    n = len(fixing)
    strike = f64(np.broadcast_to(strike, (n,)))
    notional = f64(np.ones(n) if notional is None else np.broadcast_to(notional, (n,)))
    ex = np.ascontiguousarray(np.ones(n) if exercisable is None else exercisable, dtype=np.uint8)
    v = ctypes.c_double()
    omega = np.empty((n, self.P))
    m = {"ZERO": 0, "DISCRETE_DELTA": 1}[method]
    rc = lib().orc_bermudan_aad(self._h, n, _p(ex, _U8), _p(fixing), _p(period_length), _p(payment), _p(notional),
                                _p(strike), int(callable_), basis_id, m, float(width), ctypes.byref(v), _p(omega))
    if rc != 0:
        raise ValueError(f"bermudan aad failed rc={rc}")
    return v.value, omega


Simulation.bermudan_aad = _bermudan_aad


def _bermudan_frozen(self, fixing, period_length, payment, strike, exercise_time, notional=None, callable_=True):
    fixing, period_length, payment = f64(fixing), f64(period_length), f64(payment)
    n = len(fixing)
    strike = f64(np.broadcast_to(strike, (n,)))
    notional = f64(np.ones(n) if notional is None else np.broadcast_to(notional, (n,)))
    ex = f64(exercise_time)
    v = ctypes.c_double()
    rc = lib().orc_bermudan_frozen(self._h, n, _p(fixing), _p(period_length), _p(payment), _p(notional), _p(strike),
                                   int(callable_), _p(ex), ctypes.byref(v))
    if rc != 0:
        raise ValueError(f"frozen bermudan failed rc={rc}")
    return v.value


Simulation.bermudan_frozen = _bermudan_frozen


def kahan_average(x) -> float:
    x = f64(x)
    return lib().orc_kahan_average(_p(x), len(x))


def standard_error(x) -> float:
    """getStandardError of RandomVariableFromDoubleArray.java:419-428 (Kahan mean and variance)."""
    x = f64(x)
    return lib().orc_standard_error(_p(x), len(x))
