"""The allocation-free mean / standard-error entry point, through the C ABI.

Some callers may not allocate device memory while they value: a pricing service that
reserves its whole device budget once at start-up and forbids allocator calls afterwards
(for instance a JVM host that shares one GPU between several engines, each held to a fixed
slice).  lmm_values_mean_stderr_noalloc serves them with a fixed scratch array inside the
library.  This test checks it against the product entry point's own mean and standard
error and against the oracle's Kahan mean and standard error, on two calls in a row (the
second call reuses the scratch the first one left behind), and checks that the device's
stream-ordered pool -- the one every allocation of the library comes from -- neither grows
nor hands out memory across the calls.  The test itself allocates its input with torch;
the entry point under test allocates nothing.  It sits in its own file so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

import finmath_gb300 as F
from finmath_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _call(L, values, stream):
    m, e = ctypes.c_double(), ctypes.c_double()
    rc = L.lmm_values_mean_stderr_noalloc(ctypes.c_void_p(values.data_ptr()), values.numel(),
                                          ctypes.c_void_p(stream.cuda_stream), ctypes.byref(m), ctypes.byref(e))
    assert rc == 0, L.lmm_last_error()
    return m.value, e.value


def _pool(L):
    r, u = ctypes.c_int64(), ctypes.c_int64()
    assert L.lmm_stats_pool_bytes(ctypes.byref(r), ctypes.byref(u)) == 0, L.lmm_last_error()
    return r.value, u.value


def test_noalloc_mean_stderr_matches_product_entry_point():
    import torch
    from oracle import pyoracle as po
    L = F.load()
    sim = W.build(W.LMM20, paths=5000)
    fix, plen, pay, K = W.bermudan_schedule(W.LMM20)
    ref = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate").getValues(sim, per_path=True)
    values = torch.tensor(ref["values"], dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    pool0 = _pool(L)
    for _ in range(2):
        mean, err = _call(L, values, stream)
        assert mean == pytest.approx(ref["value"], rel=1e-12)
        assert err == pytest.approx(ref["error"], rel=1e-10)
        assert mean == pytest.approx(po.kahan_average(ref["values"]), rel=1e-12)
        assert err == pytest.approx(po.standard_error(ref["values"]), rel=1e-10)
        assert _pool(L) == pool0
    sim.process.close()
    sim.process.brownianMotion.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = F.load()
    m, e = ctypes.c_double(), ctypes.c_double()
    rc = L.lmm_values_mean_stderr_noalloc(ctypes.c_void_p(16), (1 << 30) + 1, None, ctypes.byref(m), ctypes.byref(e))
    assert rc == F._lib.LMM_ERR_INVALID
    assert b"2^30" in L.lmm_last_error()
