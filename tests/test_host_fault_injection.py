"""Host-side fault injection: a device allocation failure surfaces as LMM_ERR_NOMEM.

The reference turns failures on its valuation path into CalculationException
(montecarlo/process/EulerSchemeFromProcessModel.java:211-214, 270-272) and
AbstractMonteCarloProduct.getValue(double, Model) returns null for one
(montecarlo/AbstractMonteCarloProduct.java:38-45).  The library's counterpart is an int
status and lmm_last_error(); LMM_FAULT_INJECT_ALLOC=n makes every device allocation after the
first n fail as an out-of-memory would, on the host, without calling the allocator -- no GPU
is faulted.  The first allocation of a device random variable happens before any other CUDA
call, so with n = 0 the path is testable without a GPU; the GPU test covers the valuation
path's allocations.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, sys
sys.path[:0] = [{root!r}, {root!r} + "/finmath-lib_gb300"]
import numpy as np
from finmath_gb300 import _lib
L = _lib.load()
h = ctypes.c_void_p()
x = np.arange(4, dtype=np.float64)
rc = L.lmm_rv_create(0.0, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4, ctypes.byref(h))
print(rc, h.value, L.lmm_last_error().decode())
"""


def test_injected_allocation_failure_is_nomem_with_a_message():
    env = dict(os.environ, LMM_FAULT_INJECT_ALLOC="0")
    out = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], capture_output=True, text=True, env=env,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    rc, handle, msg = out.stdout.strip().split(" ", 2)
    assert int(rc) == -2  # LMM_ERR_NOMEM
    assert handle == "None"  # no handle escapes a failed creation
    assert "injected" in msg and "random variable" in msg
