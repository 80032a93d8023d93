"""Allocation failures on the GPU valuation path, injected on the host.

With LMM_FAULT_INJECT_ALLOC=n every device allocation after the first n fails as an
out-of-memory would (no allocator call, no GPU fault).  For a range of n the child process
builds the lmm20 simulation and values a Bermudan swaption through the C ABI: each step
either succeeds or fails with LMM_ERR_NOMEM (CalculationException) and the injected message,
every handle is destroyed, and the device pool holds no memory afterwards that it did not
hold before -- nothing leaks.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, sys
sys.path[:0] = [{root!r}, {root!r} + "/finmath-lib_gb300"]
import numpy as np
import finmath_gb300 as F
from finmath_gb300 import workloads as W, _lib
L = F.load()
def pool():
    r, u = ctypes.c_int64(), ctypes.c_int64()
    L.lmm_stats_pool_bytes(ctypes.byref(r), ctypes.byref(u))
    return u.value
base = None
outcome = "ok"
sim = None
try:
    # the pool exists once the library has touched the device
    import torch
    torch.cuda.init()
    base = pool()
    sim = W.build(W.LMM20, paths=2000)
    fix, plen, pay, K = W.bermudan_schedule(W.LMM20)
    F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate").getValues(sim)
except F.CalculationException as e:
    outcome = "nomem" if e.code == _lib.LMM_ERR_NOMEM and "injected" in str(e) else "other:" + str(e)
finally:
    if sim is not None:
        sim.process.close()
        sim.process.brownianMotion.close()
torch.cuda.synchronize()
print(outcome, pool() - base)
"""


@pytest.mark.parametrize("n", [0, 1, 2, 4, 8, 16, 24])
def test_valuation_path_fails_cleanly(n):
    env = dict(os.environ, LMM_FAULT_INJECT_ALLOC=str(n))
    out = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], capture_output=True, text=True, env=env,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    outcome, leaked = out.stdout.strip().split()[-2:]
    assert outcome in ("ok", "nomem"), outcome
    assert int(leaked) == 0
