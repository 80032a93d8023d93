"""The integer accumulation behind the regression's cross-block sums (csrc/exact_sum.cuh),
compiled for the host and checked against exact rational sums.

The backward induction's last block adds the blocks' double-double X^T y partials by placing
each value into a 192-bit fixed-point accumulator (units of 2^(E - 1193), E the largest
exponent field), 32 lane accumulators joined by an xor-shuffle tree.  The driver
(tests/host_src/exact_sum_host.cu) runs the same functions on the CPU for 300 seeded sets
(one scale, a 2^200 range, zeros and subnormals, cancelling pairs, a 2^2000 range, signed
zeros): every lane ends with the same accumulator, hi is the double nearest to the exact
sum, and hi + lo is within 2^-100 of the largest input (values more than 2^170 below the
largest are dropped by design) and 2^-104 of the sum.
"""
import os
import shutil
import subprocess
from fractions import Fraction

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "finmath-lib_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("exact_sum") / "exact_sum_host")
    src = os.path.join(ROOT, "tests", "host_src", "exact_sum_host.cu")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
                    src, "-o", exe], check=True, capture_output=True)
    return exe


def test_exact_sums_match_rational_arithmetic(driver):
    out = subprocess.run([driver, "300"], check=True, capture_output=True, text=True).stdout.splitlines()
    assert len(out) == 300
    for line in out:
        left, right = line.split("|")
        tok = left.split()
        vals = [float.fromhex(t) for t in tok[1:]]
        assert len(vals) == 2 * int(tok[0])
        hi, lo = (float.fromhex(t) for t in right.split())
        exact = sum(Fraction(x) for x in vals)
        largest = max(abs(Fraction(x)) for x in vals)
        err = abs(Fraction(hi) + Fraction(lo) - exact)
        assert err <= largest * Fraction(2) ** -100 + abs(exact) * Fraction(2) ** -104
        nearest = float(exact)
        assert hi == nearest or abs(Fraction(hi) - exact) <= abs(Fraction(nearest) - exact)
