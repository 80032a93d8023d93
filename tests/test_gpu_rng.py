"""GPU MT19937 + inverse normal against the oracle (bit-exact uniforms)."""
import numpy as np
import pytest

import finmath_gb300 as F
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

# FP64 increments against the oracle's: the inverse normal's rational functions run on float
# pairs (two FP32 significands, 2^-47 relative per Horner step), 5e-14 relative at most
ICDF_REL = 5e-14


@pytest.mark.parametrize("seed", [3141, 7, 1352, -5])
@pytest.mark.parametrize("offset,count", [(0, 4096), (311, 1000), (123457, 3000), (2_500_001, 777)])
def test_uniforms_bit_exact(seed, offset, count):
    g = F.mersenne_twister_uniforms(seed, count, offset)
    o = po.mt_doubles(seed, count, skip=offset)
    assert np.array_equal(g, o)


def test_uniforms_across_many_chunks():
    # 3e6 values: the generator splits the stream into one chunk per resident CTA
    n = 3_000_000
    g = F.mersenne_twister_uniforms(7, n)
    o = po.mt_doubles(7, n)
    assert np.array_equal(g, o)


@pytest.mark.parametrize("P,T,Fk", [(5000, 20, 3), (1, 7, 2), (33, 5, 1), (1000, 13, 10)])
def test_brownian_increments_fp64(P, T, Fk):
    td = F.TimeDiscretizationFromArray(0.0, T, 0.5)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, Fk, P, 3141)
    ref = po.brownian_increments(td.getAsDoubleArray(), Fk, P, 3141)
    worst = 0.0
    for t in range(T):
        for k in range(Fk):
            g = bm.getBrownianIncrement(t, k)
            r = ref[t, k]
            worst = max(worst, float(np.max(np.abs(g - r) / np.maximum(np.abs(r), 1e-300))))
    # the GPU evaluates the same rational functions in double-float arithmetic on the FP32
    # pipe (about 2^-47 relative per Horner step, no cancellation), tails through CUDA's log
    assert worst <= ICDF_REL


def test_brownian_increments_mixed_precision():
    td = F.TimeDiscretizationFromArray(0.0, 20, 0.5)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, 3, 5000, 3141, F.PRECISION_MIXED)
    ref = po.brownian_increments(td.getAsDoubleArray(), 3, 5000, 3141)
    for t in (0, 7, 19):
        g = bm.getBrownianIncrement(t, 2)
        assert np.max(np.abs(g - ref[t, 2])) < 2e-6 * np.max(np.abs(ref[t, 2]))


@pytest.mark.parametrize("P,T,Fk", [(40000, 3, 2), (700, 80, 10), (12345, 11, 7)])
def test_increments_tile_edges_fp64(P, T, Fk):
    """The generator writes the increments through a tile of 16 (FP64) paths: fewer draws per
    path than one round (several drains per round), 800 per path, and chunk edges inside paths."""
    td = F.TimeDiscretizationFromArray(0.0, T, 0.25)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, Fk, P, 7)
    ref = po.brownian_increments(td.getAsDoubleArray(), Fk, P, 7)
    for t in sorted({0, T // 2, T - 1}):
        for k in sorted({0, Fk - 1}):
            g = bm.getBrownianIncrement(t, k)
            r = ref[t, k]
            assert float(np.max(np.abs(g - r) / np.maximum(np.abs(r), 1e-300))) <= ICDF_REL


@pytest.mark.parametrize("P,T,Fk", [(40000, 3, 2), (12345, 11, 7)])
def test_increments_tile_edges_mixed(P, T, Fk):
    """FP32 increments (tile of 32 paths) over every row against the FP64 oracle."""
    td = F.TimeDiscretizationFromArray(0.0, T, 0.25)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, Fk, P, 7, F.PRECISION_MIXED)
    ref = po.brownian_increments(td.getAsDoubleArray(), Fk, P, 7)
    for t in range(T):
        for k in range(Fk):
            g = bm.getBrownianIncrement(t, k)
            assert np.max(np.abs(g - ref[t, k])) < 2e-6 * np.max(np.abs(ref[t, k]))


def test_inverse_normal_error_distribution_fp64():
    """2^22 FP64 increments (one time step, 1 factor, unit step): the double-float inverse
    normal's error against the oracle's FP64 evaluation, worst case and mean."""
    P = 1 << 22
    td = F.TimeDiscretizationFromArray(0.0, 1, 1.0)
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, 1, P, 1352)
    g = bm.getBrownianIncrement(0, 0)
    r = po.brownian_increments(td.getAsDoubleArray(), 1, P, 1352)[0, 0]
    rel = np.abs(g - r) / np.maximum(np.abs(r), 1e-300)
    assert float(np.max(rel)) <= ICDF_REL
    assert float(np.mean(rel)) <= 1e-14
    bm.close()
