"""The oracle against independent golden vectors (CPU only).

MT19937 core + init_by_array against numpy; the nextDouble mapping of commons-math3;
the pseudo-inverse least-squares KATs of finmath-lib's LinearAlgebraTest; Wichura's
inverse normal against scipy's ndtri; tick rounding and Kahan means.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("seed", ["3141", "7", "1352", "0", "-5", str((1 << 40) + 3)])
def test_mt19937_words_match_numpy(seed):
    g = _load("mt19937_numpy.json")[seed]
    s = int(seed)
    assert po.mt_words(s, 64).tolist() == g["first"]
    assert po.mt_words(s, 64, skip=g["offset"]).tolist() == g["at_offset"]


def test_next_double_is_two_26_bit_draws():
    g = _load("mt19937_numpy.json")["3141"]["first"]
    u = po.mt_doubles(3141, 32)
    expect = [(((g[2 * i] >> 6) << 26) | (g[2 * i + 1] >> 6)) * 2.0 ** -52 for i in range(32)]
    assert u.tolist() == expect
    assert np.all((u >= 0.0) & (u < 1.0))


def test_seeded_state_is_init_by_array_of_long_halves():
    st = po.mt_seeded_state(3141)
    rs = np.random.RandomState(np.array([0, 3141], dtype=np.uint32))
    assert np.array_equal(st, rs._bit_generator.state["state"]["key"])
    assert st[0] == 0x80000000


def test_linear_algebra_pseudo_inverse_kats():
    path = os.path.join(GOLD, "linalg_kat.json")
    if not os.path.exists(path):
        pytest.skip("KAT fixture not generated")
    kat = _load("linalg_kat.json")
    assert len(kat["cases"]) >= 3
    for case in kat["cases"]:
        X = po.lstsq_pinv(np.array(case["A"]), np.array(case["B"]))
        for val, i, j in case["expected"]:
            assert abs(X[i, j] - val) <= kat["tolerance"], case["name"]


def test_icdf_against_ndtri():
    g = _load("icdf_ndtri.json")
    for p, z in zip(g["p"], g["z"]):
        v = po.icdf(p)
        assert abs(v - z) <= 1e-14 * max(1.0, abs(z)), (p, v, z)


def test_icdf_edges_and_symmetry():
    assert po.icdf(0.0) == 0.0           # r <= 0 -> 0 (NormalDistribution.java:141-142)
    assert po.icdf(0.5) == 0.0
    for p in (2.0 ** -30, 2.0 ** -7, 0.25, 0.375):  # 1 - p is exact for these
        assert po.icdf(p) == -po.icdf(1.0 - p)


def test_time_discretization_tick_rounding():
    t = po.time_discretization(0.0, 80, 0.25)
    assert t[1] == 0.25 and t[-1] == 20.0
    tick = 1.0 / (365.0 * 24.0)
    x = po.time_discretization(0.1, 3, 1.0 / 3.0)
    assert np.all(x == np.rint(x / tick) * tick)


def test_kahan_average_is_compensated():
    x = np.array([1.0] + [1e-16] * 100000)
    assert po.kahan_average(x) == pytest.approx((1.0 + 1e-11) / len(x), rel=1e-15)
