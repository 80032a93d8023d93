"""Generate the golden fixtures under tests/golden/.

    python tests/golden/make_golden.py

Sources
  mt19937_numpy.json   MT19937 words from numpy's independent MT19937 implementation
                       (RandomState seeded with the two 32-bit halves of the long seed,
                       i.e. init_by_array), which pins the oracle's MT core and seeding.
  linalg_kat.json      The pseudo-inverse known-answer tests of finmath-lib's
                       src/test/java/net/finmath/functions/LinearAlgebraTest.java,
                       read from the reference's source text when it is present.
  icdf_ndtri.json      Standard normal quantiles from scipy.special.ndtri (Cephes), an
                       independent implementation against which Wichura's AS241 agrees
                       to ~1e-15.
  oracle_lmm20.json    The oracle's own lmm20 results (5,000 paths): a snapshot that
                       detects drift of the oracle across builds and machines.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "finmath-lib_gb300"))

REF_TEST = "/root/reference/src/test/java/net/finmath/functions/LinearAlgebraTest.java"


def mt_numpy():
    out = {}
    for seed in (3141, 7, 1352, 0, -5, (1 << 40) + 3):
        u = seed & 0xFFFFFFFFFFFFFFFF
        key = np.array([u >> 32, u & 0xFFFFFFFF], dtype=np.uint64).astype(np.uint32)
        rs = np.random.RandomState(key)
        words = rs._bit_generator.random_raw(100003 + 64).astype(np.uint32)
        out[str(seed)] = {"first": [int(x) for x in words[:64]], "offset": 100003,
                          "at_offset": [int(x) for x in words[100003:100003 + 64]]}
    return out


def linalg_kat():
    if not os.path.exists(REF_TEST):
        return None
    src = open(REF_TEST).read()
    cases = []
    # every "double[][] A/matrix = new double[][] { {..},{..} };" followed by a right-hand side
    for m in re.finditer(r"public void (testSolveLinearEquationLeastSquare\w*)\(\)(.*?)\n\t}", src, re.S):
        name, body = m.group(1), m.group(2)
        mats = re.findall(r"final double\[\]\[\] (\w+) = new double\[\]\[\] \{(.*?)\};", body, re.S)
        vecs = re.findall(r"final double\[\] (\w+) = new double\[\] \{(.*?)\};", body, re.S)
        asserts = re.findall(r"assertEquals\(\"[^\"]*\",\s*([-0-9./]+),\s*(\w+)\[(\d+)\](?:\[(\d+)\])?,\s*1E-12\)", body)
        if not mats or not asserts:
            continue

        def parse_rows(txt):
            rows = re.findall(r"\{([^{}]*)\}", txt)
            return [[float(eval(v)) for v in r.split(",") if v.strip()] for r in rows]
        A = parse_rows(mats[0][1])
        if len(mats) > 1:
            B = parse_rows(mats[1][1])
        elif vecs:
            B = [[float(eval(v))] for v in vecs[0][1].split(",") if v.strip()]
        else:
            continue
        exp = [(float(eval(v)), int(i), int(j) if j else 0) for v, _, i, j in asserts]
        cases.append({"name": name, "A": A, "B": B, "expected": exp})
    return {"source": "src/test/java/net/finmath/functions/LinearAlgebraTest.java", "tolerance": 1e-12,
            "cases": cases}


def icdf():
    from scipy.special import ndtri
    p = np.concatenate([np.linspace(1e-12, 1 - 1e-12, 2001), [1e-300, 1e-100, 1e-20, 2.0 ** -52, 0.075, 0.925,
                                                              0.5, 0.5 + 1e-9, 1 - 2.0 ** -52]])
    return {"p": [float(x) for x in p], "z": [float(x) for x in ndtri(p)]}


def oracle_lmm20():
    from oracle import pyoracle as po
    from finmath_gb300 import workloads as W
    cfg = W.LMM20
    m = po.build_model(**{k: cfg[k] for k in ("dt", "T_end", "period", "tenor_end", "F", "corr_decay", "abcd",
                                              "curve_nodes", "curve_values")})
    P = cfg["paths"]
    dW = po.brownian_increments(m.times, m.F, P, cfg["seed"])
    sim = po.Simulation(m, dW)
    ex, fix, pay, K = W.swaption_schedule(cfg)
    sw = sim.swaption(ex, fix, pay, K)
    bf, bl, bp, bK = W.bermudan_schedule(cfg)
    b0 = sim.bermudan(bf, bl, bp, bK, basis_id=0)
    b1 = sim.bermudan(bf, bl, bp, bK, basis_id=1)
    return {"paths": P, "swaption": list(sw), "bermudan_reference_basis": list(b0), "bermudan_swaprate_basis": list(b1),
            "L_10_19_first8": [float(x) for x in sim.process_value(10, 19)[:8]],
            "numeraire_10_first8": [float(x) for x in sim.numeraire(10.0)[:8]],
            "dW_t3_f1_first8": [float(x) for x in dW[3, 1, :8]]}


def main():
    with open(os.path.join(HERE, "mt19937_numpy.json"), "w") as f:
        json.dump(mt_numpy(), f)
    kat = linalg_kat()
    if kat is not None:
        with open(os.path.join(HERE, "linalg_kat.json"), "w") as f:
            json.dump(kat, f, indent=1)
    with open(os.path.join(HERE, "icdf_ndtri.json"), "w") as f:
        json.dump(icdf(), f)
    with open(os.path.join(HERE, "oracle_lmm20.json"), "w") as f:
        json.dump(oracle_lmm20(), f, indent=1)


if __name__ == "__main__":
    main()
