"""Named valuation cases, run from the command line (used to profile single kernels):

    python -m finmath_gb300.cases --case valuation|greeks|portfolio --precision fp64|mixed \\
        --paths 65536 --repeat 3 [--workload lmm40] [--stride 1] [--timing]

Each repetition regenerates the increments (new seed set) and values the workload's
Bermudan swaption; 'greeks' adds its adjoint deltas and vegas; 'portfolio' runs a
16-product portfolio with Greeks through one graph launch.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import lmm as F
from . import workloads as W
from ._lib import PRECISION_FP64, PRECISION_MIXED


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=["valuation", "greeks", "portfolio"], default="valuation")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--paths", type=int, default=65536)
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--workload", default="lmm40")
    ap.add_argument("--stride", type=int, default=1)
    ap.add_argument("--timing", action="store_true", help="CUDA-event time per kernel family, after the first repetition")
    args = ap.parse_args(argv)
    from ._lib import load
    lib = load()
    if args.timing:
        lib.lmm_stats_enable_timing(1)
    cfg = W.WORKLOADS[args.workload]
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    sim = W.build(cfg, paths=args.paths, precision=prec)
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    out = None
    if args.case == "portfolio":
        pf = F.Portfolio(sim, W.portfolio_products(cfg, n=16, seed=20261203), True, args.stride, 4, 128, 0)
        for r in range(args.repeat):
            out = pf.run()["total_ms"]
            if r == 0:
                lib.lmm_stats_reset()
        pf.close()
    else:
        for r in range(args.repeat):
            sim.process.brownianMotion.setSeed(cfg["seed"] + r)
            if args.case == "greeks":
                out = berm.getGradient(sim, checkpointStride=args.stride)["value"]
            else:
                out = berm.getValue(sim)
            if r == 0:
                lib.lmm_stats_reset()
    print(json.dumps({"case": args.case, "precision": args.precision, "paths": args.paths, "last": out,
                      "kernels": F.kernel_stats()}))


if __name__ == "__main__":
    main()
