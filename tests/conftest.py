import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "finmath-lib_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


ORACLE_KEYS = ("dt", "T_end", "period", "tenor_end", "F", "corr_decay", "abcd", "curve_nodes", "curve_values")


def oracle_model(cfg, **kw):
    from oracle import pyoracle as po
    args = {k: cfg[k] for k in ORACLE_KEYS}
    args.update(kw)
    return po.build_model(**args)
