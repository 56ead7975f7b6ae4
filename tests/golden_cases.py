"""Golden fixtures (tests/golden/) and the inputs that reproduce them.

TEST INFRASTRUCTURE.  Each GEMM fixture holds the result array the reference
demo's own CPU check computed (made by tests/golden/make_golden.py); the
inputs are replayed with tests/gbgen.py.  ``gemm_case`` returns, per
transpose mode, the operand buffers as that demo passed them to the device.
"""
import json
import os

import numpy as np

import gbgen

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MODES = ("NN", "NT", "TN", "TT")


def index():
    with open(os.path.join(HERE, "golden.json")) as f:
        return json.load(f)


def expected(meta):
    return np.load(os.path.join(HERE, meta["file"]))


def gemm_names():
    return sorted(k for k, v in index().items() if v["demo"] not in ("transpose", "stencil"))


def gemm_case(name):
    """-> meta, dict mode -> (A, lda, B, ldb, ldc, C_shape)"""
    meta = index()[name]
    M, K, N = meta["M"], meta["K"], meta["N"]
    demo = meta["demo"]
    if demo == "dgemm_v11":
        d = gbgen.demo_dgemm_v11(M, K, N)
        ops = {"NN": (d["A"], d["lda"], d["B"], d["ldb"]),
               "NT": (d["A"], d["lda"], d["BT"], d["ldbT"]),
               "TN": (d["AT"], d["ldaT"], d["B"], d["ldb"]),
               "TT": (d["AT"], d["ldaT"], d["BT"], d["ldbT"])}
        ldc, crows = d["ldc"], d["M0"]
    else:
        if demo.startswith("sgemm"):
            d = gbgen.demo_sgemm(M, K, N)
        else:
            d = gbgen.demo_irr(M, K, N, np.float64 if "dgemm" in demo else np.float32)
        ops = {"NN": (d["A"], K, d["B"], N), "NT": (d["A"], K, d["BT"], K),
               "TN": (d["AT"], M, d["B"], N), "TT": (d["AT"], M, d["BT"], K)}
        ldc, crows = N, M
    return meta, ops, ldc, crows
