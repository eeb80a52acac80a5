"""balance_check! column cases of CLM.jl's test suite (tests/golden/reference_cases.json,
"balance_check_columns") and their checks.  TEST INFRASTRUCTURE."""
import json
import math
import os

import numpy as np

from clmgb import abi, colbalance

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)["balance_check_columns"]


def build(case):
    cb = colbalance.ColBalanceState(None, case["nc"])
    cb["col_itype"][:] = 1
    cb["col_active"][:] = 1
    cb["begwb"][:] = 100.0
    cb["endwb"][:] = 100.0
    for k, v in case["inputs"].items():
        cb[k][:] = v
    return cb


def check(case, cb, rep):
    for e in case["expect"]:
        if "flag" in e:
            assert rep.flags & getattr(abi, "BAL_" + e["flag"]), (case["name"], rep.flags)
            continue
        x = cb[e["field"]]
        if "exact" in e:
            assert list(x) == e["exact"], (case["name"], x)
            continue
        for i in e["index"]:
            if e.get("nonfinite"):
                assert not math.isfinite(x[i]), case["name"]
            elif e.get("nonzero"):
                assert abs(x[i]) > 0.0, case["name"]
            else:
                assert abs(x[i] - e["value"]) <= e.get("atol", 0.0) + e.get("rtol", 0.0) * abs(e["value"]), \
                    (case["name"], i, x[i])
    for s in case["stops"]:
        assert colbalance.must_stop(rep, s["dastep"], case["dtime"], s["hard_error"]) == s["stop"], (case["name"], s)


def same_report(a, b):
    for (n, _) in abi.BalanceReport._fields_:
        x, y = getattr(a, n), getattr(b, n)
        if isinstance(x, float):
            assert np.array_equal(np.float64(x).view(np.uint64), np.float64(y).view(np.uint64)) or \
                (math.isnan(x) and math.isnan(y)), (n, x, y)
        else:
            assert x == y, (n, x, y)
