"""lake_temperature! cases of CLM.jl's test suite (tests/golden/reference_cases.json,
"lake_temperature") and their checks.  TEST INFRASTRUCTURE."""
import json
import os

import numpy as np

from clmgb import abi, lake

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)["lake_temperature"]


def varpar(g):
    v = g["varpar"]
    assert v["nlevlak"] == abi.NLEVLAK
    return abi.Varpar(v["nlevsno"], v["nlevgrnd"], v["nlevsoi"], v["nlevurb"], v["nlevmaxurbgrnd"], 0)


def build(g, case):
    return lake.reference_test_state(varpar(g), case["nc"], zero_flux=case["zero_flux"])


def check(case, lk):
    for ch in case["checks"]:
        if ch == "t_lake_finite":
            assert np.all(np.isfinite(lk["t_lake"][0]))
        elif ch == "icethick_nonnegative":
            assert np.all(np.isfinite(lk["lake_icethick"])) and np.all(lk["lake_icethick"] >= 0.0)
        elif ch == "errsoi_finite":
            assert np.all(np.isfinite(lk["errsoi_col"]))
        elif ch == "errsoi_below_0.2":
            assert np.all(np.abs(lk["errsoi_col"]) < 0.2)
        else:
            raise AssertionError(ch)


def warm_state(vp, nc, seed):
    """Random lakes made ice- and snow-free over thawed soil: no phase change, so the
    energy check must close (errsoi absorbed into the sensible heat)."""
    lk = lake.random_state(vp, nc, seed=seed)
    ns, ng = vp.nlevsno, vp.nlevgrnd
    lk["lake_icefrac"][:] = 0.0
    lk["col_snl"][:] = 0
    lk["h2osno_no_layers"][:] = 0.0
    lk["t_lake"][:] = np.maximum(lk["t_lake"], 274.0)
    w = lk["h2osoi_liq"][ns:ns + ng] + lk["h2osoi_ice"][ns:ns + ng] / 0.917
    lk["t_soisno"][ns:ns + ng] = np.maximum(lk["t_soisno"][ns:ns + ng], 274.0)
    lk["h2osoi_liq"][ns:ns + ng] = w
    lk["h2osoi_ice"][ns:ns + ng] = 0.0
    return lk
