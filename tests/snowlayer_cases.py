"""Snow-layer known-answer cases of CLM.jl's test suite (tests/golden/reference_cases.json,
"snow_layers") as SnowLayerState inputs, and their checks.  TEST INFRASTRUCTURE."""
import json
import os

import numpy as np

from clmgb import snowlayers, synth

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)["snow_layers"]


def build(case):
    vp = synth.clm5_varpar()
    ns, nc = vp.nlevsno, case["nc"]
    sl = snowlayers.SnowLayerState(vp, nc, nc, 4)
    sl["lun_itype"][:] = [snowlayers.ISTSOIL, snowlayers.ISTCROP, snowlayers.ISTDLAK, snowlayers.ISTURB_MD]
    sl["lun_lakpoi"][:] = [0, 0, 1, 0]
    sl["lun_urbpoi"][:] = [0, 0, 0, 1]
    sl["col_landunit"][:] = 1
    sl["col_gridcell"][:] = 1
    sl["n_melt"][:] = 20.0
    sl["col_snl"][:] = case["snl"]
    sl["mask_nolakec"][:] = 1
    sl["mask_snow"][:] = 1
    for k, v in case["col"].items():
        sl[k][:] = v
    for k, v in case["snow"].get("all_levels", {}).items():
        sl[k][:] = v
    for k, v in case["snow"].items():
        if k == "all_levels":
            continue
        for i, x in enumerate(v):              # from the bottom snow level up
            sl[k][ns - 1 - i] = x
    # interfaces consistent with the thicknesses, the soil surface at 0
    if "dz" in case["snow"]:
        zi = np.zeros(ns + 1)
        for i in range(ns - 1, -1, -1):
            zi[i] = zi[i + 1] - sl["dz"][i, 0]
        sl["zi"][:ns + 1] = zi[:, None]
        sl["z"][:ns] = (zi[1:] - 0.5 * sl["dz"][:ns, 0])[:, None]
    return sl, snowlayers.config(), snowlayers.stage_mask(case["stages"])


def check(case, sl):
    ns = sl.vp.nlevsno
    for e in case["expect"]:
        w = e["what"]
        if w == "snl":
            assert np.all(sl["col_snl"] == e["value"]), (case["name"], sl["col_snl"])
        elif w == "bottom":
            got = sl[e["field"]][ns - 1]
            if e.get("exact"):
                assert np.all(got == e["value"]), (case["name"], got)
            else:
                np.testing.assert_allclose(got, e["value"], rtol=2.0 ** -26, err_msg=case["name"])
        elif w == "bottom_below":
            assert np.all(sl[e["field"]][ns - 1] < e["value"]), case["name"]
        elif w == "top_level_zero":
            for k in e["fields"]:
                assert np.all(sl[k][0] == 0.0), (case["name"], k)
        elif w == "masks":
            assert list(sl["mask_snow"]) == e["mask_snow"] and list(sl["mask_nosnow"]) == e["mask_nosnow"]
        else:
            raise AssertionError(w)


def active(sl):
    ns = sl.vp.nlevsno
    return np.arange(ns)[:, None] >= (ns + sl["col_snl"])[None, :]
