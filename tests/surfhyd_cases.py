"""Surface-hydrology known-answer cases of CLM.jl's test suite
(tests/golden/reference_cases.json, "surface_hydrology") as SurfHydState inputs, and
their checks.  TEST INFRASTRUCTURE."""
import json
import os

import numpy as np

from clmgb import surfhyd, synth

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)["surface_hydrology"]


def build(case):
    """(SurfHydState, config, stage mask) of a case; unset inputs are zero, masks one."""
    vp = synth.clm5_varpar()
    nc = case["nc"]
    sh = surfhyd.SurfHydState(vp, nc, nc, case["nl"], ng=case["ng"])
    sh["lun_itype"][:] = surfhyd.ISTSOIL
    sh["col_landunit"][:] = 1
    sh["col_gridcell"][:] = 1
    sh["col_cold"][:] = surfhyd.ISPVAL
    for m in ("mask_nolakec", "mask_hydrology", "mask_urban"):
        sh[m][:] = 1
    for m, v in case["masks"].items():
        sh[m][:] = v
    for k, v in case["inputs"].items():
        if k in ("icefrac3", "hksat3"):
            sh[k[:-1]][:3] = np.array(v, dtype=float).T
        elif k == "liq_top":
            sh["h2osoi_liq"][vp.nlevsno] = v
        else:
            sh[k][:] = v
    cfg = surfhyd.config(ng=case["ng"], **case["cfg"])
    return sh, cfg, surfhyd.stage_mask(case["stages"])


def check(case, before, sh):
    """The case's expectations on the host state `sh` after the call (`before`: the inputs)."""
    top = sh.vp.nlevsno
    for e in case["expect"]:
        if e["field"] == "pond_balance":
            dpond = sh["h2osoi_liq"][top] - np.array(e["pond0"])
            net = (e["rain"] - e["evap"] - sh["qflx_surf"]) * case["dtime"]
            np.testing.assert_allclose(dpond, net, rtol=0, atol=e["atol"], err_msg=case["name"])
            continue
        got = sh["h2osoi_liq"][top] if e["field"] == "liq_top" else sh[e["field"]]
        for c, v in enumerate(e["values"]):
            if v is None:
                continue
            assert abs(got[c] - v) <= e["atol"] + e["rtol"] * abs(v), (case["name"], e["field"], c, got[c], v)
    for k, cols in case["expect_nan"].items():
        assert np.all(np.isnan(sh[k][cols])), (case["name"], k)
    if any(n in case["stages"] for n in ("total_surface_runoff!", "update_urban_ponding!")):
        # only the top soil level is an urban pond; the snow levels are untouched
        assert np.array_equal(sh["h2osoi_liq"][:top], before["h2osoi_liq"][:top])
