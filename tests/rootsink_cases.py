"""Root-sink known-answer cases of CLM.jl's test suite (tests/golden/reference_cases.json,
"rootsink"), built into RootSinkState inputs, and their checks.  TEST INFRASTRUCTURE."""
import json
import os

import numpy as np

from clmgb import abi, rootsink

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)["rootsink"]


def varpar(g):
    return abi.Varpar(g["nlevsno"], g["nlevgrnd"], g["nlevsoi"], g["nlevurb"], g["nlevmaxurbgrnd"], 0)


def build(g, case):
    vp = varpar(g)
    rs = rootsink.RootSinkState(vp, case["nc"], case["np"], case["nl"])
    nsoi = g["nlevsoi"]
    rs["mask_hydrology"][:] = np.array(case["mask"], dtype=np.uint8)
    rs["col_itype"][:] = case["col_itype"]
    rs["col_landunit"][:] = case["col_landunit"]
    rs["lun_itype"][:] = case["lun_itype"]
    ppc = np.array(case["patches_per_col"])
    rs["col_patchi"][:] = np.concatenate([[1], 1 + np.cumsum(ppc)[:-1]])
    rs["col_npatches"][:] = ppc
    rs["patch_active"][:] = np.array(case["active"], dtype=np.uint8)
    rs["patch_wtcol"][:] = case["wtcol"]
    rs["rootr_patch"][:nsoi] = np.array(case["rootr"]).T
    rs["qflx_tran_veg_patch"][:] = case["tran_patch"]
    rs["qflx_tran_veg_col"][:] = case["tran_col"]
    rs["k_soil_root_patch"][:] = np.array(case["k"]).T
    rs["smp_l"][:] = np.array(case["smp"])[None, :]
    rs["vegwp_patch"][3] = case["vegwp4"]
    rs["frac_veg_nosno"][:] = case["fvn"]
    for j, z in enumerate(g["z_soil"]):
        rs["z"][g["nlevsno"] + j] = z
    return rs


def check(g, case, rs):
    """rs: host RootSinkState after the call."""
    nsoi = g["nlevsoi"]
    e = case["expect"]
    for c in range(case["nc"]):
        if "rootr_col" in e and e["rootr_col"][c] is not None:
            np.testing.assert_allclose(rs["rootr_col"][:nsoi, c], e["rootr_col"][c], rtol=0, atol=e["atol_rootr"],
                                       err_msg=case["name"])
        if "rootsoi" in e and e["rootsoi"][c] is not None:
            np.testing.assert_allclose(rs["qflx_rootsoi_col"][:nsoi, c], e["rootsoi"][c], rtol=0,
                                       atol=e["atol_rootsoi"], err_msg=case["name"])
    if "phs_neg" in e:
        np.testing.assert_allclose(rs["qflx_phs_neg_col"], e["phs_neg"], rtol=0, atol=1e-10)
    if "hydr_redist_negative" in e:
        assert np.all(rs["qflx_hydr_redist_patch"] < 0.0)
