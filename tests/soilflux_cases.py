"""soil_fluxes! scenarios of CLM.jl's test suite (tests/golden/reference_cases.json,
"soil_fluxes") as SoilFluxState inputs, and the properties that suite checks.
TEST INFRASTRUCTURE."""
import json
import os

import numpy as np

from clmgb import soilflux, synth

HERE = os.path.dirname(os.path.abspath(__file__))
LEVEL = {"t_ssbef": "t_ssbef", "t_soisno": "t_soisno", "fact": "fact", "liq": "h2osoi_liq", "ice": "h2osoi_ice"}


def load():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)["soil_fluxes"]


def build(inputs):
    vp = synth.clm5_varpar()
    fs = soilflux.SoilFluxState(vp, 1, 1, 1)
    fs["lun_itype"][:] = soilflux.ISTSOIL
    fs["col_itype"][:] = soilflux.ISTSOIL
    fs["col_patchi"][:] = 1
    fs["col_patchf"][:] = 1
    fs["patch_column"][:] = 1
    fs["patch_landunit"][:] = 1
    fs["patch_wtcol"][:] = 1.0
    fs["mask_nolakec"][:] = 1
    fs["mask_nolakep"][:] = 1
    fs["col_snl"][:] = inputs["snl"]
    for k, v in inputs.items():
        if k == "snl":
            continue
        fs[LEVEL.get(k, k)][...] = v
    return fs


def check(g, scen, fs):
    """The properties test_soil_fluxes.jl asserts, on the host state after the call."""
    hvap = g["hvap"]
    for name in ("eflx_sh_grnd", "eflx_sh_tot", "eflx_soil_grnd", "eflx_lh_tot", "eflx_lwrad_out", "eflx_lwrad_net",
                 "errsoi_patch", "errsoi_col", "qflx_evap_soi", "qflx_evap_tot", "qflx_evap_can",
                 "qflx_liqevap_from_top_layer", "qflx_solidevap_from_top_layer", "t_skin"):
        assert np.isfinite(fs[name]).all(), (scen["name"], name)
    c = scen["checks"]
    if "identities" in c:
        np.testing.assert_allclose(fs["eflx_sh_tot"], fs["eflx_sh_veg"] + fs["eflx_sh_grnd"] + fs["eflx_sh_stem"],
                                   rtol=1e-12)
        np.testing.assert_allclose(fs["qflx_evap_tot"], fs["qflx_evap_veg"] + fs["qflx_evap_soi"], rtol=1e-12)
        np.testing.assert_allclose(fs["qflx_evap_can"], fs["qflx_evap_veg"] - fs["qflx_tran_veg"], rtol=1e-12)
        np.testing.assert_allclose(fs["eflx_lh_vegt"], fs["qflx_tran_veg"] * hvap, rtol=1e-12)
        assert np.array_equal(fs["eflx_soil_grnd_r"], fs["eflx_soil_grnd"])
        assert np.array_equal(fs["eflx_lh_tot_r"], fs["eflx_lh_tot"])
    if "t_skin_range" in c:
        assert np.all((fs["t_skin"] > 200.0) & (fs["t_skin"] < 400.0))
    if "errsoi_col" in c:
        np.testing.assert_allclose(fs["errsoi_col"], fs["errsoi_patch"], rtol=1e-12)
    if "evap_partition" in c and fs["qflx_ev_snow"][0] >= 0.0:
        np.testing.assert_allclose(fs["qflx_liqevap_from_top_layer"] + fs["qflx_solidevap_from_top_layer"],
                                   fs["qflx_ev_snow"], rtol=1e-12)
    if "frost" in c:
        assert fs["qflx_soliddew_to_top_layer"][0] > 0.0
        assert fs["qflx_liqdew_to_top_layer"][0] == 0.0
        assert fs["qflx_liqevap_from_top_layer"][0] == 0.0
        assert fs["qflx_solidevap_from_top_layer"][0] == 0.0
    if "ev_snow_nonnegative" in c:
        assert fs["qflx_ev_snow"][0] >= 0.0
