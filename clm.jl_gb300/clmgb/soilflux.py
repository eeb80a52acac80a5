"""Inputs and outputs of soil_fluxes! (soil_fluxes.jl:553-697) in CLM.jl's layouts,
host (numpy) or device (torch), and the drop-in call clmgb_soil_fluxes."""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet

ISTSOIL, ISTCROP, ISTURB_MD = 1, 2, 9
ICOL_ROOF, ICOL_SUNWALL, ICOL_ROAD_IMPERV, ICOL_ROAD_PERV = 71, 72, 74, 75
HVAP = 2.501e6


class SoilFluxState(FieldSet):
    """Arrays of clmgb_soilflux_fields for nc columns, npch patches, nl landunits."""
    SPEC = abi.SOILFLUX_FIELDS
    STRUCT = abi.SoilFluxFields


def soil_fluxes(handle, fs, dtime, stream=None):
    """clmgb_soil_fluxes on a device SoilFluxState (in place)."""
    api.check(handle.lib.clmgb_soil_fluxes(handle.h, C.byref(fs.bounds()), C.byref(fs.fields()), float(dtime),
                                           api._stream(stream)), "soil_fluxes")


def random_state(vp, nc, seed=0, max_patches=3):
    """Seeded host inputs after a soil_temperature! step: 1..max_patches patches per
    column; natural vegetation, crop and urban (roof, sunwall, roads) columns; snow
    layers on a share of columns; evaporation and dew; surface water on some."""
    rng = np.random.default_rng(seed)
    npc = rng.integers(1, max_patches + 1, nc)
    npch = int(npc.sum())
    nl = 3
    fs = SoilFluxState(vp, nc, npch, nl)
    fs["lun_itype"][:] = [ISTSOIL, ISTCROP, ISTURB_MD]
    fs["lun_urbpoi"][:] = [0, 0, 1]
    kind = rng.integers(0, 3, nc)
    urb_types = np.array([ICOL_ROOF, ICOL_SUNWALL, ICOL_ROAD_IMPERV, ICOL_ROAD_PERV])
    fs["col_itype"][:] = np.where(kind == 0, ISTSOIL,
                                  np.where(kind == 1, ISTCROP, urb_types[rng.integers(0, 4, nc)]))
    fs["col_patchi"][:] = np.concatenate([[1], 1 + np.cumsum(npc)[:-1]])
    fs["col_patchf"][:] = fs["col_patchi"] + npc - 1
    pc = np.repeat(np.arange(nc), npc)
    fs["patch_column"][:] = pc + 1
    fs["patch_landunit"][:] = kind[pc] + 1
    w = rng.random(npch)
    fs["patch_wtcol"][:] = w / np.bincount(pc, weights=w, minlength=nc)[pc]
    fs["mask_nolakec"][:] = (rng.random(nc) < 0.95).astype(np.uint8)
    fs["mask_nolakep"][:] = (rng.random(npch) < 0.95).astype(np.uint8)
    fs["mask_urbanp"][:] = ((kind[pc] == 2) & (rng.random(npch) < 0.9)).astype(np.uint8)
    fs["frac_veg_nosno"][:] = rng.integers(0, 2, npch)
    # snow: 40 % of the natural/crop columns, 1..nlevsno layers
    ns = vp.nlevsno
    snl = -rng.integers(1, ns + 1, nc)
    snl[(rng.random(nc) < 0.6) | (kind == 2)] = 0
    fs["col_snl"][:] = snl
    fs["frac_sno_eff"][:] = np.where(snl < 0, rng.uniform(0.3, 1.0, nc), 0.0)
    fs["frac_h2osfc"][:] = np.where(rng.random(nc) < 0.3, rng.uniform(0.0, 0.4, nc), 0.0)
    L = ns + vp.nlevmaxurbgrnd
    fs["t_ssbef"][:] = rng.uniform(255.0, 290.0, (L, nc))
    fs["t_soisno"][:] = fs["t_ssbef"] + rng.normal(0.0, 0.5, (L, nc))
    fs["fact"][:] = rng.uniform(1e-4, 5e-2, (L, nc))
    fs["h2osoi_liq"][:] = rng.uniform(0.0, 30.0, (L, nc)) * (rng.random((L, nc)) < 0.8)
    fs["h2osoi_ice"][:] = rng.uniform(0.0, 10.0, (L, nc)) * (rng.random((L, nc)) < 0.5)
    fs["t_h2osfc_bef"][:] = rng.uniform(270.0, 285.0, nc)
    fs["t_h2osfc"][:] = fs["t_h2osfc_bef"] + rng.normal(0.0, 0.3, nc)
    fs["t_grnd"][:] = rng.uniform(255.0, 290.0, nc)
    fs["emg"][:] = rng.uniform(0.9, 0.99, nc)
    fs["htvp"][:] = np.where(rng.random(nc) < 0.5, HVAP, 2.8345e6)
    fs["xmf"][:] = rng.normal(0.0, 5.0, nc)
    fs["xmf_h2osfc"][:] = rng.normal(0.0, 1.0, nc)
    fs["c_h2osfc"][:] = rng.uniform(1e4, 1e5, nc)
    fs["eflx_h2osfc_to_snow"][:] = rng.normal(0.0, 1.0, nc)
    fs["eflx_building_heat_errsoi"][:] = rng.normal(0.0, 2.0, nc)
    fs["forc_lwrad"][:] = rng.uniform(200.0, 400.0, nc)
    for k in ("cgrnds", "cgrndl"):
        fs[k][:] = rng.uniform(0.0, 20.0 if k == "cgrnds" else 2e-3, npch)
    for k, lo, hi in (("sabg", 0, 500), ("sabg_soil", 0, 500), ("sabg_snow", 0, 300), ("dlrad", 0, 100),
                      ("ulrad", 100, 400), ("eflx_sh_veg", -50, 100), ("eflx_sh_stem", -5, 5),
                      ("eflx_wasteheat", 0, 20), ("eflx_heat_from_ac", 0, 10), ("eflx_traffic", 0, 20),
                      ("eflx_ventilation", -5, 5), ("eflx_sh_grnd", -50, 150), ("eflx_lwrad_net", -50, 100),
                      ("eflx_lwrad_out", 250, 450), ("eflx_lwrad_net_u", -50, 100)):
        fs[k][:] = rng.uniform(lo, hi, npch)
    fs["qflx_evap_veg"][:] = rng.uniform(0.0, 5e-5, npch)
    fs["qflx_tran_veg"][:] = fs["qflx_evap_veg"] * rng.uniform(0.0, 1.0, npch)
    ev = rng.normal(2e-5, 4e-5, npch)           # evaporation and dew
    big = rng.random(npch) < 0.05               # demands above the available water
    ev[big] = rng.uniform(1e-2, 1e-1, big.sum())
    fs["qflx_evap_soi"][:] = ev
    for k in ("qflx_ev_soil", "qflx_ev_h2osfc", "qflx_ev_snow"):
        fs[k][:] = ev * rng.uniform(0.5, 1.5, npch)
    for k in ("errsoi_col", "errsoi_patch", "t_skin"):
        fs[k][:] = 9.0
    return fs
