"""Inputs and outputs of the surface hydrology clm_drv_core! runs before the root sink
and soil_water! (clm_driver.jl:1938-2007) in CLM.jl's layouts, host (numpy) or device
(torch), and the drop-in call clmgb_surface_hydrology.

The reference's routines map onto stage bits (abi.SH_*): set_floodc!,
saturated_excess_runoff!, set_qflx_inputs!, infiltration_excess_runoff!,
route_infiltration_excess!, update_h2osfc!, infiltration!, total_surface_runoff!,
update_urban_ponding!.  One call with several bits is those calls in that order.
"""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet

ISTSOIL, ISTCROP, ISTURB_MD = 1, 2, 9
ICOL_ROOF, ICOL_SUNWALL, ICOL_SHADEWALL, ICOL_ROAD_IMPERV, ICOL_ROAD_PERV = 71, 72, 73, 74, 75
ISPVAL = -9999

STAGES = {"set_floodc!": abi.SH_FLOODC, "saturated_excess_runoff!": abi.SH_SAT_EXCESS,
          "set_qflx_inputs!": abi.SH_QFLX_INPUTS, "infiltration_excess_runoff!": abi.SH_INFL_EXCESS,
          "route_infiltration_excess!": abi.SH_ROUTE, "update_h2osfc!": abi.SH_UPDATE_H2OSFC,
          "infiltration!": abi.SH_INFILTRATION, "total_surface_runoff!": abi.SH_TOTAL_RUNOFF,
          "update_urban_ponding!": abi.SH_URBAN_PONDING}


class SurfHydState(FieldSet):
    """Arrays of clmgb_surfhyd_fields for nc columns, nl landunits, ng gridcells."""
    SPEC = abi.SURFHYD_FIELDS
    STRUCT = abi.SurfHydFields

    def __init__(self, vp, nc, npch=None, nl=1, arrays=None, ng=1):
        super().__init__(vp, nc, npch, nl, arrays, ng=ng)


def config(ng=1, fff=0.5, **kw):
    cfg = abi.SurfHydConfig.default(ng=ng, fff=fff)
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def stage_mask(names):
    m = 0
    for n in names:
        m |= STAGES[n]
    return m


def surface_hydrology(handle, sh, dtime, cfg=None, stages=abi.SH_ALL, stream=None):
    """clmgb_surface_hydrology on a device SurfHydState (in place)."""
    cfg = cfg if cfg is not None else config(ng=sh.ng)
    api.check(handle.lib.clmgb_surface_hydrology(handle.h, C.byref(sh.bounds()), C.byref(sh.fields()),
                                                 C.byref(cfg), int(stages), float(dtime), api._stream(stream)),
              "surface_hydrology")


def random_state(vp, nc, seed=0, ng=None):
    """Seeded host inputs: natural, crop and urban (roof, walls, roads) columns on 3
    landunits and ng gridcells; water tables above and below the frost table, frozen
    top soil on some columns, snow on some, surface water around its spill threshold,
    evaporation and dew, and flood water."""
    rng = np.random.default_rng(seed)
    ng = ng or max(1, nc // 16)
    sh = SurfHydState(vp, nc, nc, 3, ng=ng)
    sh["lun_itype"][:] = [ISTSOIL, ISTCROP, ISTURB_MD]
    kind = rng.integers(0, 3, nc)
    urb = np.array([ICOL_ROOF, ICOL_SUNWALL, ICOL_SHADEWALL, ICOL_ROAD_IMPERV, ICOL_ROAD_PERV])
    it = np.where(kind == 0, ISTSOIL, np.where(kind == 1, ISTCROP, urb[rng.integers(0, 5, nc)]))
    sh["col_itype"][:] = it
    sh["col_landunit"][:] = kind + 1
    sh["col_gridcell"][:] = rng.integers(1, ng + 1, nc)
    sh["col_urbpoi"][:] = (kind == 2).astype(np.uint8)
    sh["col_is_hillslope"][:] = (rng.random(nc) < 0.3).astype(np.uint8)
    sh["col_active"][:] = (rng.random(nc) < 0.9).astype(np.uint8)
    sh["col_cold"][:] = np.where(rng.random(nc) < 0.5, ISPVAL, rng.integers(1, nc + 1, nc))
    hydro = (kind < 2) | (it == ICOL_ROAD_PERV)
    sh["mask_nolakec"][:] = (rng.random(nc) < 0.97).astype(np.uint8)
    sh["mask_hydrology"][:] = (hydro & (rng.random(nc) < 0.95)).astype(np.uint8)
    sh["mask_urban"][:] = (kind == 2).astype(np.uint8)
    sh["col_snl"][:] = np.where(rng.random(nc) < 0.3, -rng.integers(1, vp.nlevsno + 1, nc), 0)
    sh["qflx_floodg"][:] = np.where(rng.random(ng) < 0.2, rng.uniform(0.0, 1e-3, ng), 0.0)
    sh["zwt"][:] = rng.uniform(0.0, 8.0, nc)
    sh["zwt_perched"][:] = sh["zwt"] * rng.uniform(0.0, 1.0, nc)
    sh["frost_table"][:] = rng.uniform(0.0, 8.0, nc)
    sh["wtfact"][:] = rng.uniform(0.0, 0.6, nc)
    sh["b_infil"][:] = rng.uniform(0.01, 0.5, nc)
    sh["top_max_moist"][:] = rng.uniform(50.0, 400.0, nc)
    sh["top_moist_limited"][:] = sh["top_max_moist"] * rng.uniform(0.0, 1.0, nc)
    G = vp.nlevgrnd
    frozen = rng.random(nc) < 0.3
    sh["icefrac"][:] = np.where(frozen[None, :], rng.uniform(0.0, 1.0, (G, nc)), 0.0)
    sh["hksat"][:] = rng.uniform(1e-4, 5e-2, (G, nc))
    sh["frac_sno_eff"][:] = np.where(sh["col_snl"] < 0, rng.uniform(0.2, 1.0, nc), 0.0)
    fh = np.where(rng.random(nc) < 0.5, rng.uniform(0.0, 0.8, nc), 0.0)
    sh["frac_h2osfc"][:] = fh
    sh["frac_h2osfc_nosnow"][:] = np.minimum(1.0, fh * rng.uniform(1.0, 1.5, nc))
    sh["h2osfc_thresh"][:] = rng.uniform(0.0, 40.0, nc)
    sh["h2osfc"][:] = np.where(fh > 0, sh["h2osfc_thresh"] * rng.uniform(0.0, 2.0, nc), 0.0)
    sh["h2osfc"][rng.random(nc) < 0.02] = -1e-9                    # numerical undershoot
    sh["topo_slope"][:] = rng.uniform(0.0, 60.0, nc)
    sh["qflx_rain_plus_snomelt"][:] = np.where(rng.random(nc) < 0.6, rng.exponential(5e-3, nc), 0.0)
    sh["qflx_snow_h2osfc"][:] = np.where(rng.random(nc) < 0.1, rng.uniform(0.0, 1e-4, nc), 0.0)
    ev = rng.normal(2e-5, 4e-5, nc)
    sh["qflx_liqevap_from_top_layer"][:] = np.maximum(ev, 0.0)
    sh["qflx_ev_soil"][:] = ev * rng.uniform(0.5, 1.5, nc)
    sh["qflx_ev_h2osfc"][:] = ev * rng.uniform(0.5, 1.5, nc)
    sh["h2osoi_liq"][vp.nlevsno] = rng.uniform(0.0, 1.5, nc)       # urban pond in the top soil level
    sh["xs_urban"][:] = rng.uniform(0.0, 1e-3, nc)
    for k in ("qflx_floodc", "fsat", "fcov", "qflx_sat_excess_surf", "qflx_top_soil", "qflx_in_soil",
              "qflx_top_soil_to_h2osfc", "qinmax", "qflx_infl_excess", "qflx_in_soil_limited", "qflx_in_h2osfc",
              "qflx_infl_excess_surf", "qflx_h2osfc_surf", "qflx_h2osfc_drain", "qflx_infl", "qflx_surf"):
        sh[k][:] = rng.uniform(-1e-3, 1e-3, nc)                     # what an earlier step left
    return sh
