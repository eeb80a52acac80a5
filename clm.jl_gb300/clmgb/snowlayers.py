"""Inputs and outputs of the snow layer dynamics clm_drv_core! runs after the soil solve
(clm_driver.jl:2146-2200) in CLM.jl's layouts, host (numpy) or device (torch), and the
drop-in call clmgb_snow_layers.

The reference's routines map onto stage bits (abi.SL_*): snow_compaction!,
combine_snow_layers!, divide_snow_layers!, zero_empty_snow_layers!, build_snow_filter!.
One call with several bits is those calls in that order.
"""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet

ISTSOIL, ISTCROP, ISTDLAK, ISTURB_MD = 1, 2, 5, 9
TFRZ = 273.15

STAGES = {"snow_compaction!": abi.SL_COMPACTION, "combine_snow_layers!": abi.SL_COMBINE,
          "divide_snow_layers!": abi.SL_DIVIDE, "zero_empty_snow_layers!": abi.SL_ZERO_EMPTY,
          "build_snow_filter!": abi.SL_FILTER}
AEROSOLS = ("mss_bcphi", "mss_bcpho", "mss_ocphi", "mss_ocpho", "mss_dst1", "mss_dst2", "mss_dst3", "mss_dst4")


class SnowLayerState(FieldSet):
    """Arrays of clmgb_snowlayer_fields for nc columns, nl landunits, ng gridcells."""
    SPEC = abi.SNOWLAYER_FIELDS
    STRUCT = abi.SnowLayerFields

    def __init__(self, vp, nc, npch=None, nl=1, arrays=None, ng=1):
        super().__init__(vp, nc, npch, nl, arrays, ng=ng)


def config(ng=1, **kw):
    cfg = abi.SnowLayerConfig.default(ng=ng)
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def stage_mask(names):
    m = 0
    for n in names:
        m |= STAGES[n]
    return m


def snow_layers(handle, sl, dtime, cfg=None, stages=abi.SL_ALL, stream=None):
    """clmgb_snow_layers on a device SnowLayerState (in place)."""
    cfg = cfg if cfg is not None else config(ng=sl.ng)
    api.check(handle.lib.clmgb_snow_layers(handle.h, C.byref(sl.bounds()), C.byref(sl.fields()), C.byref(cfg),
                                           int(stages), float(dtime), api._stream(stream)), "snow_layers")


def snow_water(sl):
    """Total water of each column's snow levels, unresolved snow and soil level 1 (host)."""
    ns = sl.vp.nlevsno
    return (sl["h2osoi_liq"][:ns + 1].sum(0) + sl["h2osoi_ice"][:ns + 1].sum(0) + sl["h2osno_no_layers"])


def random_state(vp, nc, seed=0, ng=None):
    """Seeded host snowpacks after a soil solve: 1..nlevsno layers of mixed thickness
    (thin, very thin and over-thick layers, layers with almost no ice), melting and
    freezing levels, aerosol masses, on soil, crop, lake and urban landunits."""
    rng = np.random.default_rng(seed)
    ng = ng or max(1, nc // 16)
    ns = vp.nlevsno
    sl = SnowLayerState(vp, nc, nc, 4, ng=ng)
    sl["lun_itype"][:] = [ISTSOIL, ISTCROP, ISTDLAK, ISTURB_MD]
    sl["lun_lakpoi"][:] = [0, 0, 1, 0]
    sl["lun_urbpoi"][:] = [0, 0, 0, 1]
    sl["col_landunit"][:] = rng.choice([1, 2, 3, 4], nc, p=[0.55, 0.25, 0.1, 0.1])
    sl["col_gridcell"][:] = rng.integers(1, ng + 1, nc)
    sl["forc_wind"][:] = rng.uniform(0.0, 15.0, ng)
    sl["n_melt"][:] = rng.uniform(1.0, 20.0, nc)
    snl = -rng.integers(0, ns + 1, nc)
    sl["col_snl"][:] = snl
    sl["mask_nolakec"][:] = (sl["col_landunit"] != 3).astype(np.uint8)
    sl["mask_snow"][:] = ((snl < 0) & (sl["mask_nolakec"] != 0)).astype(np.uint8)
    sl["mask_nosnow"][:] = 1 - sl["mask_snow"]
    sl["frac_sno"][:] = np.where(snl < 0, rng.uniform(0.2, 1.0, nc), 0.0)
    sl["frac_sno_eff"][:] = sl["frac_sno"] * rng.uniform(0.8, 1.0, nc)
    sl["frac_h2osfc"][:] = np.where(rng.random(nc) < 0.3, rng.uniform(0.0, 0.5, nc), 0.0)
    sl["int_snow"][:] = rng.uniform(0.0, 800.0, nc)
    sl["h2osno_no_layers"][:] = np.where(snl < 0, 0.0, rng.uniform(0.0, 5.0, nc))
    sl["snow_depth"][:] = 9.0
    sl["qflx_sl_top_soil"][:] = 9.0
    L = ns + vp.nlevmaxurbgrnd
    # layer thickness: a mix of normal, thin and thick; mass from a density
    dz = rng.choice([0.004, 0.012, 0.03, 0.08, 0.3], (ns, nc), p=[0.1, 0.2, 0.3, 0.3, 0.1]) * \
        rng.uniform(0.7, 1.4, (ns, nc))
    rho = rng.uniform(30.0, 450.0, (ns, nc))
    w = rho * dz * sl["frac_sno"][None, :]
    liqf = np.where(rng.random((ns, nc)) < 0.4, rng.uniform(0.0, 0.2, (ns, nc)), 0.0)
    ice = w * (1 - liqf)
    ice[rng.random((ns, nc)) < 0.05] = rng.uniform(0.0, 0.01)      # almost no ice
    active = np.arange(ns)[:, None] >= (ns + snl)[None, :]
    sl["dz"][:ns] = np.where(active, dz, 0.0)
    sl["h2osoi_ice"][:ns] = np.where(active, ice, 0.0)
    sl["h2osoi_liq"][:ns] = np.where(active, w * liqf, 0.0)
    sl["t_soisno"][:ns] = np.where(active, TFRZ - rng.uniform(0.0, 20.0, (ns, nc)) * (liqf == 0), 0.0)
    sl["h2osoi_liq"][ns:] = rng.uniform(0.0, 40.0, (L - ns, nc))
    sl["h2osoi_ice"][ns:] = rng.uniform(0.0, 10.0, (L - ns, nc))
    sl["t_soisno"][ns:] = rng.uniform(260.0, 285.0, (L - ns, nc))
    sl["dz"][ns:] = np.linspace(0.02, 1.0, L - ns)[:, None]
    zi = np.zeros((L + 1, nc))
    zi[ns + 1:] = np.cumsum(sl["dz"][ns:], axis=0)
    for k in range(ns - 1, -1, -1):
        zi[k] = np.where(active[k], zi[k + 1] - sl["dz"][k], 0.0)
    sl["zi"][:] = zi
    sl["z"][:] = np.where(np.arange(L)[:, None] >= 0, zi[1:] - 0.5 * sl["dz"], 0.0)
    sl["imelt"][:ns] = np.where(active & (rng.random((ns, nc)) < 0.3), 1, np.where(active, 2, 0))
    sl["swe_old"][:] = (sl["h2osoi_ice"][:ns] + sl["h2osoi_liq"][:ns]) * rng.uniform(0.8, 1.3, (ns, nc))
    sl["frac_iceold"][:] = np.where(active, rng.uniform(0.5, 1.0, (ns, nc)), 0.0)
    sl["snw_rds"][:] = np.where(active, rng.uniform(40.0, 1600.0, (ns, nc)), 0.0)
    for a in AEROSOLS:
        sl[a][:] = np.where(active, rng.uniform(0.0, 1e-6, (ns, nc)), 0.0)
    return sl
