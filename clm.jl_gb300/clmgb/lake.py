"""Inputs and outputs of lake_temperature! (lake_temperature.jl:1016-1295) in CLM.jl's
layouts, host (numpy) or device (torch), and the drop-in call clmgb_lake_temperature."""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet

TFRZ = 273.15
DZLAK = [0.1, 1.0, 2.0, 3.0, 4.0, 5.0, 7.0, 7.0, 10.45, 10.45]     # varcon.jl:291, nlevlak = 10


class LakeState(FieldSet):
    """Arrays of clmgb_lake_fields for nc lake columns with one patch each."""
    SPEC = abi.LAKE_FIELDS
    STRUCT = abi.LakeFields

    def bounds(self):
        return abi.Bounds(self.nc, self.np, 1, self.nc, self.np)


def config(**kw):
    cfg = abi.LakeConfig.default()
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def lake_temperature(handle, lk, dtime, cfg=None, stream=None):
    """clmgb_lake_temperature on a device LakeState (in place)."""
    cfg = cfg if cfg is not None else config()
    api.check(handle.lib.clmgb_lake_temperature(handle.h, C.byref(lk.bounds()), C.byref(lk.fields()), C.byref(cfg),
                                                float(dtime), api._stream(stream)), "lake_temperature")


def soil_grid(nlevsoi, nlevgrnd):
    """varcon_init!'s soil levels (varcon.jl:246-280): thicknesses, nodes, interfaces."""
    dz = np.zeros(nlevgrnd)
    for j in range(1, min(4, nlevsoi) + 1):
        dz[j - 1] = j * 0.02
    for j in range(5, min(13, nlevsoi) + 1):
        dz[j - 1] = dz[3] + (j - 4) * 0.04
    for j in range(14, nlevsoi + 1):
        dz[j - 1] = dz[min(13, nlevsoi) - 1] + (j - 13) * 0.10
    for j in range(nlevsoi + 1, nlevgrnd + 1):
        dz[j - 1] = dz[nlevsoi - 1] + ((j - nlevsoi) * 25.0) ** 1.5 / 100.0
    zi = np.concatenate([[0.0], np.cumsum(dz)])
    return dz, 0.5 * (zi[:-1] + zi[1:]), zi


def lake_grid():
    dzl = np.array(DZLAK)
    zl = np.zeros(len(dzl))
    zl[0] = 0.5 * dzl[0]
    for j in range(1, len(dzl)):
        zl[j] = zl[j - 1] + 0.5 * (dzl[j - 1] + dzl[j])
    return dzl, zl


def _common(vp, nc):
    lk = LakeState(vp, nc, nc, 1)
    lk["mask_lakec"][:] = 1
    lk["mask_lakep"][:] = 1
    lk["col_patchi"][:] = np.arange(1, nc + 1)
    lk["patch_column"][:] = np.arange(1, nc + 1)
    ns, ng = vp.nlevsno, vp.nlevgrnd
    dz, z, zi = soil_grid(vp.nlevsoi, ng)
    lk["dz"][ns:ns + ng] = dz[:, None]
    lk["z"][ns:ns + ng] = z[:, None]
    lk["zi"][ns:ns + ng + 1] = zi[:, None]
    dzl, zl = lake_grid()
    lk["dz_lake"][:] = dzl[:, None]
    lk["z_lake"][:] = zl[:, None]
    return lk


def reference_test_state(vp, nc, zero_flux=False):
    """create_test_data of test/test_lake_temperature.jl:24-170 (and its zero-flux
    variant, :314-337)."""
    lk = _common(vp, nc)
    ns, ng = vp.nlevsno, vp.nlevgrnd
    lk["lakedepth"][:] = 30.0
    lk["t_grnd"][:] = 280.0
    lk["t_lake"][:] = 280.0
    lk["t_soisno"][:] = 280.0
    lk["sabg"][:] = 0.0 if zero_flux else 100.0
    for k, v in (("fsds_nir_d", 30.0), ("fsds_nir_i", 20.0), ("fsr_nir_d", 5.0), ("fsr_nir_i", 3.0)):
        lk[k][:] = 0.0 if zero_flux else v
    lk["sabg_lyr"][:] = 0.0 if zero_flux else 100.0 / (ns + 1)
    for k, v in (("watsat", 0.45), ("tksatu", 1.5), ("tkmg", 3.0), ("tkdry", 0.25), ("csol", 2.0e6)):
        lk[k][:ng] = v
    lk["h2osoi_liq"][ns:ns + ng] = lk["dz"][ns:ns + ng] * 1000.0 * 0.45
    lk["eflx_gnet"][:] = 0.0 if zero_flux else 50.0
    lk["eflx_sh_tot"][:] = 20.0
    lk["eflx_sh_grnd"][:] = 20.0
    lk["eflx_soil_grnd"][:] = 50.0
    lk["etal"][:] = 0.5
    lk["ks"][:] = 0.1
    lk["ws"][:] = 0.05
    lk["lake_raw"][:] = 100.0
    lk["betaprime"][:] = 0.4
    lk["savedtke1"][:] = 0.57
    return lk


def random_state(vp, nc, seed=0):
    """Seeded lake columns: warm and frozen lakes (partly frozen levels, ice on top),
    snow layers on a share of frozen lakes, unresolved snow, shallow and deep lakes,
    light and zero solar, a few inactive patches."""
    rng = np.random.default_rng(seed)
    lk = _common(vp, nc)
    ns, ng, nsoi = vp.nlevsno, vp.nlevgrnd, vp.nlevsoi
    lk["mask_lakep"][:] = (rng.random(nc) < 0.97).astype(np.uint8)
    lk["mask_lakec"][:] = (rng.random(nc) < 0.98).astype(np.uint8)
    depth = np.where(rng.random(nc) < 0.5, rng.uniform(2.0, 24.0, nc), rng.uniform(25.0, 80.0, nc))
    lk["lakedepth"][:] = depth
    frozen = rng.random(nc) < 0.4
    nlak = abi.NLEVLAK
    t_l = np.where(frozen[None, :], TFRZ + rng.uniform(-6.0, 1.0, (nlak, nc)), TFRZ + rng.uniform(0.5, 20.0, (nlak, nc)))
    t_l = np.sort(t_l, axis=0)[::-1] if rng.random() < 0.5 else t_l      # some stable, some unstable
    lk["t_lake"][:] = t_l
    ice = np.zeros((nlak, nc))
    top_ice = frozen & (rng.random(nc) < 0.8)
    ice[0] = np.where(top_ice, rng.uniform(0.2, 1.0, nc), 0.0)
    ice[1] = np.where(top_ice & (rng.random(nc) < 0.3), rng.uniform(0.0, 0.5, nc), 0.0)
    lk["lake_icefrac"][:] = ice
    snl = np.where(frozen & (rng.random(nc) < 0.5), -rng.integers(1, min(ns, 5) + 1, nc), 0)
    lk["col_snl"][:] = snl
    lk["t_grnd"][:] = np.where(frozen, TFRZ - rng.uniform(0.0, 10.0, nc), t_l[0] + rng.normal(0.0, 0.5, nc))
    for k in range(ns):
        j = k + 1 - ns                                   # snow level index
        act = j >= snl + 1
        dzs = rng.uniform(0.02, 0.08, nc)
        lk["dz"][k] = np.where(act, dzs, 0.0)
        lk["h2osoi_ice"][k] = np.where(act, dzs * rng.uniform(100.0, 350.0, nc), 0.0)
        lk["h2osoi_liq"][k] = np.where(act & (rng.random(nc) < 0.3), rng.uniform(0.0, 2.0, nc), 0.0)
        lk["t_soisno"][k] = np.where(act, TFRZ - rng.uniform(0.0, 12.0, nc), 0.0)
    zi = np.zeros((ns + 1, nc))
    for k in range(ns - 1, -1, -1):
        zi[k] = zi[k + 1] - lk["dz"][k]
    lk["zi"][:ns] = zi[:ns]
    lk["z"][:ns] = zi[:ns] + 0.5 * lk["dz"][:ns]
    lk["h2osno_no_layers"][:] = np.where((snl == 0) & (rng.random(nc) < 0.3), rng.uniform(0.0, 8.0, nc), 0.0)
    lk["snow_depth"][:] = np.where(snl < 0, lk["dz"][:ns].sum(0), lk["h2osno_no_layers"] / 250.0)
    ws_ = rng.uniform(0.40, 0.55, (ng, nc))
    lk["watsat"][:] = ws_
    lk["tksatu"][:] = rng.uniform(1.2, 2.5, (ng, nc))
    lk["tkmg"][:] = rng.uniform(2.0, 3.5, (ng, nc))
    lk["tkdry"][:] = rng.uniform(0.2, 0.3, (ng, nc))
    lk["csol"][:] = rng.uniform(1.8e6, 2.4e6, (ng, nc))
    ts = TFRZ + rng.uniform(-3.0, 10.0, (ng, nc))
    lk["t_soisno"][ns:ns + ng] = ts
    w = lk["dz"][ns:ns + ng] * 1000.0 * ws_
    fr = np.where(ts < TFRZ, rng.uniform(0.3, 1.0, (ng, nc)), 0.0)
    lk["h2osoi_ice"][ns:ns + ng] = w * fr * 0.917
    lk["h2osoi_liq"][ns:ns + ng] = w * (1 - fr)
    lk["sabg"][:] = np.where(rng.random(nc) < 0.3, 0.0, rng.uniform(0.0, 400.0, nc))
    nir = rng.uniform(0.3, 0.6, nc) * lk["sabg"]
    lk["fsds_nir_d"][:] = nir * 0.6
    lk["fsds_nir_i"][:] = nir * 0.5
    lk["fsr_nir_d"][:] = nir * 0.06
    lk["fsr_nir_i"][:] = nir * 0.04
    lk["sabg_lyr"][:] = lk["sabg"][None, :] * rng.dirichlet(np.ones(ns + 1), nc).T
    lk["eflx_gnet"][:] = rng.normal(20.0, 60.0, nc)
    lk["eflx_sh_tot"][:] = rng.normal(10.0, 30.0, nc)
    lk["eflx_sh_grnd"][:] = rng.normal(10.0, 30.0, nc)
    lk["eflx_soil_grnd"][:] = rng.normal(20.0, 60.0, nc)
    lk["etal"][:] = np.where(rng.random(nc) < 0.5, rng.uniform(0.1, 1.0, nc), -1.0)
    lk["ks"][:] = rng.uniform(0.02, 0.5, nc)
    lk["ws"][:] = rng.uniform(0.0, 0.1, nc)
    lk["lake_raw"][:] = rng.uniform(50.0, 200.0, nc)
    lk["betaprime"][:] = 0.4
    for k in ("errsoi_col", "savedtke1", "lake_icethick", "lake_icefracsurf", "qflx_snomelt", "qflx_snofrz",
              "qflx_snow_drain", "eflx_snomelt", "lakeresist", "grnd_ch4_cond"):
        lk[k][:] = 7.0
    return lk
