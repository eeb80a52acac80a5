"""Inputs and outputs of soilwater_zengdecker2009! (soil_water_movement.jl:1616-1764)
in CLM.jl's layouts, host (numpy) or device (torch), and the drop-in call
clmgb_soil_water_zd09."""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet


def zd09_config(e_ice=6.0):
    """The configuration init_soilwater_movement builds by default: Zeng-Decker 2009 with
    the aquifer lower boundary (soil_water_movement.jl:657-668)."""
    cfg = abi.SwmConfig.clm5_default()
    cfg.soilwater_movement_method = abi.ZENGDECKER_2009
    cfg.lower_boundary_condition = abi.BC_AQUIFER
    cfg.e_ice = e_ice
    return cfg


class Zd09State(FieldSet):
    """Arrays of clmgb_zd09_fields for nc columns."""
    SPEC = abi.ZD09_FIELDS
    STRUCT = abi.Zd09Fields

    @classmethod
    def from_column_state(cls, st, zwt=None, smpmin=-1.0e8):
        """From a host ColumnState: the shared fields, h2osoi_vol from the layer water,
        smpmin (CLM's default -1e8 mm) and an optional water-table depth per column."""
        zs = cls(st.vp, st.nc, st.nc, 1)
        for (n, _, _, _) in abi.ZD09_FIELDS:
            if n in st.arrays:
                zs[n] = np.ascontiguousarray(st[n]).copy()
        vp = st.vp
        j0, j1 = vp.nlevsno, vp.nlevsno + vp.nlevgrnd
        dz = st["dz"][j0:j1]
        zs["h2osoi_vol"][:] = st["h2osoi_liq"][j0:j1] / (dz * 1000.0) + st["h2osoi_ice"][j0:j1] / (dz * 917.0)
        zs["smpmin"][:] = smpmin
        if zwt is not None:
            zs["zwt"][:] = zwt
        return zs


def soil_water_zd09(handle, zs, dtime, cfg=None, stream=None):
    """clmgb_soil_water_zd09 on a device Zd09State (in place)."""
    cfg = cfg or zd09_config()
    api.check(handle.lib.clmgb_soil_water_zd09(handle.h, C.byref(zs.bounds()), C.byref(zs.fields()),
                                               C.byref(cfg), float(dtime), api._stream(stream)),
              "soil_water_zd09")
