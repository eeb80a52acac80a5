"""Inputs and outputs of soilwater_zengdecker2009! (soil_water_movement.jl:1616-1764)
in CLM.jl's layouts, host (numpy) or device (torch), and the drop-in call
clmgb_soil_water_zd09."""
import ctypes as C

import numpy as np

from . import abi, api

_NP = {"u8": np.uint8, "i64": np.int64, "f64": np.float64}


def zd09_config(e_ice=6.0):
    """The configuration init_soilwater_movement builds by default: Zeng-Decker 2009 with
    the aquifer lower boundary (soil_water_movement.jl:657-668)."""
    cfg = abi.SwmConfig.clm5_default()
    cfg.soilwater_movement_method = abi.ZENGDECKER_2009
    cfg.lower_boundary_condition = abi.BC_AQUIFER
    cfg.e_ice = e_ice
    return cfg


class Zd09State:
    """Arrays of clmgb_zd09_fields for nc columns."""

    def __init__(self, vp, nc, arrays=None):
        self.vp, self.nc = vp, int(nc)
        if arrays is None:
            arrays = {}
            for (n, t, kind, dims) in abi.ZD09_FIELDS:
                shape = (self.nc,) if dims is None else (abi.level_count(dims, vp), self.nc)
                arrays[n] = np.zeros(shape, dtype=_NP[t])
        self.arrays = arrays

    def __getitem__(self, k):
        return self.arrays[k]

    def __setitem__(self, k, v):
        self.arrays[k] = v

    def bounds(self):
        return abi.Bounds(self.nc, self.nc, 1, self.nc, self.nc)

    def to_device(self, device="cuda"):
        import torch
        return Zd09State(self.vp, self.nc,
                         {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in self.arrays.items()})

    def to_host(self):
        return Zd09State(self.vp, self.nc,
                         {k: (v if isinstance(v, np.ndarray) else v.detach().cpu().numpy()).copy()
                          for k, v in self.arrays.items()})

    def copy(self):
        return Zd09State(self.vp, self.nc,
                         {k: (v.copy() if isinstance(v, np.ndarray) else v.clone()) for k, v in self.arrays.items()})

    def fields(self):
        s = abi.Zd09Fields()
        s.struct_size = C.sizeof(abi.Zd09Fields)
        for (n, t, _, _) in abi.ZD09_FIELDS:
            a = self.arrays[n]
            if isinstance(a, np.ndarray):
                assert a.flags.c_contiguous, n
                p = a.ctypes.data_as(abi._CT[t])
            else:
                assert a.is_contiguous(), n
                p = C.cast(C.c_void_p(a.data_ptr()), abi._CT[t])
            setattr(s, n, p)
        return s

    @classmethod
    def from_column_state(cls, st, zwt=None, smpmin=-1.0e8):
        """From a host ColumnState: the shared fields, h2osoi_vol from the layer water,
        smpmin (CLM's default -1e8 mm) and an optional water-table depth per column."""
        zs = cls(st.vp, st.nc)
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
