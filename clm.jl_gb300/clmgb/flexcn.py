"""The use_flexibleCN step of soil_water! (soil_water_movement.jl:1812-1843) in CLM.jl's
layouts, host (numpy) or device (torch), and its drop-in call
clmgb_soil_water_flexible_cn."""
import ctypes as C

from . import abi, api
from .fieldset import FieldSet


class FlexCnState(FieldSet):
    """Arrays of clmgb_flexcn_fields for nc columns."""
    SPEC = abi.FLEXCN_FIELDS
    STRUCT = abi.FlexCnFields

    @classmethod
    def from_column_state(cls, st, wa=5000.0):
        """From a host ColumnState after a soil_water! call: its mask, geometry and water,
        and an aquifer store wa (mm)."""
        fs = cls(st.vp, st.nc, st.nc, 1)
        for (n, _, _, _) in abi.FLEXCN_FIELDS:
            if n in st.arrays:
                fs[n] = st[n].copy()
        fs["wa"][:] = wa
        return fs


def soil_water_flexible_cn(handle, fs, stream=None):
    """clmgb_soil_water_flexible_cn on a device FlexCnState (in place)."""
    api.check(handle.lib.clmgb_soil_water_flexible_cn(handle.h, C.byref(fs.bounds()), C.byref(fs.fields()),
                                                      api._stream(stream)), "soil_water_flexible_cn")
