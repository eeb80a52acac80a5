"""Inputs and outputs of compute_effec_rootfrac_and_vert_tran_sink!
(soil_water_plant_sink.jl:341-451) in CLM.jl's layouts, host (numpy) or device
(torch), and the drop-in call clmgb_effec_rootfrac_vert_tran_sink.

Landunit and column type codes follow CLM (landunit_varcon.jl, column_varcon.jl).
"""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet

ISTSOIL, ISTCROP, ISTURB_MD = 1, 2, 9
ICOL_ROAD_PERV = 75


class RootSinkState(FieldSet):
    """Arrays of clmgb_rootsink_fields for nc columns, npch patches, nl landunits."""
    SPEC = abi.ROOTSINK_FIELDS
    STRUCT = abi.RootSinkFields

    def fields(self, with_hydrstress=True):
        return super().fields(skip=() if with_hydrstress else abi.HYDRSTRESS_ONLY)


def effec_rootfrac_vert_tran_sink(handle, rs, use_hydrstress=False, col_status=None, stream=None):
    """clmgb_effec_rootfrac_vert_tran_sink on a device RootSinkState (in place)."""
    f = rs.fields(with_hydrstress=use_hydrstress)
    b = rs.bounds()
    api.check(handle.lib.clmgb_effec_rootfrac_vert_tran_sink(handle.h, C.byref(b), C.byref(f),
                                                             1 if use_hydrstress else 0,
                                                             api._dptr(col_status, "col_status"),
                                                             api._stream(stream)),
              "effec_rootfrac_vert_tran_sink")


def random_state(vp, nc, seed=0, max_patches=4, hydrstress_inputs=True):
    """Seeded host inputs: 1..max_patches patches per column (some inactive, some with
    zero weight or transpiration), natural vegetation, crop and pervious-road columns,
    a hydrology mask with holes."""
    rng = np.random.default_rng(seed)
    npc = rng.integers(1, max_patches + 1, nc)
    npch = int(npc.sum())
    nl = 3
    rs = RootSinkState(vp, nc, npch, nl)
    rs["lun_itype"][:] = [ISTSOIL, ISTCROP, ISTURB_MD]
    kind = rng.integers(0, 3, nc)
    rs["col_landunit"][:] = kind + 1
    rs["col_itype"][:] = np.where(kind == 0, ISTSOIL, np.where(kind == 1, ISTCROP, ICOL_ROAD_PERV))
    rs["mask_hydrology"][:] = (rng.random(nc) < 0.9).astype(np.uint8)
    rs["col_patchi"][:] = np.concatenate([[1], 1 + np.cumsum(npc)[:-1]])
    rs["col_npatches"][:] = npc
    rs["patch_active"][:] = (rng.random(npch) < 0.85).astype(np.uint8)
    w = rng.random(npch)
    w[rng.random(npch) < 0.1] = 0.0
    rs["patch_wtcol"][:] = w
    nsoi = vp.nlevsoi
    z = np.cumsum(rng.uniform(0.02, 0.3, (nsoi, npch)), axis=0)
    r = np.exp(-rng.uniform(1.0, 6.0, npch) * z)
    rs["rootr_patch"][:nsoi] = r / r.sum(0)
    qt = rng.uniform(0.0, 1e-4, npch)
    qt[rng.random(npch) < 0.1] = 0.0
    rs["qflx_tran_veg_patch"][:] = qt
    pc = np.repeat(np.arange(nc), npc)
    rs["qflx_tran_veg_col"][:] = np.bincount(pc, weights=qt * w, minlength=nc)
    if hydrstress_inputs:
        rs["k_soil_root_patch"][:] = rng.uniform(1e-4, 2e-2, (nsoi, npch))
        rs["smp_l"][:nsoi] = -rng.uniform(50.0, 8000.0, (nsoi, nc))
        rs["vegwp_patch"][:] = -rng.uniform(100.0, 3000.0, (4, npch))
        rs["frac_veg_nosno"][:] = (rng.random(npch) < 0.8).astype(np.int64)
        zc = np.cumsum(rng.uniform(0.02, 0.3, (vp.nlevgrnd, nc)), axis=0)
        rs["z"][vp.nlevsno:vp.nlevsno + vp.nlevgrnd] = zc
    rs["rootr_col"][:] = 7.0          # untouched entries keep this
    rs["qflx_rootsoi_col"][:] = 7.0
    rs["qflx_phs_neg_col"][:] = 7.0
    rs["qflx_hydr_redist_patch"][:] = 7.0
    return rs
