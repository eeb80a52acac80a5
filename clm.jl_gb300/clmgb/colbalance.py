"""Inputs and outputs of balance_check!'s column checks (balance_check.jl:707-770,
1099-1160, 1347-1365) in CLM.jl's layouts, the drop-in call
clmgb_balance_check_columns, and the reference's stop rule."""
import ctypes as C

import numpy as np

from . import abi, api
from .fieldset import FieldSet

ICOL_SUNWALL, ICOL_SHADEWALL = 72, 73
BALANCE_CHECK_SKIP_SIZE = 3600.0      # balance_check.jl:10


class ColBalanceState(FieldSet):
    """Arrays of clmgb_colbalance_fields for nc columns."""
    SPEC = abi.COLBALANCE_FIELDS
    STRUCT = abi.ColBalanceFields

    def fields(self, skip=()):
        return super().fields(skip=skip)


def balance_check_columns(handle, cb, dtime, with_errsoi=True, stream=None):
    """clmgb_balance_check_columns on a device ColBalanceState; returns the report."""
    rep = abi.BalanceReport()
    f = cb.fields(skip=() if with_errsoi else ("errsoi",))
    api.check(handle.lib.clmgb_balance_check_columns(handle.h, C.byref(cb.bounds()), C.byref(f), float(dtime),
                                                     C.byref(rep), api._stream(stream)), "balance_check_columns")
    return rep


def skip_steps(dtime):
    """balance_check_init! (balance_check.jl:54-57)."""
    return max(2, int(round(BALANCE_CHECK_SKIP_SIZE / dtime))) + 1       # Julia round: ties to even


def must_stop(rep, dastep, dtime, hard_error=True):
    """Whether balance_check! would stop on this report (_bc_should_error, :111-112):
    a non-finite or over-threshold column water error, or a soil energy error over
    1e-4 W/m2, once DAnstep is past the startup skip."""
    live = hard_error and dastep > skip_steps(dtime)
    bad = rep.flags & (abi.BAL_H2O_NONFINITE | abi.BAL_H2O_ERROR | abi.BAL_SOI_ERROR)
    return bool(live and bad)


def random_state(nc, seed=0):
    """Seeded columns: balanced and unbalanced water budgets, walls, inactive columns,
    a few non-finite storages, soil energy residuals around the thresholds."""
    rng = np.random.default_rng(seed)
    cb = ColBalanceState(None, nc)
    cb["col_itype"][:] = np.where(rng.random(nc) < 0.1, rng.choice([ICOL_SUNWALL, ICOL_SHADEWALL], nc), 1)
    cb["col_active"][:] = (rng.random(nc) < 0.95).astype(np.uint8)
    for k in ("forc_rain", "forc_snow", "qflx_flood", "qflx_sfc_irrig", "qflx_glcice_dyn_water_flux",
              "qflx_evap_tot", "qflx_surf", "qflx_qrgwl", "qflx_drain", "qflx_drain_perched", "qflx_ice_runoff",
              "qflx_snwcp_discarded_liq", "qflx_snwcp_discarded_ice"):
        cb[k][:] = np.where(rng.random(nc) < 0.5, rng.exponential(1e-4, nc), 0.0)
    cb["begwb"][:] = rng.uniform(100.0, 5000.0, nc)
    cb["endwb"][:] = cb["begwb"] + rng.normal(0.0, 1e-3, nc)
    cb["endwb"][rng.random(nc) < 0.01] = np.nan
    cb["errsoi"][:] = rng.normal(0.0, 1e-4, nc)
    cb["errh2o"][:] = 9.0
    return cb
