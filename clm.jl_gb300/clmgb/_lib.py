"""Loads the CUDA C-ABI library (clm.jl_gb300/lib/libclmgb.so) with ctypes.

There is no fallback: if the library cannot be loaded the caller gets an error.
"""
import ctypes as C
import os

from . import abi, build

_LIB = None

P = C.c_void_p
I32, I64, F64 = C.c_int32, C.c_int64, C.c_double

_SIGS = {
    "clmgb_abi_version": ([], I32),
    "clmgb_build_info": ([], C.c_char_p),
    "clmgb_strerror": ([I32], C.c_char_p),
    "clmgb_create": ([P, P], I32),
    "clmgb_destroy": ([P], I32),
    "clmgb_device_status": ([P, P, P, I32], I32),
    "clmgb_last_cuda_error": ([P], I32),
    "clmgb_soil_temperature": ([P, P, P, F64, I32, I32, P, P], I32),
    "clmgb_soil_water_fractions": ([P, P, P, P], I32),
    "clmgb_soil_water": ([P, P, P, P, F64, P, P], I32),
    "clmgb_column_step": ([P, P, P, P, P, F64, I32, P, P, P, P], I32),
    "clmgb_phase_change_h2osfc": ([P, P, P, F64, P, P], I32),
    "clmgb_phase_change_beta": ([P, P, P, F64, P, P], I32),
    "clmgb_synth_forcing": ([P, P, P, P, P, P, P], I32),
    "clmgb_batched_band_solve": ([P, I64, I64, I32, P, P, P, P, P, P, I32, I32, I32, P], I32),
    "clmgb_tridiagonal_multi": ([P, I64, I64, I32, P, P, P, P, P, P, P, P], I32),
    "clmgb_batched_band_solve_factor": ([P, I64, I64, I32, P, P, P, P, P, P, I32, I32, I32, P, P, P], I32),
    "clmgb_batched_band_solve_adjoint": ([P, I64, I64, I32, P, P, P, P, P, P, P, P, P, I32, I32, I32, P], I32),
    "clmgb_tridiagonal_adjoint": ([P, I64, I64, I32] + [P] * 12, I32),
    "clmgb_reserve_adjoint": ([P, I64, I64], I32),
    "clmgb_soil_water_warm": ([P, P, P, P, F64, P, P, P], I32),
    "clmgb_balance_begin": ([P, P, P, P, P, P], I32),
    "clmgb_balance_residuals": ([P, P, P, P, F64, P, P, P, P, P, P, P], I32),
    "clmgb_mlp_samples": ([P, P, P, P, F64, I32, P, P, P, I64, P, P], I32),
    "clmgb_mlp_linear": ([P, I64, I32, I32, P, I64, P, P, I32, P, I64, P, I64, P], I32),
    "clmgb_mlp_linear_dw": ([P, I64, I32, I32, P, I64, P, I64, P, P, P], I32),
    "clmgb_mlp_silu_backward": ([P, I64, P, P, P, P], I32),
    "clmgb_mlp_loss": ([P, I64, P, P, C.c_float, C.c_float, P, P, P], I32),
    "clmgb_mlp_adam": ([P, I64, I64, P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, I32, P, P, P], I32),
    "clmgb_mlp_features": ([P, P, P, P, F64, P, P, P, P], I32),
    "clmgb_mlp_first_dt": ([P, I64, P, F64, C.c_float, I32, P, P], I32),
    "clmgb_column_step_vjp": ([P, P, P, P, P, F64, I32, P, P, P, P, P], I32),
    "clmgb_column_step_logged": ([P, P, P, P, P, F64, I32, P, P, P, P, P], I32),
    "clmgb_effec_rootfrac_vert_tran_sink": ([P, P, P, I32, P, P], I32),
    "clmgb_soil_water_zd09": ([P, P, P, P, F64, P], I32),
    "clmgb_soil_water_flexible_cn": ([P, P, P, P], I32),
    "clmgb_soil_fluxes": ([P, P, P, F64, P], I32),
    "clmgb_surface_hydrology": ([P, P, P, P, C.c_uint32, F64, P], I32),
    "clmgb_snow_layers": ([P, P, P, P, C.c_uint32, F64, P], I32),
    "clmgb_lake_temperature": ([P, P, P, P, F64, P], I32),
    "clmgb_balance_check_columns": ([P, P, P, F64, P, P], I32),
    "clmgb_column_step_vjp_logged": ([P, P, P, P, P, F64, I32, P, P, P, P, P, P], I32),
    "clmgb_set_option": ([P, I32, I64], I32),
    "clmgb_reserve": ([P, I64], I32),
    "clmgb_get_option": ([P, I32, P], I32),
    "clmgb_math_eval": ([P, I32, I64, P, P, P, P], I32),
    "clmgb_soil_water_noalloc": ([P, P, P, P, F64, P, P], I32),
}


def exported_names():
    return list(_SIGS)


def lib_path():
    return build.LIB


def load(build_if_missing=True):
    """Load (building first if absent) and return the ctypes library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libclmgb.so is not built (%s); run __graft_entry__.build()" % path)
        build.build()
    L = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    if L.clmgb_abi_version() != 1:
        raise RuntimeError("libclmgb ABI version mismatch")
    _LIB = L
    return L


class CLMGBError(RuntimeError):
    def __init__(self, code, what=""):
        msg = load().clmgb_strerror(code).decode()
        super().__init__("%s failed: %s (%d)" % (what, msg, code))
        self.code = code


def check(code, what=""):
    if code != abi.CLMGB_OK:
        raise CLMGBError(code, what)
    return code
