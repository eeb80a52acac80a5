"""Python mirror of CLM.jl's entry points for the soil/snow column solve, running the
hand-written sm_103a kernels through the C ABI (include/clmgb.h).

Names and argument meaning follow the reference:
  soil_temperature(...)             soil_temperature!        soil_temperature.jl:358
  set_soil_water_fractions(...)     set_soil_water_fractions! soil_hydrology.jl:394
  soil_water(...)                   soil_water!              soil_water_movement.jl:1780
  init_soilwater_movement(...)      init_soilwater_movement  soil_water_movement.jl:679
  phase_change_h2osfc / _beta       phase_change_*!          soil_temperature.jl:1857, 2232
  batched_band_solve(...)           batched_band_solve!      band_diagonal.jl:179
  tridiagonal_multi(...)            tridiagonal_multi!       tridiagonal.jl:129
  batched_band_solve_factor / _adjoint   band_solve! reverse rule   enzyme_rules.jl:80-107
  tridiagonal_adjoint(...)          tridiagonal_solve! reverse rule enzyme_rules.jl:160-201
Configurations the reference rejects with error() raise CLMGBError.  Every call
requires CUDA tensors; there is no CPU path.
"""
import ctypes as C

from . import abi
from ._lib import check, load, CLMGBError  # noqa: F401


def _stream(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def _dptr(t, what="tensor"):
    if t is None:
        return None
    if not getattr(t, "is_cuda", False):
        raise TypeError("%s must be a CUDA tensor (no CPU path)" % what)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % what)
    return C.c_void_p(t.data_ptr())


def init_soilwater_movement(use_bedrock=False, **kw):
    """init_soilwater_movement (soil_water_movement.jl:679-698): a SoilWaterMovementConfig
    with the reference's defaults (Zeng-Decker 2009, flux upper and aquifer lower
    boundaries, dtmin 60 s, verySmall 1e-8, tolerances 0.1 / 0.01, inexpensive fluxes,
    e_ice 6) and keyword overrides, validated as the reference does: Zeng-Decker 2009
    requires the aquifer lower boundary, and use_bedrock (varctl.use_bedrock) the
    zero-flux one.  Raises CLMGBError(CLMGB_ERR_CONFIG) where the reference raises."""
    vals = dict(soilwater_movement_method=abi.ZENGDECKER_2009, upper_boundary_condition=abi.BC_FLUX,
                lower_boundary_condition=abi.BC_AQUIFER, flux_calculation=1, dtmin=60.0, verySmall=1.0e-8,
                xTolerUpper=1.0e-1, xTolerLower=1.0e-2, e_ice=6.0)
    for k, v in kw.items():
        if k not in vals:
            raise TypeError("unknown SoilWaterMovementConfig field %r" % k)
        vals[k] = v
    cfg = abi.SwmConfig(**vals)
    if cfg.soilwater_movement_method == abi.ZENGDECKER_2009 and cfg.lower_boundary_condition != abi.BC_AQUIFER:
        raise CLMGBError(abi.CLMGB_ERR_CONFIG, "init_soilwater_movement: ZD09 must use bc_aquifer lower boundary "
                                               "condition")
    if use_bedrock and cfg.lower_boundary_condition != abi.BC_ZERO_FLUX:
        raise CLMGBError(abi.CLMGB_ERR_CONFIG, "init_soilwater_movement: use_bedrock requires bc_zero_flux lower "
                                               "boundary condition")
    return cfg


class Handle:
    """A library handle bound to the current CUDA device (owns the status word)."""

    def __init__(self, vp):
        self.lib = load()
        self.vp = vp
        h = C.c_void_p()
        check(self.lib.clmgb_create(C.byref(vp), C.byref(h)), "clmgb_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.clmgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, key, value):
        check(self.lib.clmgb_set_option(self.h, key, int(value)), "clmgb_set_option")

    def reserve(self, max_nc):
        """Per-column scratch for up to max_nc columns (impedance pre-pass, queue order)."""
        check(self.lib.clmgb_reserve(self.h, int(max_nc)), "clmgb_reserve")

    def reserve_adjoint(self, slots, entries):
        """Tape of column_step_vjp: `slots` columns in flight x `entries` records (32 B each)."""
        check(self.lib.clmgb_reserve_adjoint(self.h, int(slots), int(entries)), "clmgb_reserve_adjoint")

    def get_option(self, key):
        v = C.c_int64(0)
        check(self.lib.clmgb_get_option(self.h, key, C.byref(v)), "clmgb_get_option")
        return v.value

    def device_status(self, reset=True, stream=None):
        v = C.c_uint32(0)
        check(self.lib.clmgb_device_status(self.h, _stream(stream), C.byref(v), 1 if reset else 0),
              "clmgb_device_status")
        return v.value


def _require_device(state):
    if not state.on_device:
        raise TypeError("ColumnState must live on the GPU (state.to_device())")


def soil_temperature(handle, state, dtime, snow_method=abi.SNOW_JORDAN1991, use_excess_ice=False,
                     col_status=None, stream=None):
    _require_device(state)
    f = state.soiltemp_fields()
    b = state.bounds()
    check(handle.lib.clmgb_soil_temperature(handle.h, C.byref(b), C.byref(f), float(dtime), snow_method,
                                            1 if use_excess_ice else 0, _dptr(col_status, "col_status"),
                                            _stream(stream)), "soil_temperature")


def set_soil_water_fractions(handle, state, stream=None):
    _require_device(state)
    f = state.soilwater_fields()
    b = state.bounds()
    check(handle.lib.clmgb_soil_water_fractions(handle.h, C.byref(b), C.byref(f), _stream(stream)),
          "set_soil_water_fractions")


def soil_water(handle, state, dtime, cfg=None, col_status=None, stream=None):
    _require_device(state)
    cfg = cfg or abi.SwmConfig.clm5_default()
    f = state.soilwater_fields()
    b = state.bounds()
    check(handle.lib.clmgb_soil_water(handle.h, C.byref(b), C.byref(f), C.byref(cfg), float(dtime),
                                      _dptr(col_status, "col_status"), _stream(stream)), "soil_water")


def column_step(handle, state, dtime, cfg=None, snow_method=abi.SNOW_JORDAN1991, col_status=None,
                save_bef=True, stream=None):
    """soil_temperature! + set_soil_water_fractions! + soil_water! in one launch."""
    _require_device(state)
    cfg = cfg or abi.SwmConfig.clm5_default()
    ft, fw, b = state.soiltemp_fields(), state.soilwater_fields(), state.bounds()
    tss = _dptr(state["t_ssbef"]) if save_bef else None
    thb = _dptr(state["t_h2osfc_bef"]) if save_bef else None
    check(handle.lib.clmgb_column_step(handle.h, C.byref(b), C.byref(ft), C.byref(fw), C.byref(cfg),
                                       float(dtime), snow_method, tss, thb, _dptr(col_status, "col_status"),
                                       _stream(stream)), "column_step")


class SubstepLog:
    """Device buffers of a clmgb_substep_log for `nc` columns, `cap` records each; with
    `soil_temperature` (default) also the soil_temperature! records (st_rec), so the
    reverse runs neither the Richards substep loop nor soil_temperature! again."""

    def __init__(self, nc, cap=24, device="cuda", soil_temperature=True):
        import torch
        self.nc, self.cap = int(nc), int(cap)
        self.rec = torch.empty(self.nc * abi.log_stride(self.cap), dtype=torch.float64, device=device)
        self.count = torch.full((self.nc,), -1, dtype=torch.int32, device=device)
        self.st_rec = (torch.empty(self.nc * abi.LOG_ST_STRIDE, dtype=torch.float64, device=device)
                       if soil_temperature else None)

    def struct(self):
        s = abi.SubstepLog()
        s.struct_size = C.sizeof(abi.SubstepLog)
        s.rec = C.cast(C.c_void_p(self.rec.data_ptr()), abi.c_double_p)
        s.count = C.cast(C.c_void_p(self.count.data_ptr()), C.POINTER(C.c_int32))
        s.cap = self.cap
        if self.st_rec is not None:
            s.st_rec = C.cast(C.c_void_p(self.st_rec.data_ptr()), abi.c_double_p)
        return s


def column_step_logged(handle, state, dtime, log, cfg=None, snow_method=abi.SNOW_JORDAN1991, col_status=None,
                       save_bef=True, stream=None):
    """column_step that also writes the substep log `log` (a SubstepLog) for the reverse."""
    _require_device(state)
    cfg = cfg or abi.SwmConfig.clm5_default()
    ft, fw, b = state.soiltemp_fields(), state.soilwater_fields(), state.bounds()
    tss = _dptr(state["t_ssbef"]) if save_bef else None
    thb = _dptr(state["t_h2osfc_bef"]) if save_bef else None
    lg = log.struct()
    check(handle.lib.clmgb_column_step_logged(handle.h, C.byref(b), C.byref(ft), C.byref(fw), C.byref(cfg),
                                              float(dtime), snow_method, tss, thb, C.byref(lg),
                                              _dptr(col_status, "col_status"), _stream(stream)),
          "column_step_logged")


def column_step_vjp(handle, state, dtime, adj, cfg=None, snow_method=abi.SNOW_JORDAN1991, col_status=None,
                    save_bef=True, stream=None, log=None):
    """Reverse of column_step from the state it starts from (advances `state` like
    column_step does).  `adj` is a clmgb.adjoint.StepAdjointBuffers: its lam_* hold the
    adjoints of the step's outputs on entry and of its inputs on return; grad_*
    accumulate.  `log`: the SubstepLog column_step_logged wrote from the same state,
    or None."""
    _require_device(state)
    cfg = cfg or abi.SwmConfig.clm5_default()
    ft, fw, b = state.soiltemp_fields(), state.soilwater_fields(), state.bounds()
    tss = _dptr(state["t_ssbef"]) if save_bef else None
    thb = _dptr(state["t_h2osfc_bef"]) if save_bef else None
    a = adj.struct()
    lg = C.byref(log.struct()) if log is not None else None
    check(handle.lib.clmgb_column_step_vjp_logged(handle.h, C.byref(b), C.byref(ft), C.byref(fw), C.byref(cfg),
                                                  float(dtime), snow_method, tss, thb, C.byref(a), lg,
                                                  _dptr(col_status, "col_status"), _stream(stream)),
          "column_step_vjp")


def phase_change_h2osfc(handle, state, dtime, dhsdT, stream=None):
    _require_device(state)
    check(handle.lib.clmgb_phase_change_h2osfc(handle.h, C.byref(state.bounds()), C.byref(state.soiltemp_fields()),
                                               float(dtime), _dptr(dhsdT, "dhsdT"), _stream(stream)),
          "phase_change_h2osfc")


def phase_change_beta(handle, state, dtime, dhsdT, stream=None):
    _require_device(state)
    check(handle.lib.clmgb_phase_change_beta(handle.h, C.byref(state.bounds()), C.byref(state.soiltemp_fields()),
                                             float(dtime), _dptr(dhsdT, "dhsdT"), _stream(stream)),
          "phase_change_beta")


def synth_forcing(handle, state, G, I, stream=None):
    _require_device(state)
    check(handle.lib.clmgb_synth_forcing(handle.h, C.byref(state.bounds()), C.byref(state.soiltemp_fields()),
                                         C.byref(state.soilwater_fields()), _dptr(G, "G"), _dptr(I, "I"),
                                         _stream(stream)), "synth_forcing")


def batched_band_solve(handle, tvector, bmatrix, rvector, jtop, jbot, mask, kl=2, ku=2, nlevsno_off=0,
                       stream=None):
    """tvector/rvector: (nlev, nc) CUDA tensors; bmatrix (nlev, nband, nc) == Julia [nc, nband, nlev]."""
    nlev, nc = tvector.shape
    check(handle.lib.clmgb_batched_band_solve(handle.h, nc, nc, nlev, _dptr(tvector), _dptr(bmatrix),
                                              _dptr(rvector), _dptr(jtop), _dptr(jbot), _dptr(mask),
                                              kl, ku, nlevsno_off, _stream(stream)), "batched_band_solve")


def tridiagonal_multi(handle, u, a, b, c, r, jtop, mask, stream=None):
    nlevs, ncols = u.shape
    check(handle.lib.clmgb_tridiagonal_multi(handle.h, ncols, ncols, nlevs, _dptr(u), _dptr(a), _dptr(b),
                                             _dptr(c), _dptr(r), _dptr(jtop), _dptr(mask), _stream(stream)),
          "tridiagonal_multi")


def batched_band_solve_factor(handle, tvector, bmatrix, rvector, jtop, jbot, mask, lu, piv, kl=2, ku=2,
                              nlevsno_off=0, stream=None):
    """batched_band_solve that also stores its factorisation: lu (nlev, 2*kl+ku+1, nc)
    float64, piv (nlev, nc) uint8."""
    nlev, nc = tvector.shape
    check(handle.lib.clmgb_batched_band_solve_factor(handle.h, nc, nc, nlev, _dptr(tvector), _dptr(bmatrix),
                                                     _dptr(rvector), _dptr(jtop), _dptr(jbot), _dptr(mask),
                                                     kl, ku, nlevsno_off, _dptr(lu), _dptr(piv), _stream(stream)),
          "batched_band_solve_factor")


def batched_band_solve_adjoint(handle, tvector, tvector_bar, lu, piv, bmatrix_bar, rvector_bar, jtop, jbot, mask,
                               kl=2, ku=2, nlevsno_off=0, stream=None):
    """Reverse of batched_band_solve from the stored factors; bars accumulate (None = inactive)."""
    nlev, nc = tvector.shape
    check(handle.lib.clmgb_batched_band_solve_adjoint(handle.h, nc, nc, nlev, _dptr(tvector), _dptr(tvector_bar),
                                                      _dptr(lu), _dptr(piv), _dptr(bmatrix_bar),
                                                      _dptr(rvector_bar), _dptr(jtop), _dptr(jbot), _dptr(mask),
                                                      kl, ku, nlevsno_off, _stream(stream)),
          "batched_band_solve_adjoint")


def tridiagonal_adjoint(handle, u, a, b, c, u_bar, a_bar, b_bar, c_bar, r_bar, jtop, mask, stream=None):
    """tridiagonal_solve! reverse rule per column of (nlevs, ncols) tensors; bars accumulate."""
    nlevs, ncols = u.shape
    check(handle.lib.clmgb_tridiagonal_adjoint(handle.h, ncols, ncols, nlevs, _dptr(u), _dptr(a), _dptr(b),
                                               _dptr(c), _dptr(u_bar), _dptr(a_bar), _dptr(b_bar), _dptr(c_bar),
                                               _dptr(r_bar), _dptr(jtop), _dptr(mask), _stream(stream)),
          "tridiagonal_adjoint")


def balance_begin(handle, state, stream=None):
    """(t_grnd0, begwb) recorded before a step (clmgb_balance_begin)."""
    import torch
    t0 = torch.empty(state.nc, dtype=torch.float64, device="cuda")
    w0 = torch.empty(state.nc, dtype=torch.float64, device="cuda")
    check(handle.lib.clmgb_balance_begin(handle.h, C.byref(state.bounds()), C.byref(state.soiltemp_fields()),
                                         _dptr(t0), _dptr(w0), _stream(stream)), "balance_begin")
    return t0, w0


def balance_residuals(handle, state, dtime, t_grnd0, begwb, stream=None):
    """(errsoi W/m2, errh2o mm) of the step just taken (clmgb_balance_residuals)."""
    import torch
    es = torch.empty(state.nc, dtype=torch.float64, device="cuda")
    eh = torch.empty(state.nc, dtype=torch.float64, device="cuda")
    check(handle.lib.clmgb_balance_residuals(handle.h, C.byref(state.bounds()), C.byref(state.soiltemp_fields()),
                                             C.byref(state.soilwater_fields()), float(dtime),
                                             _dptr(state["t_ssbef"]), _dptr(state["t_h2osfc_bef"]), _dptr(t_grnd0),
                                             _dptr(begwb), _dptr(es), _dptr(eh), _stream(stream)),
          "balance_residuals")
    return es, eh


MATH_OPS = {"log": 0, "exp": 1, "pow": 2, "log10": 3, "sin": 4, "acos": 5, "div": 6}


def math_eval(handle, op, x, y=None, out=None, stream=None):
    """Evaluates the library's binary64 log/exp/pow/log10/sin/acos, or its division x / y
    (op "div"), on CUDA tensors."""
    import torch
    if out is None:
        out = torch.empty_like(x)
    check(handle.lib.clmgb_math_eval(handle.h, MATH_OPS[op], x.numel(), _dptr(x, "x"),
                                     _dptr(y, "y") if y is not None else None, _dptr(out, "out"),
                                     _stream(stream)), "math_eval")
    return out
