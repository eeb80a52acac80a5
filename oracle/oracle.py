"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs
import this module.  The product package never does.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
_PKG = os.path.join(ROOT, "clm.jl_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from clmgb import abi  # noqa: E402  (interface definitions only)

import importlib.util as _ilu  # noqa: E402

_spec = _ilu.spec_from_file_location("clm_oracle_build", os.path.join(HERE, "build.py"))
_build = _ilu.module_from_spec(_spec)
_spec.loader.exec_module(_build)

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.orc_soil_temperature.argtypes = [P, P, P, C.c_double, C.c_int32, P, C.c_int32]
        L.orc_soil_water_fractions.argtypes = [P, P, P, C.c_int32]
        L.orc_rootsink.argtypes = [P, P, P, C.c_int32]
        L.orc_soil_water_zd09.argtypes = [P, P, P, C.c_double, C.c_double]
        L.orc_soil_fluxes.argtypes = [P, P, P, C.c_double]
        L.orc_surface_hydrology.argtypes = [P, P, P, P, C.c_uint32, C.c_double]
        L.orc_snow_layers.argtypes = [P, P, P, P, C.c_uint32, C.c_double]
        L.orc_lake_temperature.argtypes = [P, P, P, P, C.c_double]
        L.orc_balance_check_columns.argtypes = [P, P, C.c_double, P]
        L.orc_soil_water.argtypes = [P, P, P, P, C.c_double, P, P, P, C.c_int32]
        L.orc_run_steps.argtypes = [P, P, P, P, P, C.c_double, C.c_int32, C.c_int32, P, P,
                                    C.c_int64, P, P, P, C.c_int32]
        L.orc_batched_band_solve.argtypes = [C.c_int64, C.c_int64, C.c_int32, P, P, P, P, P, P,
                                             C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        L.orc_tridiagonal_multi.argtypes = [C.c_int64, C.c_int64, C.c_int32, P, P, P, P, P, P, P, C.c_int32]
        L.orc_tridiagonal_solve.argtypes = [P, P, P, P, P, C.c_int32, C.c_int32]
        L.orc_tridiagonal_col.argtypes = [P, P, P, P, P, C.c_int32, C.c_int32, C.c_int32]
        L.orc_ice_impedance.argtypes = [C.c_double, C.c_double]
        L.orc_ice_impedance.restype = C.c_double
        L.orc_phase_change_h2osfc.argtypes = [P, P, P, C.c_double, P]
        L.orc_phase_change_beta.argtypes = [P, P, P, C.c_double, P]
        L.orc_init_soil_properties.argtypes = [C.c_int64] + [P] * 11
        L.orc_tridiagonal_adjoint.argtypes = [P] * 9 + [C.c_int32, C.c_int32]
        L.orc_tridiagonal_adjoint_multi.argtypes = [C.c_int64, C.c_int64, C.c_int32] + [P] * 11 + [C.c_int32]
        L.orc_batched_band_solve_adjoint.argtypes = [C.c_int64, C.c_int64, C.c_int32] + [P] * 8 + \
            [C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        L.orc_soil_water_flexible_cn.argtypes = [P, P, P]
        L.orc_compute_rhs_moisture_form.argtypes = [C.c_int32] + [P] * 6
        L.orc_compute_rhs_moisture_form.restype = None
        L.orc_compute_lhs_moisture_form.argtypes = [C.c_int32] + [P] * 8
        L.orc_compute_lhs_moisture_form.restype = None
        L.orc_set_perturbation.argtypes = [C.c_int32, C.c_double, C.c_uint64]
        L.orc_set_perturbation.restype = None
        _lib = L
    return _lib


def default_threads():
    return int(os.environ.get("CLMGB_ORACLE_THREADS", os.cpu_count() or 1))


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _chk(rc):
    if rc != 0:
        raise RuntimeError("oracle returned %d" % rc)


def soil_temperature(st, dtime, snow_method=abi.SNOW_JORDAN1991, nthreads=None):
    """soil_temperature! on a host ColumnState (in place); returns per-column status."""
    vp, b, f = st.vp, st.bounds(), st.soiltemp_fields()
    status = np.zeros(st.nc, dtype=np.uint32)
    _chk(lib().orc_soil_temperature(C.byref(vp), C.byref(b), C.byref(f), dtime, snow_method,
                                    _p(status), nthreads or default_threads()))
    return status


def soil_water_fractions(st, nthreads=None):
    vp, b, f = st.vp, st.bounds(), st.soilwater_fields()
    _chk(lib().orc_soil_water_fractions(C.byref(vp), C.byref(b), C.byref(f), nthreads or default_threads()))


def rootsink(rs, use_hydrstress=False):
    """compute_effec_rootfrac_and_vert_tran_sink! in place on a host RootSinkState;
    returns 1 where the reference would raise its filter-count error, else 0."""
    vp, b, f = rs.vp, rs.bounds(), rs.fields(with_hydrstress=True)
    rc = lib().orc_rootsink(C.byref(vp), C.byref(b), C.byref(f), 1 if use_hydrstress else 0)
    if rc < 0:
        _chk(rc)
    return rc


def soil_fluxes(fs, dtime):
    """soil_fluxes! in place on a host SoilFluxState."""
    _chk(lib().orc_soil_fluxes(C.byref(fs.vp), C.byref(fs.bounds()), C.byref(fs.fields()), float(dtime)))


def balance_check_columns(cb, dtime):
    """balance_check!'s column checks on a host ColBalanceState; returns the report."""
    rep = abi.BalanceReport()
    _chk(lib().orc_balance_check_columns(C.byref(cb.bounds()), C.byref(cb.fields()), float(dtime), C.byref(rep)))
    return rep


def lake_temperature(lk, dtime, cfg):
    """lake_temperature! in place on a host LakeState."""
    _chk(lib().orc_lake_temperature(C.byref(lk.vp), C.byref(lk.bounds()), C.byref(lk.fields()), C.byref(cfg),
                                    float(dtime)))


def snow_layers(sl, dtime, cfg, stages):
    """The snow-layer routines selected by `stages`, in place on a host SnowLayerState."""
    _chk(lib().orc_snow_layers(C.byref(sl.vp), C.byref(sl.bounds()), C.byref(sl.fields()), C.byref(cfg),
                               int(stages), float(dtime)))


def surface_hydrology(sh, dtime, cfg, stages):
    """The surface-hydrology routines selected by `stages`, in place on a host SurfHydState."""
    _chk(lib().orc_surface_hydrology(C.byref(sh.vp), C.byref(sh.bounds()), C.byref(sh.fields()), C.byref(cfg),
                                     int(stages), float(dtime)))


def soil_water_zd09(zs, dtime, e_ice=6.0):
    """soilwater_zengdecker2009! in place on a host Zd09State."""
    _chk(lib().orc_soil_water_zd09(C.byref(zs.vp), C.byref(zs.bounds()), C.byref(zs.fields()), float(e_ice),
                                   float(dtime)))


def soil_water(st, dtime, cfg=None, capture=False, nthreads=None):
    """soil_water! (moisture form) in place; returns status (and captured qin/qout)."""
    cfg = cfg or abi.SwmConfig.clm5_default()
    vp, b, f = st.vp, st.bounds(), st.soilwater_fields()
    status = np.zeros(st.nc, dtype=np.uint32)
    qin = qout = None
    if capture:
        qin = np.zeros((vp.nlevsoi, st.nc))
        qout = np.zeros((vp.nlevsoi, st.nc))
    rc = lib().orc_soil_water(C.byref(vp), C.byref(b), C.byref(f), C.byref(cfg), dtime,
                              _p(status), _p(qin), _p(qout), nthreads or default_threads())
    if rc != 0:
        return rc
    if capture:
        return status, qin, qout
    return status


def run_steps(st, dtime, G, I, cfg=None, snow_method=abi.SNOW_JORDAN1991, nthreads=None):
    """Run len(G) synthetic steps (forcing + path) in place.  G, I: [nsteps, nc]."""
    cfg = cfg or abi.SwmConfig.clm5_default()
    G = np.ascontiguousarray(G, dtype=np.float64)
    I = np.ascontiguousarray(I, dtype=np.float64)
    nsteps = G.shape[0]
    vp, b = st.vp, st.bounds()
    ft, fw = st.soiltemp_fields(), st.soilwater_fields()
    status = np.zeros(st.nc, dtype=np.uint32)
    _chk(lib().orc_run_steps(C.byref(vp), C.byref(b), C.byref(ft), C.byref(fw), C.byref(cfg),
                             dtime, snow_method, nsteps, _p(G), _p(I), st.nc,
                             _p(st["t_ssbef"]), _p(st["t_h2osfc_bef"]), _p(status),
                             nthreads or default_threads()))
    return status


def batched_band_solve(tvector, bmatrix, rvector, jtop, jbot, mask, kl=2, ku=2, nlevsno_off=0,
                       nthreads=None):
    """bmatrix: numpy (nlev, nband, nc) == Julia [nc, nband, nlev]; vectors (nlev, nc)."""
    nlev, nc = tvector.shape
    _chk(lib().orc_batched_band_solve(nc, nc, nlev, _p(tvector), _p(bmatrix), _p(rvector),
                                      _p(jtop), _p(jbot), _p(mask), kl, ku, nlevsno_off,
                                      nthreads or default_threads()))


def tridiagonal_multi(u, a, b, c, r, jtop, mask, nthreads=None):
    nlevs, ncols = u.shape
    _chk(lib().orc_tridiagonal_multi(ncols, ncols, nlevs, _p(u), _p(a), _p(b), _p(c), _p(r),
                                     _p(jtop), _p(mask), nthreads or default_threads()))


def tridiagonal_solve(a, b, c, r, jtop, nlevs):
    u = np.zeros(nlevs)
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (a, b, c, r)]
    lib().orc_tridiagonal_solve(_p(u), *[_p(x) for x in arr], jtop, nlevs)
    return u


def tridiagonal_col(a, b, c, r, jtop, lbj, ubj, u=None):
    n = ubj - lbj + 1
    u = np.zeros(n) if u is None else np.array(u, dtype=np.float64)
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (a, b, c, r)]
    lib().orc_tridiagonal_col(_p(u), *[_p(x) for x in arr], jtop, lbj, ubj)
    return u


def tridiagonal_adjoint(u, a, b, c, ubar, jtop, n):
    """tridiagonal_solve! reverse rule for one system; returns (abar, bbar, cbar, rbar)
    accumulated from zero, and consumes ubar (a float64 array, modified in place)."""
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (u, a, b, c)]
    outs = [np.zeros(n) for _ in range(4)]
    lib().orc_tridiagonal_adjoint(*[_p(x) for x in arr], _p(ubar), *[_p(x) for x in outs], jtop, n)
    return tuple(outs)


def tridiagonal_adjoint_multi(u, a, b, c, ubar, abar, bbar, cbar, rbar, jtop, mask, nthreads=None):
    """Batched rule over (nlevs, ncols) arrays; the bar arrays accumulate in place (None = inactive)."""
    nlevs, ncols = u.shape
    _chk(lib().orc_tridiagonal_adjoint_multi(ncols, ncols, nlevs, _p(u), _p(a), _p(b), _p(c), _p(ubar),
                                             _p(abar), _p(bbar), _p(cbar), _p(rbar), _p(jtop), _p(mask),
                                             nthreads or default_threads()))


def batched_band_solve_adjoint(tvector, tbar, bmatrix, bbar, rbar, jtop, jbot, mask, kl=2, ku=2,
                               nlevsno_off=0, nthreads=None):
    """band_solve! reverse rule on the batched layout; bbar/rbar accumulate (None = inactive)."""
    nlev, nc = tvector.shape
    _chk(lib().orc_batched_band_solve_adjoint(nc, nc, nlev, _p(tvector), _p(tbar), _p(bmatrix), _p(bbar),
                                              _p(rbar), _p(jtop), _p(jbot), _p(mask), kl, ku, nlevsno_off,
                                              nthreads or default_threads()))


def ice_impedance(icefrac, e_ice):
    return lib().orc_ice_impedance(float(icefrac), float(e_ice))


def phase_change_h2osfc(st, dtime, dhsdT):
    dh = np.ascontiguousarray(dhsdT, dtype=np.float64)
    _chk(lib().orc_phase_change_h2osfc(C.byref(st.vp), C.byref(st.bounds()),
                                       C.byref(st.soiltemp_fields()), dtime, _p(dh)))


def phase_change_beta(st, dtime, dhsdT):
    dh = np.ascontiguousarray(dhsdT, dtype=np.float64)
    _chk(lib().orc_phase_change_beta(C.byref(st.vp), C.byref(st.bounds()),
                                     C.byref(st.soiltemp_fields()), dtime, _p(dh)))


def init_soil_properties(sand, clay, om, zsoi):
    sand, clay, om, zsoi = [np.ascontiguousarray(np.broadcast_to(x, np.broadcast(sand, clay, om, zsoi).shape),
                                                 dtype=np.float64) for x in (sand, clay, om, zsoi)]
    n = sand.size
    outs = {k: np.zeros(sand.shape) for k in ("watsat", "bsw", "sucsat", "hksat", "tkmg", "tkdry", "csol")}
    lib().orc_init_soil_properties(n, _p(sand), _p(clay), _p(om), _p(zsoi),
                                   *[_p(outs[k]) for k in ("watsat", "bsw", "sucsat", "hksat", "tkmg",
                                                           "tkdry", "csol")])
    return outs


def set_perturbation(mode=0, frac=0.0, salt=0):
    """The oracle's pow/log10 sensitivity hook (clm_oracle.c): 0 off, 1 every result
    +-1 ulp, 2 a fraction `frac` of them, 3 the previous single-precision-log library."""
    lib().orc_set_perturbation(int(mode), float(frac), int(salt))


def soil_water_flexible_cn(fs):
    """soil_water!'s use_flexibleCN step in place on a host FlexCnState."""
    _chk(lib().orc_soil_water_flexible_cn(C.byref(fs.vp), C.byref(fs.bounds()), C.byref(fs.fields())))


def compute_rhs_moisture_form(vert_trans_sink, vwc_liq, qin, qout, dt_dz):
    """compute_RHS_moisture_form! on one column's vectors; returns rmx."""
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (vert_trans_sink, vwc_liq, qin, qout, dt_dz)]
    rmx = np.empty(len(a[0]))
    lib().orc_compute_rhs_moisture_form(len(rmx), *[_p(v) for v in a], _p(rmx))
    return rmx


def compute_lhs_moisture_form(dt_dz, dqidw0, dqidw1, dqodw1, dqodw2):
    """compute_LHS_moisture_form! on one column's vectors; returns (amx, bmx, cmx)."""
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (dt_dz, dqidw0, dqidw1, dqodw1, dqodw2)]
    n = len(a[0])
    amx, bmx, cmx = np.empty(n), np.empty(n), np.empty(n)
    lib().orc_compute_lhs_moisture_form(n, *[_p(v) for v in a], _p(amx), _p(bmx), _p(cmx))
    return amx, bmx, cmx
