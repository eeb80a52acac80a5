"""Writes tests/golden/reference_cases.json: the known-answer fixtures of CLM.jl's
own test suite for this path, transcribed from its test files (cited per case).

CLM.jl is Julia and cannot run here, so these are the reference's hand-built inputs
and analytic answers (x = 1:n solutions, [1,1,1], impedance powers, conservation
identities), not outputs captured from a run.  Run:  python tests/golden/make_golden.py
"""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def penta(n):
    # test_band_diagonal.jl:52-89 (n=5) and :114-139 (n=6): diag 10, +-1 off -2, +-2 off -1
    A = np.diag(np.full(n, 10.0)) + np.diag(np.full(n - 1, -2.0), -1) + np.diag(np.full(n - 1, -2.0), 1) \
        + np.diag(np.full(n - 2, -1.0), -2) + np.diag(np.full(n - 2, -1.0), 2)
    return A


def tri(n, d, o):
    return np.diag(np.full(n, d)) + np.diag(np.full(n - 1, o), -1) + np.diag(np.full(n - 1, o), 1)


def band_case(A, x, jtop, nlevs, kl, ku, tol, src):
    n = A.shape[0]
    nband = kl + ku + 1
    rhs = A @ x
    bm = np.zeros((nband, nlevs))
    r = np.zeros(nlevs)
    for i in range(n):
        lev = jtop - 1 + i
        r[lev] = rhs[i]
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            band = (i - j) + kl  # 0-based: band 1 = A[i, i+ku]
            bm[band, lev] = A[i, j]
    return dict(bmatrix=bm.tolist(), rvector=r.tolist(), x_exact=x.tolist(), jtop=jtop,
                jbot=jtop + n - 1, nlevs=nlevs, kl=kl, ku=ku, atol=tol, source=src)


def surface_hydrology_cases():
    """The known answers of the surface-hydrology routines' tests, one case per call:
    test/test_sat_excess_runoff.jl, test/test_infilt_excess_runoff.jl and
    test/test_soil_hydrology_mod.jl.  Column vectors are per column; "icefrac3" and
    "hksat3" give soil levels 1-3 per column; "liq_top" the top soil level's liquid.
    Expected values are the tests' own formulas with their tolerances (isapprox's
    default rtol is sqrt(eps) = 1.49e-8)."""
    RT = 2.0 ** -26
    ISTSOIL, ISTCROP, SUNWALL, SHADEWALL, ROOF, ROAD_IMPERV, ISPVAL = 1, 2, 72, 73, 71, 74, -9999
    out = []

    def case(name, src, stages, nc, inputs, expect, cfg=None, nl=1, ng=1, dtime=1800.0, masks=None, nan=None,
             error=False):
        out.append(dict(name=name, source=src, stages=stages, nc=nc, nl=nl, ng=ng, dtime=dtime, cfg=cfg or {},
                        inputs=inputs, masks=masks or {}, expect=expect, expect_nan=nan or {}, error=error))

    def ex(field, values, rtol=RT, atol=0.0):
        return dict(field=field, values=values, rtol=rtol, atol=atol)

    sat = ["saturated_excess_runoff!"]

    def sat_inputs(nc, **kw):
        d = dict(col_landunit=[1] * nc, col_urbpoi=[0] * nc, col_active=[1] * nc, col_is_hillslope=[0] * nc,
                 col_cold=[ISPVAL] * nc, qflx_floodc=[0.0] * nc)
        d.update(kw)
        return d

    e = [0.4 * math.exp(-0.5 * 0.5 * 2.0), 0.4 * math.exp(-0.5 * 0.5 * 1.0), 0.4 * math.exp(-0.5 * 0.5 * 2.0)]
    case("sat_topmodel", "test/test_sat_excess_runoff.jl:182-245", sat, 3,
         sat_inputs(3, frost_table=[5.0, 1.5, 0.5], zwt=[2.0] * 3, zwt_perched=[1.0] * 3, wtfact=[0.4] * 3,
                    qflx_rain_plus_snomelt=[5.0, 10.0, 2.0]),
         [ex("fsat", e), ex("qflx_sat_excess_surf", [e[0] * 5.0, e[1] * 10.0, e[2] * 2.0]), ex("fcov", e)],
         cfg=dict(fff=0.5), nl=1)
    f1, f2 = 1.0 - (1.0 - 50.0 / 100.0) ** 0.5, 1.0 - (1.0 - 150.0 / 200.0) ** (2.0 / 3.0)
    case("sat_vic", "test/test_sat_excess_runoff.jl:250-305", sat, 2,
         sat_inputs(2, b_infil=[1.0, 2.0], top_max_moist=[100.0, 200.0], top_moist_limited=[50.0, 150.0],
                    qflx_rain_plus_snomelt=[8.0, 4.0]),
         [ex("fsat", [f1, f2]), ex("qflx_sat_excess_surf", [f1 * 8.0, f2 * 4.0])], cfg=dict(fsat_method=2))
    e1 = 0.4 * math.exp(-0.5 * 0.5 * 1.0)
    case("sat_crop_fsat_zero", "test/test_sat_excess_runoff.jl:310-364", sat, 2,
         sat_inputs(2, col_landunit=[1, 2], lun_itype=[ISTSOIL, ISTCROP], frost_table=[5.0] * 2, zwt=[1.0] * 2,
                    zwt_perched=[10.0] * 2, wtfact=[0.4] * 2, qflx_rain_plus_snomelt=[10.0] * 2),
         [ex("fsat", [e1, 0.0]), ex("qflx_sat_excess_surf", [e1 * 10.0, 0.0])],
         cfg=dict(fff=0.5, crop_fsat_equals_zero=1), nl=2)
    case("sat_hillslope_fsat_zero", "test/test_sat_excess_runoff.jl:369-428", sat, 3,
         sat_inputs(3, col_is_hillslope=[0, 1, 1], col_cold=[ISPVAL, 3, ISPVAL], frost_table=[5.0] * 3,
                    zwt=[1.0] * 3, zwt_perched=[10.0] * 3, wtfact=[0.4] * 3, qflx_rain_plus_snomelt=[10.0] * 3),
         [ex("fsat", [e1, 0.0, e1]), ex("qflx_sat_excess_surf", [None, 0.0, e1 * 10.0])],
         cfg=dict(fff=0.5, hillslope_fsat_equals_zero=1))
    e3 = 0.3 * math.exp(-0.5 * 0.5 * 1.0)
    case("sat_urban_flood", "test/test_sat_excess_runoff.jl:433-478", sat, 2,
         sat_inputs(2, col_urbpoi=[1, 0], frost_table=[5.0] * 2, zwt=[1.0] * 2, zwt_perched=[10.0] * 2,
                    wtfact=[0.3] * 2, qflx_rain_plus_snomelt=[5.0] * 2, qflx_floodc=[2.0] * 2),
         [ex("qflx_sat_excess_surf", [e3 * 5.0 + 2.0, e3 * 5.0])], cfg=dict(fff=0.5))
    e5 = 0.5 * math.exp(-0.5 * 1.0 * 1.0)
    case("sat_mask", "test/test_sat_excess_runoff.jl:483-530", sat, 4,
         sat_inputs(4, frost_table=[5.0] * 4, zwt=[1.0] * 4, zwt_perched=[10.0] * 4, wtfact=[0.5] * 4,
                    qflx_rain_plus_snomelt=[3.0] * 4, fsat=[float("nan")] * 4),
         [ex("fsat", [e5, None, e5, None]), ex("qflx_sat_excess_surf", [e5 * 3.0, None, e5 * 3.0, None])],
         cfg=dict(fff=1.0), masks=dict(mask_hydrology=[1, 0, 1, 0]), nan=dict(fsat=[1, 3]))
    case("sat_invalid_method", "test/test_sat_excess_runoff.jl:535-570", sat, 1, sat_inputs(1), [],
         cfg=dict(fsat_method=99), error=True)
    case("sat_crop_and_hillslope", "test/test_sat_excess_runoff.jl:575-630", sat, 3,
         sat_inputs(3, col_landunit=[1, 2, 2], lun_itype=[ISTCROP, ISTSOIL], col_is_hillslope=[0, 1, 0],
                    col_cold=[ISPVAL, 3, ISPVAL], frost_table=[5.0] * 3, zwt=[1.0] * 3, zwt_perched=[10.0] * 3,
                    wtfact=[0.4] * 3, qflx_rain_plus_snomelt=[10.0] * 3),
         [ex("fsat", [0.0, 0.0, e1], atol=0.0), ex("qflx_sat_excess_surf", [0.0, 0.0, e1 * 10.0])],
         cfg=dict(fff=0.5, crop_fsat_equals_zero=1, hillslope_fsat_equals_zero=1), nl=2)

    inf = ["infiltration_excess_runoff!"]

    def inf_inputs(nc, ice, hk, fsat, qin, fh):
        return dict(icefrac3=ice, hksat3=hk, fsat=fsat, qflx_in_soil=qin, frac_h2osfc=fh)

    v = [10.0 ** (-6.0 * 0.1) * 0.01, 10.0 ** (-6.0 * 0.2) * 0.02, 10.0 ** (-6.0 * 0.3) * 0.03]
    case("qinmax_hksat", "test/test_infilt_excess_runoff.jl:71-124 (qinmax with fsat = 0 is qinmax_on_unsaturated_area)",
         inf, 3, inf_inputs(3, [[0.1, 0.2, 0.3], [0.0] * 3, [0.5] * 3], [[0.01, 0.02, 0.03], [0.05] * 3, [0.01] * 3],
                            [0.0] * 3, [0.0] * 3, [0.0] * 3),
         [ex("qinmax", [min(v), 0.05, 10.0 ** (-6.0 * 0.5) * 0.01], rtol=0.0, atol=1e-15)])
    case("infl_excess_hksat", "test/test_infilt_excess_runoff.jl:128-170", inf, 2,
         inf_inputs(2, [[0.0] * 3] * 2, [[0.01] * 3] * 2, [0.1, 0.2], [0.02, 0.005], [0.0, 0.0]),
         [ex("qinmax", [0.9 * 0.01, 0.8 * 0.01], rtol=0.0, atol=1e-15),
          ex("qflx_infl_excess", [max(0.0, 0.02 - 0.009), 0.0], rtol=0.0, atol=1e-15)])
    case("infl_excess_none", "test/test_infilt_excess_runoff.jl:175-210", inf, 2,
         inf_inputs(2, [[0.0] * 3] * 2, [[0.01] * 3] * 2, [0.0, 0.0], [100.0, 200.0], [0.0, 0.0]),
         [ex("qinmax", [1.0e200, 1.0e200], rtol=0.0, atol=1e190), ex("qflx_infl_excess", [0.0, 0.0], rtol=0.0)],
         cfg=dict(qinmax_method=0))
    case("infl_excess_mask", "test/test_infilt_excess_runoff.jl:215-252", inf, 3,
         dict(inf_inputs(3, [[0.0] * 3] * 3, [[0.01] * 3] * 3, [0.0] * 3, [0.02] * 3, [0.0] * 3),
              qinmax=[float("nan")] * 3),
         [ex("qinmax", [None, 0.01, None], rtol=0.0, atol=1e-15)], masks=dict(mask_hydrology=[0, 1, 0]),
         nan=dict(qinmax=[0, 2]))
    case("qinmax_zero_ice", "test/test_infilt_excess_runoff.jl:257-280", inf, 1,
         inf_inputs(1, [[0.0] * 3], [[0.05, 0.03, 0.04]], [0.0], [0.0], [0.0]),
         [ex("qinmax", [0.03], rtol=0.0, atol=1e-15)])
    fz = 10.0 ** (-6.0) * 0.01
    case("infl_excess_fully_frozen", "test/test_infilt_excess_runoff.jl:284-330", inf, 1,
         inf_inputs(1, [[1.0] * 3], [[0.01] * 3], [0.0], [0.001], [0.0]),
         [ex("qinmax", [fz], rtol=0.0, atol=1e-20), ex("qflx_infl_excess", [max(0.0, 0.001 - fz)], rtol=0.0, atol=1e-12)])
    for fs, qm, exv in ((0.5, 0.5 * 0.02, 0.0), (0.9, 0.1 * 0.02, 0.003)):
        case("infl_excess_fsat_%g" % fs, "test/test_infilt_excess_runoff.jl:335-378", inf, 1,
             inf_inputs(1, [[0.0] * 3], [[0.02] * 3], [fs], [0.005], [0.0]),
             [ex("qinmax", [qm], rtol=0.0, atol=1e-15), ex("qflx_infl_excess", [exv], rtol=0.0, atol=1e-15)])
    for fh, exv in ((0.0, 0.005), (0.5, max(0.0, 0.015 - 0.5 * 0.01)), (1.0, 0.015)):
        case("infl_excess_frac_h2osfc_%g" % fh, "test/test_infilt_excess_runoff.jl:383-428", inf, 1,
             inf_inputs(1, [[0.0] * 3], [[0.01] * 3], [0.0], [0.015], [fh]),
             [ex("qflx_infl_excess", [exv], rtol=0.0, atol=1e-15)])
    q3 = 10.0 ** (-6.0 * 0.8) * 0.01
    case("infl_excess_heterogeneous", "test/test_infilt_excess_runoff.jl:433-488", inf, 4,
         inf_inputs(4, [[0.0] * 3, [0.0] * 3, [0.8] * 3, [0.0] * 3], [[0.01] * 3, [0.1] * 3, [0.01] * 3, [0.01] * 3],
                    [0.0, 0.0, 0.0, 0.5], [0.005] * 4, [0.0] * 4),
         [ex("qflx_infl_excess", [0.0, 0.0, None, 0.0], rtol=0.0, atol=1e-15),
          ex("qflx_infl_excess", [None, None, max(0.0, 0.005 - q3), None], rtol=0.0, atol=1e-12),
          ex("qinmax", [None, None, q3, 0.005], rtol=0.0, atol=1e-15)])
    case("infl_invalid_method", "test/test_infilt_excess_runoff.jl:493-520", inf, 1,
         inf_inputs(1, [[0.0] * 3], [[0.01] * 3], [0.0], [0.01], [0.0]), [], cfg=dict(qinmax_method=99), error=True)
    for ei in (3.0, 9.0):
        case("qinmax_e_ice_%g" % ei, "test/test_infilt_excess_runoff.jl:525-555", inf, 1,
             inf_inputs(1, [[0.5] * 3], [[0.01] * 3], [0.0], [0.0], [0.0]),
             [ex("qinmax", [10.0 ** (-ei * 0.5) * 0.01], rtol=0.0, atol=1e-15)], cfg=dict(e_ice=ei))

    case("set_floodc", "test/test_soil_hydrology_mod.jl:117-131", ["set_floodc!"], 4,
         dict(qflx_floodg=[0.5, 0.3], col_gridcell=[1, 1, 2, 2], col_itype=[1, SUNWALL, 1, SHADEWALL]),
         [ex("qflx_floodc", [0.5, 0.0, 0.3, 0.0])], ng=2)
    case("infiltration", "test/test_soil_hydrology_mod.jl:136-150", ["infiltration!"], 3,
         dict(qflx_in_soil_limited=[0.1, 0.2, 0.3], qflx_h2osfc_drain=[0.01, 0.02, 0.03]),
         [ex("qflx_infl", [0.11, 0.22, 0.33])])
    # The truncation test calls the partial-update kernel alone with an outflow; through
    # update_h2osfc! the same arithmetic is an inflow of the opposite sign, the store
    # below its spill threshold (no runoff) and no drainage (frac_h2osfc = 0).
    for rel, res in ((5.0e-11, 5.0e-11), (5.0e-14, 0.0)):
        case("h2osfc_truncation_%g" % rel, "test/test_soil_hydrology_mod.jl:152-173", ["update_h2osfc!"], 1,
             dict(h2osfc=[1.0], qflx_in_h2osfc=[-(1.0 - rel) / 1800.0], h2osfc_thresh=[10.0], frac_h2osfc=[0.0],
                  frac_h2osfc_nosnow=[0.0], qinmax=[0.0], topo_slope=[5.0]),
             [ex("h2osfc", [res], rtol=0.0, atol=1e-15 if res else 0.0)])
    urb = ["total_surface_runoff!", "update_urban_ponding!"]

    def urb_inputs(rain, evap, pond0):
        return dict(col_snl=[0, 0], col_itype=[ROOF, ROAD_IMPERV], qflx_rain_plus_snomelt=[rain] * 2,
                    qflx_liqevap_from_top_layer=[evap] * 2, qflx_floodc=[0.0] * 2, xs_urban=[0.0] * 2,
                    qflx_surf=[0.0] * 2, liq_top=pond0, qflx_sat_excess_surf=[0.0] * 2,
                    qflx_infl_excess_surf=[0.0] * 2, qflx_h2osfc_surf=[0.0] * 2)

    um = dict(mask_hydrology=[0, 0], mask_urban=[1, 1])
    case("urban_pond_light_rain", "test/test_soil_hydrology_mod.jl:495-534", urb, 2, urb_inputs(1.0e-4, 0.0, [0.0, 0.0]),
         [ex("xs_urban", [0.0, 0.0], rtol=0.0, atol=1e-12), ex("qflx_surf", [0.0, 0.0], rtol=0.0, atol=1e-12),
          ex("liq_top", [1.0e-4 * 3600.0] * 2)], dtime=3600.0, masks=um)
    xs = 1.0e-2 - 1.0 / 3600.0
    case("urban_pond_heavy_rain", "test/test_soil_hydrology_mod.jl:536-556", urb, 2, urb_inputs(1.0e-2, 0.0, [0.0, 0.0]),
         [ex("xs_urban", [xs] * 2, rtol=1e-10), ex("qflx_surf", [xs] * 2, rtol=1e-10), ex("liq_top", [1.0, 1.0])],
         dtime=3600.0, masks=um)
    case("urban_pond_balance", "test/test_soil_hydrology_mod.jl:558-582", urb, 2, urb_inputs(5.0e-4, 1.0e-4, [0.2, 0.5]),
         [dict(field="pond_balance", rain=5.0e-4, evap=1.0e-4, pond0=[0.2, 0.5], atol=1e-10)],
         dtime=3600.0, masks=um)
    return dict(cases=out)


def balance_check_cases():
    """Column water-balance cases of test/test_balance_check.jl (make_bc_test_data: 4
    soil columns, begwb = endwb = 100 mm, zero fluxes, dtime 1800 s, errsoi 0); each
    sets the inputs it changes and the answers and stop decisions the test asserts.
    The stop rule is _bc_should_error: hard_error and DAnstep > skip_steps (3)."""
    out = []
    dt = 1800.0

    def case(name, src, inputs, expect, stops=()):
        out.append(dict(name=name, source=src, nc=4, dtime=dt, inputs=inputs, expect=expect, stops=list(stops)))

    case("perfect_balance", "test/test_balance_check.jl:309-378", {}, [dict(field="errh2o", exact=[0.0] * 4)],
         stops=[dict(dastep=100, hard_error=True, stop=False)])
    case("water_error_detection", "test/test_balance_check.jl:381-429", dict(endwb=[200.0] * 4),
         [dict(field="errh2o", exact=[100.0] * 4)], stops=[dict(dastep=100, hard_error=True, stop=True)])
    case("urban_walls_take_no_precipitation", "test/test_balance_check.jl:432-477",
         dict(col_itype=[1, 72, 73, 1], forc_rain=[5.0] * 4, forc_snow=[2.0] * 4),
         [dict(field="errh2o", index=[1, 2], atol=1e-15, value=0.0), dict(field="errh2o", index=[0], nonzero=True)],
         stops=[dict(dastep=1, hard_error=True, stop=False)])
    q = 5.7e-1
    case("ice_runoff_closes_the_balance", "test/test_balance_check.jl:533-592 (a)",
         dict(begwb=[12000.0] * 4, endwb=[12000.0 - q * dt] * 4, qflx_ice_runoff=[q] * 4),
         [dict(field="errh2o", index=[0, 1, 2, 3], atol=1e-10, value=0.0)])
    case("ice_runoff_missing", "test/test_balance_check.jl:533-592 (b)",
         dict(begwb=[12000.0] * 4, endwb=[12000.0 - q * dt] * 4),
         [dict(field="errh2o", index=[0, 1, 2, 3], rtol=1e-12, value=-q * dt), dict(flag="H2O_ERROR")],
         stops=[dict(dastep=2, hard_error=True, stop=False)])
    case("unbalanced_column_stops_past_skip", "test/test_balance_check.jl:639-700", dict(endwb=[150.0] * 4),
         [dict(field="errh2o", index=[0], rtol=1e-12, value=50.0), dict(flag="H2O_ERROR")],
         stops=[dict(dastep=4, hard_error=True, stop=True), dict(dastep=500, hard_error=True, stop=True),
                dict(dastep=2, hard_error=True, stop=False), dict(dastep=500, hard_error=False, stop=False)])
    for field, val in (("endwb", "nan"), ("begwb", "nan"), ("endwb", "inf")):
        case("nonfinite_%s_%s" % (field, val), "test/test_balance_check.jl:709-765",
             {field: [float(val), 100.0, 100.0, 100.0]},
             [dict(field="errh2o", index=[0], nonfinite=True), dict(flag="H2O_NONFINITE")],
             stops=[dict(dastep=4, hard_error=True, stop=True)])
    return dict(cases=out)


def snow_layer_cases():
    """Known answers of test/test_snow_hydrology.jl for the snow-layer routines, each
    through the public routine that uses it.  "snow" level values are listed from the
    bottom snow level up (j = 0, -1, ...); every column has the same values."""
    TFRZ = 273.15
    out = []

    def case(name, src, stages, nc, snl, snow, col, expect):
        out.append(dict(name=name, source=src, stages=stages, nc=nc, snl=snl, snow=snow, col=col, expect=expect))

    case("zero_empty_interface_regression", "test/test_snow_hydrology.jl:264-286", ["zero_empty_snow_layers!"], 1,
         [-1], dict(all_levels=dict(dz=0.1, z=-0.05, zi=-0.1, t_soisno=TFRZ - 2.0, h2osoi_ice=1.0, h2osoi_liq=0.5)),
         {}, [dict(what="top_level_zero", fields=["h2osoi_ice", "h2osoi_liq", "zi"])])
    # combo_scalar's answer (:421-433) through combine_snow_layers!: the top layer is
    # thinner than dzmin (frac_sno_eff * dz = 0.009 < 0.01) and merges into the one below
    t1, t2 = TFRZ - 5.0, TFRZ - 10.0
    case("combine_merges_thin_top_layer", "test/test_snow_hydrology.jl:421-433", ["combine_snow_layers!"], 1, [-2],
         dict(dz=[0.05, 0.03], h2osoi_liq=[2.0, 1.0], h2osoi_ice=[8.0, 5.0], t_soisno=[t2, t1]),
         dict(frac_sno=0.3, frac_sno_eff=0.3, int_snow=100.0),
         [dict(what="snl", value=-1), dict(what="bottom", field="dz", value=0.08),
          dict(what="bottom", field="h2osoi_liq", value=3.0), dict(what="bottom", field="h2osoi_ice", value=13.0),
          dict(what="bottom_below", field="t_soisno", value=TFRZ)])
    # mass_weighted_snow_radius's answers (:435-447) through divide_snow_layers!: the top
    # layer (0.04 m > dzmax_u 0.02 m) hands half its 10 kg/m2 to the layer below (5 kg/m2)
    for name, r1, r2, want in (("radius_weighted", 100.0, 200.0, 150.0), ("radius_clamped_min", 10.0, 20.0, 54.526),
                               ("radius_clamped_max", 2000.0, 2000.0, 1500.0)):
        case("divide_" + name, "test/test_snow_hydrology.jl:435-447", ["divide_snow_layers!"], 1, [-2],
             dict(dz=[0.03, 0.04], h2osoi_liq=[0.0, 0.0], h2osoi_ice=[5.0, 10.0], t_soisno=[TFRZ - 3.0] * 2,
                  snw_rds=[r2, r1]),
             dict(frac_sno=1.0, frac_sno_eff=1.0, int_snow=100.0),
             [dict(what="snl", value=-2), dict(what="bottom", field="snw_rds", value=want, exact=name != "radius_weighted")])
    case("build_snow_filter", "test/test_snow_hydrology.jl:451-465", ["build_snow_filter!"], 4, [-2, 0, -1, 0], {}, {},
         [dict(what="masks", mask_snow=[1, 0, 1, 0], mask_nosnow=[0, 1, 0, 1])])
    return dict(cases=out)


def soil_fluxes_cases():
    """test/test_soil_fluxes.jl: one soil patch on one column, the inputs of its three
    scenarios (level values are the same on every level) and the properties it checks."""
    HVAP, HSUB = 2.501e6, 2.501e6 + 3.337e5
    base = dict(snl=0, t_grnd=280.0, t_h2osfc=280.0, t_h2osfc_bef=279.5, emg=0.96, xmf=0.0, xmf_h2osfc=0.0,
                c_h2osfc=4.188e6, t_skin=280.0, t_ssbef=279.5, t_soisno=280.0, fact=1.0e7, liq=20.0, ice=5.0,
                frac_sno_eff=0.0, frac_h2osfc=0.0, cgrnds=10.0, cgrndl=0.001, htvp=HVAP, eflx_sh_grnd=50.0,
                eflx_sh_veg=10.0, eflx_sh_stem=2.0, dlrad=300.0, ulrad=350.0, qflx_evap_soi=1.0e-5,
                qflx_evap_veg=2.0e-5, qflx_tran_veg=1.0e-5, qflx_ev_snow=5.0e-6, qflx_ev_soil=5.0e-6,
                qflx_ev_h2osfc=0.0, frac_veg_nosno=0, sabg_soil=100.0, sabg_snow=0.0, sabg=100.0,
                forc_lwrad=300.0)
    dew = dict(base, t_grnd=265.0, t_h2osfc=265.0, t_h2osfc_bef=265.0, t_skin=265.0, t_ssbef=265.0,
               t_soisno=265.0, liq=10.0, ice=10.0, htvp=HSUB, eflx_sh_grnd=30.0, eflx_sh_veg=5.0,
               eflx_sh_stem=1.0, dlrad=250.0, ulrad=280.0, qflx_evap_soi=-1.0e-5, qflx_evap_veg=0.0,
               qflx_tran_veg=0.0, qflx_ev_snow=-1.0e-5, qflx_ev_soil=-1.0e-5, sabg_soil=50.0, sabg=50.0,
               forc_lwrad=250.0)
    snow = dict(base, snl=-3, t_grnd=270.0, t_h2osfc=270.0, t_h2osfc_bef=269.5, emg=0.97, t_skin=270.0,
                t_ssbef=269.5, t_soisno=270.0, liq=5.0, ice=50.0, frac_sno_eff=0.8, cgrnds=8.0, cgrndl=0.0005,
                htvp=HSUB, eflx_sh_grnd=20.0, eflx_sh_veg=3.0, eflx_sh_stem=0.5, dlrad=220.0, ulrad=240.0,
                qflx_evap_soi=5.0e-6, qflx_evap_veg=0.0, qflx_tran_veg=0.0, qflx_ev_snow=5.0e-6,
                qflx_ev_soil=0.0, sabg_soil=30.0, sabg_snow=80.0)
    return dict(hvap=HVAP, dtime=1800.0, scenarios=[
        dict(name="smoke", source="test/test_soil_fluxes.jl:3-210", inputs=base,
             checks=["finite", "identities", "t_skin_range", "errsoi_col", "evap_partition"]),
        dict(name="dew_below_freezing", source="test/test_soil_fluxes.jl:257-368", inputs=dew,
             checks=["finite", "frost"]),
        dict(name="snow_layers", source="test/test_soil_fluxes.jl:370-485", inputs=snow,
             checks=["finite", "ev_snow_nonnegative"])])


def rootsink_cases():
    """test/test_soil_water_plant_sink.jl: varpar nlevsno 5, nlevgrnd 10, nlevsoi 4 (:8-21);
    z[c, j + nlevsno] = 0.1 j (:57-61); the expected values are the test's own formulas."""
    ISTSOIL, ISTCROP, ISTURB_MD, ROAD = 1, 2, 9, 75
    nsoi = 4
    zs = [0.1 * j for j in range(1, nsoi + 1)]
    out = []

    def case(name, src, method, col_itype, col_landunit, lun_itype, ppc, rootr, tran_p, tran_c, wt, active,
             expect, mask=None, fvn=None, k=None, smp=None, vegwp4=None, use_hydrstress=False):
        nc = len(col_itype)
        out.append(dict(name=name, source=src, method=method, use_hydrstress=use_hydrstress,
                        nc=nc, np=len(wt), nl=len(lun_itype), col_itype=col_itype, col_landunit=col_landunit,
                        lun_itype=lun_itype, patches_per_col=ppc, rootr=rootr, tran_patch=tran_p,
                        tran_col=tran_c, wtcol=wt, active=active, mask=mask or [True] * nc,
                        fvn=fvn or [0] * len(wt), k=k or [[0.0] * nsoi for _ in wt],
                        smp=smp or [0.0] * nc, vegwp4=vegwp4 or [0.0] * len(wt), expect=expect))

    r = [0.4, 0.3, 0.2, 0.1]
    case("default_single", "test/test_soil_water_plant_sink.jl:131-163", "default", [ISTSOIL], [1], [ISTSOIL], [1],
         [r], [0.002], [0.002], [1.0], [True],
         dict(rootr_col=[r], rootsoi=[[x * 0.002 for x in r]], atol_rootr=1e-12, atol_rootsoi=1e-14))
    r1, r2 = [0.1, 0.2, 0.3, 0.4], [0.5, 0.3, 0.15, 0.05]
    tp, wt = [0.001, 0.003], [0.4, 0.6]
    temp = tp[0] * wt[0] + tp[1] * wt[1]
    ex = [(r1[j] * tp[0] * wt[0] + r2[j] * tp[1] * wt[1]) / temp for j in range(nsoi)]
    case("default_two_patches", "test/test_soil_water_plant_sink.jl:165-207", "default", [ISTSOIL], [1], [ISTSOIL],
         [2], [r1, r2], tp, [temp], wt, [True, True],
         dict(rootr_col=[ex], rootsoi=[[x * temp for x in ex]], atol_rootr=1e-12, atol_rootsoi=1e-14))
    case("default_zero_transpiration", "test/test_soil_water_plant_sink.jl:209-238", "default", [ISTSOIL], [1],
         [ISTSOIL], [1], [[0.25] * 4], [0.0], [0.0], [1.0], [True],
         dict(rootr_col=[[0.0] * 4], rootsoi=[[0.0] * 4], atol_rootr=1e-14, atol_rootsoi=1e-14))
    case("default_inactive_patch", "test/test_soil_water_plant_sink.jl:240-270", "default", [ISTSOIL], [1],
         [ISTSOIL], [2], [[0.4, 0.3, 0.2, 0.1], [0.1, 0.1, 0.1, 0.7]], [0.002, 0.005], [0.001], [0.5, 0.5],
         [True, False], dict(rootr_col=[[0.4, 0.3, 0.2, 0.1]], atol_rootr=1e-12))
    rr = [0.3, 0.3, 0.2, 0.2]
    case("hydstress_roads", "test/test_soil_water_plant_sink.jl:272-304", "hydstress_roads", [ROAD], [1],
         [ISTURB_MD], [1], [rr], [0.001], [0.001], [1.0], [True],
         dict(rootr_col=[rr], rootsoi=[[x * 0.001 for x in rr]], atol_rootr=1e-12, atol_rootsoi=1e-14),
         use_hydrstress=True)
    fl = [0.01 * (-500.0 - (-1000.0) - z * 1000.0) for z in zs]
    case("hydstress_single", "test/test_soil_water_plant_sink.jl:306-346", "hydstress", [ISTSOIL], [1], [ISTSOIL],
         [1], [[0.0] * 4], [0.002], [0.002], [1.0], [True],
         dict(rootsoi=[fl], atol_rootsoi=1e-10), fvn=[1], k=[[0.01] * 4], smp=[-500.0], vegwp4=[-1000.0],
         use_hydrstress=True)
    fl = [0.01 * (-5000.0 - (-500.0) - z * 1000.0) for z in zs]
    case("hydstress_negative", "test/test_soil_water_plant_sink.jl:348-389", "hydstress", [ISTSOIL], [1],
         [ISTSOIL], [1], [[0.0] * 4], [0.002], [0.002], [1.0], [True],
         dict(rootsoi=[fl], phs_neg=[sum(fl)], hydr_redist_negative=[True], atol_rootsoi=1e-10),
         fvn=[1], k=[[0.01] * 4], smp=[-5000.0], vegwp4=[-500.0], use_hydrstress=True)
    fl = [0.01 * (-500.0 - (-1000.0) - z * 1000.0) * 0.6 for z in zs]
    case("hydstress_noveg_patch", "test/test_soil_water_plant_sink.jl:391-434", "hydstress",
         [ISTSOIL], [1], [ISTSOIL], [2], [[0.0] * 4, [0.0] * 4], [0.002, 0.003], [0.002], [0.6, 0.4],
         [True, True], dict(rootsoi=[fl], atol_rootsoi=1e-10), fvn=[1, 0], k=[[0.01] * 4, [0.01] * 4],
         smp=[-500.0], vegwp4=[-1000.0, -200.0], use_hydrstress=True)
    rw = [[0.25] * 4, [0.4, 0.3, 0.2, 0.1], [0.1, 0.2, 0.3, 0.4]]
    tc = [0.001, 0.002, 0.003]
    case("wrapper_default_types", "test/test_soil_water_plant_sink.jl:436-482", "wrapper", [ROAD, ISTCROP, ISTSOIL],
         [1, 2, 3], [ISTURB_MD, ISTCROP, ISTSOIL], [1, 1, 1], rw, tc, tc, [1.0, 1.0, 1.0], [True] * 3,
         dict(rootr_col=rw, rootsoi=[[x * tc[c] for x in rw[c]] for c in range(3)], atol_rootr=1e-12,
              atol_rootsoi=1e-14))
    case("wrapper_hydstress_dispatch", "test/test_soil_water_plant_sink.jl:520-572", "wrapper", [ROAD, ISTSOIL],
         [1, 2], [ISTURB_MD, ISTSOIL], [1, 1], [[0.25] * 4, [0.0] * 4], [0.001, 0.002], [0.001, 0.002],
         [1.0, 1.0], [True, True],
         dict(rootr_col=[[0.25] * 4, None], rootsoi=[None, [0.005 * (-300.0 - (-600.0) - z * 1000.0) for z in zs]],
              atol_rootr=1e-12, atol_rootsoi=1e-10),
         fvn=[1, 1], k=[[0.005] * 4, [0.005] * 4], smp=[-300.0, -300.0], vegwp4=[-800.0, -600.0],
         use_hydrstress=True)
    case("wrapper_mask", "test/test_soil_water_plant_sink.jl:612-652", "wrapper", [ISTSOIL, ISTSOIL], [1, 1],
         [ISTSOIL], [1, 1], [[0.4, 0.3, 0.2, 0.1], [0.1, 0.2, 0.3, 0.4]], [0.001, 0.002], [0.001, 0.002],
         [1.0, 1.0], [True, True], dict(rootr_col=[[0.4, 0.3, 0.2, 0.1], [0.0] * 4], atol_rootr=1e-12),
         mask=[True, False])
    return dict(nlevsno=5, nlevgrnd=10, nlevsoi=nsoi, nlevurb=5, nlevmaxurbgrnd=10, z_soil=zs, cases=out)


def main():
    cases = {}
    cases["band_penta5"] = band_case(penta(5), np.arange(1.0, 6.0), 1, 5, 2, 2, 1e-10,
                                     "test/test_band_diagonal.jl:52-89")
    cases["band_penta6"] = band_case(penta(6), np.arange(1.0, 7.0), 1, 6, 2, 2, 1e-10,
                                     "test/test_band_diagonal.jl:114-139")
    cases["band_tri4"] = band_case(tri(4, 4.0, -1.0), np.array([1.0, 2.0, 3.0, 4.0]), 1, 4, 1, 1, 1e-12,
                                   "test/test_band_diagonal.jl:6-49")
    cases["band_partial"] = band_case(tri(4, 5.0, -1.0), np.array([2.0, 4.0, 6.0, 8.0]), 3, 8, 1, 1, 1e-12,
                                      "test/test_band_diagonal.jl:174-202")
    cases["tridiag_3x3"] = dict(a=[0.0, -1.0, -1.0], b=[2.0, 2.0, 2.0], c=[-1.0, -1.0, 0.0],
                                r=[1.0, 0.0, 1.0], jtop=1, u=[1.0, 1.0, 1.0], atol=1e-12,
                                source="test/test_tridiagonal.jl:6-16")
    cases["tridiag_identity"] = dict(a=[0.0] * 5, b=[1.0] * 5, c=[0.0] * 5, r=[1.0, 2.0, 3.0, 4.0, 5.0],
                                     jtop=1, u=[1.0, 2.0, 3.0, 4.0, 5.0], atol=1e-14,
                                     source="test/test_tridiagonal.jl:18-28")
    cases["tridiag_partial"] = dict(a=[0.0, 0.0, 0.0, -1.0, -1.0], b=[1.0, 1.0, 2.0, 2.0, 2.0],
                                    c=[0.0, 0.0, -1.0, -1.0, 0.0], r=[0.0, 0.0, 1.0, 0.0, 1.0], jtop=3,
                                    u=[None, None, 1.0, 1.0, 1.0], atol=1e-12,
                                    source="test/test_tridiagonal.jl:30-45")
    coeff = 1.0e-6 * 3600.0 / (0.1 ** 2)
    cases["tridiag_residual"] = dict(a=[0.0] + [-coeff] * 9, b=[1.0 + 2.0 * coeff] * 10,
                                     c=[-coeff] * 9 + [0.0], r=[300.0 - 2.0 * j for j in range(1, 11)],
                                     jtop=1, atol=1e-10, source="test/test_tridiagonal.jl:47-68")
    cases["tridiag_col_3x3"] = dict(a=[0.0, -1.0, -1.0], b=[2.0, 2.0, 2.0], c=[-1.0, -1.0, 0.0],
                                    r=[1.0, 0.0, 1.0], jtop=1, lbj=1, ubj=3, u=[1.0, 1.0, 1.0], atol=1e-12,
                                    source="test/test_soil_water_movement.jl:95-118")
    cases["tridiag_col_jtop"] = dict(a=[0.0, 0.0, -1.0, -1.0], b=[1.0, 2.0, 2.0, 2.0], c=[0.0, -1.0, -1.0, 0.0],
                                     r=[0.0, 1.0, 0.0, 1.0], jtop=2, lbj=1, ubj=4, atol=1e-12,
                                     source="test/test_soil_water_movement.jl:120-134")
    # test/test_enzyme_smoke.jl:194-248 — fixed 9-level system, jtop=3, objective sum(w .* u)
    cases["tridiag_adjoint9"] = dict(
        n=9, jtop=3,
        a=[0.0, 0.0, 0.0, 0.31, -0.22, 0.44, -0.17, 0.28, -0.39],
        b=[3.4, 3.1, 3.9, 3.2, 3.7, 3.3, 3.5, 3.8, 3.6],
        c=[-0.25, 0.33, -0.41, 0.19, -0.29, 0.37, -0.21, 0.24, 0.0],
        r=[0.7, -1.2, 0.4, 1.9, -0.6, 0.3, -1.1, 0.8, 0.2],
        w=[0.9, -0.4, 1.3, 0.2, -1.7, 0.6, 0.5, -0.8, 1.1],
        tol_vs_exact=1e-10, tol_vs_fd=1e-6, source="test/test_enzyme_smoke.jl:194-248")
    cases["ice_impedance"] = dict(values=[[0.0, 6.0, 1.0], [1.0, 6.0, 1.0e-6], [0.5, 6.0, 10.0 ** -3.0],
                                          [0.5, 4.0, 10.0 ** -2.0]],
                                  source="test/test_soil_water_movement.jl:76-88")
    cases["swm_config_defaults"] = dict(dtmin=60.0, verySmall=1.0e-8, xTolerUpper=1.0e-1, xTolerLower=1.0e-2,
                                        expensive=42, inexpensive=1, flux_calculation=1, e_ice=6.0,
                                        source="test/test_soil_water_movement.jl:18-31")
    cases["rhs_moisture_form"] = dict(nlayers=3, vert_trans_sink=[0.1, 0.2, 0.05], vwc_liq=[0.3, 0.35, 0.25],
                                      qin=[1.0, 0.8, 0.6], qout=[0.8, 0.6, 0.3], dt_dz=[0.01, 0.012, 0.008],
                                      expect="rmx[j] = -(qin[j] - qout[j] - vert_trans_sink[j]) * dt_dz[j]",
                                      atol=1e-15, source="test/test_soil_water_movement.jl:151-170")
    cases["lhs_moisture_form"] = dict(nlayers=4, dt_dz=[0.01, 0.012, 0.008, 0.01], dqidw0=[0.0, 0.5, 0.4, 0.3],
                                      dqidw1=[0.1, 0.2, 0.15, 0.12], dqodw1=[0.3, 0.25, 0.2, 0.18],
                                      dqodw2=[0.4, 0.35, 0.28, 0.0],
                                      expect="amx[1] = 0, amx[j] = dqidw0[j] dt_dz[j]; "
                                             "bmx[j] = -1 - (-dqidw1[j] + dqodw1[j]) dt_dz[j]; "
                                             "cmx[j] = -dqodw2[j] dt_dz[j], cmx[nlayers] = 0",
                                      rtol=2.0 ** -26, source="test/test_soil_water_movement.jl:172-202")
    # (method, lower BC, use_bedrock, raises) of init_soilwater_movement's checks
    cases["init_soilwater_movement"] = dict(
        default=dict(method=0, upper=1, lower=4),
        checks=[[0, 1, False, True], [1, 1, False, False], [0, 4, True, True], [1, 2, True, False],
                [0, 4, False, False]],
        source="test/test_soil_water_movement.jl:207-256 (ZD09 = 0, MOISTURE_FORM = 1; BC_FLUX = 1, "
               "BC_ZERO_FLUX = 2, BC_AQUIFER = 4)")
    # test/test_soil_water_movement.jl:272-336
    cases["moisture_form_conservation"] = dict(nc=12, nlev=10, nlevsno=5, dtime=1800.0, dz=0.05,
                                               watsat=0.45, hksat=0.02, bsw=5.0, sucsat=100.0,
                                               qflx_infl=1.0e-5, liq_profile="(0.30+0.01*j)*watsat*dz*1000",
                                               rtol=1e-10, source="test/test_soil_water_movement.jl:272-336")
    # test/test_soil_temperature.jl:1-226 (setup_soil_column!)
    cases["soiltemp_fixture"] = dict(nlevsno=5, nlevgrnd=10, nlevurb=5, nlevmaxurbgrnd=10, nlevsoi=8, nc=4,
                                     t=280.0, liq=5.0, watsat=0.45, bsw=5.0, sucsat=100.0, tkmg=2.0,
                                     tkdry=0.25, csol=2.0e6, emg=0.97, dlrad=50.0, cgrnd=5.0, sh=10.0,
                                     sabg=100.0, sabg_soil=100.0, sabg_snow=0.0, sabg_lyr_top=100.0,
                                     source="test/test_soil_temperature.jl:41-226")
    cases["phase_change_melt"] = dict(j=2, ice=5.0, liq=2.0, dT=2.0, dtime=1800.0, dhsdT=-5.0,
                                      source="test/test_soil_temperature.jl:566-599")
    cases["phase_change_mass"] = dict(layers=[[4.0, 1.0, 3.0], [0.0, 6.0, -3.0], [7.0, 0.0, -1.0],
                                              [0.0, 0.0, -1.0], [0.5, 0.05, 0.5]],
                                      atol=1e-12, rtol=1e-12, dtime=1800.0, dhsdT=-5.0,
                                      source="test/test_soil_temperature.jl:613-666")
    cases["phase_change_h2osfc_depth"] = dict(snl=-1, ice0=40.0, snow_depth=0.10, frac_sno_eff=1.0,
                                              frac_h2osfc=0.5, h2osfc=20.0, dT=-1.0, fact0=1.0, c_h2osfc=0.0,
                                              dtime=1800.0, dhsdT=-1000.0,
                                              source="test/test_soil_temperature.jl:498-532")
    cases["rootsink"] = rootsink_cases()
    cases["soil_fluxes"] = soil_fluxes_cases()
    cases["surface_hydrology"] = surface_hydrology_cases()
    cases["snow_layers"] = snow_layer_cases()
    cases["balance_check_columns"] = balance_check_cases()
    cases["lake_temperature"] = dict(
        varpar=dict(nlevsno=5, nlevsoi=10, nlevgrnd=15, nlevlak=10, nlevurb=5, nlevmaxurbgrnd=15),
        source="test/test_lake_temperature.jl:9-17 (setup_lake_params!), :24-170 (create_test_data)",
        cases=[dict(name="runs_finite", source="test/test_lake_temperature.jl:285-311", nc=2, zero_flux=False,
                    checks=["t_lake_finite", "icethick_nonnegative", "errsoi_finite"]),
               dict(name="energy_conservation_zero_input", source="test/test_lake_temperature.jl:314-337", nc=1,
                    zero_flux=True, checks=["errsoi_below_0.2"])])
    with open(os.path.join(HERE, "reference_cases.json"), "w") as fh:
        json.dump(cases, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
