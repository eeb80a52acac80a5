"""Pins the CPU oracle against CLM.jl's own known-answer tests (tests/golden)."""
import numpy as np
import pytest

from clmgb import abi, synth
from fixtures import golden, moisture_fixture, soil_column_fixture, TFRZ
from oracle import oracle as orc

G = golden()


def _band_arrays(case):
    nlevs, kl, ku = case["nlevs"], case["kl"], case["ku"]
    nband = kl + ku + 1
    bm = np.zeros((nlevs, nband, 1))
    bm[:, :, 0] = np.array(case["bmatrix"]).T
    rv = np.array(case["rvector"]).reshape(nlevs, 1)
    tv = np.zeros((nlevs, 1))
    one = np.ones(1, dtype=np.int64)
    jtop = one * case["jtop"]
    jbot = one * case["jbot"]
    return bm, rv, tv, jtop, jbot


@pytest.mark.parametrize("name", ["band_penta5", "band_penta6", "band_tri4", "band_partial"])
def test_band_known_answers(name):
    case = G[name]
    bm, rv, tv, jtop, jbot = _band_arrays(case)
    mask = np.ones(1, dtype=np.uint8)
    # jtop/jbot are 1-based rows here: nlevsno_off = -1 makes row = jtop
    orc.batched_band_solve(tv, bm, rv, jtop, jbot, mask, case["kl"], case["ku"], -1)
    x = tv[case["jtop"] - 1:case["jbot"], 0]
    np.testing.assert_allclose(x, case["x_exact"], atol=case["atol"], rtol=0)
    assert np.all(tv[:case["jtop"] - 1, 0] == 0.0)
    assert np.all(tv[case["jbot"]:, 0] == 0.0)


@pytest.mark.parametrize("name", ["tridiag_3x3", "tridiag_identity", "tridiag_partial"])
def test_tridiagonal_known_answers(name):
    c = G[name]
    n = len(c["b"])
    u = orc.tridiagonal_solve(c["a"], c["b"], c["c"], c["r"], c["jtop"], n)
    for got, want in zip(u, c["u"]):
        if want is not None:
            assert abs(got - want) <= c["atol"]
    # batched kernel form, same system in every column
    ncols = 3
    arr = {k: np.repeat(np.array(c[k], dtype=np.float64)[:, None], ncols, 1) for k in "abcr"}
    um = np.zeros((n, ncols))
    orc.tridiagonal_multi(um, arr["a"], arr["b"], arr["c"], arr["r"],
                          np.full(ncols, c["jtop"], dtype=np.int64), np.ones(ncols, dtype=np.uint8))
    for col in range(ncols):
        for got, want in zip(um[:, col], c["u"]):
            if want is not None:
                assert abs(got - want) <= c["atol"]


def test_tridiagonal_residual():
    c = G["tridiag_residual"]
    a, b, cc, r = (np.array(c[k]) for k in ("a", "b", "c", "r"))
    u = orc.tridiagonal_solve(a, b, cc, r, 1, 10)
    res = b * u + a * np.r_[0.0, u[:-1]] + cc * np.r_[u[1:], 0.0] - r
    assert np.max(np.abs(res)) < c["atol"]


def test_tridiagonal_col_known_answers():
    c = G["tridiag_col_3x3"]
    u = orc.tridiagonal_col(c["a"], c["b"], c["c"], c["r"], 1, 1, 3)
    np.testing.assert_allclose(u, c["u"], atol=c["atol"])
    c = G["tridiag_col_jtop"]
    u = orc.tridiagonal_col(c["a"], c["b"], c["c"], c["r"], 2, 1, 4)
    assert abs(2 * u[1] - u[2] - 1.0) < c["atol"]
    assert abs(-u[1] + 2 * u[2] - u[3]) < c["atol"]
    assert abs(-u[2] + 2 * u[3] - 1.0) < c["atol"]


@pytest.mark.parametrize("nlevs,jt", [(20, 1), (5, 1), (25, 1), (20, 4), (21, 1)])
def test_tridiagonal_multi_vs_dense(nlevs, jt):
    # property of test_tridiagonal.jl:123-144 (its MersenneTwister values are Julia-only)
    rng = np.random.default_rng(nlevs * 10 + jt)
    ncols = 48
    a = -0.5 * np.ones((nlevs, ncols))
    c = -0.5 * np.ones((nlevs, ncols))
    b = 2 + 0.5 * rng.random((nlevs, ncols))
    r = rng.random((nlevs, ncols))
    a[0] = 0.0
    c[-1] = 0.0
    u = np.zeros((nlevs, ncols))
    orc.tridiagonal_multi(u, a, b, c, r, np.full(ncols, jt, dtype=np.int64), np.ones(ncols, dtype=np.uint8))
    for col in range(ncols):
        n = nlevs - jt + 1
        M = np.zeros((n, n))
        for i in range(n):
            M[i, i] = b[jt - 1 + i, col]
            if i > 0:
                M[i, i - 1] = a[jt - 1 + i, col]
            if i < n - 1:
                M[i, i + 1] = c[jt - 1 + i, col]
        np.testing.assert_allclose(u[jt - 1:, col], np.linalg.solve(M, r[jt - 1:, col]), atol=1e-10)


def test_band_dense_matches_numpy_with_pivoting():
    from fixtures import random_band_system
    rng = np.random.default_rng(5)
    nc, nlev = 64, 38
    bm, rv = random_band_system(nc, nlev, 2, 2, rng, pivot_frac=0.3)
    tv = np.zeros((nlev, nc))
    jtop = rng.integers(1, 13, nc).astype(np.int64)
    jbot = np.full(nc, nlev, dtype=np.int64)
    orc.batched_band_solve(tv, bm, rv, jtop, jbot, np.ones(nc, dtype=np.uint8), 2, 2, -1)
    for c in range(nc):
        n = nlev - jtop[c] + 1
        A = np.zeros((n, n))
        for i in range(n):
            for j in range(max(0, i - 2), min(n, i + 3)):
                A[i, j] = bm[jtop[c] - 1 + i, (i - j) + 2, c]
        x = np.linalg.solve(A, rv[jtop[c] - 1:, c])
        np.testing.assert_allclose(tv[jtop[c] - 1:, c], x, rtol=1e-9, atol=1e-9)


def test_ice_impedance():
    for icefrac, e_ice, want in G["ice_impedance"]["values"]:
        assert orc.ice_impedance(icefrac, e_ice) == pytest.approx(want, rel=1e-14)


def test_config_defaults():
    g = G["swm_config_defaults"]
    cfg = abi.SwmConfig.clm5_default()
    assert cfg.dtmin == g["dtmin"] and cfg.verySmall == g["verySmall"]
    assert cfg.xTolerUpper == g["xTolerUpper"] and cfg.xTolerLower == g["xTolerLower"]
    assert cfg.e_ice == g["e_ice"] and cfg.flux_calculation == g["inexpensive"]
    assert cfg.soilwater_movement_method == abi.MOISTURE_FORM
    assert cfg.lower_boundary_condition == abi.BC_ZERO_FLUX


def test_moisture_form_conserves_mass():
    g = G["moisture_form_conservation"]
    st = moisture_fixture()
    joff = st.vp.nlevsno
    liq0 = st["h2osoi_liq"][joff:joff + g["nlev"]].sum(0).copy()
    status, qin, qout = orc.soil_water(st, g["dtime"], capture=True)
    assert np.all(status == 0)
    dliq = st["h2osoi_liq"][joff:joff + g["nlev"]].sum(0) - liq0
    np.testing.assert_allclose(dliq, g["qflx_infl"] * g["dtime"], rtol=g["rtol"])
    for j in range(1, g["nlev"]):
        assert np.array_equal(qin[j], qout[j - 1])
    assert np.all(qin[0] == g["qflx_infl"])


def test_moisture_form_rejects_unsupported_config():
    st = moisture_fixture()
    cfg = abi.SwmConfig.clm5_default()
    cfg.upper_boundary_condition = abi.BC_HEAD
    assert orc.soil_water(st, 1800.0, cfg) == abi.CLMGB_ERR_CONFIG
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_AQUIFER
    assert orc.soil_water(st, 1800.0, cfg) == abi.CLMGB_ERR_CONFIG


def test_soil_temperature_fixture_properties():
    st = soil_column_fixture()
    status = orc.soil_temperature(st, 1800.0)
    assert np.all(status == 0)
    joff = st.vp.nlevsno
    T = st["t_soisno"]
    assert np.all(np.isfinite(T[joff:]))
    assert np.all(st["fact"][joff:] > 0.0)
    # column 1 (the reference fixture): no ice above freezing -> no phase change
    assert np.all(st["imelt"][joff:, 0] == 0)
    assert st["xmf"][0] == 0.0 and st["qflx_snomelt"][0] == 0.0
    # dG/dT < 0 is visible through eflx_gnet derivative per patch
    assert np.all(st["dgnetdT"] < 0.0)
    # snow column: finite snow temperatures and conductivity
    assert np.all(np.isfinite(T[joff - 2:joff, 1]))
    assert np.all(st["thk"][joff - 2:joff, 1] > 0.0)


def test_phase_change_melt():
    g = G["phase_change_melt"]
    st = soil_column_fixture(1)
    joff = st.vp.nlevsno
    jj = g["j"] + joff
    st["h2osoi_ice"][jj - 1, 0] = g["ice"]
    st["h2osoi_liq"][jj - 1, 0] = g["liq"]
    st["t_soisno"][jj - 1, 0] = TFRZ + g["dT"]
    for j in range(1, st.vp.nlevgrnd + 1):
        st["fact"][j + joff - 1, 0] = g["dtime"] / (2.0e6 * st["dz"][j + joff - 1, 0])
    orc.phase_change_beta(st, g["dtime"], np.full(1, g["dhsdT"]))
    assert st["imelt"][jj - 1, 0] == 1
    assert abs(st["t_soisno"][jj - 1, 0] - TFRZ) <= 2.0
    assert st["h2osoi_ice"][jj - 1, 0] < g["ice"]


def test_phase_change_no_change_above_freezing():
    st = soil_column_fixture(1)
    joff = st.vp.nlevsno
    st["fact"][joff:, 0] = 1.0
    orc.phase_change_beta(st, 1800.0, np.full(1, -5.0))
    assert st["xmf"][0] == 0.0 and st["qflx_snomelt"][0] == 0.0 and st["qflx_snofrz"][0] == 0.0
    assert np.all(st["imelt"][joff:, 0] == 0)


def test_phase_change_conserves_mass():
    g = G["phase_change_mass"]
    st = soil_column_fixture(1)
    joff = st.vp.nlevsno
    for j in range(1, st.vp.nlevgrnd + 1):
        st["fact"][j + joff - 1, 0] = g["dtime"] / (2.0e6 * st["dz"][j + joff - 1, 0])
    for j, (ice, liq, dT) in enumerate(g["layers"], start=1):
        st["h2osoi_ice"][j + joff - 1, 0] = ice
        st["h2osoi_liq"][j + joff - 1, 0] = liq
        st["t_soisno"][j + joff - 1, 0] = TFRZ + dT
    w0 = st["h2osoi_ice"][joff:, 0] + st["h2osoi_liq"][joff:, 0]
    orc.phase_change_beta(st, g["dtime"], np.full(1, g["dhsdT"]))
    w1 = st["h2osoi_ice"][joff:, 0] + st["h2osoi_liq"][joff:, 0]
    np.testing.assert_allclose(w1, w0, atol=g["atol"], rtol=g["rtol"])
    assert np.all(st["h2osoi_liq"][joff:, 0] >= 0) and np.all(st["h2osoi_ice"][joff:, 0] >= 0)
    assert st["imelt"][joff, 0] == 1   # layer 1 melts


def test_phase_change_h2osfc_no_water():
    st = soil_column_fixture(1)
    orc.phase_change_h2osfc(st, 1800.0, np.full(1, -5.0))
    assert st["xmf_h2osfc"][0] == 0.0 and st["qflx_h2osfc_to_ice"][0] == 0.0


def test_phase_change_h2osfc_snow_depth_closed_form():
    g = G["phase_change_h2osfc_depth"]
    st = soil_column_fixture(1)
    joff = st.vp.nlevsno
    st["col_snl"][0] = g["snl"]
    st["h2osoi_ice"][joff - 1, 0] = g["ice0"]
    st["h2osoi_liq"][joff - 1, 0] = 0.0
    st["snow_depth"][0] = g["snow_depth"]
    st["frac_sno_eff"][0] = g["frac_sno_eff"]
    st["frac_h2osfc"][0] = g["frac_h2osfc"]
    st["h2osfc"][0] = g["h2osfc"]
    st["t_h2osfc"][0] = TFRZ + g["dT"]
    st["t_soisno"][joff - 1, 0] = TFRZ
    st["fact"][joff - 1, 0] = g["fact0"]
    st["c_h2osfc"][0] = g["c_h2osfc"]
    dt, dh = g["dtime"], g["dhsdT"]
    xm = g["frac_h2osfc"] * (dh * 1.0 - 1.0 * g["c_h2osfc"] / dt) * dt / 3.337e5
    rho = min(800.0, g["ice0"] / (g["frac_sno_eff"] * g["snow_depth"]))
    expect = (g["ice0"] - xm) / (rho * g["frac_sno_eff"])
    orc.phase_change_h2osfc(st, dt, np.full(1, dh))
    assert st["snow_depth"][0] == pytest.approx(expect, rel=1e-12)


def test_soil_properties_numpy_matches_c():
    rng = np.random.default_rng(3)
    n = 500
    sand = rng.uniform(5, 90, n)
    clay = rng.uniform(5, 60, n)
    om = rng.uniform(0, 1.0, n)
    zs = rng.uniform(0, 8, n)
    py = synth.init_soil_properties(sand, clay, om, zs)
    cc = orc.init_soil_properties(sand, clay, om, zs)
    for k in py:
        np.testing.assert_allclose(py[k], cc[k], rtol=1e-14, err_msg=k)


def test_workload_water_balance_closes():
    # multi-step oracle run: column water change == infiltration - transpiration
    wl = synth.make_workload(1, nc=256, nsteps=6)
    st = wl.state
    w0 = st["h2osoi_liq"].sum(0) + st["h2osoi_ice"].sum(0) + st["h2osno_no_layers"] + st["h2osfc"]
    G_, I_ = wl.forcing_block(range(6))
    status = orc.run_steps(st, wl.dtime, G_, I_)
    assert np.all(status == 0)
    w1 = st["h2osoi_liq"].sum(0) + st["h2osoi_ice"].sum(0) + st["h2osno_no_layers"] + st["h2osfc"]
    expect = I_.sum(0) * wl.dtime - st["qflx_rootsoi"].sum(0) * wl.dtime * 6
    np.testing.assert_allclose(w1 - w0, expect, atol=1e-9)


def test_oracle_root_sink_known_answers():
    """compute_effec_rootfrac_and_vert_tran_sink! known answers of
    test_soil_water_plant_sink.jl, through the oracle's wrapper restatement."""
    import rootsink_cases as RC
    from oracle import oracle as O
    g = RC.load()
    for case in g["cases"]:
        rs = RC.build(g, case)
        assert O.rootsink(rs, case["use_hydrstress"]) == 0
        RC.check(g, case, rs)


def test_oracle_root_sink_filter_error():
    """A pervious road on a natural-vegetation landunit sits in two of the wrapper's
    filters: the counts disagree, where the reference raises its error."""
    import rootsink_cases as RC
    from oracle import oracle as O
    g = RC.load()
    case = dict(g["cases"][0])
    case["col_itype"] = [75]
    rs = RC.build(g, case)
    assert O.rootsink(rs, False) == 1


def test_rhs_moisture_form_known_answer():
    """compute_RHS_moisture_form! (test_soil_water_movement.jl:151-170)."""
    g = G["rhs_moisture_form"]
    rmx = orc.compute_rhs_moisture_form(g["vert_trans_sink"], g["vwc_liq"], g["qin"], g["qout"], g["dt_dz"])
    for j in range(g["nlayers"]):
        fluxnet = g["qin"][j] - g["qout"][j] - g["vert_trans_sink"][j]
        assert abs(rmx[j] - (-fluxnet * g["dt_dz"][j])) <= g["atol"]


def test_lhs_moisture_form_known_answer():
    """compute_LHS_moisture_form! (test_soil_water_movement.jl:172-202), the same
    expressions the solve forms for its matrix (soil_water_movement.jl:1380-1397)."""
    g = G["lhs_moisture_form"]
    n, dt, d0, d1, o1, o2 = (g[k] for k in ("nlayers", "dt_dz", "dqidw0", "dqidw1", "dqodw1", "dqodw2"))
    amx, bmx, cmx = orc.compute_lhs_moisture_form(dt, d0, d1, o1, o2)
    rt = g["rtol"]
    assert amx[0] == 0.0 and cmx[n - 1] == 0.0
    for j in range(n):
        assert bmx[j] == pytest.approx(-1.0 - (-d1[j] + o1[j]) * dt[j], rel=rt)
        if j > 0:
            assert amx[j] == pytest.approx(d0[j] * dt[j], rel=rt)
        if j < n - 1:
            assert cmx[j] == pytest.approx(-o2[j] * dt[j], rel=rt)


def test_init_soilwater_movement_checks():
    """init_soilwater_movement's defaults and consistency checks, the use_bedrock one
    included (test_soil_water_movement.jl:207-256)."""
    from clmgb import api
    g = G["init_soilwater_movement"]
    cfg = api.init_soilwater_movement()
    d = g["default"]
    assert (cfg.soilwater_movement_method, cfg.upper_boundary_condition, cfg.lower_boundary_condition) == \
        (d["method"], d["upper"], d["lower"])
    assert cfg.dtmin == 60.0 and cfg.e_ice == 6.0 and cfg.flux_calculation == 1
    for method, lower, bedrock, raises in g["checks"]:
        if raises:
            with pytest.raises(api.CLMGBError) as e:
                api.init_soilwater_movement(use_bedrock=bedrock, soilwater_movement_method=method,
                                            lower_boundary_condition=lower)
            assert e.value.code == abi.CLMGB_ERR_CONFIG
        else:
            c = api.init_soilwater_movement(use_bedrock=bedrock, soilwater_movement_method=method,
                                            lower_boundary_condition=lower)
            assert c.lower_boundary_condition == lower
