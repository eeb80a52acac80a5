"""GPU parity: the sm_103a kernels through the C ABI against the CPU oracle.

Tolerance (stated by the workload definition): 1e-10 relative in temperatures and
water/ice contents (atol 1e-12), level indices and phase flags (imelt) exact, and no
column outside it.  The kernels and the oracle share one binary64 log/exp/pow, so
most tests also require identical bits; the band and tridiagonal solves involve no
transcendental and must match bit for bit too.
"""
import numpy as np
import pytest

from clmgb import abi, api, synth
from fixtures import golden, moisture_fixture, random_band_system, soil_column_fixture, TFRZ
from oracle import oracle as orc
from parity import bit_mismatches, compare

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

G = golden()


@pytest.fixture(scope="module")
def handle_factory():
    assert torch.cuda.is_available()
    hs = {}

    def get(vp):
        key = (vp.nlevsno, vp.nlevgrnd, vp.nlevsoi, vp.nlevurb, vp.nlevmaxurbgrnd)
        if key not in hs:
            hs[key] = api.Handle(vp)
        return hs[key]
    yield get
    for h in hs.values():
        h.close()


# the soil_temperature! outputs compared bit for bit
FLOAT_OUT_ST = ["t_soisno", "h2osoi_liq", "h2osoi_ice", "t_h2osfc", "t_grnd", "fact", "thk", "xmf", "imelt",
                "eflx_fgr12", "eflx_fgr", "snow_depth", "qflx_snomelt", "qflx_snofrz"]


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# ---------------------------------------------------------------- solvers
@pytest.mark.parametrize("kl", [1, 2])
def test_band_solve_bit_exact_vs_oracle(handle_factory, kl):
    h = handle_factory(synth.clm5_varpar())
    rng = np.random.default_rng(11 + kl)
    nc, nlev = 4099, 38
    bm, rv = random_band_system(nc, nlev, kl, kl, rng, pivot_frac=0.25)
    jtop = rng.integers(1, 14, nc).astype(np.int64)
    jbot = np.full(nc, nlev, dtype=np.int64)
    jbot[::7] = rng.integers(20, nlev + 1, len(jbot[::7]))
    mask = (rng.random(nc) < 0.95).astype(np.uint8)
    tv_ref = np.full((nlev, nc), -7.0)
    orc.batched_band_solve(tv_ref, bm, rv, jtop, jbot, mask, kl, kl, -1)
    tv = _dev(np.full((nlev, nc), -7.0))
    api.batched_band_solve(h, tv, _dev(bm), _dev(rv), _dev(jtop), _dev(jbot), _dev(mask), kl, kl, -1)
    got = tv.cpu().numpy()
    assert np.array_equal(got, tv_ref), "max |diff| %g" % np.nanmax(np.abs(got - tv_ref))


@pytest.mark.parametrize("kl", [1, 2])
def test_band_solve_short_systems_and_pivoting_everywhere(handle_factory, kl):
    """Systems of 1 to 8 rows (the elimination window reaching past the last row) and
    systems whose every diagonal is weak, so that nearly every step exchanges rows:
    the bits of the oracle's dense elimination."""
    h = handle_factory(synth.clm5_varpar())
    rng = np.random.default_rng(31 + kl)
    nc, nlev = 4096, 38
    bm, rv = random_band_system(nc, nlev, kl, kl, rng, pivot_frac=0.0)
    weak = np.arange(nc) % 2 == 1                            # odd columns: every diagonal weak
    bm[:, kl, weak] *= 1e-3
    jtop = rng.integers(1, nlev - 8, nc).astype(np.int64)
    jbot = jtop + (np.arange(nc) // 2) % 8                   # 1..8 rows
    jbot[::64] = nlev                                         # and some full-length ones
    mask = np.ones(nc, dtype=np.uint8)
    tv_ref = np.full((nlev, nc), -7.0)
    orc.batched_band_solve(tv_ref, bm, rv, jtop, jbot, mask, kl, kl, -1)
    tv = _dev(np.full((nlev, nc), -7.0))
    api.batched_band_solve(h, tv, _dev(bm), _dev(rv), _dev(jtop), _dev(jbot), _dev(mask), kl, kl, -1)
    got = tv.cpu().numpy()
    assert np.array_equal(got.view(np.uint64), tv_ref.view(np.uint64))


@pytest.mark.parametrize("name", ["band_penta5", "band_penta6", "band_tri4", "band_partial"])
def test_band_solve_known_answers(handle_factory, name):
    h = handle_factory(synth.clm5_varpar())
    case = G[name]
    nlevs, kl = case["nlevs"], case["kl"]
    bm = np.array(case["bmatrix"]).T.reshape(nlevs, 2 * kl + 1, 1).copy()
    rv = np.array(case["rvector"]).reshape(nlevs, 1)
    tv = _dev(np.zeros((nlevs, 1)))
    one = np.ones(1, dtype=np.int64)
    api.batched_band_solve(h, tv, _dev(bm), _dev(rv), _dev(one * case["jtop"]), _dev(one * case["jbot"]),
                           _dev(np.ones(1, dtype=np.uint8)), kl, kl, -1)
    x = tv.cpu().numpy()[case["jtop"] - 1:case["jbot"], 0]
    np.testing.assert_allclose(x, case["x_exact"], atol=case["atol"], rtol=0)


def test_tridiagonal_bit_exact_vs_oracle(handle_factory):
    h = handle_factory(synth.clm5_varpar())
    rng = np.random.default_rng(7)
    ncols, nlevs = 5000, 25
    a = rng.uniform(-1, 0, (nlevs, ncols))
    c = rng.uniform(-1, 0, (nlevs, ncols))
    b = 2.2 + rng.random((nlevs, ncols))
    b[3, ::13] = 0.0     # exercises the 1e-30 guard
    r = rng.uniform(-5, 5, (nlevs, ncols))
    jtop = rng.integers(1, 5, ncols).astype(np.int64)
    mask = np.ones(ncols, dtype=np.uint8)
    u_ref = np.zeros((nlevs, ncols))
    orc.tridiagonal_multi(u_ref, a, b, c, r, jtop, mask)
    u = _dev(np.zeros((nlevs, ncols)))
    api.tridiagonal_multi(h, u, *[_dev(x) for x in (a, b, c, r, jtop, mask)])
    assert np.array_equal(u.cpu().numpy(), u_ref)


# ---------------------------------------------------------------- soil temperature
def _run_soiltemp_both(st, dtime, handle_factory, snow_method=abi.SNOW_JORDAN1991):
    ref = st.copy()
    orc.soil_temperature(ref, dtime, snow_method)
    d = st.to_device()
    h = handle_factory(st.vp)
    status = torch.zeros(st.nc, dtype=torch.int32, device="cuda")
    api.soil_temperature(h, d, dtime, snow_method, col_status=status)
    torch.cuda.synchronize()
    return d.to_host(), ref, status.cpu().numpy()


@pytest.mark.parametrize("snow_method", [abi.SNOW_JORDAN1991, abi.SNOW_STURM1997])
def test_soil_temperature_fixture(handle_factory, snow_method):
    st = soil_column_fixture()
    got, ref, status = _run_soiltemp_both(st, 1800.0, handle_factory, snow_method)
    assert np.all(status == 0)
    rep, bad = compare(got, ref)
    assert not bad, rep


@pytest.mark.parametrize("cfg_id,nc", [(0, 1024), (1, 8192), (2, 8192)])
def test_soil_temperature_workloads(handle_factory, cfg_id, nc):
    wl = synth.make_workload(cfg_id, nc=nc)
    got, ref, status = _run_soiltemp_both(wl.state, wl.dtime, handle_factory)
    assert np.all(status == 0)
    rep, bad = compare(got, ref)
    assert not bad, (len(bad), rep)
    assert not bit_mismatches(got, ref, FLOAT_OUT_ST)


def test_soil_temperature_edge_columns(handle_factory):
    """Full snowpack (snl = -12), one-layer snow, melting snow, ponded water above and
    below freezing, unresolved snow, masked columns and a zero-weight patch."""
    from fixtures import set_snowpack
    wl = synth.make_workload(1, nc=512, seed=99)
    st = wl.state
    a = st.arrays
    rng = np.random.default_rng(4)
    for c in range(0, 8):
        set_snowpack(st, c, 12, rng)
    for c in range(8, 16):
        set_snowpack(st, c, 1, rng)
    for c in range(100, 110):                 # snow at and above freezing -> melt
        set_snowpack(st, c, 3, rng, t_range=(272.5, 274.5))
    a["mask_nolakec"][16:24] = 0
    a["frac_h2osfc"][24:48] = 0.25
    a["h2osfc"][24:48] = np.linspace(0.0, 30.0, 24)
    a["t_h2osfc"][24:48] = TFRZ - np.linspace(-0.5, 3.0, 24)
    for c in range(48, 64):
        set_snowpack(st, c, 0, rng)
    a["h2osno_no_layers"][48:64] = 3.0
    a["frac_sno_eff"][48:64] = 0.4
    a["snow_depth"][48:64] = 0.02
    a["patch_wtcol"][96:100] = 0.0
    synth.apply_forcing_host(st, *wl.forcing(0))
    got, ref, status = _run_soiltemp_both(st, wl.dtime, handle_factory)
    assert np.all(status[np.r_[0:16, 24:512]] == 0)
    rep, bad = compare(got, ref)
    assert not bad, (sorted(bad), rep)
    # masked columns are untouched
    for k in ("t_soisno", "h2osoi_liq", "fact"):
        assert np.array_equal(got[k][:, 16:24], st[k][:, 16:24])


def test_soil_temperature_special_landunits(handle_factory):
    wl = synth.make_workload(1, nc=256, seed=5)
    st = wl.state
    nl = 3
    from clmgb.state import ColumnState
    arrs = dict(st.arrays)
    arrs["lun_itype"] = np.array([1, 6, 4], dtype=np.int64)    # soil, wetland, glacier
    arrs["lun_urbpoi"] = np.zeros(nl, dtype=np.uint8)
    lu = (np.arange(st.nc) % 3 + 1).astype(np.int64)
    arrs["col_landunit"] = lu
    arrs["patch_landunit"] = lu.copy()
    st3 = ColumnState(st.vp, st.nc, st.np, nl, arrs)
    got, ref, status = _run_soiltemp_both(st3, wl.dtime, handle_factory)
    assert np.all(status == 0)
    rep, bad = compare(got, ref)
    assert not bad, rep


def test_urban_column_reports_status(handle_factory):
    wl = synth.make_workload(0, nc=64)
    st = wl.state
    st["lun_urbpoi"][:] = 1
    d = st.to_device()
    h = handle_factory(st.vp)
    h.device_status(reset=True)
    status = torch.zeros(st.nc, dtype=torch.int32, device="cuda")
    api.soil_temperature(h, d, wl.dtime, col_status=status)
    assert np.all(status.cpu().numpy() == abi.COL_URBAN)
    assert h.device_status(reset=True) == abi.COL_URBAN
    # untouched state
    assert np.array_equal(d["t_soisno"].cpu().numpy(), st["t_soisno"])


# ---------------------------------------------------------------- phase change
def test_phase_change_golden_on_gpu(handle_factory):
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
    ref = st.copy()
    orc.phase_change_beta(ref, g["dtime"], np.full(1, g["dhsdT"]))
    d = st.to_device()
    h = handle_factory(st.vp)
    api.phase_change_beta(h, d, g["dtime"], _dev(np.full(1, g["dhsdT"])))
    got = d.to_host()
    w1 = got["h2osoi_ice"][joff:, 0] + got["h2osoi_liq"][joff:, 0]
    np.testing.assert_allclose(w1, w0, atol=g["atol"], rtol=g["rtol"])
    rep, bad = compare(got, ref)
    assert not bad, rep


def test_phase_change_h2osfc_golden_on_gpu(handle_factory):
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
    d = st.to_device()
    h = handle_factory(st.vp)
    api.phase_change_h2osfc(h, d, dt, _dev(np.full(1, dh)))
    assert float(d["snow_depth"][0]) == pytest.approx(expect, rel=1e-12)


# ---------------------------------------------------------------- soil water
def test_moisture_form_conserves_mass_gpu(handle_factory):
    g = G["moisture_form_conservation"]
    st = moisture_fixture()
    joff = st.vp.nlevsno
    ref = st.copy()
    orc.soil_water(ref, g["dtime"])
    d = st.to_device()
    h = handle_factory(st.vp)
    api.soil_water(h, d, g["dtime"])
    got = d.to_host()
    liq0 = st["h2osoi_liq"][joff:joff + g["nlev"]].sum(0)
    dliq = got["h2osoi_liq"][joff:joff + g["nlev"]].sum(0) - liq0
    np.testing.assert_allclose(dliq, g["qflx_infl"] * g["dtime"], rtol=g["rtol"])
    rep, bad = compare(got, ref, fields=["h2osoi_liq", "smp_l", "hk_l", "qcharge", "num_substeps"])
    assert not bad, rep


@pytest.mark.parametrize("schedule", ["queue", "queue_reserved", "waves"])
@pytest.mark.parametrize("lower_bc", [abi.BC_ZERO_FLUX, abi.BC_FLUX, abi.BC_WATERTABLE])
@pytest.mark.parametrize("cfg_id", [0, 2])
def test_soil_water_workloads(cfg_id, lower_bc, schedule):
    wl = synth.make_workload(cfg_id, nc=4096)
    st = wl.state
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = lower_bc
    orc.soil_water_fractions(st)
    st["zwt"][:] = np.linspace(0.5, 9.0, st.nc)
    st["num_substeps"][:] = np.arange(st.nc) % 9     # a previous-call history for the queue order
    st["mask_hydrology"][::11] = 0
    ref = st.copy()
    orc.soil_water(ref, wl.dtime, cfg)
    d = st.to_device()
    h = api.Handle(st.vp)
    if schedule != "queue":
        h.reserve(st.nc)
    if schedule == "waves":
        h.set_option(abi.OPT_STEP_SCHEDULE, abi.SCHEDULE_WAVES)
    status = torch.full((st.nc,), 5, dtype=torch.int32, device="cuda")
    api.soil_water(h, d, wl.dtime, cfg, col_status=status)
    got = d.to_host()
    h.close()
    rep, bad = compare(got, ref, fields=["h2osoi_liq", "smp_l", "hk_l", "qcharge", "num_substeps"])
    assert not bad, (len(bad), rep)
    assert np.all(status.cpu().numpy() == 0)


@pytest.mark.parametrize("schedule", ["fused", "queue", "queue_reserved", "waves"])
def test_soil_water_watertable_runs_compute_qcharge(schedule):
    """BC_WATERTABLE: soilwater_moisture_form! runs compute_qcharge! after the solve
    (soil_water_movement.jl:1575-1598).  Water tables from the surface to below the soil
    column and ragged bedrock, so some columns drain to the table in the solve and still
    get their recharge overwritten.  Every output bit for bit against the oracle."""
    from test_oracle_qcharge import _watertable_case, qcharge_numpy
    for cfg_id in (0, 2):
        wl, st = _watertable_case(cfg_id, nc=2048)
        cfg = abi.SwmConfig.clm5_default()
        cfg.lower_boundary_condition = abi.BC_WATERTABLE
        ref = st.copy()
        assert np.all(orc.soil_water(ref, wl.dtime, cfg) == 0)
        d = st.to_device()
        h = api.Handle(st.vp)
        if schedule in ("queue_reserved", "waves"):
            h.reserve(st.nc)
        if schedule == "waves":
            h.set_option(abi.OPT_STEP_SCHEDULE, abi.SCHEDULE_WAVES)
        if schedule == "fused":
            h.set_option(abi.OPT_STEP_SCHEDULE, abi.SCHEDULE_FUSED)
        status = torch.full((st.nc,), 5, dtype=torch.int32, device="cuda")
        api.soil_water(h, d, wl.dtime, cfg, col_status=status)
        got = d.to_host()
        h.close()
        assert np.all(status.cpu().numpy() == 0)
        assert not bit_mismatches(got, ref, ["h2osoi_liq", "smp_l", "hk_l", "qcharge", "num_substeps"])
        jwt, q = qcharge_numpy(ref, wl.dtime)
        over = ~np.isnan(q)
        assert over.sum() > st.nc // 2
        assert np.array_equal(got["qcharge"][over].view(np.uint64), q[over].view(np.uint64))


def test_soil_water_rejects_configs(handle_factory):
    st = moisture_fixture()
    d = st.to_device()
    h = handle_factory(st.vp)
    cfg = abi.SwmConfig.clm5_default()
    cfg.soilwater_movement_method = abi.ZENGDECKER_2009
    with pytest.raises(api.CLMGBError) as e:
        api.soil_water(h, d, 1800.0, cfg)
    assert e.value.code == abi.CLMGB_ERR_UNSUPPORTED
    cfg = abi.SwmConfig.clm5_default()
    cfg.upper_boundary_condition = abi.BC_HEAD
    with pytest.raises(api.CLMGBError) as e:
        api.soil_water(h, d, 1800.0, cfg)
    assert e.value.code == abi.CLMGB_ERR_CONFIG
    # soilwm_moisture_form_solve! rejects the aquifer boundary with error() (:1502-1505)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_AQUIFER
    with pytest.raises(api.CLMGBError) as e:
        api.soil_water(h, d, 1800.0, cfg)
    assert e.value.code == abi.CLMGB_ERR_CONFIG
    with pytest.raises(api.CLMGBError) as e:
        api.soil_temperature(h, d, 1800.0, use_excess_ice=True)
    assert e.value.code == abi.CLMGB_ERR_UNSUPPORTED


def test_empty_bounds_is_noop(handle_factory):
    wl = synth.make_workload(0, nc=8)
    st = wl.state
    d = st.to_device()
    h = handle_factory(st.vp)
    import ctypes as C
    b = abi.Bounds(0, 0, 1, 8, 8)
    assert h.lib.clmgb_soil_temperature(h.h, C.byref(b), C.byref(d.soiltemp_fields()), 1800.0, 1, 0, None,
                                        None) == 0
    assert np.array_equal(d["t_soisno"].cpu().numpy(), st["t_soisno"])


# ---------------------------------------------------------------- shared math
@pytest.mark.parametrize("op", ["log", "exp", "pow", "log10", "sin", "acos"])
def test_math_bit_identical_to_cpu_build(handle_factory, op):
    import ctypes as C
    h = handle_factory(synth.clm5_varpar())
    rng = np.random.default_rng(hash(op) & 0xffff)
    n = 200000
    if op == "exp":
        x = rng.uniform(-745, 709, n)
    elif op == "sin":
        x = np.concatenate([rng.uniform(-1e5, 1e5, n // 2), rng.uniform(-4.0, 4.0, n - n // 2)])
    elif op == "acos":
        x = rng.uniform(-1.0, 1.0, n)
    else:
        x = np.concatenate([10 ** rng.uniform(-300, 300, n // 2), rng.uniform(0.0, 3.0, n - n // 2)])
    y = rng.uniform(-50, 50, n)
    got = api.math_eval(h, op, _dev(x), _dev(y) if op == "pow" else None).cpu().numpy()
    f = getattr(orc.lib(), "orc_cm_" + op)
    f.restype = C.c_double
    f.argtypes = [C.c_double] * (2 if op == "pow" else 1)
    sel = rng.choice(n, 5000, replace=False)
    ref = np.array([f(float(x[i]), float(y[i])) if op == "pow" else f(float(x[i])) for i in sel])
    assert np.array_equal(got[sel].view(np.uint64), ref.view(np.uint64))


def test_division_is_ieee_with_zero_numerators(handle_factory):
    """The kernels' division (jl_div: a zero numerator over a finite nonzero divisor
    answered from the sign bits, normal operands by cm_div on the integer pipes, the
    rest by the hardware division) against IEEE division on the host, over every pairing of zeros, subnormals, normals, extremes, infinities
    and NaN, and 4 M random pairs: numerators a fifth zero, random bit patterns (every
    exponent class), divisors with short significands, quotients next to a
    representable value."""
    h = handle_factory(synth.clm5_varpar())
    tiny = np.nextafter(0.0, 1.0)
    special = np.array([0.0, -0.0, tiny, -tiny, 2.2250738585072014e-308, 1e-300, 1e-20, 0.5, 1.0, 917.0, 3.0e8,
                        1e300, np.finfo(np.float64).max, -1.0, -917.0, np.inf, -np.inf, np.nan])
    xs, ys = np.meshgrid(special, special, indexing="ij")
    rng = np.random.default_rng(61)
    n = 4_000_000
    xr = rng.uniform(-50.0, 50.0, n) * 10.0 ** rng.integers(-30, 30, n)
    xr[rng.random(n) < 0.2] = 0.0
    xr[rng.random(n) < 0.05] *= -0.0
    yr = rng.uniform(-50.0, 50.0, n) * 10.0 ** rng.integers(-30, 30, n)
    k = n // 4                                                # random bit patterns: every exponent
    xr[:k] = rng.integers(0, 2 ** 64, k, dtype=np.uint64).view(np.float64)
    yr[:k] = rng.integers(0, 2 ** 64, k, dtype=np.uint64).view(np.float64)
    yb = yr[k:2 * k].view(np.uint64)                          # divisors with short significands
    yb &= ~np.uint64(0x000FFFFFFFFFFF00)
    q = rng.uniform(1.0, 2.0, k)                              # quotients next to a representable value
    with np.errstate(all="ignore"):
        xr[2 * k:3 * k] = q * yr[2 * k:3 * k]
    x = np.concatenate([xs.ravel(), xr])
    y = np.concatenate([ys.ravel(), yr])
    got = api.math_eval(h, "div", _dev(x), _dev(y)).cpu().numpy()
    with np.errstate(all="ignore"):
        want = x / y
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)                 # NaN payloads differ between hosts
    assert np.array_equal(got[~nan].view(np.uint64), want[~nan].view(np.uint64))


# ---------------------------------------------------------------- multi-step column step
# ---------------------------------------------------------------- multi-step column step
@pytest.mark.parametrize("mode", ["queue", "queue_reserved", "waves", "fused"])
@pytest.mark.parametrize("cfg_id,nc,nsteps", [(0, 1024, 48), (1, 4096, 48), (2, 4096, 24)])
def test_column_step_multistep_vs_oracle(cfg_id, nc, nsteps, mode):
    wl = synth.make_workload(cfg_id, nc=nc)
    st = wl.state
    Gf, If = wl.forcing_block(range(nsteps))
    ref = st.copy()
    status_ref = orc.run_steps(ref, wl.dtime, Gf, If)
    d = st.to_device()
    h = api.Handle(st.vp)       # own handle: reserve state must not leak into other tests
    h.set_option(abi.OPT_STEP_SCHEDULE, {"fused": abi.SCHEDULE_FUSED, "waves": abi.SCHEDULE_WAVES}.get(
        mode, abi.SCHEDULE_QUEUE))
    if mode == "waves":
        assert h.get_option(abi.OPT_WAVES_OCCUPANCY) > 0
    if mode in ("queue_reserved", "waves"):
        h.reserve(nc)
        assert h.get_option(abi.OPT_RESERVED_COLUMNS) == nc
    Gd, Id = _dev(Gf), _dev(If)
    for t in range(nsteps):
        api.synth_forcing(h, d, Gd[t], Id[t])
        api.column_step(h, d, wl.dtime)
    torch.cuda.synchronize()
    assert h.device_status() == 0
    assert np.all(status_ref == 0)
    h.close()
    got = d.to_host()
    rep, bad = compare(got, ref)
    assert not bad, (len(bad), rep)
    # GPU and oracle share their transcendentals and operation order: identical bits
    for k in ("t_soisno", "h2osoi_liq", "h2osoi_ice", "num_substeps", "qcharge", "t_grnd", "imelt"):
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("nlevs,jt", [(20, 1), (21, 4), (38, 1), (64, 7), (5, 5)])
def test_tridiagonal_pcr_matches_thomas(nlevs, jt):
    """CLMGB_TRIDIAG_PCR (one warp per column) against the Thomas path (the oracle's
    bits) on diagonally dominant systems with ragged masks: agreement to 1e-13
    relative, masked columns untouched."""
    from clmgb import autotune
    ncols = 777
    a, b, c, r = autotune.diagonally_dominant_systems(ncols, nlevs, seed=nlevs + jt)
    jtop = torch.full((ncols,), jt, dtype=torch.int64, device="cuda")
    mask = torch.ones(ncols, dtype=torch.uint8, device="cuda")
    mask[::11] = 0
    h = api.Handle(synth.clm5_varpar())
    out = {}
    for method in (abi.TRIDIAG_THOMAS, abi.TRIDIAG_PCR):
        h.set_option(abi.OPT_TRIDIAG_METHOD, method)
        assert h.get_option(abi.OPT_TRIDIAG_METHOD) == method
        u = torch.full((nlevs, ncols), 7.0, dtype=torch.float64, device="cuda")
        api.tridiagonal_multi(h, u, a, b, c, r, jtop, mask)
        torch.cuda.synchronize()
        out[method] = u.cpu().numpy()
    h.close()
    ut, up = out[abi.TRIDIAG_THOMAS], out[abi.TRIDIAG_PCR]
    m = mask.cpu().numpy() != 0
    # Thomas is the oracle's restatement bit for bit
    u_ref = np.full((nlevs, ncols), 7.0)
    orc.tridiagonal_multi(u_ref, a.cpu().numpy(), b.cpu().numpy(), c.cpu().numpy(), r.cpu().numpy(),
                          jtop.cpu().numpy(), mask.cpu().numpy())
    assert np.array_equal(ut.view(np.uint64), u_ref.view(np.uint64))
    sl = slice(jt - 1, nlevs)
    scale = np.max(np.abs(ut[sl][:, m]), axis=0)
    assert np.max(np.abs(up[sl][:, m] - ut[sl][:, m]) / scale) < 1e-13
    assert np.all(up[:, ~m] == 7.0) and np.all(up[:jt - 1] == 7.0)


def test_tridiagonal_pcr_known_answers():
    """The reference's tridiagonal known answers (test_tridiagonal.jl, test_soil_water_
    movement.jl: all-ones solutions, the identity, a partial system below jtop) through
    the PCR path, within each case's tolerance."""
    G = golden()
    h = api.Handle(synth.clm5_varpar())
    h.set_option(abi.OPT_TRIDIAG_METHOD, abi.TRIDIAG_PCR)
    ran = 0
    for name in ("tridiag_3x3", "tridiag_col_3x3", "tridiag_identity", "tridiag_partial"):
        c = G[name]
        n, ncols = len(c["b"]), 3
        arr = {k: _dev(np.repeat(np.array(c[k], dtype=np.float64)[:, None], ncols, 1)) for k in "abcr"}
        u = torch.zeros((n, ncols), dtype=torch.float64, device="cuda")
        api.tridiagonal_multi(h, u, arr["a"], arr["b"], arr["c"], arr["r"],
                              _dev(np.full(ncols, c["jtop"], dtype=np.int64)), _dev(np.ones(ncols, dtype=np.uint8)))
        torch.cuda.synchronize()
        got = u.cpu().numpy()
        for col in range(ncols):
            for g, want in zip(got[:, col], c["u"]):
                if want is not None:
                    assert abs(g - want) <= c["atol"], (name, col, g, want)
        ran += 1
    h.close()
    assert ran == 4


@pytest.mark.parametrize("mode", ["queue", "queue_reserved", "waves", "fused"])
@pytest.mark.parametrize("cfg_id", [1, 2])
def test_column_step_at_maximum_level_counts(cfg_id, mode):
    """The largest level counts the ABI accepts (12 snow, 25 ground, 25 soil levels:
    37 levels and a 38-row band system, the Richards solve over 25 levels, the packed
    refresh's shared block and the record pre-pass at their largest), with ragged bedrock
    depths and a partial last tile of columns: the oracle's bits after 6 steps."""
    vp = abi.Varpar(abi.MAX_NLEVSNO, abi.MAX_NLEVGRND, abi.MAX_NLEVSOI, 5, abi.MAX_NLEVGRND, 0)
    nsteps, nc = 6, 3000
    wl = synth.make_workload(cfg_id, nc=nc, seed=77 + cfg_id, nsteps=nsteps, vp=vp)
    st = wl.state
    rng = np.random.default_rng(cfg_id)
    st["col_nbedrock"][:] = rng.integers(1, vp.nlevsoi + 1, nc)
    Gf, If = wl.forcing_block(range(nsteps))
    ref = st.copy()
    status_ref = orc.run_steps(ref, wl.dtime, Gf, If)
    assert np.all(status_ref == 0)
    d = st.to_device()
    h = api.Handle(st.vp)
    h.set_option(abi.OPT_STEP_SCHEDULE, {"fused": abi.SCHEDULE_FUSED, "waves": abi.SCHEDULE_WAVES}.get(
        mode, abi.SCHEDULE_QUEUE))
    if mode in ("queue_reserved", "waves"):
        h.reserve(nc)
    Gd, Id = _dev(Gf), _dev(If)
    for t in range(nsteps):
        api.synth_forcing(h, d, Gd[t], Id[t])
        api.column_step(h, d, wl.dtime)
    torch.cuda.synchronize()
    assert h.device_status() == 0
    h.close()
    got = d.to_host()
    for k in ("t_soisno", "h2osoi_liq", "h2osoi_ice", "num_substeps", "qcharge", "t_grnd", "imelt", "smp_l",
              "hk_l", "fact", "icefrac"):
        assert np.array_equal(got[k].view(np.uint64) if got[k].dtype == np.float64 else got[k],
                              ref[k].view(np.uint64) if ref[k].dtype == np.float64 else ref[k]), k


def test_zero_columns_is_a_no_op():
    """Calls over zero columns return CLMGB_OK before they read a field (the reference's
    loops over an empty filter do nothing); the handle's device status stays 0."""
    import ctypes as C
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    lib = h.lib
    b = abi.Bounds(0, 0, 0, 0, 0)
    ft, fw = abi.SoilTempFields(), abi.SoilWaterFields()
    ft.struct_size, fw.struct_size = C.sizeof(ft), C.sizeof(fw)
    cfg = abi.SwmConfig.clm5_default()
    ok = abi.CLMGB_OK
    assert lib.clmgb_soil_temperature(h.h, C.byref(b), C.byref(ft), 1800.0, 1, 0, None, None) == ok
    assert lib.clmgb_soil_water_fractions(h.h, C.byref(b), C.byref(fw), None) == ok
    assert lib.clmgb_soil_water(h.h, C.byref(b), C.byref(fw), C.byref(cfg), 1800.0, None, None) == ok
    assert lib.clmgb_column_step(h.h, C.byref(b), C.byref(ft), C.byref(fw), C.byref(cfg), 1800.0, 1, None, None,
                                 None, None) == ok
    assert lib.clmgb_synth_forcing(h.h, C.byref(b), C.byref(ft), C.byref(fw), None, None, None) == ok
    assert lib.clmgb_tridiagonal_multi(h.h, 0, 0, 20, None, None, None, None, None, None, None, None) == ok
    assert lib.clmgb_batched_band_solve(h.h, 0, 0, 38, None, None, None, None, None, None, 2, 2, 12, None) == ok
    assert lib.clmgb_soil_water_noalloc(C.byref(vp), C.byref(b), C.byref(fw), C.byref(cfg), 1800.0, None,
                                        None) == ok
    torch.cuda.synchronize()
    assert h.device_status() == 0
    h.close()
