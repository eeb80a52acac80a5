"""compute_qcharge! after the moisture-form solve (the water-table lower boundary).

soilwater_moisture_form! (soil_water_movement.jl:1575-1598) runs compute_qcharge!
(:1153-1215) when use_aquifer_layer(cfg) holds; among the lower boundaries the
moisture form accepts, that is BC_WATERTABLE.  It passes freshly zeroed dwat, smp and
imped rows, so the recharge it writes for a column whose water table lies within the
soil column (jwt < nlevsoi) is -ka*(wh_zwt - wh)/den with ka = 0*hksat*s1^(2b+3): a
zero whose sign follows (wh_zwt - wh) (+0 whenever the suction head at the table lies
below that of the level above it, as on these workloads).  The reference's own tests hold no case
for it, so the oracle's restatement is pinned here against a second, numpy
restatement written from the reference's text, bit for bit (signs of zero included).
"""
import numpy as np

from clmgb import abi, synth
from oracle import oracle as orc


def qcharge_numpy(st, dtime):
    """compute_qcharge! on the solved state `st` (host), numpy.  Returns (jwt, qcharge)
    with qcharge NaN where the routine leaves the solve's value."""
    vp, nc = st.vp, st.nc
    joff, nlevsoi = vp.nlevsno, vp.nlevsoi
    zi, z, dz = st["zi"], st["z"], st["dz"]
    liq = st["h2osoi_liq"]
    jwt = np.full(nc, nlevsoi, dtype=np.int64)
    for c in range(nc):
        for j in range(1, nlevsoi + 1):
            if st["zwt"][c] <= zi[joff + 1 + j - 1, c]:     # Julia zi[c, joff_zi + j]
                jwt[c] = j - 1
                break
    out = np.full(nc, np.nan)
    for c in range(nc):
        if not st["mask_hydrology"][c] or jwt[c] >= nlevsoi:
            continue
        nl = int(st["col_nbedrock"][c])
        jp = jwt[c] + 1
        vwc = 0.0
        if jp <= min(nl, nlevsoi):
            vwc = max(liq[joff + jp - 1, c], 1.0e-6) / (dz[joff + jp - 1, c] * 1000.0)
        s1 = min(1.0, max(vwc / st["watsat"][jp - 1, c], 0.01))
        ka = 0.0 * st["hksat"][jp - 1, c] * s1 ** (2.0 * st["bsw"][jp - 1, c] + 3.0)
        zwt = st["zwt"][c]
        wh_zwt = -st["sucsat"][jp - 1, c] - zwt * 1000.0
        jm = max(1, jwt[c])
        smp1 = max(st["smpmin"][c], 0.0)
        wh = smp1 - z[joff + jm - 1, c] * 1000.0
        if jwt[c] == 0:
            q = -ka * (wh_zwt - wh) / ((zwt + 1.0e-3) * 1000.0)
        else:
            q = -ka * (wh_zwt - wh) / ((zwt - z[joff + jwt[c] - 1, c]) * 1000.0 * 2.0)
        q = max(-10.0 / dtime, q) if not np.isnan(q) else q
        q = min(10.0 / dtime, q) if not np.isnan(q) else q
        out[c] = q
    return jwt, out


def _watertable_case(cfg_id, nc=384, seed=5):
    wl = synth.make_workload(cfg_id, nc=nc, seed=seed)
    st = wl.state
    orc.soil_water_fractions(st)
    # water tables from the surface to below the soil column (jwt = 0 .. nlevsoi) and
    # bedrock depths from 5 levels to the whole soil column
    st["zwt"][:] = np.linspace(0.0, 12.0, st.nc)
    st["col_nbedrock"][:] = 5 + np.arange(st.nc) % (st.vp.nlevsoi - 4)
    st["mask_hydrology"][::13] = 0
    return wl, st


def test_oracle_qcharge_matches_numpy_restatement_bit_for_bit():
    for cfg_id in (0, 2):
        wl, st = _watertable_case(cfg_id)
        cfg = abi.SwmConfig.clm5_default()
        cfg.lower_boundary_condition = abi.BC_WATERTABLE
        status = orc.soil_water(st, wl.dtime, cfg)
        assert np.all(status == 0)
        jwt, q = qcharge_numpy(st, wl.dtime)
        over = ~np.isnan(q)
        nlevsoi = st.vp.nlevsoi
        assert over.sum() > 0.5 * st.nc and (jwt == nlevsoi).sum() > 10 and (jwt == 0).sum() >= 1
        got = st["qcharge"]
        assert np.array_equal(got[over].view(np.uint64), q[over].view(np.uint64))
        assert np.all(got[over] == 0.0)
        # columns whose bedrock lies above the water table drain to it in the solve
        # (the bottom flux of the water-table boundary, :1345-1358), and compute_qcharge!
        # still overwrites their recharge when the table lies within the soil column
        drains = over & (st["col_nbedrock"] <= jwt)
        assert drains.sum() > 5
        # the others keep the solve's accumulated bottom flux: nonzero where they drain
        keep = ~over & (st["mask_hydrology"] == 1)
        assert np.all(np.isfinite(got[keep])) and np.any(got[keep] != 0.0)


def test_oracle_qcharge_other_boundaries_untouched():
    """Under the flux and zero-flux lower boundaries use_aquifer_layer is false
    (soil_water_movement.jl:707-710): qcharge is the solve's own value."""
    wl, st = _watertable_case(0, nc=128)
    for bc in (abi.BC_FLUX, abi.BC_ZERO_FLUX):
        cfg = abi.SwmConfig.clm5_default()
        cfg.lower_boundary_condition = bc
        s = st.copy()
        orc.soil_water(s, wl.dtime, cfg)
        m = st["mask_hydrology"] == 1
        if bc == abi.BC_ZERO_FLUX:
            assert np.all(s["qcharge"][m] == 0.0)
        else:
            assert np.all(s["qcharge"][m] > 0.0)
