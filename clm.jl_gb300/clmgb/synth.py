"""Seeded synthetic column inputs for the soil/snow column solve.

No dataset is involved: CLM.jl's benchmarks of this path run on site data that is
not available, so every workload is generated here from numpy ``default_rng(seed)``
with the shapes, value ranges and distributions of the workload definitions:

  cfg 0  1,024 columns, no snow, dtime 1800 s, 48 steps
  cfg 1  65,536 columns, snl uniform 0..12, frozen top soil, dtime 1800 s, 48 steps
  cfg 2  262,144 columns, snl 60% 0 / 40% 1..12, diurnal ground flux and
         Bernoulli(0.1) infiltration pulses, dtime 3600 s, 1,000 steps

Soil parameters come from sand/clay/organic fraction through the reference's
soil-parameter routine (init_soil_properties!, cold_start.jl:225-391) restated in
``init_soil_properties`` below, on CLM5's 20SL_8.5m grid (varcon.jl:241-280).
The ground heat flux is injected through the real ground-flux code: one patch per
column with wtcol=1, frac_veg_nosno=0, emg=0.97, zero sensible/latent fluxes,
sabg = sabg_soil = sabg_snow = G and sabg_lyr[top active layer] = G, and
forc_lwrad = SB*t_grnd^4 each step so the net long-wave is ~0.
"""
import math

import numpy as np

from . import abi
from .state import ColumnState

SB = 5.67e-8
HVAP = 2.501e6
TFRZ = 273.15
ISTSOIL = 1


def clm5_varpar():
    """varpar for CLM5 20SL_8.5m with 12 snow layers and 5 urban levels."""
    return abi.Varpar(12, 25, 20, 5, 25, 0)


def soil_grid(nlevsoi=20, nlevgrnd=25):
    """dzsoi, zsoi, zisoi of the 20SL_8.5m structure (varcon_init!, varcon.jl:241-280)."""
    dz = np.zeros(nlevgrnd)
    for j in range(1, min(4, nlevsoi) + 1):
        dz[j - 1] = j * 0.02
    for j in range(5, min(13, nlevsoi) + 1):
        dz[j - 1] = dz[3] + (j - 4) * 0.04
    for j in range(14, nlevsoi + 1):
        dz[j - 1] = dz[min(13, nlevsoi) - 1] + (j - 13) * 0.10
    for j in range(nlevsoi + 1, nlevgrnd + 1):
        dz[j - 1] = dz[nlevsoi - 1] + (((j - nlevsoi) * 25.0) ** 1.5) / 100.0
    zi = np.zeros(nlevgrnd + 1)
    for j in range(1, nlevgrnd + 1):
        zi[j] = zi[j - 1] + dz[j - 1]
    z = np.array([0.5 * (zi[j] + zi[j + 1]) for j in range(nlevgrnd)])
    return dz, z, zi


def init_soil_properties(sand, clay, om_frac, zsoi):
    """init_soil_properties! (cold_start.jl:276-375) with SoilStateParams defaults
    (types/soil_state.jl:19-35).  Arrays broadcast elementwise; returns a dict."""
    sand = np.asarray(sand, dtype=np.float64)
    clay = np.asarray(clay, dtype=np.float64)
    om_frac = np.asarray(om_frac, dtype=np.float64)
    zsoi = np.asarray(zsoi, dtype=np.float64)
    tkd_sand, tkd_clay, tkd_om, tkm_om = 8.8, 2.92, 0.05, 0.25
    csol_sand, csol_clay, csol_om, pd = 2.128, 2.385, 2.5, 2700.0
    watsat_mineral = 0.489 - 0.00126 * sand
    bsw_mineral = 2.91 + 0.159 * clay
    sucsat_mineral = 10.0 * np.power(10.0, 1.88 - 0.0131 * sand)
    xksat_mineral = 0.0070556 * np.power(10.0, -0.884 + 0.0153 * sand)
    depth_ratio = zsoi / 0.5
    watsat_organic = np.maximum(0.93 - 0.1 * depth_ratio, 0.83)
    bsw_organic = np.minimum(2.7 + 9.3 * depth_ratio, 12.0)
    sucsat_organic = np.minimum(10.3 - 0.2 * depth_ratio, 10.1)
    xksat_organic = np.maximum(0.28 - 0.2799 * depth_ratio, xksat_mineral)
    watsat = np.minimum(1.0 * ((1.0 - om_frac) * watsat_mineral + om_frac * watsat_organic), 0.93)
    bsw = 1.0 * ((1.0 - om_frac) * bsw_mineral + om_frac * bsw_organic)
    sucsat = 1.0 * ((1.0 - om_frac) * sucsat_mineral + om_frac * sucsat_organic)
    pcalpha, pcbeta = 0.5, 0.139
    perc_norm = np.power(1.0 - pcalpha, -pcbeta)
    perc_frac = np.where(om_frac > pcalpha,
                         perc_norm * np.power(np.maximum(om_frac - pcalpha, 0.0), pcbeta), 0.0)
    uncon_frac = (1.0 - om_frac) + (1.0 - perc_frac) * om_frac
    with np.errstate(divide="ignore", invalid="ignore"):
        uncon_hksat = np.where(uncon_frac > 0.0,
                               uncon_frac / ((1.0 - om_frac) / xksat_mineral +
                                             ((1.0 - perc_frac) * om_frac) / xksat_organic), 0.0)
    hksat = 1.0 * (uncon_frac * uncon_hksat + (perc_frac * om_frac) * xksat_organic)
    bd = (1.0 - watsat_mineral) * pd
    sc = sand + clay
    tkm = np.where(sc > 0.0, (1.0 - om_frac) * (tkd_sand * sand + tkd_clay * clay) / np.where(sc > 0, sc, 1.0)
                   + tkm_om * om_frac, tkm_om)
    tkmg = np.power(tkm, 1.0 - watsat)
    tkdry = ((0.135 * bd + 64.7) / (pd - 0.947 * bd)) * (1.0 - om_frac) + tkd_om * om_frac
    csol_min = np.where(sc > 0.0, (csol_sand * 1.0e6 * sand + csol_clay * 1.0e6 * clay) / np.where(sc > 0, sc, 1.0),
                        csol_om * 1.0e6)
    csol = (1.0 - om_frac) * csol_min + csol_om * 1.0e6 * om_frac
    return dict(watsat=watsat, bsw=bsw, sucsat=sucsat, hksat=hksat, tkmg=tkmg, tkdry=tkdry, csol=csol)


CONFIGS = {
    0: dict(nc=1024, dtime=1800.0, nsteps=48, seed=20240, snow="none"),
    1: dict(nc=65536, dtime=1800.0, nsteps=48, seed=20241, snow="uniform"),
    2: dict(nc=262144, dtime=3600.0, nsteps=1000, seed=20242, snow="mix"),
}


class Workload:
    """A generated workload: initial host state plus per-step forcing."""

    def __init__(self, cfg_id, state, dtime, nsteps, G0, A, infl0, seed, pulses):
        self.cfg_id = cfg_id
        self.state = state
        self.dtime = float(dtime)
        self.nsteps = int(nsteps)
        self.G0 = G0
        self.A = A
        self.infl0 = infl0
        self.seed = seed
        self.pulses = pulses

    def forcing(self, step, cols=None):
        """(G, I) rows [nc] for timestep `step` (0-based)."""
        G0 = self.G0 if cols is None else self.G0[cols]
        I0 = self.infl0 if cols is None else self.infl0[cols]
        if self.A is None:
            return G0.copy(), I0.copy()
        A = self.A if cols is None else self.A[cols]
        s = math.sin(2.0 * math.pi * (step * self.dtime) / 86400.0)
        G = G0 + A * s
        I = I0.copy()
        if self.pulses:
            r = np.random.default_rng([self.seed, 7, step])
            hit = r.random(self.state.nc) < 0.1
            amp = r.uniform(1.0e-4, 2.0e-3, self.state.nc)
            if cols is not None:
                hit, amp = hit[cols], amp[cols]
            I = I + np.where(hit, amp, 0.0)
        return G, I

    def forcing_block(self, steps, cols=None):
        """Stacked forcing [len(steps), nc] arrays (G, I)."""
        rows = [self.forcing(t, cols) for t in steps]
        return np.stack([r[0] for r in rows]), np.stack([r[1] for r in rows])


def make_workload(cfg_id, nc=None, seed=None, vp=None, nsteps=None):
    """Build workload `cfg_id` (0, 1 or 2), optionally with fewer columns."""
    spec = dict(CONFIGS[cfg_id])
    if nc is not None:
        spec["nc"] = int(nc)
    if seed is not None:
        spec["seed"] = int(seed)
    if nsteps is not None:
        spec["nsteps"] = int(nsteps)
    vp = vp or clm5_varpar()
    nc = spec["nc"]
    rng = np.random.default_rng(spec["seed"])
    nlevsno, nlevgrnd, nlevsoi = vp.nlevsno, vp.nlevgrnd, vp.nlevsoi
    L = nlevsno + vp.nlevmaxurbgrnd
    joff = nlevsno
    st = ColumnState(vp, nc, nc, 1)
    a = st.arrays

    # ---- texture (rejection-sample sand+clay <= 95) ----
    sand = rng.uniform(5.0, 90.0, nc)
    clay = rng.uniform(5.0, 60.0, nc)
    bad = sand + clay > 95.0
    while bad.any():
        k = int(bad.sum())
        sand[bad] = rng.uniform(5.0, 90.0, k)
        clay[bad] = rng.uniform(5.0, 60.0, k)
        bad = sand + clay > 95.0
    om = rng.uniform(0.0, 0.3, nc)
    dzs, zs, zis = soil_grid(nlevsoi, nlevgrnd)
    props = init_soil_properties(sand[None, :], clay[None, :], om[None, :], zs[:, None])
    for k in ("watsat", "bsw", "sucsat", "hksat", "tkmg", "tkdry", "csol"):
        a[k][:] = props[k]

    # ---- topology: one landunit (soil), one patch per column ----
    idx = np.arange(1, nc + 1, dtype=np.int64)
    a["mask_nolakec"][:] = 1
    a["mask_nolakep"][:] = 1
    a["mask_hydrology"][:] = 1
    a["col_itype"][:] = ISTSOIL
    a["col_landunit"][:] = 1
    a["col_patchi"][:] = idx
    a["col_patchf"][:] = idx
    a["lun_itype"][:] = ISTSOIL
    a["lun_urbpoi"][:] = 0
    a["patch_column"][:] = idx
    a["patch_landunit"][:] = 1
    a["patch_wtcol"][:] = 1.0
    a["frac_veg_nosno"][:] = 0
    a["col_nbedrock"][:] = nlevsoi

    # ---- soil geometry ----
    for j in range(1, nlevgrnd + 1):
        a["dz"][joff + j - 1] = dzs[j - 1]
        a["z"][joff + j - 1] = zs[j - 1]
    for j in range(0, nlevgrnd + 1):
        a["zi"][joff + j] = zis[j]     # Julia index j + nlevsno + 1 (1-based) -> row j + nlevsno

    # ---- soil water and temperature ----
    wfrac = rng.uniform(0.3, 0.9, (nlevsoi, nc))
    watsat = a["watsat"]
    for j in range(1, nlevsoi + 1):
        a["h2osoi_liq"][joff + j - 1] = wfrac[j - 1] * watsat[j - 1] * dzs[j - 1] * 1000.0
    ttop = rng.uniform(275.0, 300.0, nc)
    tbot = rng.uniform(278.0, 290.0, nc)
    for j in range(1, nlevgrnd + 1):
        a["t_soisno"][joff + j - 1] = ttop + (tbot - ttop) * ((j - 1) / (nlevgrnd - 1))
    infl0 = rng.uniform(0.0, 5.0e-4, nc)
    qtran = rng.uniform(0.0, 1.0e-4, nc)
    adec = rng.uniform(1.0, 6.0, nc)
    rootfr = np.exp(-adec[None, :] * zs[:nlevsoi, None])
    rootfr = rootfr / rootfr.sum(axis=0, keepdims=True)
    a["qflx_rootsoi"][:] = qtran[None, :] * rootfr
    G0 = rng.normal(50.0, 100.0, nc)

    # ---- snow and frozen soil ----
    snl = np.zeros(nc, dtype=np.int64)
    if spec["snow"] == "uniform":
        snl = -rng.integers(0, nlevsno + 1, nc)
    elif spec["snow"] == "mix":
        has = rng.random(nc) < 0.4
        snl = np.where(has, -rng.integers(1, nlevsno + 1, nc), 0)
    if spec["snow"] != "none":
        sdz = rng.uniform(0.01, 0.5, (nlevsno, nc))
        rho = rng.uniform(100.0, 500.0, (nlevsno, nc))
        tsn = rng.uniform(240.0, 273.0, (nlevsno, nc))
        ifrac = rng.uniform(0.0, 0.8, (5, nc))
        tfz = rng.uniform(265.0, 275.0, (5, nc))
        for j in range(1, 6):
            tot = a["h2osoi_liq"][joff + j - 1].copy()
            a["h2osoi_ice"][joff + j - 1] = ifrac[j - 1] * tot
            a["h2osoi_liq"][joff + j - 1] = (1.0 - ifrac[j - 1]) * tot
            a["t_soisno"][joff + j - 1] = tfz[j - 1]
        # snow layers j = 0, -1, ..., snl+1 (row jj-1 = j + nlevsno - 1)
        zi_below = np.zeros(nc)
        depth = np.zeros(nc)
        for j in range(0, -nlevsno, -1):
            act = j >= snl + 1
            r = j + nlevsno - 1
            dzj = sdz[j + nlevsno - 1]
            a["dz"][r] = np.where(act, dzj, 0.0)
            a["z"][r] = np.where(act, zi_below - 0.5 * dzj, 0.0)
            zi_above = zi_below - dzj
            a["zi"][r] = np.where(act, zi_above, 0.0)   # Julia zi index j+nlevsno (Fortran j-1)
            a["h2osoi_ice"][r] = np.where(act, rho[j + nlevsno - 1] * dzj, 0.0)
            a["h2osoi_liq"][r] = 0.0
            a["t_soisno"][r] = np.where(act, tsn[j + nlevsno - 1], 0.0)
            depth = depth + np.where(act, dzj, 0.0)
            zi_below = np.where(act, zi_above, zi_below)
        a["snow_depth"][:] = depth
        a["frac_sno_eff"][:] = np.where(snl < 0, 1.0, 0.0)
    a["col_snl"][:] = snl

    # ---- surface / ground flux injection ----
    a["emg"][:] = 0.97
    a["htvp"][:] = HVAP
    a["eflx_bot"][:] = 0.0
    a["frac_h2osfc"][:] = 0.0
    a["h2osfc"][:] = 0.0
    a["t_h2osfc"][:] = a["t_soisno"][joff]
    top = np.where(snl < 0, a["t_soisno"][np.clip(snl + joff, 0, L - 1), np.arange(nc)], a["t_soisno"][joff])
    fse = a["frac_sno_eff"]
    a["t_grnd"][:] = np.where(snl < 0, fse * top + (1.0 - fse) * a["t_soisno"][joff], a["t_soisno"][joff])
    a["zwt"][:] = zis[nlevsoi]
    a["smpmin"][:] = -1.0e8          # cold_start.jl:763
    A = None
    if spec["snow"] == "mix":
        A = rng.uniform(50.0, 300.0, nc)
    wl = Workload(cfg_id, st, spec["dtime"], spec["nsteps"], G0, A, infl0, spec["seed"],
                  pulses=(spec["snow"] == "mix"))
    G, I = wl.forcing(0)
    apply_forcing_host(st, G, I)
    return wl


def pow4(x):
    """Julia's Float64 x^4 (Base.Math.pow_body compensated squaring), elementwise:
    x2 = x*x, x4 = x2*x2, result x4 + (lo(x2*x2) + x2*2*lo(x*x)), where lo(a*b) is the
    exact rounding error of the product (what fma(a, b, -a*b) returns)."""
    x = np.asarray(x, dtype=np.float64)
    x2 = x * x
    lo1 = _prod_lo(x, x, x2)
    x4 = x2 * x2
    lo2 = _prod_lo(x2, x2, x4)
    xnlo = lo2 + (x2 * 2.0 * lo1)
    out = x4 + xnlo
    return np.where(np.isfinite(x4) & np.isfinite(xnlo), out, x4)


def _prod_lo(a, b, p):
    """Exact a*b - p for p = fl(a*b), by Dekker's splitting (no overflow assumed)."""
    s = 134217729.0
    ah = a * s
    ah = ah - (ah - a)
    al = a - ah
    bh = b * s
    bh = bh - (bh - b)
    bl = b - bh
    return ((ah * bh - p) + ah * bl + al * bh) + al * bl


def apply_forcing_host(st, G, I):
    """The per-step harness forcing on a host state (one patch per column)."""
    a = st.arrays
    nlevsno = st.vp.nlevsno
    a["sabg"][:] = G
    a["sabg_soil"][:] = G
    a["sabg_snow"][:] = G
    a["sabg_lyr"][:] = 0.0
    rows = (a["col_snl"] + nlevsno).astype(np.int64)   # 0-based row of Julia index snl+1+nlevsno
    a["sabg_lyr"][rows, np.arange(st.np)] = G
    a["forc_lwrad"][:] = SB * pow4(a["t_grnd"])
    a["qflx_infl"][:] = I
