"""Seeded inputs of the Zeng-Decker 2009 solve from the synthetic workloads, with the
water table at the surface, inside the soil column and below it.  TEST INFRASTRUCTURE."""
import numpy as np

from clmgb import synth, zd09


def make(cfg_id, nc, seed, nsteps_spin=0):
    wl = synth.make_workload(cfg_id, nc=nc, seed=seed, nsteps=1)
    st = wl.state
    vp = st.vp
    rng = np.random.default_rng(seed + 1)
    zi = st["zi"]                      # row nlevsno + j: interface below soil layer j
    top = zi[vp.nlevsno + 1]
    bot = zi[vp.nlevsno + vp.nlevsoi]
    kind = rng.integers(0, 3, nc)
    zwt = np.where(kind == 0, rng.uniform(0.0, 0.9, nc) * top,
                   np.where(kind == 1, top + rng.uniform(0.05, 0.95, nc) * (bot - top),
                            bot + rng.uniform(0.3, 5.0, nc)))
    zs = zd09.Zd09State.from_column_state(st, zwt=zwt)
    return wl, zs, kind


def balance(zs0, zs1, dtime):
    """Soil water change + recharge (water table below the soil column) minus
    (infiltration - root sink) dtime, per column, and the scale of the terms."""
    vp = zs0.vp
    j0, j1 = vp.nlevsno, vp.nlevsno + vp.nlevsoi
    dliq = (zs1["h2osoi_liq"][j0:j1] - zs0["h2osoi_liq"][j0:j1]).sum(0)
    bot = zs0["zi"][vp.nlevsno + vp.nlevsoi]
    below = zs0["zwt"] > bot
    flux = (zs0["qflx_infl"] - zs0["qflx_rootsoi"][:vp.nlevsoi].sum(0)) * dtime
    resid = dliq + np.where(below, zs1["qcharge"] * dtime, 0.0) - flux
    scale = np.abs(zs0["h2osoi_liq"][j0:j1]).sum(0) + np.abs(flux)
    return resid, scale
