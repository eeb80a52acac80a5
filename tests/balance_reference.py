"""Balance residuals of a column step in numpy (TEST INFRASTRUCTURE ONLY): errsoi
(soil_fluxes.jl:321-328, :380-447) and the path's part of errh2o
(balance_check.jl:741-768), in the same operation order as clmgb_balance_residuals.
Host states with one patch per column."""
import numpy as np

from clmgb.synth import pow4

SB = 5.67e-8


def storage(st):
    vp = st.vp
    out = np.zeros(st.nc)
    for c in range(st.nc):
        snl = int(st["col_snl"][c])
        w = 0.0
        for jj in range(snl + 1 + vp.nlevsno, vp.nlevsno + vp.nlevgrnd + 1):
            w += st["h2osoi_liq"][jj - 1, c] + st["h2osoi_ice"][jj - 1, c]
        out[c] = w + st["h2osfc"][c] + st["h2osno_no_layers"][c]
    return out


def residuals(st, dtime, t_grnd0, begwb):
    vp = st.vp
    ns = vp.nlevsno
    es = np.zeros(st.nc)
    eh = np.zeros(st.nc)
    end = storage(st)
    for c in range(st.nc):
        snl = int(st["col_snl"][c])
        p = c
        fsno, fh, eg = st["frac_sno_eff"][c], st["frac_h2osfc"][c], st["emg"][c]
        tg0 = t_grnd0[c]
        tinc = st["t_grnd"][c] - tg0
        tsb = st["t_ssbef"]
        lw = (fsno * pow4(np.float64(tsb[snl + ns, c])) + (1.0 - fsno - fh) * pow4(np.float64(tsb[ns, c])) +
              fh * pow4(np.float64(st["t_h2osfc_bef"][c])))
        gs = (((1.0 - fsno) * st["sabg_soil"][p] + fsno * st["sabg_snow"][p]) + st["dlrad"][p] +
              (1.0 - float(st["frac_veg_nosno"][p])) * eg * st["forc_lwrad"][c] - eg * SB * lw -
              eg * SB * (tg0 * tg0 * tg0) * (4.0 * tinc) -
              (st["eflx_sh_grnd"][p] + st["qflx_evap_soi"][p] * st["htvp"][c]))
        e = gs - st["xmf"][c] - st["xmf_h2osfc"][c] - fh * (st["t_h2osfc"][c] - st["t_h2osfc_bef"][c]) * (
            st["c_h2osfc"][c] / dtime)
        e += st["eflx_h2osfc_to_snow"][c]
        for j in range(snl + 1, vp.nlevgrnd + 1):
            jj = j + ns
            d = (st["t_soisno"][jj - 1, c] - tsb[jj - 1, c]) / st["fact"][jj - 1, c]
            e = e - fsno * d if j < 1 else e - d
        es[c] = e * st["patch_wtcol"][p]
        nl = int(st["col_nbedrock"][c])
        sink = 0.0
        for j in range(1, min(nl, vp.nlevsoi) + 1):
            sink += st["qflx_rootsoi"][j - 1, c]
        eh[c] = end[c] - begwb[c] - (st["qflx_infl"][c] - sink - st["qcharge"][c]) * dtime
    return es, eh
