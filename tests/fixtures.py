"""Column states built from CLM.jl's own hand-built test fixtures (tests/golden)."""
import json
import os

import numpy as np

from clmgb import abi
from clmgb.state import ColumnState

HERE = os.path.dirname(os.path.abspath(__file__))
HVAP = 2.501e6
TFRZ = 273.15


def golden():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return json.load(fh)


def soil_column_fixture(ncols=4):
    """setup_soil_column! (test_soil_temperature.jl:92-226) on every column, with
    column 2 given the two-layer snowpack of the Jordan1991 test (:259-287),
    column 3 a frozen layer and column 4 ponded surface water at the freezing point."""
    g = golden()["soiltemp_fixture"]
    vp = abi.Varpar(g["nlevsno"], g["nlevgrnd"], g["nlevsoi"], g["nlevurb"], g["nlevmaxurbgrnd"], 0)
    nlevsno, nlevgrnd, nlevmax = vp.nlevsno, vp.nlevgrnd, vp.nlevmaxurbgrnd
    joff = nlevsno
    st = ColumnState(vp, ncols, ncols, ncols)
    a = st.arrays
    idx = np.arange(1, ncols + 1, dtype=np.int64)
    a["mask_nolakec"][:] = 1
    a["mask_nolakep"][:] = 1
    a["mask_hydrology"][:] = 1
    a["col_landunit"][:] = idx
    a["col_itype"][:] = 1
    a["lun_itype"][:] = 1
    a["lun_urbpoi"][:] = 0
    a["col_snl"][:] = 0
    a["col_nbedrock"][:] = nlevgrnd
    a["patch_column"][:] = idx
    a["patch_landunit"][:] = idx
    a["patch_wtcol"][:] = 1.0
    a["col_patchi"][:] = idx
    a["col_patchf"][:] = idx
    for j in range(1, nlevmax + 1):
        jj = j + joff
        a["dz"][jj - 1] = 0.1 * j
        a["z"][jj - 1] = sum(0.1 * k for k in range(1, j + 1)) - 0.5 * 0.1 * j
    a["zi"][joff] = 0.0
    for j in range(1, nlevmax + 1):
        a["zi"][j + joff] = a["zi"][j + joff - 1] + a["dz"][j + joff - 1]
    for j in range(1, nlevmax + 1):
        a["t_soisno"][j + joff - 1] = g["t"]
        a["h2osoi_liq"][j + joff - 1] = g["liq"]
    a["t_grnd"][:] = g["t"]
    a["t_h2osfc"][:] = g["t"]
    a["emg"][:] = g["emg"]
    for k in ("watsat", "bsw", "sucsat", "tkmg", "tkdry", "csol"):
        a[k][:] = g[k]
    a["hksat"][:] = 0.01
    a["htvp"][:] = HVAP
    a["dlrad"][:] = g["dlrad"]
    a["cgrnd"][:] = g["cgrnd"]
    for k in ("eflx_sh_grnd", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc"):
        a[k][:] = g["sh"]
    a["sabg"][:] = g["sabg"]
    a["sabg_soil"][:] = g["sabg_soil"]
    a["sabg_snow"][:] = g["sabg_snow"]
    a["sabg_lyr"][nlevsno] = g["sabg_lyr_top"]          # Julia index nlevsno+1 = soil layer 1
    a["forc_lwrad"][:] = 300.0
    a["zwt"][:] = a["zi"][joff + vp.nlevsoi]
    a["smpmin"][:] = -1.0e8
    if ncols >= 2:   # two snow layers (test_soil_temperature.jl:259-287)
        c = 1
        a["col_snl"][c] = -2
        a["frac_sno_eff"][c] = 1.0
        for j in (-1, 0):
            jj = j + joff
            a["dz"][jj - 1, c] = 0.1
            a["z"][jj - 1, c] = (j - 0.5) * 0.1
            a["h2osoi_ice"][jj - 1, c] = 10.0
            a["h2osoi_liq"][jj - 1, c] = 1.0
            a["t_soisno"][jj - 1, c] = 270.0
        a["zi"][joff - 2, c] = -0.2
        a["zi"][joff - 1, c] = -0.1
        a["zi"][joff, c] = 0.0
        a["snow_depth"][c] = 0.2
        a["sabg_lyr"][:, c] = 0.0
        a["sabg_lyr"][nlevsno - 2, c] = g["sabg_lyr_top"]   # top active layer j = -1
    if ncols >= 3:   # frozen top soil
        c = 2
        for j in (1, 2, 3):
            jj = j + joff
            a["h2osoi_ice"][jj - 1, c] = 4.0
            a["h2osoi_liq"][jj - 1, c] = 1.0
            a["t_soisno"][jj - 1, c] = TFRZ - 2.0 + 0.5 * j
        a["t_grnd"][c] = TFRZ - 1.5
    if ncols >= 4:   # ponded surface water below freezing
        c = 3
        a["frac_h2osfc"][c] = 0.3
        a["h2osfc"][c] = 8.0
        a["t_h2osfc"][c] = TFRZ - 0.5
        a["h2osno_no_layers"][c] = 2.0
        a["snow_depth"][c] = 0.01
        a["frac_sno_eff"][c] = 0.2
    return st


def moisture_fixture():
    """test_soil_water_movement.jl:272-336: 12 columns x 10 levels, zero-flux bottom."""
    g = golden()["moisture_form_conservation"]
    nc, nlev, nlevsno = g["nc"], g["nlev"], g["nlevsno"]
    vp = abi.Varpar(nlevsno, nlev, nlev, 5, nlev, 0)
    joff = nlevsno
    st = ColumnState(vp, nc, nc, 1)
    a = st.arrays
    dzv = g["dz"]
    a["mask_hydrology"][:] = 1
    a["col_nbedrock"][:] = nlev
    for j in range(1, nlev + 1):
        a["dz"][joff + j - 1] = dzv
        a["z"][joff + j - 1] = (j - 0.5) * dzv
        a["zi"][joff + j] = j * dzv      # Julia index joff_zi + j
    a["watsat"][:] = g["watsat"]
    a["hksat"][:] = g["hksat"]
    a["bsw"][:] = g["bsw"]
    a["sucsat"][:] = g["sucsat"]
    a["icefrac"][:] = 0.0
    a["zwt"][:] = nlev * dzv
    a["smpmin"][:] = -1.0e8
    for j in range(1, nlev + 1):
        a["h2osoi_liq"][joff + j - 1] = (0.30 + 0.01 * j) * g["watsat"] * dzv * 1000.0
    a["qflx_infl"][:] = g["qflx_infl"]
    return st


def random_band_system(nc, nlev, kl, ku, rng, pivot_frac=0.0):
    """Random banded systems [nlev, nband, nc] / [nlev, nc] (numpy layout of Julia
    [nc, nband, nlev]); a fraction of columns get weak diagonals so pivoting fires."""
    nband = kl + ku + 1
    bm = rng.uniform(-1.0, 1.0, (nlev, nband, nc))
    bm[:, kl, :] = rng.uniform(2.5, 4.0, (nlev, nc)) * np.where(rng.random((nlev, nc)) < 0.5, 1.0, -1.0)
    if pivot_frac > 0:
        weak = rng.random((nlev, nc)) < pivot_frac
        bm[:, kl, :] = np.where(weak, bm[:, kl, :] * 1e-3, bm[:, kl, :])
    rv = rng.uniform(-10.0, 10.0, (nlev, nc))
    return bm, rv


def set_snowpack(st, c, k, rng, t_range=(240.0, 273.0)):
    """Give column c exactly k resolved snow layers (snl = -k), geometry as in the
    synthetic workloads: z = zi_below - dz/2, zi_above = zi_below - dz."""
    a = st.arrays
    nlevsno = st.vp.nlevsno
    zi_below = 0.0
    depth = 0.0
    for j in range(0, -nlevsno, -1):
        r = j + nlevsno - 1
        if j >= -k + 1:
            dz = rng.uniform(0.01, 0.5)
            a["dz"][r, c] = dz
            a["z"][r, c] = zi_below - 0.5 * dz
            a["zi"][r, c] = zi_below - dz
            a["h2osoi_ice"][r, c] = rng.uniform(100.0, 500.0) * dz
            a["h2osoi_liq"][r, c] = 0.0
            a["t_soisno"][r, c] = rng.uniform(*t_range)
            zi_below -= dz
            depth += dz
        else:
            a["dz"][r, c] = a["z"][r, c] = a["zi"][r, c] = 0.0
            a["h2osoi_ice"][r, c] = a["h2osoi_liq"][r, c] = a["t_soisno"][r, c] = 0.0
    a["col_snl"][c] = -k
    a["snow_depth"][c] = depth
    a["frac_sno_eff"][c] = 1.0 if k > 0 else 0.0
