"""The use_flexibleCN step of soil_water! (soil_water_movement.jl:1812-1843): the
oracle's restatement against a numpy restatement written from the reference's loops,
bit for bit, on columns with negative liquid water at every level position."""
import numpy as np

from clmgb import flexcn, synth
from oracle import oracle as orc


def flexcn_numpy(fs):
    out = {k: v.copy() for k, v in fs.arrays.items()}
    vp = fs.vp
    joff, nlevsoi = vp.nlevsno, vp.nlevsoi
    liq, m = out["h2osoi_liq"], fs["mask_hydrology"] == 1
    for j in range(1, nlevsoi):
        lj = liq[joff + j - 1]
        xs = np.where(lj >= 0.0, 0.0, 0.001 - lj)
        liq[joff + j - 1] = np.where(m, lj + xs, lj)
        liq[joff + j] = np.where(m, liq[joff + j] - xs, liq[joff + j])
    lj = liq[joff + nlevsoi - 1]
    xs = np.where((lj - 0.001) >= 0.0, 0.0, 0.001 - lj)
    liq[joff + nlevsoi - 1] = np.where(m, lj + xs, lj)
    out["wa"] = np.where(m, out["wa"] - xs, out["wa"])
    for j in range(1, nlevsoi + 1):
        dz = fs["dz"][joff + j - 1]
        v = liq[joff + j - 1] / (dz * 1000.0) + fs["h2osoi_ice"][joff + j - 1] / (dz * 917.0)
        out["h2osoi_vol"][j - 1] = np.where(m, v, out["h2osoi_vol"][j - 1])
    return out


def flexcn_case(nc=512, seed=3):
    wl = synth.make_workload(1, nc=nc, seed=seed)
    st = wl.state
    fs = flexcn.FlexCnState.from_column_state(st)
    rng = np.random.default_rng(seed)
    joff, nsoi = st.vp.nlevsno, st.vp.nlevsoi
    for c in range(nc):                       # a few negative levels per column, bottom included
        for j in rng.choice(nsoi, size=rng.integers(0, 4), replace=False):
            fs["h2osoi_liq"][joff + j, c] = -rng.uniform(0.0, 2.0)
    fs["h2osoi_liq"][joff + nsoi - 1, ::5] = 0.0005          # bottom below watmin, not negative
    fs["mask_hydrology"][::9] = 0
    fs["h2osoi_vol"][:] = -1.0
    return fs


def test_oracle_flexible_cn_matches_numpy_restatement():
    fs = flexcn_case()
    want = flexcn_numpy(fs)
    orc.soil_water_flexible_cn(fs)
    for k in ("h2osoi_liq", "h2osoi_vol", "wa"):
        assert np.array_equal(fs[k].view(np.uint64), want[k].view(np.uint64)), k
    joff, nsoi = fs.vp.nlevsno, fs.vp.nlevsoi
    m = fs["mask_hydrology"] == 1
    assert np.all(fs["h2osoi_liq"][joff:joff + nsoi - 1][:, m] >= 0.0)       # no negative level left above the bottom
    assert np.all(fs["h2osoi_liq"][joff + nsoi - 1][m] >= 0.001 - 1e-15)
    assert np.all(fs["h2osoi_vol"][:, ~m] == -1.0)
