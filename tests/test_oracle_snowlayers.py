"""CPU checks of the oracle's restatement of the snow layer dynamics after the soil solve
(clm_driver.jl:2146-2200): the known answers of test_snow_hydrology.jl through the
public routines, and conservation of water, depth and layer bookkeeping on seeded packs."""
import numpy as np

import snowlayer_cases as S
from clmgb import abi, snowlayers, synth
from oracle import oracle as O


def test_snow_layers_known_answers():
    g = S.load()
    assert len(g["cases"]) == 6
    for case in g["cases"]:
        sl, cfg, st = S.build(case)
        O.snow_layers(sl, 1800.0, cfg, st)
        S.check(case, sl)


def test_snow_layers_conserve_water_and_keep_layers_valid():
    vp = synth.clm5_varpar()
    ns = vp.nlevsno
    for seed in range(2):
        sl = snowlayers.random_state(vp, 3000, seed=seed)
        before = sl.copy()
        O.snow_layers(sl, 1800.0, snowlayers.config(ng=sl.ng), abi.SL_ALL)
        m = before["mask_snow"] != 0
        w0, w1 = snowlayers.snow_water(before), snowlayers.snow_water(sl)
        np.testing.assert_allclose(w1[m], w0[m], rtol=1e-14, atol=1e-12)
        snl = sl["col_snl"]
        assert np.all((snl <= 0) & (snl >= -ns))
        act = S.active(sl)
        # active layers are within the thickness limits' reach and ordered by depth
        assert np.all(sl["dz"][:ns][act] > 0.0)
        zi = sl["zi"][:ns + 1]
        assert np.all((zi[1:] - zi[:-1])[act] > 0.0)
        # emptied snow levels are zeroed (zero_empty_snow_layers!)
        emptied = (~act) & (snl > -ns)[None, :] & m[None, :]
        for k in ("dz", "h2osoi_ice", "h2osoi_liq", "t_soisno", "z", "zi"):
            assert np.all(sl[k][:ns][emptied] == 0.0), k
        # the filter follows snl
        nl = sl["mask_nolakec"] != 0
        assert np.array_equal(sl["mask_snow"] != 0, nl & (snl < 0))
        assert np.array_equal(sl["mask_nosnow"] != 0, nl & (snl >= 0))


def test_snow_layers_compaction_only_changes_thickness():
    vp = synth.clm5_varpar()
    sl = snowlayers.random_state(vp, 2000, seed=9)
    before = sl.copy()
    O.snow_layers(sl, 1800.0, snowlayers.config(ng=sl.ng, wind_dependent_snow_density=1), abi.SL_COMPACTION)
    for (n, _, _, _) in abi.SNOWLAYER_FIELDS:
        if n != "dz":
            assert np.array_equal(sl[n], before[n], equal_nan=True), n
    ns = vp.nlevsno
    act = S.active(before)
    m = (before["mask_snow"] != 0)[None, :] & act
    # no layer is compacted below the thickness of its ice and water (melt can also
    # thicken a layer when the melt-time snow cover exceeds frac_sno)
    assert np.any(sl["dz"][:ns][m] < before["dz"][:ns][m])
    fs = np.where(before["frac_sno"] > 0, before["frac_sno"], 1.0)
    solid = (before["h2osoi_ice"][:ns] / 917.0 + before["h2osoi_liq"][:ns] / 1000.0) / fs[None, :]
    assert np.all(sl["dz"][:ns][m] >= solid[m] * (1 - 1e-15))
