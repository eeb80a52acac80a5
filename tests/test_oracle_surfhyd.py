"""CPU checks of the oracle's restatement of the surface hydrology before soil_water!
(clm_driver.jl:1938-2007): the known answers of CLM.jl's tests for those routines,
the error on unknown methods, and water bookkeeping identities on seeded states."""
import numpy as np
import pytest

import surfhyd_cases as S
from clmgb import abi, surfhyd, synth
from oracle import oracle as O


def test_surface_hydrology_known_answers():
    g = S.load()
    assert len(g["cases"]) == 30
    for case in g["cases"]:
        sh, cfg, st = S.build(case)
        before = sh.copy()
        if case["error"]:
            with pytest.raises(RuntimeError):
                O.surface_hydrology(sh, case["dtime"], cfg, st)
            continue
        O.surface_hydrology(sh, case["dtime"], cfg, st)
        S.check(case, before, sh)


def test_surface_hydrology_identities_on_seeded_state():
    vp = synth.clm5_varpar()
    sh = surfhyd.random_state(vp, 2000, seed=4)
    before = sh.copy()
    dt = 1800.0
    O.surface_hydrology(sh, dt, surfhyd.config(ng=sh.ng), abi.SH_ALL)
    m = sh["mask_hydrology"] != 0
    # surface inputs split between soil and surface water, less evaporation
    np.testing.assert_allclose(sh["qflx_infl"][m], (sh["qflx_in_soil_limited"] + sh["qflx_h2osfc_drain"])[m],
                               rtol=1e-15)
    # the surface-water store changes by inflow - runoff - drainage (up to truncation)
    dh = (sh["h2osfc"] - before["h2osfc"])[m]
    flux = ((sh["qflx_in_h2osfc"] - sh["qflx_h2osfc_surf"] - sh["qflx_h2osfc_drain"]) * dt)[m]
    np.testing.assert_allclose(dh, flux, rtol=0, atol=1e-9)
    assert np.all(sh["fsat"][m] >= 0.0) and np.all(sh["fsat"][m] <= 1.0)
    assert np.all(sh["qflx_infl_excess"][m] >= 0.0)
    # columns outside every filter keep what an earlier step left
    off = (sh["mask_hydrology"] == 0) & (sh["mask_urban"] == 0) & (sh["mask_nolakec"] == 0)
    for k in ("qflx_infl", "qflx_surf", "qflx_floodc", "fsat"):
        assert np.array_equal(sh[k][off], before[k][off]), k
