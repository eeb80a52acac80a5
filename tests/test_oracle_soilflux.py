"""CPU checks of the oracle's soil_fluxes! restatement: the scenarios and properties of
test_soil_fluxes.jl, and energy bookkeeping identities on seeded multi-patch states."""
import numpy as np

import soilflux_cases as S
from clmgb import soilflux, synth
from oracle import oracle as O


def test_soil_fluxes_reference_scenarios():
    g = S.load()
    for scen in g["scenarios"]:
        fs = S.build(scen["inputs"])
        O.soil_fluxes(fs, g["dtime"])
        S.check(g, scen, fs)


def test_soil_fluxes_identities_on_seeded_states():
    fs = soilflux.random_state(synth.clm5_varpar(), 800, seed=5)
    O.soil_fluxes(fs, 1800.0)
    m = fs["mask_nolakep"] != 0
    for k in ("eflx_soil_grnd", "errsoi_patch", "eflx_lwrad_out", "qflx_evap_soi"):
        assert np.isfinite(fs[k][m]).all(), k
    np.testing.assert_allclose(fs["qflx_evap_tot"][m], (fs["qflx_evap_veg"] + fs["qflx_evap_soi"])[m], rtol=1e-12)
    np.testing.assert_allclose(fs["eflx_lh_grnd"][m], (fs["qflx_evap_soi"] * fs["htvp"][fs["patch_column"] - 1])[m],
                               rtol=1e-12)
    assert np.all(fs["qflx_liqevap_from_top_layer"][m] >= 0.0)
