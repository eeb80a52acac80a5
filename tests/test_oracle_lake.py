"""CPU checks of the oracle's restatement of lake_temperature!: the reference's own tests
(test_lake_temperature.jl), energy closure without phase change, and the physical
ranges of ice and temperatures on seeded lakes."""
import numpy as np

import lake_cases as L
from clmgb import lake, synth
from oracle import oracle as O


def test_lake_temperature_reference_cases():
    g = L.load()
    for case in g["cases"]:
        lk = L.build(g, case)
        O.lake_temperature(lk, 1800.0, lake.config())
        L.check(case, lk)


def test_lake_energy_closes_without_phase_change():
    vp = synth.clm5_varpar()
    lk = L.warm_state(vp, 1500, seed=3)
    before = lk.copy()
    O.lake_temperature(lk, 1800.0, lake.config())
    m = (before["mask_lakec"] != 0) & (before["mask_lakep"] != 0)
    assert np.all(lk["errsoi_col"][m] == 0.0)
    # the residual moved into the patch fluxes is below 0.1 W/m2
    assert np.all(np.abs(lk["eflx_gnet"] - before["eflx_gnet"])[m] < 0.1)


def test_lake_ranges_on_seeded_lakes():
    vp = synth.clm5_varpar()
    lk = lake.random_state(vp, 1500, seed=4)
    before = lk.copy()
    O.lake_temperature(lk, 1800.0, lake.config(use_lch4=1))
    m = before["mask_lakec"] != 0
    assert np.all((lk["lake_icefrac"][:, m] >= 0.0) & (lk["lake_icefrac"][:, m] <= 1.0))
    assert np.all(np.isfinite(lk["t_lake"][:, m]))
    assert np.all(lk["lake_icethick"][m] >= 0.0)
    assert np.all(lk["grnd_ch4_cond"][m] >= 0.0)
    # columns outside the lake filter are untouched
    off = ~m
    assert np.array_equal(lk["t_lake"][:, off], before["t_lake"][:, off])
