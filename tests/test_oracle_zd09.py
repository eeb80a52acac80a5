"""CPU checks of the oracle's Zeng-Decker 2009 restatement: the implicit solve
conserves water (its linearised fluxes telescope), all three water-table cases occur,
and the outputs are finite and within the reference's limits."""
import numpy as np

import zd09_cases as Z
from oracle import oracle as O


def test_zd09_oracle_conserves_water():
    for cfg_id, seed in ((0, 3), (1, 4)):
        wl, zs, kind = Z.make(cfg_id, 600, seed)
        zs0 = zs.copy()
        O.soil_water_zd09(zs, wl.dtime)
        resid, scale = Z.balance(zs0, zs, wl.dtime)
        assert np.all(np.abs(resid) <= 1e-10 * scale), np.max(np.abs(resid) / scale)
        assert set(np.unique(kind)) == {0, 1, 2}
        assert np.isfinite(zs["qcharge"]).all() and np.isfinite(zs["h2osoi_liq"]).all()
        assert np.all(np.abs(zs["qcharge"]) <= 10.0 / wl.dtime + 1e-300)
        assert np.all(zs["qflx_deficit"] >= 0.0)
