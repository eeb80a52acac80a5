"""GPU tests of soil_water! with the Zeng-Decker 2009 method (clmgb_soil_water_zd09):
bit-for-bit parity with the oracle's stage-by-stage restatement, water conservation,
and the configuration checks of init_soilwater_movement."""
import ctypes as C

import numpy as np
import pytest

import zd09_cases as Z
from clmgb import abi, api, zd09
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg_id,seed", [(0, 11), (1, 12), (2, 13)])
def test_zd09_matches_oracle_bits(cfg_id, seed):
    wl, zs, kind = Z.make(cfg_id, 4000, seed)
    h = api.Handle(zs.vp)
    try:
        ref = zs.copy()
        O.soil_water_zd09(ref, wl.dtime)
        d = zs.to_device()
        zd09.soil_water_zd09(h, d, wl.dtime)
        torch.cuda.synchronize()
        out = d.to_host()
        for (n, _, _, _) in abi.ZD09_FIELDS:
            assert np.array_equal(out[n], ref[n], equal_nan=True), n
        resid, scale = Z.balance(zs, out, wl.dtime)
        assert np.all(np.abs(resid) <= 1e-10 * scale)
    finally:
        h.close()


def test_zd09_config_checks():
    wl, zs, _ = Z.make(0, 64, 1)
    h = api.Handle(zs.vp)
    try:
        d = zs.to_device()
        bad = zd09.zd09_config()
        bad.lower_boundary_condition = abi.BC_FLUX       # ZD09 needs the aquifer boundary
        with pytest.raises(api.CLMGBError):
            zd09.soil_water_zd09(h, d, wl.dtime, bad)
        mf = abi.SwmConfig.clm5_default()                 # the moisture form goes to clmgb_soil_water
        with pytest.raises(api.CLMGBError):
            zd09.soil_water_zd09(h, d, wl.dtime, mf)
        st = wl.state.to_device()                         # and clmgb_soil_water rejects ZD09
        with pytest.raises(api.CLMGBError):
            api.soil_water(h, st, wl.dtime, zd09.zd09_config())
    finally:
        h.close()
