"""clmgb_soil_water_flexible_cn (soil_water!'s use_flexibleCN step,
soil_water_movement.jl:1812-1843) on the GPU: the oracle's bits."""
import numpy as np
import pytest

from clmgb import api, flexcn
from oracle import oracle as orc
from test_oracle_flexcn import flexcn_case

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_flexible_cn_matches_oracle_bits():
    fs = flexcn_case(nc=4099, seed=17)
    ref = fs.copy()
    orc.soil_water_flexible_cn(ref)
    h = api.Handle(fs.vp)
    d = fs.to_device()
    flexcn.soil_water_flexible_cn(h, d)
    torch.cuda.synchronize()
    got = d.to_host()
    h.close()
    for k in ("h2osoi_liq", "h2osoi_vol", "wa"):
        assert np.array_equal(got[k].view(np.uint64), ref[k].view(np.uint64)), k
