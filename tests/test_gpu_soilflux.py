"""GPU tests of soil_fluxes! (clmgb_soil_fluxes): the scenarios and properties of
test_soil_fluxes.jl, and bit-for-bit parity with the oracle's loop-by-loop restatement
on seeded multi-patch states with natural, crop and urban columns."""
import numpy as np
import pytest

import soilflux_cases as S
from clmgb import abi, api, soilflux, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(h, host, dtime):
    d = host.to_device()
    soilflux.soil_fluxes(h, d, dtime)
    torch.cuda.synchronize()
    return d.to_host()


def test_soil_fluxes_reference_scenarios():
    g = S.load()
    h = api.Handle(synth.clm5_varpar())
    try:
        for scen in g["scenarios"]:
            host = S.build(scen["inputs"])
            ref = host.copy()
            O.soil_fluxes(ref, g["dtime"])
            out = _run(h, host, g["dtime"])
            S.check(g, scen, out)
            for (n, _, _, _) in abi.SOILFLUX_FIELDS:
                assert np.array_equal(out[n], ref[n]), (scen["name"], n)
        assert h.device_status() == 0
    finally:
        h.close()


@pytest.mark.parametrize("seed,nc", [(1, 3000), (2, 5000), (3, 257)])
def test_soil_fluxes_matches_oracle_bits(seed, nc):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = soilflux.random_state(vp, nc, seed=seed)
        ref = host.copy()
        O.soil_fluxes(ref, 1800.0)
        out = _run(h, host, 1800.0)
        for (n, _, _, _) in abi.SOILFLUX_FIELDS:
            assert np.array_equal(out[n], ref[n]), n
        assert h.device_status() == 0
    finally:
        h.close()


def test_soil_fluxes_flags_bad_patch_range():
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = soilflux.random_state(vp, 64, seed=4)
        host["mask_nolakec"][7] = 1
        host["col_patchf"][7] = host.np + 3
        _run(h, host, 1800.0)
        assert h.device_status() & abi.COL_PATCH_RANGE
        with pytest.raises(api.CLMGBError):
            soilflux.soil_fluxes(h, host.to_device(), 0.0)
    finally:
        h.close()
