"""GPU tests of the snow layer dynamics after the soil solve (clmgb_snow_layers): the
known answers of test_snow_hydrology.jl through the public routines, and bit-for-bit
parity with the oracle's routine-by-routine restatement for each routine alone and for
the driver's whole sequence under each overburden and wind-drift option."""
import numpy as np
import pytest

import snowlayer_cases as S
from clmgb import abi, api, snowlayers, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(h, host, dtime, cfg, stages):
    d = host.to_device()
    snowlayers.snow_layers(h, d, dtime, cfg, stages)
    torch.cuda.synchronize()
    return d.to_host()


def _same(out, ref, what):
    for (n, _, _, _) in abi.SNOWLAYER_FIELDS:
        assert np.array_equal(out[n], ref[n], equal_nan=True), (what, n)


def test_snow_layers_known_answers():
    g = S.load()
    h = api.Handle(synth.clm5_varpar())
    try:
        for case in g["cases"]:
            sl, cfg, st = S.build(case)
            ref = sl.copy()
            O.snow_layers(ref, 1800.0, cfg, st)
            out = _run(h, sl, 1800.0, cfg, st)
            S.check(case, out)
            _same(out, ref, case["name"])
        assert h.device_status() == 0
    finally:
        h.close()


CFGS = {"default": {}, "vionnet_wind": dict(overburden_method=abi.OVERBURDEN_VIONNET2012,
                                            wind_dependent_snow_density=1),
        "no_subgrid": dict(use_subgrid_fluxes=0), "lake_divide": dict(is_lake=1)}


@pytest.mark.parametrize("name", sorted(CFGS))
def test_snow_layers_sequence_matches_oracle_bits(name):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = snowlayers.random_state(vp, 6000, seed=len(name) + 3)
        cfg = snowlayers.config(ng=host.ng, **CFGS[name])
        ref = host.copy()
        O.snow_layers(ref, 1800.0, cfg, abi.SL_ALL)
        out = _run(h, host, 1800.0, cfg, abi.SL_ALL)
        _same(out, ref, name)
        assert h.device_status() == 0
    finally:
        h.close()


@pytest.mark.parametrize("stage", sorted(snowlayers.STAGES))
def test_snow_layers_single_stage_matches_oracle_bits(stage):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = snowlayers.random_state(vp, 3000, seed=21)
        cfg = snowlayers.config(ng=host.ng, wind_dependent_snow_density=1)
        ref = host.copy()
        O.snow_layers(ref, 1800.0, cfg, snowlayers.STAGES[stage])
        out = _run(h, host, 1800.0, cfg, snowlayers.STAGES[stage])
        _same(out, ref, stage)
    finally:
        h.close()


def test_snow_layers_argument_checks():
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = snowlayers.random_state(vp, 64, seed=2)
        with pytest.raises(api.CLMGBError) as e:
            snowlayers.snow_layers(h, host.to_device(), 1800.0, snowlayers.config(overburden_method=7))
        assert e.value.code == abi.CLMGB_ERR_CONFIG
        with pytest.raises(api.CLMGBError) as e:
            snowlayers.snow_layers(h, host.to_device(), 1800.0, snowlayers.config(), 64)
        assert e.value.code == abi.CLMGB_ERR_CONFIG
        # only the selected stages' pointers are required
        import ctypes as C
        d = host.to_device()
        f = d.fields()
        for n in snowlayers.AEROSOLS + ("snw_rds", "imelt", "swe_old", "frac_iceold", "n_melt", "forc_wind"):
            setattr(f, n, None)
        cfg = snowlayers.config(ng=host.ng)
        b = d.bounds()
        assert h.lib.clmgb_snow_layers(h.h, C.byref(b), C.byref(f), C.byref(cfg), abi.SL_ZERO_EMPTY | abi.SL_FILTER,
                                       1800.0, None) == 0
        assert h.lib.clmgb_snow_layers(h.h, C.byref(b), C.byref(f), C.byref(cfg), abi.SL_DIVIDE,
                                       1800.0, None) == abi.CLMGB_ERR_NULL_ARG
        torch.cuda.synchronize()
        ref = host.copy()
        O.snow_layers(ref, 1800.0, cfg, abi.SL_ZERO_EMPTY | abi.SL_FILTER)
        _same(d.to_host(), ref, "zero_empty+filter")
        host["col_snl"][3] = -vp.nlevsno - 1                 # snl outside -nlevsno..0
        host["mask_snow"][3] = 1
        out = _run(h, host, 1800.0, snowlayers.config(ng=host.ng), abi.SL_COMBINE)
        assert h.device_status() & abi.COL_LEVEL_RANGE
        assert np.array_equal(out["dz"][:, 3], host["dz"][:, 3])
    finally:
        h.close()
