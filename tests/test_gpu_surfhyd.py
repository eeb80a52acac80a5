"""GPU tests of the surface hydrology before soil_water! (clmgb_surface_hydrology):
the known answers of CLM.jl's tests for those routines, bit-for-bit parity with the
oracle's routine-by-routine restatement for every stage alone and for the driver's
whole sequence under each method and flag, and the argument checks."""
import ctypes as C

import numpy as np
import pytest

import surfhyd_cases as S
from clmgb import abi, api, surfhyd, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(h, host, dtime, cfg, stages):
    d = host.to_device()
    surfhyd.surface_hydrology(h, d, dtime, cfg, stages)
    torch.cuda.synchronize()
    return d.to_host()


def test_surface_hydrology_known_answers():
    g = S.load()
    h = api.Handle(synth.clm5_varpar())
    try:
        for case in g["cases"]:
            sh, cfg, st = S.build(case)
            if case["error"]:
                with pytest.raises(api.CLMGBError) as e:
                    surfhyd.surface_hydrology(h, sh.to_device(), case["dtime"], cfg, st)
                assert e.value.code == abi.CLMGB_ERR_CONFIG
                continue
            ref = sh.copy()
            O.surface_hydrology(ref, case["dtime"], cfg, st)
            out = _run(h, sh, case["dtime"], cfg, st)
            S.check(case, sh, out)
            for (n, _, _, _) in abi.SURFHYD_FIELDS:
                assert np.array_equal(out[n], ref[n], equal_nan=True), (case["name"], n)
        assert h.device_status() == 0
    finally:
        h.close()


CFGS = {
    "default": {},
    "vic_none": dict(fsat_method=abi.FSAT_VIC, qinmax_method=abi.QINMAX_NONE),
    "zeroed_fsat": dict(crop_fsat_equals_zero=1, hillslope_fsat_equals_zero=1, fff=2.5),
    "h2osfcflag_0": dict(h2osfcflag=0, update_h2osfcflag=0),
    "update_flag_2": dict(update_h2osfcflag=2),
}


@pytest.mark.parametrize("name", sorted(CFGS))
def test_surface_hydrology_sequence_matches_oracle_bits(name):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = surfhyd.random_state(vp, 6000, seed=len(name))
        cfg = surfhyd.config(ng=host.ng, **CFGS[name])
        ref = host.copy()
        O.surface_hydrology(ref, 1800.0, cfg, abi.SH_ALL)
        out = _run(h, host, 1800.0, cfg, abi.SH_ALL)
        for (n, _, _, _) in abi.SURFHYD_FIELDS:
            assert np.array_equal(out[n], ref[n], equal_nan=True), n
        assert h.device_status() == 0
    finally:
        h.close()


@pytest.mark.parametrize("stage", sorted(surfhyd.STAGES))
def test_surface_hydrology_single_stage_matches_oracle_bits(stage):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = surfhyd.random_state(vp, 3000, seed=77)
        cfg = surfhyd.config(ng=host.ng)
        st = surfhyd.STAGES[stage]
        ref = host.copy()
        O.surface_hydrology(ref, 1800.0, cfg, st)
        out = _run(h, host, 1800.0, cfg, st)
        for (n, _, _, _) in abi.SURFHYD_FIELDS:
            assert np.array_equal(out[n], ref[n], equal_nan=True), (stage, n)
    finally:
        h.close()


def test_surface_hydrology_argument_checks():
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = surfhyd.random_state(vp, 64, seed=2)
        d = host.to_device()
        with pytest.raises(api.CLMGBError) as e:                       # unknown stage bit
            surfhyd.surface_hydrology(h, d, 1800.0, surfhyd.config(ng=host.ng), 1024)
        assert e.value.code == abi.CLMGB_ERR_CONFIG
        with pytest.raises(api.CLMGBError) as e:                       # dtime <= 0
            surfhyd.surface_hydrology(h, d, 0.0, surfhyd.config(ng=host.ng))
        assert e.value.code == abi.CLMGB_ERR_CONFIG
        # only the selected stages' pointers are required
        f = d.fields()
        f.topo_slope = None
        b = d.bounds()
        cfg = surfhyd.config(ng=host.ng)
        assert h.lib.clmgb_surface_hydrology(h.h, C.byref(b), C.byref(f), C.byref(cfg), abi.SH_INFILTRATION,
                                             1800.0, None) == 0
        assert h.lib.clmgb_surface_hydrology(h.h, C.byref(b), C.byref(f), C.byref(cfg), abi.SH_UPDATE_H2OSFC,
                                             1800.0, None) == abi.CLMGB_ERR_NULL_ARG
        # a gridcell index outside 1..ng is flagged and the column skipped
        host["col_gridcell"][5] = host.ng + 1
        host["mask_nolakec"][5] = 1
        out = _run(h, host, 1800.0, cfg, abi.SH_FLOODC)
        assert h.device_status() & abi.COL_PATCH_RANGE
        assert out["qflx_floodc"][5] == host["qflx_floodc"][5]
    finally:
        h.close()
