"""GPU tests of lake_temperature! (clmgb_lake_temperature): the reference's own tests and
bit-for-bit parity with the oracle's kernel-by-kernel restatement on seeded lakes
(frozen, snow-covered, warm, deep) under each lake option."""
import ctypes as C

import numpy as np
import pytest

import lake_cases as L
from clmgb import abi, api, lake, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(h, host, cfg):
    d = host.to_device()
    lake.lake_temperature(h, d, 1800.0, cfg)
    torch.cuda.synchronize()
    return d.to_host()


def _same(out, ref, what):
    for (n, _, _, _) in abi.LAKE_FIELDS:
        assert np.array_equal(out[n], ref[n], equal_nan=True), (what, n)


def test_lake_temperature_reference_cases():
    g = L.load()
    h = api.Handle(L.varpar(g))
    try:
        for case in g["cases"]:
            host = L.build(g, case)
            ref = host.copy()
            O.lake_temperature(ref, 1800.0, lake.config())
            out = _run(h, host, lake.config())
            L.check(case, out)
            _same(out, ref, case["name"])
        assert h.device_status() == 0
    finally:
        h.close()


CFGS = {"default": {}, "lch4": dict(use_lch4=1), "puddling": dict(lakepuddling=1, lake_puddle_thick=0.05),
        "no_ed": dict(lake_no_ed=1, deepmixing_depthcrit=10.0)}


@pytest.mark.parametrize("name", sorted(CFGS))
def test_lake_temperature_matches_oracle_bits(name):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = lake.random_state(vp, 4000, seed=len(name) + 11)
        cfg = lake.config(**CFGS[name])
        ref = host.copy()
        O.lake_temperature(ref, 1800.0, cfg)
        out = _run(h, host, cfg)
        _same(out, ref, name)
        assert h.device_status() == 0
    finally:
        h.close()


def test_lake_temperature_argument_checks():
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = lake.random_state(vp, 64, seed=5)
        d = host.to_device()
        b = d.bounds()
        f = d.fields()
        bad = lake.config(nlevlak=abi.MAX_NLEVLAK + 1)
        assert h.lib.clmgb_lake_temperature(h.h, C.byref(b), C.byref(f), C.byref(bad), 1800.0, None) == \
            abi.CLMGB_ERR_DIMS
        f.lakeresist = None                                  # only use_lch4 writes it
        cfg = lake.config()
        assert h.lib.clmgb_lake_temperature(h.h, C.byref(b), C.byref(f), C.byref(cfg), 1800.0, None) == 0
        cfg4 = lake.config(use_lch4=1)
        assert h.lib.clmgb_lake_temperature(h.h, C.byref(b), C.byref(f), C.byref(cfg4), 1800.0, None) == \
            abi.CLMGB_ERR_NULL_ARG
        torch.cuda.synchronize()
        host["mask_lakec"][4] = 1
        host["col_patchi"][4] = 9                          # a patch of another column
        _run(h, host, cfg)
        assert h.device_status() & abi.COL_PATCH_RANGE
    finally:
        h.close()
