"""clmgb_soil_water_noalloc: the allocation-free soil_water! entry point.

Callers that cannot allocate GPU memory (a runtime that owns the device memory
pool, code running under stream capture, allocator-free embedded hosts) cannot
create a handle, whose scratch comes from cudaMalloc.  This entry point keeps its
scratch in a static device array instead.  Here it is called through the C ABI on
two calls in a row and must give what the handle entry point clmgb_soil_water
gives, within the parity tolerance of the other GPU tests (1e-10 relative,
atol 1e-12).  The file sorts last so a failure here stops a -x run only after every
other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from clmgb import abi, api, synth
from parity import compare

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-10, 1e-12
FIELDS = ["h2osoi_liq", "smp_l", "hk_l", "qcharge", "num_substeps"]


def _noalloc(lib, state, cfg, dtime, status):
    vp, b = state.vp, state.bounds()
    f = state.soilwater_fields()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.clmgb_soil_water_noalloc(C.byref(vp), C.byref(b), C.byref(f), C.byref(cfg), float(dtime),
                                        C.c_void_p(status.data_ptr()), stream)


def test_noalloc_matches_handle_entry_point_on_two_calls():
    assert torch.cuda.is_available()
    wl = synth.make_workload(2, nc=20000, seed=321)
    st = wl.state
    st["mask_hydrology"][::17] = 0
    cfg = abi.SwmConfig.clm5_default()
    a = st.to_device()          # advanced by the handle entry point
    b = st.to_device()          # advanced by the allocation-free entry point
    h = api.Handle(st.vp)
    lib = h.lib
    for call in range(2):
        _, infl = wl.forcing(call)
        for s in (a, b):
            s["qflx_infl"].copy_(torch.from_numpy(infl))
            api.set_soil_water_fractions(h, s)
        status_a = torch.full((st.nc,), 7, dtype=torch.int32, device="cuda")
        status_b = torch.full((st.nc,), 7, dtype=torch.int32, device="cuda")
        api.soil_water(h, a, wl.dtime, cfg, col_status=status_a)
        assert _noalloc(lib, b, cfg, wl.dtime, status_b) == abi.CLMGB_OK
        torch.cuda.synchronize()
        ga, gb = a.to_host(), b.to_host()
        rep, bad = compare(gb, ga, rtol=RTOL, atol=ATOL, fields=FIELDS)
        assert not bad, (call, rep)
        assert np.array_equal(status_a.cpu().numpy(), status_b.cpu().numpy())
        assert np.all(status_b.cpu().numpy() == 0)
    h.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    st = synth.make_workload(0, nc=64).state.to_device()
    lib = api.load()
    cfg = abi.SwmConfig.clm5_default()
    big = abi.Bounds(abi.CLMGB_NOALLOC_MAX_COLUMNS + 1, 1, 1, abi.CLMGB_NOALLOC_MAX_COLUMNS + 1, 1)
    f = st.soilwater_fields()
    rc = lib.clmgb_soil_water_noalloc(C.byref(st.vp), C.byref(big), C.byref(f), C.byref(cfg), 1800.0, None, None)
    assert rc == abi.CLMGB_ERR_DIMS
