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


def _padded(st, ldc):
    """The host state `st` widened to leading dimension ldc > nc (the extra columns
    filled with a marker), for calls whose bounds say nc columns, ldc stride."""
    from clmgb.state import ColumnState
    arrs = {}
    for k, a in st.arrays.items():
        if st.spec[k][2] == "c":
            w = np.full(a.shape[:-1] + (ldc,), 7 if a.dtype != np.float64 else -7.25, dtype=a.dtype)
            w[..., :st.nc] = a
            arrs[k] = w
        else:
            arrs[k] = a.copy()
    return ColumnState(st.vp, ldc, st.np, st.nl, arrs)


@pytest.mark.parametrize("lower_bc", [abi.BC_ZERO_FLUX, abi.BC_FLUX, abi.BC_WATERTABLE])
def test_noalloc_matches_oracle_under_each_lower_boundary(lower_bc):
    """Against the CPU oracle (soilwater_moisture_form!, compute_qcharge! included),
    bit for bit, with masked columns, ragged bedrock, water tables from the surface to
    below the column, and a leading dimension larger than the column count."""
    wl = synth.make_workload(2, nc=6000, seed=77)
    st = wl.state
    from oracle import oracle as orc
    from parity import bit_mismatches
    orc.soil_water_fractions(st)
    st["mask_hydrology"][::7] = 0
    st["col_nbedrock"][:] = 5 + np.arange(st.nc) % (st.vp.nlevsoi - 4)
    st["zwt"][:] = np.linspace(0.0, 12.0, st.nc)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = lower_bc
    ref = st.copy()
    assert np.all(orc.soil_water(ref, wl.dtime, cfg) == 0)
    ldc = st.nc + 37
    pad = _padded(st, ldc).to_device()
    lib = api.load()
    b = abi.Bounds(st.nc, st.np, st.nl, ldc, st.np)
    f = pad.soilwater_fields()
    status = torch.full((ldc,), 9, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.clmgb_soil_water_noalloc(C.byref(st.vp), C.byref(b), C.byref(f), C.byref(cfg), float(wl.dtime),
                                      C.c_void_p(status.data_ptr()), stream)
    assert rc == abi.CLMGB_OK
    torch.cuda.synchronize()
    got = pad.to_host()
    cut = {k: got[k][..., :st.nc] for k in FIELDS}
    assert not bit_mismatches(cut, ref, FIELDS)
    s = status.cpu().numpy()
    assert np.all(s[:st.nc] == 0) and np.all(s[st.nc:] == 9)
    for k in FIELDS:                      # the padding is never touched
        assert np.all(got[k][..., st.nc:] == -7.25)


def test_noalloc_more_columns_than_threads_and_two_calls():
    """More columns than the solve kernel has threads (each lane takes many columns
    from the queue), ldc > nc, two calls in a row: the handle entry point's bits."""
    nc = 400_000
    wl = synth.make_workload(0, nc=nc, seed=5)
    st = wl.state
    st["mask_hydrology"][::17] = 0
    cfg = abi.SwmConfig.clm5_default()
    ldc = nc + 5
    a = _padded(st, ldc).to_device()
    bdev = _padded(st, ldc).to_device()
    h = api.Handle(st.vp)
    b = abi.Bounds(nc, st.np, st.nl, ldc, st.np)
    from parity import bit_mismatches
    for call in range(2):
        for s_ in (a, bdev):
            f = s_.soilwater_fields()
            api.check(h.lib.clmgb_soil_water_fractions(h.h, C.byref(b), C.byref(f), None), "fractions")
        fa = a.soilwater_fields()
        api.check(h.lib.clmgb_soil_water(h.h, C.byref(b), C.byref(fa), C.byref(cfg), float(wl.dtime), None, None),
                  "soil_water")
        fb = bdev.soilwater_fields()
        rc = h.lib.clmgb_soil_water_noalloc(C.byref(st.vp), C.byref(b), C.byref(fb), C.byref(cfg),
                                            float(wl.dtime), None, None)
        assert rc == abi.CLMGB_OK
        torch.cuda.synchronize()
        ga, gb = a.to_host(), bdev.to_host()
        assert not bit_mismatches(gb, ga, FIELDS), call
    h.close()


def test_noalloc_under_stream_capture():
    """After a first call (which loads the module), the call is captured into a CUDA
    graph by torch.cuda.graph and replayed: the replay gives the eager call's bits."""
    wl = synth.make_workload(1, nc=5000, seed=19)
    st = wl.state
    cfg = abi.SwmConfig.clm5_default()
    lib = api.load()
    eager = st.to_device()
    status = torch.zeros(st.nc, dtype=torch.int32, device="cuda")
    assert _noalloc(lib, eager, cfg, wl.dtime, status) == abi.CLMGB_OK      # first call, outside capture
    torch.cuda.synchronize()
    want = eager.to_host()
    cap = st.to_device()
    start = st.to_device()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc = _noalloc(lib, cap, cfg, wl.dtime, status)
    assert rc == abi.CLMGB_OK
    torch.cuda.current_stream().wait_stream(s)
    for k in cap.arrays:              # the graph advances `cap` from the eager run's start state
        cap[k].copy_(start[k])
    g.replay()
    torch.cuda.synchronize()
    from parity import bit_mismatches
    assert not bit_mismatches(cap.to_host(), want, FIELDS)


def test_noalloc_rejects_the_aquifer_boundary():
    st = synth.make_workload(0, nc=64).state.to_device()
    lib = api.load()
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_AQUIFER
    f = st.soilwater_fields()
    b = st.bounds()
    rc = lib.clmgb_soil_water_noalloc(C.byref(st.vp), C.byref(b), C.byref(f), C.byref(cfg), 1800.0, None, None)
    assert rc == abi.CLMGB_ERR_CONFIG
