"""GPU test of the packed hydraulic refresh of the work-queue Richards kernel
(CLMGB_OPT_QUEUE_PACKED_REFRESH): a warp refreshes its waiting lanes' columns
together, (column, level) pairs spread over its 32 lanes.  The results are the bits
of the per-lane refresh and the oracle's, for every lower boundary condition, both
flux calculations, ragged bedrock depths, deferral on and off, and any batch size."""
import numpy as np
import pytest

from clmgb import abi, api, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OUT = ("h2osoi_liq", "qcharge", "num_substeps", "smp_l", "hk_l")


def _ragged(wl, seed):
    """Bedrock depths 1..nlevsoi per column, a few columns outside the solve's range
    and a few outside the hydrology mask."""
    rng = np.random.default_rng(seed)
    st = wl.state
    nlev = st.vp.nlevsoi
    nb = rng.integers(1, nlev + 1, st.nc).astype(st["col_nbedrock"].dtype)
    nb[rng.choice(st.nc, 7, replace=False)] = 0
    nb[rng.choice(st.nc, 5, replace=False)] = nlev + 1
    st["col_nbedrock"][:] = nb
    st["mask_hydrology"][rng.choice(st.nc, 11, replace=False)] = 0
    return wl


def _solve(wl, cfg, packed, defer, batch, steps=2):
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        h.set_option(abi.OPT_STEP_SCHEDULE, abi.SCHEDULE_QUEUE)
        h.set_option(abi.OPT_QUEUE_PACKED_REFRESH, packed)
        h.set_option(abi.OPT_QUEUE_DEFER, defer)
        h.set_option(abi.OPT_QUEUE_FRESH_BATCH, batch)
        d = wl.state.to_device()
        G, I = wl.forcing_block(range(steps))
        Gd, Id = torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()
        status = torch.zeros(wl.state.nc, dtype=torch.int32, device="cuda")
        for t in range(steps):
            api.synth_forcing(h, d, Gd[t], Id[t])
            api.soil_temperature(h, d, wl.dtime)
            api.set_soil_water_fractions(h, d)
            api.soil_water(h, d, wl.dtime, cfg, col_status=status)
        torch.cuda.synchronize()
        assert h.get_option(abi.OPT_QUEUE_PACKED_REFRESH) == packed
        return d.to_host(), status.cpu().numpy(), h.device_status()
    finally:
        h.close()


@pytest.mark.parametrize("bc", [abi.BC_ZERO_FLUX, abi.BC_FLUX, abi.BC_WATERTABLE])
@pytest.mark.parametrize("flux", [1, 42])
def test_packed_refresh_keeps_the_bits(bc, flux):
    wl = _ragged(synth.make_workload(2, nc=12000, seed=8, nsteps=2), 3)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = bc
    cfg.flux_calculation = flux
    ref, st_ref, ds_ref = _solve(wl, cfg, 0, 0, 20)
    assert (st_ref & abi.COL_LEVEL_RANGE).any()
    for defer, batch in ((0, 1), (0, 8), (6, 20), (24, 32)):
        out, st, ds = _solve(wl, cfg, 1, defer, batch)
        for k in OUT:
            assert np.array_equal(out[k], ref[k], equal_nan=True), (defer, batch, k)
        assert np.array_equal(st, st_ref) and ds == ds_ref, (defer, batch)


def test_packed_refresh_matches_oracle():
    wl = _ragged(synth.make_workload(2, nc=3000, seed=9, nsteps=1), 4)
    cfg = abi.SwmConfig.clm5_default()
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        h.set_option(abi.OPT_QUEUE_PACKED_REFRESH, 1)
        st = wl.state
        G, I = wl.forcing_block(range(1))
        d = st.to_device()
        api.synth_forcing(h, d, torch.from_numpy(G[0]).cuda(), torch.from_numpy(I[0]).cuda())
        api.soil_temperature(h, d, wl.dtime)
        api.set_soil_water_fractions(h, d)
        host = d.to_host()
        api.soil_water(h, d, wl.dtime, cfg)
        torch.cuda.synchronize()
        out = d.to_host()
        O.soil_water(host, wl.dtime, cfg)
        m = (host["mask_hydrology"] != 0) & (host["col_nbedrock"] >= 1) & (host["col_nbedrock"] <= st.vp.nlevsoi)
        for k in ("h2osoi_liq", "qcharge", "num_substeps", "smp_l", "hk_l"):
            assert np.array_equal(out[k][..., m], host[k][..., m]), k
    finally:
        h.close()


def _logged(wl, cfg, packed, cap):
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        h.set_option(abi.OPT_QUEUE_PACKED_REFRESH, packed)
        d = wl.state.to_device()
        G, I = wl.forcing_block(range(1))
        api.synth_forcing(h, d, torch.from_numpy(G[0]).cuda(), torch.from_numpy(I[0]).cuda())
        log = api.SubstepLog(wl.state.nc, cap)
        log.rec.fill_(float("nan"))
        api.column_step_logged(h, d, wl.dtime, log, cfg)
        torch.cuda.synchronize()
        return d.to_host(), log.rec.cpu().numpy(), log.count.cpu().numpy(), h.device_status()
    finally:
        h.close()


@pytest.mark.parametrize("bc", [abi.BC_FLUX, abi.BC_WATERTABLE])
@pytest.mark.parametrize("cap", [3, 24])
def test_packed_refresh_writes_the_same_substep_log(bc, cap):
    """The logged solve (the step adjoint's recompute) writes the same records."""
    wl = _ragged(synth.make_workload(1, nc=6000, seed=10, nsteps=1), 5)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = bc
    ref, rec_ref, cnt_ref, ds_ref = _logged(wl, cfg, 0, cap)
    out, rec, cnt, ds = _logged(wl, cfg, 1, cap)
    assert (cnt_ref > cap).any() or cap == 24
    assert np.array_equal(cnt, cnt_ref) and ds == ds_ref
    assert np.array_equal(rec, rec_ref, equal_nan=True)
    for k in OUT:
        assert np.array_equal(out[k], ref[k], equal_nan=True), k


@pytest.mark.parametrize("nc", [3000, 2999])
def test_column_records_tensor_copies_and_plain_loads(nc):
    """The Richards pre-pass stages its tiles of 32 columns with 2-D tensor copies
    (CLMGB_OPT_RECORDS_TMA = 1) or plain loads (0); both give the oracle's bits.  3000
    columns end in a partial tile (the copy fills the missing columns with zeros);
    2999 columns give an odd row stride, which the tensor copy cannot address, so the
    pre-pass takes plain loads whatever the option says."""
    wl = _ragged(synth.make_workload(2, nc=nc, seed=21, nsteps=1), 6)
    cfg = abi.SwmConfig.clm5_default()
    st = wl.state
    G, I = wl.forcing_block(range(1))
    host = None
    outs = {}
    for tma in (1, 0):
        h = api.Handle(st.vp)
        try:
            h.reserve(st.nc)
            h.set_option(abi.OPT_RECORDS_TMA, tma)
            d = st.to_device()
            api.synth_forcing(h, d, torch.from_numpy(G[0]).cuda(), torch.from_numpy(I[0]).cuda())
            api.soil_temperature(h, d, wl.dtime)
            api.set_soil_water_fractions(h, d)
            if host is None:
                host = d.to_host()
            api.soil_water(h, d, wl.dtime, cfg)
            torch.cuda.synchronize()
            assert h.get_option(abi.OPT_RECORDS_TMA_USED) == (1 if (tma and nc % 2 == 0) else 0)
            assert h.device_status() & abi.COL_COPY_WAIT == 0
            outs[tma] = d.to_host()
        finally:
            h.close()
    O.soil_water(host, wl.dtime, cfg)
    m = (host["mask_hydrology"] != 0) & (host["col_nbedrock"] >= 1) & (host["col_nbedrock"] <= st.vp.nlevsoi)
    for tma in (1, 0):
        for k in OUT:
            assert np.array_equal(outs[tma][k][..., m], host[k][..., m]), (tma, k)
            assert np.array_equal(outs[tma][k], outs[0][k], equal_nan=True), (tma, k)
