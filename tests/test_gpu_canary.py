"""Out-of-bounds writes, caught without a sanitizer: every field of the device state
lives in the middle of a larger buffer whose guard regions hold a sentinel pattern.
The column step (every schedule), the logged step (with its substep log and
soil_temperature! records) and its reverse (with its adjoint buffers), the
allocation-free solve and both tridiagonal solvers run on such buffers, with ragged
bedrock depths, masked columns and a partial last tile of columns; afterwards every
guard must still hold its sentinel, and the column step's results must be the same bits
as a run on plain buffers.  The guards are 64 elements (16-byte aligned, so the tensor copies of the
Richards pre-pass still apply)."""
import ctypes as C

import numpy as np
import pytest

from clmgb import abi, adjoint, api, synth
from clmgb.state import ColumnState

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PAD = 64
SENTINEL = {torch.float64: float.fromhex("-0x1.dead0badcafep+777"), torch.int64: 0x5A5A5A5A5A5A5A5A,
            torch.int32: 0x5A5A5A5A, torch.uint8: 0xA5, torch.float32: -1.2345e30}


def _guarded(dev):
    """A copy of the device state whose arrays sit between two guard regions; returns
    (state, [(field, buffer, numel)])."""
    arrs, bufs = {}, []
    for k, a in dev.arrays.items():
        n = a.numel()
        buf = torch.full((n + 2 * PAD,), SENTINEL[a.dtype], dtype=a.dtype, device=a.device)
        view = buf[PAD:PAD + n].view(a.shape)
        view.copy_(a)
        arrs[k] = view
        bufs.append((k, buf, n))
    return ColumnState(dev.vp, dev.nc, dev.np, dev.nl, arrs), bufs


def _check_guards(bufs):
    bad = []
    for k, buf, n in bufs:
        s = SENTINEL[buf.dtype]
        lo, hi = buf[:PAD], buf[PAD + n:]
        if buf.dtype == torch.float64:
            ok = torch.equal(lo.view(torch.int64), torch.full_like(lo, s).view(torch.int64)) and \
                torch.equal(hi.view(torch.int64), torch.full_like(hi, s).view(torch.int64))
        else:
            ok = bool((lo == s).all()) and bool((hi == s).all())
        if not ok:
            bad.append(k)
    return bad


def _workload(cfg_id, nc, nsteps, seed):
    wl = synth.make_workload(cfg_id, nc=nc, seed=seed, nsteps=nsteps)
    st = wl.state
    rng = np.random.default_rng(seed)
    st["col_nbedrock"][:] = rng.integers(1, st.vp.nlevsoi + 1, nc)
    st["mask_hydrology"][::13] = 0
    G, I = wl.forcing_block(range(nsteps))
    return wl, torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()


@pytest.mark.parametrize("mode", ["packed", "queue", "waves", "fused"])
def test_column_step_writes_only_inside_its_fields(mode):
    nc, nsteps = 1000, 3
    wl, G, I = _workload(1, nc, nsteps, seed=41)
    outs = {}
    for guarded in (False, True):
        h = api.Handle(wl.state.vp)
        if mode in ("packed", "waves", "queue"):
            h.reserve(nc)
        if mode == "queue":
            h.set_option(abi.OPT_QUEUE_PACKED_REFRESH, 0)
        h.set_option(abi.OPT_STEP_SCHEDULE, {"fused": abi.SCHEDULE_FUSED, "waves": abi.SCHEDULE_WAVES}.get(
            mode, abi.SCHEDULE_QUEUE))
        d = wl.state.to_device()
        bufs = []
        if guarded:
            d, bufs = _guarded(d)
        for t in range(nsteps):
            api.synth_forcing(h, d, G[t], I[t])
            api.column_step(h, d, wl.dtime)
        torch.cuda.synchronize()
        if guarded:
            assert _check_guards(bufs) == []
            if mode == "packed":
                assert h.get_option(abi.OPT_RECORDS_TMA_USED) == 1
        h.close()
        outs[guarded] = d.to_host()
    for k in ("t_soisno", "h2osoi_liq", "h2osoi_ice", "smp_l", "hk_l", "qcharge", "num_substeps"):
        assert np.array_equal(outs[True][k].view(np.uint64), outs[False][k].view(np.uint64)), k


def _guard_tensor(t):
    buf = torch.full((t.numel() + 2 * PAD,), SENTINEL[t.dtype], dtype=t.dtype, device=t.device)
    view = buf[PAD:PAD + t.numel()].view(t.shape)
    view.copy_(t)
    return view, buf


def test_logged_step_and_reverse_write_only_inside_their_fields():
    """The logged step writes its state, its substep log and its soil_temperature!
    records; the reverse writes the state and the adjoint buffers: all inside."""
    nc = 700
    wl, G, I = _workload(1, nc, 1, seed=43)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_FLUX
    h = api.Handle(wl.state.vp)
    h.reserve(nc)
    h.reserve_adjoint(1024, 256)
    d1, bufs1 = _guarded(wl.state.to_device())
    log = api.SubstepLog(nc, 4)             # a small cap: some columns run their substep loop again
    gb = []
    log.rec, b = _guard_tensor(log.rec)
    gb.append(("rec", b, log.rec.numel()))
    log.count, b = _guard_tensor(log.count)
    gb.append(("count", b, log.count.numel()))
    log.st_rec, b = _guard_tensor(log.st_rec)
    gb.append(("st_rec", b, log.st_rec.numel()))
    api.synth_forcing(h, d1, G[0], I[0])
    api.column_step_logged(h, d1, wl.dtime, log, cfg)
    torch.cuda.synchronize()
    assert _check_guards(bufs1) == [] and _check_guards(gb) == []
    d2, bufs2 = _guarded(wl.state.to_device())
    adj = adjoint.StepAdjointBuffers(d2)
    ab = []
    for name in ("lam_t_soisno", "lam_h2osoi_liq", "lam_h2osoi_ice", "lam_t_grnd", "lam_t_h2osfc", "lam_qcharge",
                 "lam_forc_lwrad"):
        v, b = _guard_tensor(getattr(adj, name).fill_(1.0))
        setattr(adj, name, v)
        ab.append((name, b, v.numel()))
    for p in adjoint.PARAMS:
        adj.grad[p], b = _guard_tensor(adj.grad[p])
        ab.append((p, b, adj.grad[p].numel()))
    status = torch.zeros(nc, dtype=torch.int32, device="cuda")
    api.synth_forcing(h, d2, G[0], I[0])
    api.column_step_vjp(h, d2, wl.dtime, adj, cfg, col_status=status, log=log)
    torch.cuda.synchronize()
    assert _check_guards(bufs2) == [] and _check_guards(ab) == [] and _check_guards(gb) == []
    for p in adjoint.PARAMS:
        assert torch.isfinite(adj.grad[p]).all()
    h.close()


def test_noalloc_and_tridiagonal_write_only_inside_their_fields():
    nc = 999
    wl, G, I = _workload(2, nc, 1, seed=45)
    vp = wl.state.vp
    d, bufs = _guarded(wl.state.to_device())
    h = api.Handle(vp)
    api.synth_forcing(h, d, G[0], I[0])
    api.soil_temperature(h, d, wl.dtime)
    api.set_soil_water_fractions(h, d)
    cfg = abi.SwmConfig.clm5_default()
    b, fw = d.bounds(), d.soilwater_fields()
    assert h.lib.clmgb_soil_water_noalloc(C.byref(vp), C.byref(b), C.byref(fw), C.byref(cfg), float(wl.dtime),
                                          None, None) == abi.CLMGB_OK
    torch.cuda.synchronize()
    assert _check_guards(bufs) == []
    # tridiagonal systems in guarded buffers, both solvers
    nlevs = 38
    g = torch.Generator().manual_seed(3)
    tri = {}
    for name in "abcr":
        tri[name] = torch.rand((nlevs, nc), generator=g, dtype=torch.float64) - (0.0 if name == "r" else 1.0)
    tri["b"] = 3.0 + tri["b"].abs()
    host = dict(tri, u=torch.zeros((nlevs, nc), dtype=torch.float64),
                jtop=torch.from_numpy(np.arange(nc) % 7 + 1).to(torch.int64),
                mask=torch.from_numpy((np.arange(nc) % 5 != 0).astype(np.uint8)))
    for method in (abi.TRIDIAG_THOMAS, abi.TRIDIAG_PCR):
        h.set_option(abi.OPT_TRIDIAG_METHOD, method)
        views, tb = {}, []
        for k, v in host.items():
            dv = v.cuda()
            buf = torch.full((dv.numel() + 2 * PAD,), SENTINEL[dv.dtype], dtype=dv.dtype, device="cuda")
            view = buf[PAD:PAD + dv.numel()].view(dv.shape)
            view.copy_(dv)
            views[k] = view
            tb.append((k, buf, dv.numel()))
        api.tridiagonal_multi(h, views["u"], views["a"], views["b"], views["c"], views["r"], views["jtop"],
                              views["mask"])
        torch.cuda.synchronize()
        assert _check_guards(tb) == [], method
    h.close()
