"""GPU test of the deferral of long columns from the work-queue Richards kernel to the
warp-per-column finish (CLMGB_OPT_QUEUE_DEFER): the results are the bits of the solve
without deferral, for every lower boundary condition and both flux calculations, and
the oracle's."""
import numpy as np
import pytest

from clmgb import abi, api, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OUT = ("h2osoi_liq", "qcharge", "num_substeps", "smp_l", "hk_l")


def _cfg(bc, flux):
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = bc
    cfg.flux_calculation = flux
    return cfg


def _solve(wl, cfg, defer, steps=3):
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        h.set_option(abi.OPT_STEP_SCHEDULE, abi.SCHEDULE_QUEUE)
        h.set_option(abi.OPT_QUEUE_DEFER, defer)
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
        assert h.get_option(abi.OPT_QUEUE_DEFER) == defer
        return d.to_host(), status.cpu().numpy(), h.device_status()
    finally:
        h.close()


@pytest.mark.parametrize("bc", [abi.BC_ZERO_FLUX, abi.BC_FLUX, abi.BC_WATERTABLE])
@pytest.mark.parametrize("flux", [1, 42])
def test_deferral_keeps_the_bits(bc, flux):
    wl = synth.make_workload(2, nc=20000, seed=5, nsteps=3)
    cfg = _cfg(bc, flux)
    ref, st_ref, ds_ref = _solve(wl, cfg, 0)
    for defer in (2, 6):
        out, st, ds = _solve(wl, cfg, defer)
        for k in OUT:
            assert np.array_equal(out[k], ref[k], equal_nan=True), (defer, k)
        assert np.array_equal(st, st_ref) and ds == ds_ref


def test_deferral_matches_oracle():
    wl = synth.make_workload(2, nc=4096, seed=6, nsteps=1)
    cfg = abi.SwmConfig.clm5_default()
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        h.set_option(abi.OPT_QUEUE_DEFER, 3)
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
        for k in ("h2osoi_liq", "qcharge", "num_substeps"):
            assert np.array_equal(out[k], host[k]), k
        assert (out["num_substeps"] > 3).any()             # some columns took the deferred path
    finally:
        h.close()
