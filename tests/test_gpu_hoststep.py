"""GPU test of the host-buffer stepper (clmgb.hoststep): a run whose state lives in
pinned host memory, with only the step's inputs moved in and its outputs moved out
(overlapped with the Richards solve), ends with the same bits as a device-resident
run of the same steps."""
import numpy as np
import pytest

from clmgb import abi, api, hoststep, synth
from clmgb.state import ColumnRange

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_host_stepper_matches_device_steps():
    nsteps = 5
    wl = synth.make_workload(2, nc=3000, seed=11, nsteps=nsteps)
    cfg = abi.SwmConfig.clm5_default()
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        G, I = wl.forcing_block(range(nsteps))
        Gd, Id = torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()
        d = wl.state.to_device()
        for t in range(nsteps):
            api.synth_forcing(h, d, Gd[t], Id[t])
            api.soil_temperature(h, d, wl.dtime)
            api.set_soil_water_fractions(h, d)
            api.soil_water(h, d, wl.dtime, cfg)
        host = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in wl.state.arrays.items()}
        hs = hoststep.HostStepper(h, host, wl.state.to_device(), wl.dtime, cfg)
        for t in range(nsteps):
            hs.step(forcing=lambda dv, t=t: api.synth_forcing(h, dv, Gd[t], Id[t]))
        torch.cuda.synchronize()
        written = set(hoststep.WRITTEN_TEMPERATURE) | set(hoststep.WRITTEN_WATER)
        for k in written:
            assert torch.equal(host[k], d[k].cpu()), k
        assert hs.h2d_bytes < 0.4 * hoststep.nbytes(host, list(host))
    finally:
        h.close()


@pytest.mark.parametrize("ranges", [2, 3, 7])
def test_column_ranges_match_whole_calls(ranges):
    """The drop-in calls run over column ranges (column pointers advanced by the range's
    first column, CLMGB_OPT_COLUMN_BASE set to it, patch arrays whole), as a caller that
    splits its columns does: the same bits as calls over all columns."""
    nsteps = 3
    wl = synth.make_workload(2, nc=3001, seed=12, nsteps=nsteps)
    cfg = abi.SwmConfig.clm5_default()
    h = api.Handle(wl.state.vp)
    try:
        h.reserve(wl.state.nc)
        G, I = wl.forcing_block(range(nsteps))
        Gd, Id = torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()
        d = wl.state.to_device()
        for t in range(nsteps):
            api.synth_forcing(h, d, Gd[t], Id[t])
            api.soil_temperature(h, d, wl.dtime)
            api.set_soil_water_fractions(h, d)
            api.soil_water(h, d, wl.dtime, cfg)
        r = wl.state.to_device()
        edges = np.linspace(0, wl.state.nc, ranges + 1).astype(np.int64)
        for t in range(nsteps):
            for a, b in zip(edges[:-1], edges[1:]):
                v = ColumnRange(r, int(a), int(b))
                h.set_option(abi.OPT_COLUMN_BASE, int(a))
                api.synth_forcing(h, v, Gd[t][a:b], Id[t][a:b])
                api.soil_temperature(h, v, wl.dtime)
                api.set_soil_water_fractions(h, v)
                api.soil_water(h, v, wl.dtime, cfg)
        h.set_option(abi.OPT_COLUMN_BASE, 0)
        torch.cuda.synchronize()
        for k in set(hoststep.WRITTEN_TEMPERATURE) | set(hoststep.WRITTEN_WATER):
            assert torch.equal(r[k], d[k]), k
        assert h.device_status() == 0
    finally:
        h.close()
