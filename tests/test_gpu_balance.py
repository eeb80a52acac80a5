"""GPU balance residuals (clmgb_balance_residuals) against the numpy restatement on
the oracle's state: the same numbers, bit for bit, and both within the reference's
warning thresholds (balance_check.jl:713 H2O_WARNING_THRESH 1e-9 mm,
:1352-1360 errsoi 1e-5 W/m2)."""
import numpy as np
import pytest

from balance_reference import residuals, storage
from clmgb import api, synth
from oracle import oracle as orc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg_id", [0, 1, 2])
def test_residuals_match_oracle_and_thresholds(cfg_id):
    h = api.Handle(synth.clm5_varpar())
    try:
        wl = synth.make_workload(cfg_id, nc=384, seed=71 + cfg_id, nsteps=3)
        st = wl.state
        G, I = wl.forcing_block(range(3))
        ref = st.copy()
        d = st.to_device()
        for t in range(3):
            g0, w0 = ref["t_grnd"].copy(), storage(ref)
            orc.run_steps(ref, wl.dtime, G[t:t + 1], I[t:t + 1])
            es_r, eh_r = residuals(ref, wl.dtime, g0, w0)
            api.synth_forcing(h, d, torch.from_numpy(G[t]).cuda(), torch.from_numpy(I[t]).cuda())
            tg0, bw = api.balance_begin(h, d)
            api.column_step(h, d, wl.dtime)
            es, eh = api.balance_residuals(h, d, wl.dtime, tg0, bw)
            es, eh = es.cpu().numpy(), eh.cpu().numpy()
            assert np.array_equal(es, es_r), np.max(np.abs(es - es_r))
            assert np.array_equal(eh, eh_r), np.max(np.abs(eh - eh_r))
            assert np.max(np.abs(eh)) < 1e-9 * max(1.0, float(np.max(w0))), np.max(np.abs(eh))
            assert np.max(np.abs(es)) < 1e-5, np.max(np.abs(es))
    finally:
        h.close()
