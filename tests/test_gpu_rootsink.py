"""GPU tests of compute_effec_rootfrac_and_vert_tran_sink! (clmgb_effec_rootfrac_vert_tran_sink):
the reference's known answers, and bit-for-bit parity with the oracle on seeded
multi-patch inputs for both methods."""
import numpy as np
import pytest

import rootsink_cases as RC
from clmgb import abi, api, rootsink, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(h, rs_host, hydr):
    d = rs_host.to_device()
    status = torch.zeros(rs_host.nc, dtype=torch.int32, device="cuda")
    rootsink.effec_rootfrac_vert_tran_sink(h, d, hydr, col_status=status)
    torch.cuda.synchronize()
    return d.to_host(), status.cpu().numpy()


def test_root_sink_known_answers():
    g = RC.load()
    h = api.Handle(RC.varpar(g))
    try:
        for case in g["cases"]:
            out, st = _run(h, RC.build(g, case), case["use_hydrstress"])
            assert np.all(st == 0), case["name"]
            RC.check(g, case, out)
    finally:
        h.close()


@pytest.mark.parametrize("hydr", [False, True])
def test_root_sink_matches_oracle_bits(hydr):
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = rootsink.random_state(vp, 5000, seed=17 + int(hydr))
        ref = host.copy()
        assert O.rootsink(ref, hydr) == 0
        out, st = _run(h, host, hydr)
        assert np.all(st == 0)
        for k in ("rootr_col", "qflx_rootsoi_col", "qflx_phs_neg_col", "qflx_hydr_redist_patch"):
            assert np.array_equal(out[k], ref[k]), k
        # columns outside the hydrology mask are untouched
        off = host["mask_hydrology"] == 0
        assert np.all(out["qflx_rootsoi_col"][:, off] == 7.0)
    finally:
        h.close()


def test_root_sink_flags_double_filter_and_bad_patch_range():
    vp = synth.clm5_varpar()
    h = api.Handle(vp)
    try:
        host = rootsink.random_state(vp, 64, seed=3)
        host["mask_hydrology"][:] = 1
        host["col_itype"][5] = rootsink.ICOL_ROAD_PERV
        host["col_landunit"][5] = 1                      # natural-vegetation landunit
        host["col_npatches"][9] = host.np + 5            # beyond the patch arrays
        ref = host.copy()
        assert O.rootsink(_fixed(ref), False) == 1
        out, st = _run(h, host, False)
        assert st[5] & abi.COL_FILTER
        assert st[9] & abi.COL_PATCH_RANGE
        assert np.all(np.delete(st, [5, 9]) == 0)
        assert h.device_status() & abi.COL_FILTER
    finally:
        h.close()


def _fixed(rs):
    """The oracle has no range checks: give it the valid patch range back."""
    rs["col_npatches"][9] = 1
    return rs
