"""Failure detection on the GPU, with every failure made on the host side.

None of these tests faults, traps or hangs the GPU.  Bad inputs are planted in
host arrays (NaN and infinite state, a zero layer thickness, snow-layer counts and
bedrock depths outside the level range); the attempt cap and the deferred-column
wait are shortened through handle options.  Each test checks the per-column status
the kernels report and that every other column is left bit for bit as a clean run
leaves it, matching the oracle.  The reference's own mechanisms are the non-finite
scan of balance_check! (balance_check.jl:128-160) and substep halving bounded by
dtmin (soil_water_movement.jl:1460-1463); Julia raises BoundsError for level counts
out of range.
"""
import numpy as np
import pytest

from clmgb import abi, api, synth
from oracle import oracle as orc
from parity import bit_mismatches

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

STEP_FIELDS = ["t_soisno", "h2osoi_liq", "h2osoi_ice", "t_grnd", "t_h2osfc", "fact", "imelt", "qcharge",
               "num_substeps", "smp_l", "hk_l", "icefrac"]
WATER_FIELDS = ["h2osoi_liq", "smp_l", "hk_l", "qcharge", "num_substeps"]


def _step(st, wl, reserve=True, options=()):
    """One forcing + column step on the GPU; returns (host state, col_status, device status)."""
    h = api.Handle(st.vp)
    if reserve:
        h.reserve(st.nc)
    for k, v in options:
        h.set_option(k, v)
    d = st.to_device()
    G, I = wl.forcing(0)
    api.synth_forcing(h, d, torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda())
    status = torch.full((st.nc,), 0, dtype=torch.int32, device="cuda")
    api.column_step(h, d, wl.dtime, col_status=status)
    torch.cuda.synchronize()
    dev = h.device_status()
    h.close()
    return d.to_host(), status.cpu().numpy().astype(np.uint32), dev


def _cols_equal(a, b, cols, fields):
    sa, sb = {}, {}
    for k in fields:
        sa[k] = a[k][..., cols]
        sb[k] = b[k][..., cols]
    return bit_mismatches(sa, sb, fields)


def test_bad_inputs_flag_their_columns_and_leave_the_rest():
    wl = synth.make_workload(1, nc=1024, seed=31, nsteps=1)
    clean = wl.state
    joff = clean.vp.nlevsno
    bad = clean.copy()
    bad["t_soisno"][joff + 2, 10] = np.nan          # non-finite temperature
    bad["h2osoi_liq"][joff + 4, 11] = np.inf        # non-finite water
    bad["h2osoi_ice"][joff + 1, 12] = -np.inf
    bad["dz"][joff + 3, 13] = 0.0                   # a zero layer thickness
    bad["col_snl"][14] = -(clean.vp.nlevsno + 1)    # more snow layers than levels
    bad["col_snl"][15] = 1                          # a positive snow-layer count
    bad["col_nbedrock"][16] = 0                     # bedrock depth out of 1..nlevsoi
    bad["col_nbedrock"][17] = clean.vp.nlevsoi + 1
    planted = np.arange(10, 18)
    got_clean, st_clean, dev_clean = _step(clean, wl)
    got_bad, st_bad, dev_bad = _step(bad, wl)
    assert np.all(st_clean == 0) and dev_clean == 0
    for c in (10, 11, 12, 13):
        assert st_bad[c] & abi.COL_NONFINITE, (c, st_bad[c])
    for c in (14, 15, 16, 17):
        assert st_bad[c] & abi.COL_LEVEL_RANGE, (c, st_bad[c])
    others = np.setdiff1d(np.arange(clean.nc), planted)
    assert np.all(st_bad[others] == 0)
    assert dev_bad & abi.COL_NONFINITE and dev_bad & abi.COL_LEVEL_RANGE
    assert not _cols_equal(got_bad, got_clean, others, STEP_FIELDS)
    # columns whose snl is out of range are not touched by soil_temperature!
    for c in (14, 15):
        for k in ("t_soisno", "h2osoi_ice", "fact"):
            assert np.array_equal(got_bad[k][:, c].view(np.uint64), bad[k][:, c].view(np.uint64))
    # the oracle flags the same columns
    ref = bad.copy()
    G, I = wl.forcing_block(range(1))
    s_ref = orc.run_steps(ref, wl.dtime, G, I)
    for c in planted:
        assert (s_ref[c] != 0) and (st_bad[c] != 0)
    ref_clean = clean.copy()
    orc.run_steps(ref_clean, wl.dtime, G, I)
    assert not bit_mismatches(got_clean, ref_clean, STEP_FIELDS)


@pytest.mark.parametrize("schedule", ["packed", "queue", "fused"])
def test_attempt_cap_flags_long_columns_only(schedule):
    wl = synth.make_workload(2, nc=4096, seed=8)
    st = wl.state
    orc.soil_water_fractions(st)
    cfg = abi.SwmConfig.clm5_default()
    ref = st.copy()
    orc.soil_water(ref, wl.dtime, cfg)
    cap = 3
    h = api.Handle(st.vp)
    if schedule == "packed":
        h.reserve(st.nc)
    if schedule == "fused":
        h.set_option(abi.OPT_STEP_SCHEDULE, abi.SCHEDULE_FUSED)
    h.set_option(abi.OPT_ATTEMPT_CAP, cap)
    assert h.get_option(abi.OPT_ATTEMPT_CAP) == cap
    d = st.to_device()
    status = torch.zeros(st.nc, dtype=torch.int32, device="cuda")
    api.soil_water(h, d, wl.dtime, cfg, col_status=status)
    got = d.to_host()
    dev = h.device_status()
    h.close()
    s = status.cpu().numpy().astype(np.uint32)
    m = st["mask_hydrology"] == 1
    long_cols = m & (ref["num_substeps"] > cap)
    short_cols = m & (ref["num_substeps"] <= cap)
    assert long_cols.sum() > 100 and short_cols.sum() > 100
    assert np.all(s[long_cols] & abi.COL_SUBSTEP_CAP)
    assert np.all(s[short_cols] == 0)
    assert dev & abi.COL_SUBSTEP_CAP
    # the capped columns stopped after cap + 1 trips, the others are the oracle's bits
    assert np.all(got["num_substeps"][long_cols] == cap + 1)
    assert not _cols_equal(got, ref, np.nonzero(short_cols)[0], WATER_FIELDS)


def test_attempt_cap_option_range():
    h = api.Handle(synth.clm5_varpar())
    for v in (0, 4097, -1):
        with pytest.raises(api.CLMGBError):
            h.set_option(abi.OPT_ATTEMPT_CAP, v)
    with pytest.raises(api.CLMGBError):
        h.set_option(abi.OPT_QUEUE_POLL_LIMIT, -1)
    with pytest.raises(api.CLMGBError):
        h.set_option(abi.OPT_QUEUE_PUBLISH_DELAY, 20_000_000)
    h.close()


def test_deferred_slot_wait_runs_out_and_every_column_is_finished():
    """A finishing warp that finds a deferred column's index still on its way waits a
    bounded number of polls.  With no polls allowed and the index of every even slot
    written only after a finishing warp has taken the slot (test option), the waits run
    out: the slots are given back, the deferring lanes finish their own columns,
    CLMGB_COL_QUEUE_WAIT is recorded in the device status, the call returns normally
    and every result is the oracle's."""
    wl = synth.make_workload(2, nc=16384, seed=12)
    st = wl.state
    orc.soil_water_fractions(st)
    st["num_substeps"][:] = np.arange(st.nc) % 9
    cfg = abi.SwmConfig.clm5_default()
    ref = st.copy()
    orc.soil_water(ref, wl.dtime, cfg)
    runs = {}
    for name, opts in (("normal", ()),
                       ("given_back", ((abi.OPT_QUEUE_POLL_LIMIT, 0), (abi.OPT_QUEUE_PUBLISH_DELAY, 5_000_000)))):
        h = api.Handle(st.vp)
        h.reserve(st.nc)
        h.set_option(abi.OPT_QUEUE_DEFER, 4)      # many deferred columns
        for k, v in opts:
            h.set_option(k, v)
        d = st.to_device()
        status = torch.full((st.nc,), 3, dtype=torch.int32, device="cuda")
        api.soil_water(h, d, wl.dtime, cfg, col_status=status)
        got = d.to_host()
        dev = h.device_status()
        h.close()
        assert np.all(status.cpu().numpy() == 0), name
        assert not bit_mismatches(got, ref, WATER_FIELDS), name
        runs[name] = dev
    assert runs["normal"] == 0
    assert runs["given_back"] & abi.COL_QUEUE_WAIT
    assert runs["given_back"] & ~np.uint32(abi.COL_QUEUE_WAIT) == 0
