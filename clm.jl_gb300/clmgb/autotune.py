"""Autotuner for the column-step schedule.

Times each candidate schedule on a scratch copy of the caller's device state (so
every candidate does the same work) and leaves the fastest one set on the handle:

  * CLMGB_SCHEDULE_QUEUE with 1..4 resident 128-thread blocks per SM of the
    work-queue Richards kernel (fewer resident warps give each lane more columns to
    balance over; more warps hide more latency);
  * CLMGB_SCHEDULE_FUSED (one column per thread, whole step in one kernel);
  * CLMGB_SCHEDULE_WAVES (all columns in synchronous rounds; needs clmgb_reserve).

Results never depend on the choice: the per-column arithmetic is the same in every
schedule, only the order in which columns are visited changes.
"""
import torch

from . import abi, api

DEFAULT_CANDIDATES = [(abi.SCHEDULE_QUEUE, 1), (abi.SCHEDULE_QUEUE, 2), (abi.SCHEDULE_QUEUE, 3),
                      (abi.SCHEDULE_QUEUE, 4), (abi.SCHEDULE_FUSED, 0), (abi.SCHEDULE_WAVES, 0)]


def tune_column_step(handle, state, dtime, cfg=None, G=None, I=None, candidates=None, steps=2, warm=1,
                     stream=None):
    """Returns {"best": (schedule, blocks_per_sm), "ms_per_step": {...}} and sets the best option."""
    cfg = cfg or abi.SwmConfig.clm5_default()
    candidates = candidates or DEFAULT_CANDIDATES
    stream = stream or torch.cuda.current_stream()
    timings = {}
    for sched, bps in candidates:
        handle.set_option(abi.OPT_STEP_SCHEDULE, sched)
        handle.set_option(abi.OPT_QUEUE_BLOCKS_PER_SM, bps)
        scratch = state.copy()
        for t in range(warm + steps):
            if t == warm:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            if G is not None:
                api.synth_forcing(handle, scratch, G[t % G.shape[0]], I[t % I.shape[0]], stream=stream)
            api.column_step(handle, scratch, dtime, cfg, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        timings["%d/%d" % (sched, bps)] = e0.elapsed_time(e1) / steps
        del scratch
    best = min(timings, key=timings.get)
    sched, bps = (int(x) for x in best.split("/"))
    handle.set_option(abi.OPT_STEP_SCHEDULE, sched)
    handle.set_option(abi.OPT_QUEUE_BLOCKS_PER_SM, bps)
    return {"best": {"schedule": sched, "queue_blocks_per_sm": bps}, "ms_per_step": timings}


def capture_steps(handle, state, dtime, G, I, nsteps, first_step=0, cfg=None):
    """Captures `nsteps` column steps (forcing rows first_step.. of G/I, then the step)
    into one CUDA graph; replaying it runs the whole timestep sequence."""
    cfg = cfg or abi.SwmConfig.clm5_default()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            for t in range(first_step, first_step + nsteps):
                api.synth_forcing(handle, state, G[t], I[t])
                api.column_step(handle, state, dtime, cfg)
    torch.cuda.current_stream().wait_stream(s)
    return g


def diagonally_dominant_systems(ncols, nlevs, seed=0, device="cuda"):
    """Random tridiagonal systems [nlevs, ncols] with |b| > |a| + |c| (the shape of the
    soil-water systems), right-hand sides of order one: (a, b, c, r)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    a = -torch.rand((nlevs, ncols), generator=g, dtype=torch.float64)
    c = -torch.rand((nlevs, ncols), generator=g, dtype=torch.float64)
    b = 1.0 + a.abs() + c.abs() + torch.rand((nlevs, ncols), generator=g, dtype=torch.float64)
    r = torch.randn((nlevs, ncols), generator=g, dtype=torch.float64)
    return tuple(x.to(device) for x in (a, b, c, r))


def tune_tridiagonal(handle, ncols, nlevs, exact=True, jtop=1, reps=20, warm=3, stream=None):
    """Times clmgb_tridiagonal_multi on `ncols` columns of `nlevs` levels with Thomas (one
    thread per column) and with parallel cyclic reduction (one warp per column), on
    diagonally dominant systems of that shape.  With exact=False it sets the faster
    method on the handle; with exact=True (the default) it keeps Thomas, whose results
    are the reference's bits, and only reports what PCR would give.  Returns
    {"method": ..., "ms": {"thomas": ..., "pcr": ...}, "faster": ...}."""
    stream = stream or torch.cuda.current_stream()
    a, b, c, r = diagonally_dominant_systems(ncols, nlevs)
    u = torch.zeros_like(r)
    jt = torch.full((ncols,), int(jtop), dtype=torch.int64, device=r.device)
    mask = torch.ones(ncols, dtype=torch.uint8, device=r.device)
    prev = handle.get_option(abi.OPT_TRIDIAG_METHOD)
    ms = {}
    for name, method in (("thomas", abi.TRIDIAG_THOMAS), ("pcr", abi.TRIDIAG_PCR)):
        handle.set_option(abi.OPT_TRIDIAG_METHOD, method)
        for _ in range(warm):
            api.tridiagonal_multi(handle, u, a, b, c, r, jt, mask, stream=stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            api.tridiagonal_multi(handle, u, a, b, c, r, jt, mask, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms[name] = e0.elapsed_time(e1) / reps
    faster = min(ms, key=ms.get)
    method = abi.TRIDIAG_PCR if (faster == "pcr" and not exact) else abi.TRIDIAG_THOMAS
    handle.set_option(abi.OPT_TRIDIAG_METHOD, method if not exact else prev)
    return {"method": "pcr" if method == abi.TRIDIAG_PCR else "thomas", "ms": ms, "faster": faster,
            "ncols": ncols, "nlevs": nlevs}
