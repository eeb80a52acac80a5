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
