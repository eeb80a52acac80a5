"""Benchmark: column-steps/s of the soil/snow column solve on GB300.

Workload (default): 262,144 synthetic columns, snl 60% 0 / 40% 1..12, dtime 3600 s,
diurnal ground heat flux and Bernoulli(0.1) infiltration pulses (the 262,144-column
scale/roofline workload).  One step = the synthetic forcing update + soil_temperature!
+ set_soil_water_fractions! + soil_water! (moisture form) over every column, through
the C ABI (clmgb_column_step: a soil-temperature kernel and the work-queue Richards
kernel, schedule chosen by the autotuner before timing).  The same sequence is also
replayed as one captured CUDA graph ("graph" in the output line).  The state (~1.6 GB) is far larger than
L2 (129 MB), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of CLM.jl's Float64 path (the oracle;
the Julia reference itself cannot run here) on the host cores, on a bounded sample
of the same workload.  Under torchrun each rank owns a disjoint column shard
(weak scaling, no collective on the data path).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "clm.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "column-steps/s, plain FP64 vs MLP warm-start at equal error; adjoint/forward time"
UNIT = "column-steps/s"
WORKLOAD = "scale/roofline: 262,144 columns, snl 60% 0 / 40% 1..12, dtime 3600 s, diurnal G, infiltration pulses"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nc", type=int, default=262144)
    ap.add_argument("--cfg", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--cpu-steps", type=int, default=5, help="steps of the CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 probe and the work count")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--schedule", type=int, default=None, help="CLMGB_OPT_STEP_SCHEDULE override")
    ap.add_argument("--queue-bps", type=int, default=None, help="CLMGB_OPT_QUEUE_BLOCKS_PER_SM override")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-reserve", action="store_true", help="run without clmgb_reserve scratch")
    ap.add_argument("--queue-order", type=int, default=None)
    ap.add_argument("--fresh-batch", type=int, default=None, help="CLMGB_OPT_QUEUE_FRESH_BATCH override")
    ap.add_argument("--defer", type=int, default=None, help="CLMGB_OPT_QUEUE_DEFER override")
    ap.add_argument("--st-block", type=int, default=None, choices=[128, 320, 640],
                    help="CLMGB_OPT_ST_BLOCK override (columns sorted together per soil-temperature block)")
    ap.add_argument("--records-tma", type=int, default=None, choices=[0, 1],
                    help="CLMGB_OPT_RECORDS_TMA override (tensor copies or plain loads in the Richards pre-pass)")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint calibration leg")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the adjoint calibration leg and print its JSON (profiling)")
    ap.add_argument("--adj-nc", type=int, default=65536)
    ap.add_argument("--adj-steps", type=int, default=48)
    ap.add_argument("--adj-k", type=int, default=8,
                    help="checkpoint every k steps (8, the calibration workload's interval: 6 checkpoints of "
                         "0.45 GB at 65,536 columns)")
    ap.add_argument("--adj-k2", type=int, default=2,
                    help="a second checkpoint interval reported beside it (0: none)")
    ap.add_argument("--adj-slots", type=int, default=65536)
    ap.add_argument("--adj-entries", type=int, default=256,
                    help="tape entries per slot (the recording kernel only; the default adjoint needs none)")
    ap.add_argument("--no-warm", action="store_true", help="skip the learned warm-start leg")
    ap.add_argument("--warm-train-nc", type=int, default=65536)
    ap.add_argument("--warm-train-steps", type=int, default=1000,
                    help="length of the training trajectory (pairs recorded every --warm-record-every steps)")
    ap.add_argument("--warm-record-every", type=int, default=31)
    ap.add_argument("--warm-eval-steps", type=int, default=1000,
                    help="steps of the warm-start evaluation (the learned warm start's workload: 1,000 steps of "
                         "the scale workload)")
    ap.add_argument("--warm-epochs", type=int, default=3)
    return ap.parse_args()


def richards_launch_count(h, nc):
    """This library's kernels in one clmgb_soil_water call under the handle's schedule."""
    from clmgb import abi
    if h.get_option(abi.OPT_STEP_SCHEDULE) == abi.SCHEDULE_QUEUE and h.get_option(abi.OPT_RESERVED_COLUMNS) >= nc:
        order = 3 if h.get_option(abi.OPT_QUEUE_ORDER) == 1 else 0
        packed = h.get_option(abi.OPT_QUEUE_PACKED_REFRESH) == 1
        return 1 + order + 1 + (1 if packed else 0)
    return 1


def shard_seed(cfg_id, rank):
    """Seed of rank `rank`'s column shard: every rank solves its own disjoint set of
    columns (weak scaling), so a shard's results do not depend on the world size."""
    from clmgb import synth
    return synth.CONFIGS[cfg_id]["seed"] + 1000 * rank


def aggregate_throughput(elapsed_ms, units_per_rank, world, device="cuda"):
    """Whole-job throughput: the units all ranks processed over the slowest rank's
    time (a MAX all-reduce of the timed region; the only collective of the bench).
    Returns (value, max elapsed ms)."""
    if world > 1:
        import torch
        t = torch.tensor([elapsed_ms], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    return units_per_rank * world / (elapsed_ms / 1000.0), elapsed_ms


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """Per-column-step DRAM bytes of the column-step kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return None


def fp64_probe():
    """(DFMA/s, divisions/s, pow/s, log10/s, integer-pipe divisions/s) of this device from
    libclmgb_probe.so, or None."""
    import ctypes as C
    from clmgb import build
    try:
        lib = C.CDLL(build.build_probe())
    except OSError:
        return None
    out = (C.c_double * 5)()
    lib.clmgb_probe_fp64.argtypes = [C.c_int, C.POINTER(C.c_double)]
    if lib.clmgb_probe_fp64(4, out) != 0:
        return None
    return [float(v) for v in out]


def cpu_baseline_sample(wl, cfg, nsample, nsteps=1):
    """Times the oracle (CPU restatement of the reference path) on the first `nsample`
    columns for `nsteps` steps with every host thread."""
    from oracle import oracle as orc
    cols = np.arange(min(nsample, wl.state.nc))
    st = wl.state.subset(cols)
    G, I = wl.forcing_block(range(nsteps), cols=cols)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    orc.run_steps(st, wl.dtime, G, I, cfg, nthreads=threads)
    dt = time.perf_counter() - t0
    state_mb = sum(a.nbytes for a in st.arrays.values()) / 1e6
    return {"value": len(cols) * nsteps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d columns x %d steps of the same workload (its first columns and forcing), OpenMP over "
                      "columns; the sample's state (%.0f MB) fits in the host's caches, unlike the full "
                      "workload's, so the rate is an upper bound of the CPU path's" % (len(cols), nsteps, state_mb)}


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's Float64 path."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from clmgb import abi, synth
    from oracle import oracle as orc
    cfg = abi.SwmConfig.clm5_default()
    nsample = min(args.cpu_sample, args.nc)
    wl = synth.make_workload(args.cfg, nc=nsample, nsteps=args.warmup + args.steps)
    st = wl.state
    threads = os.cpu_count() or 1
    for t in range(args.warmup):
        G, I = wl.forcing_block([t])
        orc.run_steps(st, wl.dtime, G, I, cfg, nthreads=threads)
    t0 = time.perf_counter()
    for t in range(args.warmup, args.warmup + args.steps):
        G, I = wl.forcing_block([t])
        orc.run_steps(st, wl.dtime, G, I, cfg, nthreads=threads)
    dt = time.perf_counter() - t0
    value = nsample * args.steps / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "nc": nsample, "dtime": wl.dtime, "variant": "plain FP64",
                       "note": "CPU restatement of CLM.jl's Float64 path (Julia is not installed)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d columns per step of the same workload" % nsample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def adjoint_leg(args):
    """Calibration gradient: 65,536 columns of the snow / frozen-soil workload, 48 steps
    of 1800 s, free-drainage lower boundary; loss sum_t (drainage + top-10 cm water -
    target)^2 with the target from the same model with bsw, hksat, watsat, sucsat
    perturbed by lognormal(0.2); gradient w.r.t. those 4 x 20 parameters per column,
    checkpoints every k steps.  Times the plain forward (48 production steps) and the
    gradient pass (forward with checkpoints, then reverse)."""
    import torch
    from clmgb import abi, adjoint, api, synth
    nc, nsteps = args.adj_nc, args.adj_steps
    wl = synth.make_workload(1, nc=nc, seed=synth.CONFIGS[1]["seed"] + 4000, nsteps=nsteps)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_FLUX
    h = api.Handle(wl.state.vp)
    h.reserve(nc)
    h.reserve_adjoint(min(nc, args.adj_slots), args.adj_entries)
    G, I = wl.forcing_block(range(nsteps))
    Gd, Id = torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()

    def forcing(t, st):
        api.synth_forcing(h, st, Gd[t], Id[t])
    traj = adjoint.Trajectory(h, nsteps, wl.dtime, forcing, cfg, forcing_reverse=adjoint.synth_forcing_reverse)
    st0 = wl.state.to_device()
    pert = wl.state.copy()
    adjoint.perturb_parameters(pert, np.random.default_rng(4242))
    tl = adjoint.CalibrationLoss(st0, wl.dtime)
    s = pert.to_device()
    for t in range(nsteps):
        traj.step(t, s)
        tl.observe(t, s)
    target = torch.stack(tl.y)
    del s, pert
    # warm-up: two steps forward and back
    warm = adjoint.Trajectory(h, 2, wl.dtime, forcing, cfg, forcing_reverse=adjoint.synth_forcing_reverse)
    wloss = adjoint.CalibrationLoss(st0, wl.dtime, target[:2])
    adjoint.multistep_reverse(warm, st0.copy(), wloss.seed, wloss.observe, checkpoint_every=args.adj_k)
    torch.cuda.synchronize()
    # the plain forward
    st = st0.copy()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for t in range(nsteps):
        traj.step(t, st)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1)
    del st
    # the gradient pass
    loss = adjoint.CalibrationLoss(st0, wl.dtime, target)
    st = st0.copy()
    status = torch.zeros(nc, dtype=torch.int32, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    adj = adjoint.multistep_reverse(traj, st, loss.seed, loss.observe, checkpoint_every=args.adj_k,
                                    col_status=status, events=ev)
    torch.cuda.synchronize()
    fwd_ckpt_ms = ev[0].elapsed_time(ev[1])
    rev_ms = ev[1].elapsed_time(ev[2])
    sts = status.cpu().numpy()
    finite = all(bool(torch.isfinite(adj.grad[p]).all()) for p in adjoint.PARAMS)
    out = {"workload": "adjoint calibration: %d columns, snow + frozen soil, %d steps x %g s, free drainage, "
                       "checkpoints every %d steps" % (nc, nsteps, wl.dtime, args.adj_k),
           "forward_ms": fwd_ms, "forward_with_checkpoints_ms": fwd_ckpt_ms, "reverse_ms": rev_ms,
           "adjoint_over_forward": rev_ms / fwd_ms,
           "gradient_over_forward": (fwd_ckpt_ms + rev_ms) / fwd_ms,
           "loss": float(loss.per_column().sum()),
           "gradients_finite": finite,
           "tape_entries_max": h.get_option(abi.OPT_ADJ_TAPE_USED),
           "tape": {"slots": h.get_option(abi.OPT_ADJ_TAPE_SLOTS), "entries": h.get_option(abi.OPT_ADJ_TAPE_ENTRIES)},
           "columns_flagged": int(np.count_nonzero(sts & (abi.COL_TAPE_FULL | abi.COL_ADJ_UNSUPPORTED |
                                                          abi.COL_ADJ_REPLAY))),
           "note": "adjoint_over_forward = reverse pass / plain forward; gradients checked against "
                   "complex-step and central differences in tests/test_gpu_adjoint_step.py"}
    h.close()
    return out


def adjoint_legs(args):
    """The adjoint leg at the calibration workload's checkpoint interval, and at a
    second interval beside it."""
    out = adjoint_leg(args)
    if args.adj_k2 and args.adj_k2 != args.adj_k:
        import copy
        import torch
        torch.cuda.empty_cache()
        a2 = copy.copy(args)
        a2.adj_k = args.adj_k2
        o2 = adjoint_leg(a2)
        out["other_interval"] = {k: o2[k] for k in ("workload", "forward_ms", "forward_with_checkpoints_ms",
                                                    "reverse_ms", "adjoint_over_forward", "gradient_over_forward")}
    return out


def warm_leg(args, wl_eval):
    """Learned warm start: training pairs from the plain solver on the scale workload's
    column distribution with another seed, GPU training, then the plain and the
    warm-started step timed on the scale workload itself."""
    import torch
    from clmgb import abi, api, mlp, synth
    cfg = abi.SwmConfig.clm5_default()
    h = api.Handle(wl_eval.state.vp)
    h.reserve(max(args.warm_train_nc, wl_eval.state.nc))
    t0 = time.time()
    # ---- training pairs (first substep of every column-step) ----
    wt = synth.make_workload(2, nc=args.warm_train_nc, seed=synth.CONFIGS[2]["seed"] + 777,
                             nsteps=args.warm_train_steps + 4)
    Gt, It = wt.forcing_block(range(args.warm_train_steps + 4))
    Gt, It = torch.from_numpy(Gt).cuda(), torch.from_numpy(It).cuda()
    st = wt.state.to_device()
    F, T = mlp.generate_samples(h, st, Gt, It, args.warm_train_steps, wt.dtime, per_column=1,
                                record_every=args.warm_record_every)
    gen_s = time.time() - t0
    n_pairs = int(F.shape[0])
    model = mlp.WarmStartMLP(h, seed=0)
    t1 = time.time()
    hist = model.train(F, T, epochs=args.warm_epochs, batch=4096, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.time() - t1
    del F, T

    def run(state, G, I, steps, warm, t_first=0, timed=True):
        dt = torch.empty(state.nc, dtype=torch.float64, device="cuda")
        nsub = torch.zeros(state.nc, dtype=torch.float64, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for k in range(steps):
            t = t_first + k
            api.synth_forcing(h, state, G[t], I[t])
            api.soil_temperature(h, state, wl_eval.dtime)
            api.set_soil_water_fractions(h, state)
            if warm:
                model.propose_first_dt(state, wl_eval.dtime, cfg, out=dt)
                mlp.soil_water_warm(h, state, wl_eval.dtime, dt, cfg)
            else:
                api.soil_water(h, state, wl_eval.dtime, cfg)
            nsub += state["num_substeps"]
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), float(nsub.sum()) / (steps * state.nc)

    # ---- decision margin, chosen on the training workload ----
    # (from the state at the end of the training trajectory)
    tune = {}
    for m in (0.0, 0.5, 1.0):
        model.margin = m
        s2 = st.copy()
        ms, att = run(s2, Gt, It, 4, True, t_first=args.warm_train_steps)
        tune[m] = {"ms": ms, "attempts": att}
        del s2
    model.margin = min(tune, key=lambda m: tune[m]["ms"])
    del st
    # ---- evaluation on the scale workload ----
    ne = args.warm_eval_steps
    G, I = wl_eval.forcing_block(range(ne + 2))
    G, I = torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()
    res = {}
    for mode in ("plain", "warm"):
        s2 = wl_eval.state.to_device()
        run(s2, G, I, 2, mode == "warm")               # warm-up
        ms, att = run(s2, G, I, ne, mode == "warm", t_first=2)
        res[mode] = {"ms_per_step": ms / ne, "value": ne * s2.nc / (ms / 1000.0), "attempts_per_column_step": att}
        del s2
    # ---- balance residuals of one warm-started step ----
    s2 = wl_eval.state.to_device()
    dtv = torch.empty(s2.nc, dtype=torch.float64, device="cuda")
    api.synth_forcing(h, s2, G[0], I[0])
    tg0, bw = api.balance_begin(h, s2)
    s2["t_ssbef"].copy_(s2["t_soisno"])          # the driver records these before soil_temperature!
    s2["t_h2osfc_bef"].copy_(s2["t_h2osfc"])
    api.soil_temperature(h, s2, wl_eval.dtime, col_status=None)
    api.set_soil_water_fractions(h, s2)
    model.propose_first_dt(s2, wl_eval.dtime, cfg, out=dtv)
    mlp.soil_water_warm(h, s2, wl_eval.dtime, dtv, cfg)
    es, eh = api.balance_residuals(h, s2, wl_eval.dtime, tg0, bw)
    warm_balance = {"errsoi_max_abs_w_m2": float(es.abs().max()), "errh2o_max_abs_mm": float(eh.abs().max())}
    del s2
    # ---- where the time goes: levels of attempts and of hydraulic refreshes per
    #      column-step in each arm (kernel-counted, an untimed pass of 20 steps) ----
    work = {}
    for mode in ("plain", "warm"):
        s2 = wl_eval.state.to_device()
        run(s2, G, I, 2, mode == "warm")
        h.set_option(abi.OPT_COUNT_WORK, 1)
        run(s2, G, I, 20, mode == "warm", t_first=2)
        la, lr = h.get_option(abi.OPT_WORK_LEVEL_ATTEMPTS), h.get_option(abi.OPT_WORK_LEVEL_REFRESHES)
        h.set_option(abi.OPT_COUNT_WORK, 0)
        nl = float(wl_eval.state["col_nbedrock"].mean())
        work[mode] = {"attempts_per_column_step": la / (20 * s2.nc * nl),
                      "refreshes_per_column_step": lr / (20 * s2.nc * nl)}
        del s2
    # ---- the proposal's share of the warm-started step ----
    s2 = wl_eval.state.to_device()
    api.synth_forcing(h, s2, G[0], I[0])
    api.soil_temperature(h, s2, wl_eval.dtime)
    api.set_soil_water_fractions(h, s2)
    dtv = torch.empty(s2.nc, dtype=torch.float64, device="cuda")
    X = torch.empty((s2.nc, mlp.IN), dtype=torch.bfloat16, device="cuda")
    b, fw = s2.bounds(), s2.soilwater_fields()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        model.propose_first_dt(s2, wl_eval.dtime, cfg, out=dtv)
    reps = 10
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        model.propose_first_dt(s2, wl_eval.dtime, cfg, out=dtv)
    e1.record()
    torch.cuda.synchronize()
    prop_ms = e0.elapsed_time(e1) / reps
    model.features(s2, wl_eval.dtime, cfg, out=X)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        model.forward(X)
    e1.record()
    torch.cuda.synchronize()
    layers_ms = e0.elapsed_time(e1) / reps
    del s2, X
    # ---- error against the FP64 oracle on a sample of columns, and of both arms
    #      against a converged solution (the oracle with both tolerances / 100), after
    #      one step (the per-step error) and after all the evaluated steps (where the
    #      trajectories of different tolerances have drifted apart) ----
    from oracle import oracle as orc
    cols = np.linspace(0, wl_eval.state.nc - 1, 256).astype(np.int64)
    sub = wl_eval.state.subset(cols)
    Gh, Ih = wl_eval.forcing_block(range(ne + 2), cols=cols)
    conv_cfg = abi.SwmConfig.clm5_default()
    conv_cfg.xTolerUpper = cfg.xTolerUpper / 100.0
    conv_cfg.xTolerLower = cfg.xTolerLower / 100.0
    Gs, Is = torch.from_numpy(np.ascontiguousarray(Gh)).cuda(), torch.from_numpy(np.ascontiguousarray(Ih)).cuda()

    def gpu_liq(mode, n):
        d = sub.to_device()
        dtv = torch.empty(d.nc, dtype=torch.float64, device="cuda")
        for t in range(n):
            api.synth_forcing(h, d, Gs[t], Is[t])
            if mode == "plain":
                api.column_step(h, d, wl_eval.dtime, cfg)
            else:
                api.soil_temperature(h, d, wl_eval.dtime)
                api.set_soil_water_fractions(h, d)
                model.propose_first_dt(d, wl_eval.dtime, cfg, out=dtv)
                mlp.soil_water_warm(h, d, wl_eval.dtime, dtv, cfg)
        return d["h2osoi_liq"].cpu().numpy()

    def oracle_liq(c, n):
        o = sub.copy()
        orc.run_steps(o, wl_eval.dtime, Gh[:n], Ih[:n], c)
        return o["h2osoi_liq"]

    errs, errs_conv, errs1, errs1_conv = {}, {}, {}, {}
    for n, e_ref, e_conv in ((1, errs1, errs1_conv), (ne + 2, errs, errs_conv)):
        ref_l, conv_l = oracle_liq(cfg, n), oracle_liq(conv_cfg, n)
        for mode in ("plain", "warm"):
            liq = gpu_liq(mode, n)
            e_ref[mode] = float(np.max(np.abs(liq - ref_l)))
            e_conv[mode] = float(np.max(np.abs(liq - conv_l)))
    out = {"workload": "learned warm start: MLP 64-128-128-21 (SiLU, bf16/fp32), trained on %d pairs from the "
                       "plain solver (%d columns, every %d-th of %d steps, other seed); evaluated on the scale "
                       "workload, %d steps" % (n_pairs, args.warm_train_nc, args.warm_record_every,
                                               args.warm_train_steps, ne),
           "plain": res["plain"], "warm": res["warm"],
           "speedup": res["warm"]["value"] / res["plain"]["value"],
           "attempt_ratio": res["warm"]["attempts_per_column_step"] / res["plain"]["attempts_per_column_step"],
           "work_per_column_step": work,
           "max_abs_liq_error_vs_oracle_mm": errs,
           "max_abs_liq_error_vs_converged_mm": errs_conv,
           "first_step_max_abs_liq_error_vs_oracle_mm": errs1,
           "first_step_max_abs_liq_error_vs_converged_mm": errs1_conv,
           "converged_reference": "the oracle with xTolerUpper and xTolerLower / 100",
           "error_sample_columns": 256, "balance": warm_balance,
           "proposal_ms": prop_ms, "proposal_share_of_warm_step": prop_ms / res["warm"]["ms_per_step"],
           "mlp_layers_ms": layers_ms, "mlp_layers_share_of_warm_step": layers_ms / res["warm"]["ms_per_step"],
           "margin": model.margin, "margin_tuning": tune, "train_loss": hist,
           "sample_generation_s": gen_s, "training_s": train_s,
           "note": "both paths meet the same accept tolerance (xTolerUpper); the warm path only changes the "
                   "first substep each column tries"}
    h.close()
    return out


def run_ours(args):
    import torch
    from clmgb import abi, api, bytes_model, synth
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg = abi.SwmConfig.clm5_default()
    nsteps = args.warmup + args.steps
    seed = shard_seed(args.cfg, rank)
    wl = synth.make_workload(args.cfg, nc=args.nc, seed=seed, nsteps=nsteps)
    st = wl.state
    nc = st.nc
    h = api.Handle(st.vp)
    if not args.no_reserve:
        h.reserve(nc)
    if args.schedule is not None:
        h.set_option(abi.OPT_STEP_SCHEDULE, args.schedule)
    if args.queue_bps is not None:
        h.set_option(abi.OPT_QUEUE_BLOCKS_PER_SM, args.queue_bps)
    if args.queue_order is not None:
        h.set_option(abi.OPT_QUEUE_ORDER, args.queue_order)
    if args.fresh_batch is not None:
        h.set_option(abi.OPT_QUEUE_FRESH_BATCH, args.fresh_batch)
    if args.defer is not None:
        h.set_option(abi.OPT_QUEUE_DEFER, args.defer)
    if args.records_tma is not None:
        h.set_option(abi.OPT_RECORDS_TMA, args.records_tma)
    if args.st_block is not None:
        h.set_option(abi.OPT_ST_BLOCK, args.st_block)
    d = st.to_device()
    # per-step forcing, resident in HBM before the timed region
    Gd = torch.empty((nsteps, nc), dtype=torch.float64, device="cuda")
    Id = torch.empty((nsteps, nc), dtype=torch.float64, device="cuda")
    for t in range(nsteps):
        g, i = wl.forcing(t)
        Gd[t].copy_(torch.from_numpy(g))
        Id[t].copy_(torch.from_numpy(i))
    stream = torch.cuda.current_stream()
    tune = None
    if not args.no_autotune and args.schedule is None and args.queue_bps is None:
        from clmgb import autotune
        tune = autotune.tune_column_step(h, d, wl.dtime, cfg, Gd, Id, steps=2, warm=1)
        # the tridiagonal solver of clmgb_tridiagonal_multi (Thomas or warp-cooperative
        # PCR) for soil-water-sized systems at three batch sizes; Thomas is kept (the
        # reference's bits), the timings say where PCR would be faster
        tune["tridiagonal"] = [autotune.tune_tridiagonal(h, n, st.vp.nlevsoi, exact=True)
                               for n in (nc, 4096, 256)]

    def step(t, ev=None):
        # one timestep through the drop-in entry points, in the driver's order
        api.synth_forcing(h, d, Gd[t], Id[t], stream=stream)
        api.soil_temperature(h, d, wl.dtime, stream=stream)
        api.set_soil_water_fractions(h, d, stream=stream)
        if ev is not None:
            ev[0].record(stream)
        api.soil_water(h, d, wl.dtime, cfg, stream=stream)
        if ev is not None:
            ev[1].record(stream)

    for t in range(args.warmup):
        step(t)
    torch.cuda.synchronize()
    # the state entering the timed steps, for the graph leg to replay the same steps from
    d_timed0 = None if args.no_graph else d.copy()
    d_count0 = None if args.no_fp64 else d.copy()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    t_start.record(stream)
    for k in range(args.steps):
        step(args.warmup + k, evs[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if world > 1:
        torch.distributed.barrier()
    elapsed_ms = t_start.elapsed_time(t_end)
    kern_ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    status = h.device_status()
    # balance residuals of one more step (soil_fluxes.jl errsoi, balance_check.jl errh2o)
    tg0, bw = api.balance_begin(h, d)
    api.synth_forcing(h, d, Gd[nsteps - 1], Id[nsteps - 1], stream=stream)
    api.column_step(h, d, wl.dtime, cfg, stream=stream)
    es, eh = api.balance_residuals(h, d, wl.dtime, tg0, bw)
    balance = {"errsoi_max_abs_w_m2": float(es.abs().max()), "errh2o_max_abs_mm": float(eh.abs().max()),
               "columns_errh2o_above_1e-9_mm": int((eh.abs() > 1e-9).sum()),
               "thresholds": {"errsoi_w_m2": 1e-5, "errh2o_mm": 1e-9},
               "note": "state after the timed steps; the path is bit-identical to the oracle, so these are the "
                       "reference's residuals.  Water residuals come from phase change clamping a level's liquid "
                       "water at zero (liq = max(0, wmass0 - ice), soil_temperature.jl:2168) after the moisture-form "
                       "update left it negative"}
    graph = None
    if not args.no_graph:
        # the same timestep sequence captured once as a CUDA graph and replayed
        from clmgb import autotune
        gsteps = min(args.steps, nsteps - args.warmup)
        g = autotune.capture_steps(h, d, wl.dtime, Gd, Id, gsteps, first_step=args.warmup, cfg=cfg)
        g.replay()
        torch.cuda.synchronize()
        for k, v in d_timed0.arrays.items():     # replay the timed steps from their own start
            d.arrays[k].copy_(v)
        del d_timed0
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        g.replay()
        g1.record(stream)
        torch.cuda.synchronize()
        gms = g0.elapsed_time(g1)
        graph = {"steps": gsteps, "ms_per_step": gms / gsteps,
                 "value": gsteps * nc * world / (gms / 1000.0),
                 "launches_per_step": 2 + richards_launch_count(h, nc),
                 "note": "the timed steps again, from the same state, as clmgb_column_step (fused entry) "
                         "calls replayed from one captured graph"}
        del g
    value, elapsed_ms = aggregate_throughput(elapsed_ms, args.steps * nc, world)

    # FP64 work of the timed Richards calls: the same steps again from the same state
    # (untimed) with the kernel counting the levels of its attempts and refreshes, and
    # the device's DFMA, division and pow rates from the probe (clmgb/flops_model.py)
    fp64 = None
    if d_count0 is not None:
        for k, v in d_count0.arrays.items():
            d.arrays[k].copy_(v)
        del d_count0
        h.set_option(abi.OPT_COUNT_WORK, 1)
        for k in range(args.steps):
            step(args.warmup + k)
        torch.cuda.synchronize()
        la = h.get_option(abi.OPT_WORK_LEVEL_ATTEMPTS)
        lr = h.get_option(abi.OPT_WORK_LEVEL_REFRESHES)
        h.set_option(abi.OPT_COUNT_WORK, 0)
        probe = fp64_probe()
        if probe is not None and la > 0:
            from clmgb import flops_model
            fp64 = flops_model.fp64_roofline(la, lr, args.steps, kern_ms, probe)

    # roofline of the dominant kernel: the work-queue Richards solve (soil_water!)
    bytes_launch = bytes_model.richards_bytes_per_call(nc, st.vp.nlevsoi)
    peak, peak_kind = measured_peaks()
    achieved = bytes_launch / (kern_ms / 1000.0) / 1e9
    kname = {abi.SCHEDULE_FUSED: "k_moisture_form", abi.SCHEDULE_QUEUE: "k_moisture_form_queue",
             abi.SCHEDULE_WAVES: "k_moisture_form_waves"}[h.get_option(abi.OPT_STEP_SCHEDULE)]
    if kname == "k_moisture_form_queue" and h.get_option(abi.OPT_QUEUE_PACKED_REFRESH) and not args.no_reserve:
        kname = "k_moisture_form_packed"
    tr = profile_traffic()
    traffic = None
    if tr and tr.get(kname + "_bytes_per_column"):
        traffic = tr[kname + "_bytes_per_column"] * nc
    step_bytes = bytes_model.bytes_per_step(st["col_snl"], st.vp.nlevgrnd, st.vp.nlevsoi)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_kind": peak_kind, "kernel": kname,
                "kernel_ms": kern_ms, "kernel_share_of_step": kern_ms / (elapsed_ms / args.steps),
                "algorithmic_bytes_per_launch": bytes_launch,
                "step_algorithmic_bytes": step_bytes,
                "step_achieved_gbs": step_bytes / (elapsed_ms / args.steps / 1000.0) / 1e9,
                "fp64": fp64, "fp64_frac": fp64["frac"] if fp64 else None,
                "note": "HBM is not the bound: the kernel runs thousands of FP64 operations per 2 KB of traffic. "
                        "fp64 is its FP64-pipe work in DFMA-equivalents (clmgb/flops_model.py, levels counted by "
                        "the kernel) over its time and the DFMA rate the probe measures on this device; its "
                        "divisions run on the integer pipes (fp64.integer_pipe_divisions_per_launch), and with "
                        "them off the FP64 pipe the kernel is bound by latency at 7-10 warps per SM; ncu "
                        "summaries in profiles/"}

    # end to end with the state in pinned host memory (clmgb.hoststep): each step moves
    # the fields it reads that the rest of the model changes (parameters, geometry and
    # topology stay resident), runs the four drop-in calls, and reads back every field
    # it writes, the soil-temperature outputs overlapped with the Richards solve
    e2e = None
    if args.e2e_steps > 0:
        from clmgb import hoststep
        host = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in st.arrays.items()}
        hs = hoststep.HostStepper(h, host, d, wl.dtime, cfg)

        def e2e_step(k):
            G, I = Gd[k % nsteps], Id[k % nsteps]
            hs.step(stream, forcing=lambda dv: api.synth_forcing(h, dv, G, I, stream=stream))

        for k in range(2):
            e2e_step(k)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(args.e2e_steps):
            e2e_step(k)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1)
        e2e = {"value": args.e2e_steps * nc * world / (e2e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": hs.h2d_bytes, "d2h_bytes_per_step": hs.d2h_bytes,
               "note": "host-resident state: per step H2D of the inputs other modules change, D2H of every "
                       "written field, the soil-temperature outputs read back during the Richards solve; "
                       "parameters/geometry/topology uploaded once"}
        del host, hs

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(wl, cfg, args.cpu_sample, args.cpu_steps)

    state_gb = sum(v.numel() * v.element_size() for v in d.arrays.values()) / 1e9
    adj_line = None
    warm_line = None
    if rank == 0 and (not args.no_adjoint or not args.no_warm):
        del d, Gd, Id
        torch.cuda.empty_cache()
        if not args.no_warm:
            warm_line = warm_leg(args, wl)
            torch.cuda.empty_cache()
        if not args.no_adjoint:
            adj_line = adjoint_legs(args)

    # this library's kernels per timed step: forcing, soil temperature, water fractions,
    # then the Richards call (work queue with reserved scratch: the impedance / column
    # record pass, the three longest-first ordering kernels, the solve, and with the
    # packed refresh the post-pass that writes the columns' outputs from their records)
    richards_launches = richards_launch_count(h, nc)
    launches_per_step = 3 + richards_launches
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "nc_per_gpu": nc, "dtime": wl.dtime, "variant": "plain FP64",
                           "l2": "inputs larger than L2 (state %.2f GB per GPU)" % state_gb,
                           "device_status": status, "parallelism": "replicas over disjoint column shards",
                           "schedule": h.get_option(abi.OPT_STEP_SCHEDULE),
                           "queue_blocks_per_sm": h.get_option(abi.OPT_QUEUE_BLOCKS_PER_SM),
                           "queue_occupancy": h.get_option(abi.OPT_QUEUE_OCCUPANCY),
                           "reserved_columns": h.get_option(abi.OPT_RESERVED_COLUMNS),
                           "queue_order": h.get_option(abi.OPT_QUEUE_ORDER)},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "graph": graph, "autotune": tune,
                "adjoint": adj_line, "warm_start": warm_line, "balance": balance,
                "gpu_launches": launches_per_step * args.steps, "launches_per_step": launches_per_step,
                "clocks": clocks}
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.adjoint_only:
        print(json.dumps(adjoint_legs(args)))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
