"""Reverse mode over a trajectory of column steps, with checkpoints.

Mirrors the reference's checkpointed reverse engines (canopy_fluxes_reverse.jl):
  * `reverse_step`         _reverse_step_into! (:447-465): reverse one step from the
                           state it starts from, threading the adjoint backwards;
  * `multistep_reverse`    multistep_reverse! (:495-517) with the coarse checkpoints
                           kept every `checkpoint_every` steps instead of every step
                           (the steps in between are recomputed forward, then reversed);
  * `multistep_reverse_binomial`  multistep_reverse_binomial! (:536-570): recursive
                           bisection, O(log n) live checkpoints.
The per-step reverse is the hand-written GPU kernel behind clmgb_column_step_vjp; the
forward steps are the production clmgb_column_step.  Checkpoints are device copies
of the column state.

The loss is a sum of per-step terms l_t(state after step t, qcharge of step t);
`seed(t, state_after_t, adj)` adds dl_t/d(outputs of step t) into the adjoint buffers
before step t is reversed.  Gradients are taken w.r.t. the hydraulic parameters
watsat, bsw, sucsat, hksat of levels 1..nlevsoi of every column, and the adjoint
left in the buffers at the end is dL/d(initial state).

`calibration_*` build the benchmark's calibration problem: the loss
sum_t sum_c (y_tc - target_tc)^2 with y = drainage of the step (qcharge * dtime, mm;
free-drainage lower boundary, since under the zero-flux boundary qcharge is 0) plus
the water (liquid + ice, mm) of the top 10 cm of soil.
"""
import numpy as np

from . import abi, api

PARAMS = ("watsat", "bsw", "sucsat", "hksat")


class StepAdjointBuffers:
    """Device buffers of clmgb_step_adjoint for a column state."""

    def __init__(self, state):
        import torch
        dev = state["t_soisno"].device
        z = lambda shape: torch.zeros(shape, dtype=torch.float64, device=dev)  # noqa: E731
        nc = state.nc
        L = state["t_soisno"].shape
        nsoi = state.vp.nlevsoi
        self.lam_t_soisno, self.lam_h2osoi_liq, self.lam_h2osoi_ice = z(L), z(L), z(L)
        self.lam_t_grnd, self.lam_t_h2osfc, self.lam_qcharge = z(nc), z(nc), z(nc)
        self.lam_forc_lwrad = z(nc)
        self.grad = {p: z((nsoi, nc)) for p in PARAMS}

    def struct(self):
        s = abi.StepAdjoint()
        s.struct_size = C_sizeof(abi.StepAdjoint)
        for name, _ in abi.STEP_ADJOINT_MEMBERS:
            t = self.grad[name[5:]] if name.startswith("grad_") else getattr(self, name)
            setattr(s, name, _cptr(t))
        return s

    def zero_(self):
        for t in (self.lam_t_soisno, self.lam_h2osoi_liq, self.lam_h2osoi_ice, self.lam_t_grnd, self.lam_t_h2osfc,
                  self.lam_qcharge):
            t.zero_()
        for t in self.grad.values():
            t.zero_()


def C_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)


def _cptr(t):
    import ctypes
    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), abi.c_double_p)


def copy_state_(dst, src, full=False):
    """dst <- src (device to device).  Unless `full`, the geometry, parameter and
    topology fields (hoststep.STATIC) are left as they are: neither the forcing nor the
    column step writes them, so two states of one trajectory hold the same values
    there (the states the reverse passes copy between all descend from one state)."""
    from .hoststep import STATIC
    for k, v in src.arrays.items():
        if full or k not in STATIC:
            dst.arrays[k].copy_(v)


class Trajectory:
    """A sequence of column steps: forcing(t, state) sets step t's inputs, then the
    production column step runs.  When the forcing reads the state (the synthetic
    forcing sets forc_lwrad from t_grnd), forcing_reverse(t, state_before_forcing, adj)
    adds the forcing's share to the adjoint after the step has been reversed."""

    def __init__(self, handle, nsteps, dtime, forcing, cfg=None, snow_method=abi.SNOW_JORDAN1991,
                 forcing_reverse=None):
        self.handle, self.nsteps, self.dtime, self.forcing = handle, nsteps, dtime, forcing
        self.cfg = cfg or abi.SwmConfig.clm5_default()
        self.snow_method = snow_method
        self.forcing_reverse = forcing_reverse

    def step(self, t, state, log=None):
        """Step t in place; with `log` (an api.SubstepLog) the Richards solve also
        writes the substep log the step's reverse can read."""
        self.forcing(t, state)
        if log is None:
            api.column_step(self.handle, state, self.dtime, self.cfg, self.snow_method)
        else:
            api.column_step_logged(self.handle, state, self.dtime, log, self.cfg, self.snow_method)

    def reverse_step(self, t, state_in, adj, col_status=None, log=None):
        """_reverse_step_into!: state_in is the state entering step t (before its forcing);
        `log`: the substep log of step t from the same state, or None."""
        before = None
        if self.forcing_reverse is not None:
            before = {"t_grnd": state_in["t_grnd"].clone()}
        self.forcing(t, state_in)
        api.column_step_vjp(self.handle, state_in, self.dtime, adj, self.cfg, self.snow_method, col_status,
                            log=log)
        if self.forcing_reverse is not None:
            self.forcing_reverse(t, before, adj)


SB = 5.67e-8


def synth_forcing_reverse(t, before, adj):
    """Reverse of clmgb_synth_forcing's forc_lwrad = SB*t_grnd^4."""
    tg = before["t_grnd"]
    adj.lam_t_grnd += 4.0 * SB * tg * tg * tg * adj.lam_forc_lwrad


def multistep_reverse(traj, state, seed, observe=None, checkpoint_every=8, col_status=None, events=None,
                      log_cap=24, log_soil_temperature=True):
    """Forward through traj from `state` (left holding the final state), keeping a
    checkpoint every `checkpoint_every` steps; then reverse, recomputing each segment's
    step-entry states from its checkpoint.  observe(t, state_after_t) runs after every
    forward step (the loss's forward half).  `events`, three CUDA events, are recorded
    at the start, between the forward and the reverse pass, and at the end.  The
    recomputed steps, and the last step of every segment in the forward pass, write
    substep logs (`log_cap` records per column; 0: no logs) so that no reverse runs the
    Richards substep loop again, and with `log_soil_temperature` the soil_temperature!
    records too, so that no reverse runs soil_temperature! again.  Returns the adjoint
    buffers."""
    k = max(1, int(checkpoint_every))
    if events is not None:
        events[0].record()
    ckpt = []
    nseg = (traj.nsteps + k - 1) // k
    # the last step of a segment is not recomputed: the forward pass logs it
    mklog = lambda: api.SubstepLog(state.nc, log_cap, soil_temperature=log_soil_temperature)  # noqa: E731
    last_logs = [mklog() for _ in range(nseg)] if log_cap > 0 else []
    for t in range(traj.nsteps):
        if t % k == 0:
            ckpt.append(state.copy())
        last = t % k == k - 1 or t == traj.nsteps - 1
        traj.step(t, state, last_logs[t // k] if (last_logs and last) else None)
        if observe is not None:
            observe(t, state)
    if events is not None:
        events[1].record()
    adj = StepAdjointBuffers(state)
    seg_states = [state.copy() for _ in range(min(k, traj.nsteps))]
    logs = [mklog() for _ in range(min(k, traj.nsteps) - 1)] if log_cap > 0 else []
    for s in range(len(ckpt) - 1, -1, -1):
        t0, t1 = s * k, min((s + 1) * k, traj.nsteps)
        copy_state_(seg_states[0], ckpt[s])
        for t in range(t0, t1 - 1):
            copy_state_(seg_states[t - t0 + 1], seg_states[t - t0])
            traj.step(t, seg_states[t - t0 + 1], logs[t - t0] if logs else None)
        for t in range(t1 - 1, t0 - 1, -1):
            seed(t, adj)
            lg = None
            if logs:
                lg = logs[t - t0] if t < t1 - 1 else last_logs[s]
            traj.reverse_step(t, seg_states[t - t0], adj, col_status, log=lg)
    if events is not None:
        events[2].record()
    return adj


def multistep_reverse_binomial(traj, state, seed, observe=None, col_status=None, peak=None):
    """Recursive bisection (multistep_reverse_binomial!): O(log nsteps) live states.
    `peak`, a one-element list, receives the most states held at once."""
    b0 = state.copy()
    for t in range(traj.nsteps):
        traj.step(t, state)
        if observe is not None:
            observe(t, state)
    adj = StepAdjointBuffers(state)
    live = [0, 0]

    def bump(d):
        live[0] += d
        live[1] = max(live[1], live[0])

    def rev_seg(lo, hi, b_lo):
        if hi - lo == 1:
            seed(lo, adj)
            tmp = b_lo.copy()
            traj.reverse_step(lo, tmp, adj, col_status)
            return
        mid = (lo + hi) // 2
        b_mid = b_lo.copy()
        bump(1)
        for t in range(lo, mid):
            traj.step(t, b_mid)
        rev_seg(mid, hi, b_mid)
        del b_mid
        bump(-1)
        rev_seg(lo, mid, b_lo)

    bump(1)
    if traj.nsteps >= 1:
        rev_seg(0, traj.nsteps, b0)
    if peak is not None:
        peak[:] = [live[1]]
    return adj


# ---------------------------------------------------------------- calibration problem
def top_layer_weights(state, depth=0.1):
    """Fraction of each soil layer (1..nlevsoi) inside the top `depth` metres, from zi."""
    import torch
    vp = state.vp
    zi = state["zi"]                         # (nlevsno+1+nlevgrnd, nc): level jj holds zi(jj - nlevsno - 1)
    top = zi[vp.nlevsno:vp.nlevsno + vp.nlevsoi]        # interface above layer j (zi(j-1))
    bot = zi[vp.nlevsno + 1:vp.nlevsno + 1 + vp.nlevsoi]   # interface below layer j
    w = (torch.clamp(torch.minimum(bot, torch.full_like(bot, depth)) - top, min=0.0)) / (bot - top)
    return w


class CalibrationLoss:
    """L = sum_t sum_c (y_tc - target_tc)^2,  y = qcharge*dtime + sum_j w_j (liq_j + ice_j)."""

    def __init__(self, state, dtime, target=None):
        import torch
        self.vp = state.vp
        self.dtime = dtime
        self.w = top_layer_weights(state)
        self.target = target
        self.y = []
        self._torch = torch

    def observe_value(self, state):
        vp = self.vp
        j0, j1 = vp.nlevsno, vp.nlevsno + vp.nlevsoi
        water = state["h2osoi_liq"][j0:j1] + state["h2osoi_ice"][j0:j1]
        return state["qcharge"] * self.dtime + (self.w * water).sum(0)

    def observe(self, t, state):
        y = self.observe_value(state)
        if t < len(self.y):
            self.y[t] = y
        else:
            self.y.append(y)

    def per_column(self):
        """Per-column loss (None while no target is set)."""
        if self.target is None:
            return None
        Y = self._torch.stack(self.y)
        return ((Y - self.target) ** 2).sum(0)

    def seed(self, t, adj):
        vp = self.vp
        r = 2.0 * (self.y[t] - self.target[t])
        j0, j1 = vp.nlevsno, vp.nlevsno + vp.nlevsoi
        adj.lam_qcharge.copy_(r * self.dtime)
        adj.lam_h2osoi_liq[j0:j1] += r * self.w
        adj.lam_h2osoi_ice[j0:j1] += r * self.w


def perturb_parameters(state, rng, sigma=0.2):
    """Multiply bsw, hksat, watsat, sucsat of levels 1..nlevsoi by lognormal(0, sigma)
    factors (host state, in place)."""
    nsoi = state.vp.nlevsoi
    for p in PARAMS:
        a = state[p]
        a[:nsoi] = a[:nsoi] * np.exp(rng.normal(0.0, sigma, size=a[:nsoi].shape))
