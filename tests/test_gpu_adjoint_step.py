"""GPU tests of the reverse mode through the column step (clmgb_column_step_vjp) and
the checkpointed trajectory reverse (clmgb.adjoint).

* The replay inside the adjoint is the production step: it leaves every field bit
  for bit as clmgb_column_step does.
* Gradients are checked against FP64 central finite differences with h = 1e-6
  relative (the reference's own adjoint check, test_enzyme_smoke.jl:216-231, uses
  central FD with the error measure max|g - fd| / max|fd| < 1e-6, per column here).
  A difference quotient is only a derivative where it resolves one: a perturbation
  can move a discrete decision (a substep accepted instead of rejected, a doubled
  substep, a layer that starts to freeze), and a loss that hardly depends on a
  parameter changes by less than its own rounding.  Entries whose quotients at
  h and 2h disagree, or whose substep counts / phase flags change, are left out;
  the tests require that the entries carrying the gradient are resolved and bound
  the share left out.  A column whose loss residual y - target sits at the rounding
  level of y is left out whole: its gradient is 2 (y - target) dy/dtheta with a
  factor that each run rounds differently.
* The moisture-form part is also checked against complex-step derivatives (exact
  to rounding) of a numpy restatement.
* The flat, every-k and bisection checkpoint schedules give the same bits.
"""
import numpy as np
import pytest

from clmgb import abi, adjoint, api, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _cfg_flux():
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_FLUX
    return cfg


@pytest.fixture(scope="module")
def handle():
    assert torch.cuda.is_available()
    h = api.Handle(synth.clm5_varpar())
    h.reserve_adjoint(4096, 8192)
    yield h
    h.close()


def _workload_cfg(cfg_id, nc, nsteps, seed):
    wl = synth.make_workload(cfg_id, nc=nc, seed=seed, nsteps=nsteps)
    G, I = wl.forcing_block(range(nsteps))
    return wl, torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda()


def _workload(nc, nsteps, seed=20241):
    return _workload_cfg(1, nc, nsteps, seed)


def _traj(h, wl, G, I, nsteps, cfg):
    def forcing(t, st):
        api.synth_forcing(h, st, G[t], I[t])
    return adjoint.Trajectory(h, nsteps, wl.dtime, forcing, cfg, forcing_reverse=adjoint.synth_forcing_reverse)


@pytest.mark.parametrize("st_mode", [abi.ADJ_ST_CLOSED_FORM, abi.ADJ_ST_RECORDED])
def test_replay_is_the_production_step(handle, st_mode):
    cfg = _cfg_flux()
    wl, G, I = _workload(700, 6)
    a = wl.state.to_device()
    b = a.copy()
    adj = adjoint.StepAdjointBuffers(a)
    status = torch.zeros(a.nc, dtype=torch.int32, device="cuda")
    handle.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, st_mode)
    try:
        for t in range(6):
            api.synth_forcing(handle, a, G[t], I[t])
            api.column_step(handle, a, wl.dtime, cfg)
            api.synth_forcing(handle, b, G[t], I[t])
            adj.zero_()
            api.column_step_vjp(handle, b, wl.dtime, adj, cfg, col_status=status)
            torch.cuda.synchronize()
            for k in a.arrays:
                assert torch.equal(a[k], b[k]), "step %d field %s" % (t, k)
    finally:
        handle.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_CLOSED_FORM)
    st = status.cpu().numpy()
    assert np.all((st & abi.COL_TAPE_FULL) == 0)
    if st_mode == abi.ADJ_ST_RECORDED:
        assert handle.get_option(abi.OPT_ADJ_TAPE_USED) > 1000


def _params_and_decisions(traj, st0, loss, steps):
    """Forward run: per-column loss plus the discrete record (substeps, imelt)."""
    st = st0.copy()
    loss.y = []
    nsub, imelt = [], []
    for t in range(steps):
        traj.step(t, st)
        loss.observe(t, st)
        nsub.append(st["num_substeps"].clone())
        imelt.append(st["imelt"].clone())
    return loss.per_column(), torch.stack(nsub), torch.stack(imelt)


def _fd_check(traj, st0, loss, steps, grads, params, tol):
    """Central differences at h = 1e-6 relative (the calibration workload's step),
    checked against quotients at 1.37e-6 (not commensurate, so a difference quantised
    to a few ulps of the loss cannot agree with itself by accident) and at 1e-5 (ten
    times the step: rounding noise of the loss is ten times smaller there, and two
    quotients that share the same noise no longer agree).  An entry is resolved when
    the discrete record matches the base run for every step size, the change of the
    loss is at least ~2e8 ulps of it, and the three quotients agree to 1e-7.  Every
    resolved entry must satisfy max|g - fd| <= tol * max|fd| over the resolved entries
    of its column, fd the quotient at h = 1e-6."""
    base_L, base_n, base_m = _params_and_decisions(traj, st0, loss, steps)
    L0 = base_L.cpu().numpy()
    # dL/dtheta = sum 2 (y - target) dy/dtheta: where |y - target| is at the rounding
    # level of y, every run rounds it differently and no quotient can resolve it
    Y = torch.stack(loss.y).cpu().numpy()
    resid = np.abs(Y - loss.target.cpu().numpy()).max(0)
    conditioned = resid >= 1e-6 * np.abs(Y).max(0)
    nc = st0.nc
    nsoi = st0.vp.nlevsoi
    G, F1, F2, F3, OK = [], [], [], [], []
    for p in params:
        for j in range(nsoi):
            theta = st0[p][j].clone()
            fds, same = [], torch.ones(nc, dtype=torch.bool, device="cuda")
            dl = None
            for rel in (1e-6, 1.37e-6, 1e-5):
                h = rel * theta.abs()
                res = []
                for sgn in (1.0, -1.0):
                    st = st0.copy()
                    st[p][j] = theta + sgn * h
                    res.append(_params_and_decisions(traj, st, loss, steps))
                (Lp, np_, mp), (Lm, nm, mm) = res
                same &= ((np_ == nm).all(0) & (np_ == base_n).all(0) &
                         (mp == mm).all(0).all(0) & (mp == base_m).all(0).all(0))
                fds.append(((Lp - Lm) / (2.0 * h)).cpu().numpy())
                if dl is None:
                    dl = (Lp - Lm).abs().cpu().numpy()
            G.append(grads[p][j].cpu().numpy())
            F1.append(fds[0])
            F2.append(fds[1])
            F3.append(fds[2])
            OK.append(same.cpu().numpy() & (dl >= 4e-8 * np.abs(L0)))
    G, F1, F2, F3, OK = (np.array(x) for x in (G, F1, F2, F3, OK))     # [nparam, nc]
    resolved = (OK & (np.abs(F1 - F2) <= 1e-7 * np.abs(F1)) & (np.abs(F1 - F3) <= 1e-7 * np.abs(F1)) &
                conditioned[None, :])
    scale = np.max(np.where(resolved, np.abs(F1), 0.0), axis=0)
    err = np.where(resolved, np.abs(G - F1), 0.0) / np.maximum(scale, 1e-300)
    rel = err.max(axis=0)
    bad = np.where(rel > tol)[0]
    if len(bad):
        lines = []
        for c in bad[:10]:
            k = int(np.argmax(err[:, c]))
            p, j = params[k // nsoi], k % nsoi + 1
            lines.append("col %d %s[%d]: adj %.10e fd(h) %.10e fd(1.37h) %.10e scale %.3e" %
                         (c, p, j, G[k, c], F1[k, c], F2[k, c], scale[c]))
        raise AssertionError("%d columns above tol:\n" % len(bad) + "\n".join(lines))
    # a quotient with h = 1e-6 resolves an entry only where the loss moves by enough
    # ulps (relative sensitivity (theta/L) dL/dtheta above ~1e-2): require that the
    # largest entry is checked in a good share of the columns
    gbig = np.argmax(np.abs(G), axis=0)
    top_resolved = resolved[gbig, np.arange(nc)][conditioned].mean()
    assert top_resolved >= 0.4, top_resolved
    return rel, resolved.mean(), top_resolved


def test_one_step_gradient_vs_finite_differences(handle):
    cfg = _cfg_flux()
    wl, G, I = _workload(64, 1, seed=777)
    traj = _traj(handle, wl, G, I, 1, cfg)
    st0 = wl.state.to_device()
    loss = adjoint.CalibrationLoss(st0, wl.dtime)
    # target: the same model with perturbed parameters
    pert = wl.state.copy()
    adjoint.perturb_parameters(pert, np.random.default_rng(5))
    tl = adjoint.CalibrationLoss(st0, wl.dtime)
    _params_and_decisions(traj, pert.to_device(), tl, 1)
    loss.target = torch.stack(tl.y)
    st = st0.copy()
    adj = adjoint.multistep_reverse(traj, st, loss.seed, loss.observe, checkpoint_every=1)
    rel, frac, top = _fd_check(traj, st0, loss, 1, adj.grad, adjoint.PARAMS, 1e-6)
    print("one step: max rel err %.3g over resolved entries (%.1f%% resolved, largest entry resolved in "
          "%.0f%% of columns)" % (rel.max(), 100 * frac, 100 * top))


def test_calibration_gradient_48_steps_vs_finite_differences(handle):
    cfg = _cfg_flux()
    nsteps = 48
    wl, G, I = _workload(64, nsteps, seed=4242)
    traj = _traj(handle, wl, G, I, nsteps, cfg)
    st0 = wl.state.to_device()
    pert = wl.state.copy()
    adjoint.perturb_parameters(pert, np.random.default_rng(9))
    tl = adjoint.CalibrationLoss(st0, wl.dtime)
    _params_and_decisions(traj, pert.to_device(), tl, nsteps)
    loss = adjoint.CalibrationLoss(st0, wl.dtime, torch.stack(tl.y))
    st = st0.copy()
    status = torch.zeros(st.nc, dtype=torch.int32, device="cuda")
    adj = adjoint.multistep_reverse(traj, st, loss.seed, loss.observe, checkpoint_every=8, col_status=status)
    assert int((status.cpu().numpy() & (abi.COL_TAPE_FULL | abi.COL_ADJ_UNSUPPORTED)).sum()) == 0
    for p in adjoint.PARAMS:
        assert torch.isfinite(adj.grad[p]).all()
    rel, frac, top = _fd_check(traj, st0, loss, nsteps, adj.grad, adjoint.PARAMS, 1e-6)
    print("48 steps: max rel err %.3g over resolved entries (%.1f%% resolved, largest entry resolved in "
          "%.0f%% of columns)" % (rel.max(), 100 * frac, 100 * top))


def test_richards_gradient_vs_complex_step(handle):
    """Exact reference: the moisture-form solve restated in complex arithmetic
    (tests/adjoint_reference.py, pinned to the oracle), differentiated by complex step
    for every parameter of every level.  On the no-frost workload the soil-temperature
    step leaves the water alone, so this is the whole step's gradient of the
    calibration loss."""
    from adjoint_reference import moisture_form
    cfg = _cfg_flux()
    nc = 16
    wl, G, I = _workload_cfg(0, nc, 1, seed=1234)
    traj = _traj(handle, wl, G, I, 1, cfg)
    st0 = wl.state.to_device()
    loss = adjoint.CalibrationLoss(st0, wl.dtime, torch.zeros((1, nc), dtype=torch.float64, device="cuda"))
    st = st0.copy()
    status = torch.zeros(nc, dtype=torch.int32, device="cuda")
    adj = adjoint.multistep_reverse(traj, st, loss.seed, loss.observe, checkpoint_every=1, col_status=status)
    assert int(status.cpu().numpy().sum()) == 0
    h0 = wl.state
    w = loss.w.cpu().numpy()
    Ih = I.cpu().numpy()[0]
    joff = h0.vp.nlevsno
    nsoi = h0.vp.nlevsoi
    worst = 0.0
    for c in range(nc):
        nl = int(h0["col_nbedrock"][c])
        lv = slice(joff, joff + nl)
        base = {p: h0[p][:nl, c].astype(complex) for p in adjoint.PARAMS}

        def y_of(theta):
            liq, qc, _ = moisture_form(h0["h2osoi_liq"][lv, c], h0["dz"][lv, c], h0["z"][lv, c],
                                       theta["watsat"], theta["bsw"], theta["sucsat"], theta["hksat"],
                                       np.ones(nl), Ih[c], h0["qflx_rootsoi"][:nl, c], wl.dtime, cfg, "flux")
            y = qc * wl.dtime + np.sum(w[:nl, c] * (liq + h0["h2osoi_ice"][lv, c]))
            return y * y
        ref = np.zeros((len(adjoint.PARAMS), nsoi))
        for k, p in enumerate(adjoint.PARAMS):
            for j in range(nl):
                th = {q: v.copy() for q, v in base.items()}
                th[p][j] += 1e-30j
                ref[k, j] = y_of(th).imag / 1e-30
        got = np.array([adj.grad[p][:, c].cpu().numpy() for p in adjoint.PARAMS])
        assert np.isfinite(got).all(), c
        e = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert np.isfinite(e), c
        worst = max(worst, e)
    print("complex-step: max rel err %.3g" % worst)
    assert worst < 1e-9


@pytest.mark.parametrize("bc", [abi.BC_FLUX, abi.BC_WATERTABLE, abi.BC_ZERO_FLUX])
def test_closed_form_substep_reverse_matches_recorded_replay(handle, bc):
    """The hand-written reverse of a Richards substep and the recorded replay of the
    same substep differentiate the same arithmetic: they agree to rounding (both with
    soil_temperature! recorded, so only the substep reverse differs), for each lower
    boundary condition."""
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = bc
    nsteps = 4
    wl, G, I = _workload(256, nsteps, seed=555)
    traj = _traj(handle, wl, G, I, nsteps, cfg)
    st0 = wl.state.to_device()
    if bc == abi.BC_WATERTABLE:
        st0["zwt"][::2] += 1.5     # water table below the soil column: drainage to it is active
    tgt = torch.zeros((nsteps, st0.nc), dtype=torch.float64, device="cuda")
    out = {}
    handle.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_RECORDED)
    try:
        for mode in (abi.ADJ_RICHARDS_CLOSED_FORM, abi.ADJ_RICHARDS_RECORDED):
            handle.set_option(abi.OPT_ADJ_RICHARDS, mode)
            loss = adjoint.CalibrationLoss(st0, wl.dtime, tgt)
            status = torch.zeros(st0.nc, dtype=torch.int32, device="cuda")
            adj = adjoint.multistep_reverse(traj, st0.copy(), loss.seed, loss.observe, checkpoint_every=2,
                                            col_status=status)
            assert int(status.cpu().numpy().sum()) == 0
            out[mode] = np.array([adj.grad[p].cpu().numpy() for p in adjoint.PARAMS] +
                                 [adj.lam_h2osoi_liq.cpu().numpy()[st0.vp.nlevsno:st0.vp.nlevsno + 20]])
    finally:
        handle.set_option(abi.OPT_ADJ_RICHARDS, abi.ADJ_RICHARDS_CLOSED_FORM)
        handle.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_CLOSED_FORM)
    a, b = out[abi.ADJ_RICHARDS_CLOSED_FORM], out[abi.ADJ_RICHARDS_RECORDED]
    assert np.isfinite(a).all() and np.isfinite(b).all()
    scale = np.max(np.abs(b), axis=(0, 1))
    rel = np.max(np.abs(a - b), axis=(0, 1)) / np.maximum(scale, 1e-300)
    print("closed form vs recorded: max rel diff %.3g" % rel.max())
    assert rel.max() < 1e-11


def test_checkpoint_schedules_give_the_same_bits(handle):
    cfg = _cfg_flux()
    nsteps = 13
    wl, G, I = _workload(300, nsteps, seed=99)
    traj = _traj(handle, wl, G, I, nsteps, cfg)
    st0 = wl.state.to_device()
    tgt = torch.zeros((nsteps, st0.nc), dtype=torch.float64, device="cuda")
    outs = []
    for sched in ("k1", "k8", "k5", "binomial"):
        loss = adjoint.CalibrationLoss(st0, wl.dtime, tgt)
        st = st0.copy()
        if sched == "binomial":
            peak = [0]
            adj = adjoint.multistep_reverse_binomial(traj, st, loss.seed, loss.observe, peak=peak)
            assert peak[0] <= 1 + int(np.ceil(np.log2(nsteps)))
        else:
            adj = adjoint.multistep_reverse(traj, st, loss.seed, loss.observe, checkpoint_every=int(sched[1:]))
        outs.append((adj, st))
    ref, ref_st = outs[0]
    for adj, st in outs[1:]:
        for p in adjoint.PARAMS:
            assert torch.equal(adj.grad[p], ref.grad[p])
        assert torch.equal(adj.lam_t_soisno, ref.lam_t_soisno)
        assert torch.equal(adj.lam_h2osoi_liq, ref.lam_h2osoi_liq)
        assert torch.equal(st["t_soisno"], ref_st["t_soisno"])


def test_tape_overflow_and_unsupported_state_are_flagged():
    h = api.Handle(synth.clm5_varpar())
    try:
        cfg = _cfg_flux()
        wl, G, I = _workload(128, 1, seed=5)
        st = wl.state.to_device()
        st["frac_h2osfc"][3] = 0.2
        st["h2osfc"][3] = 5.0
        api.synth_forcing(h, st, G[0], I[0])
        adj = adjoint.StepAdjointBuffers(st)
        status = torch.zeros(st.nc, dtype=torch.int32, device="cuda")
        h.reserve_adjoint(128, 256)
        h.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_RECORDED)   # only the recording kernel has a tape
        api.column_step_vjp(h, st.copy(), wl.dtime, adj, cfg, col_status=status)
        s = status.cpu().numpy()
        assert np.all(s & abi.COL_TAPE_FULL)
        h.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_CLOSED_FORM)
        api.column_step_vjp(h, st.copy(), wl.dtime, adj, cfg, col_status=status)
        s = status.cpu().numpy()
        assert s[3] & abi.COL_ADJ_UNSUPPORTED
        assert np.all((np.delete(s, 3) & (abi.COL_ADJ_UNSUPPORTED | abi.COL_TAPE_FULL)) == 0)
        h.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_RECORDED)
        h.reserve_adjoint(128, 8192)
        api.column_step_vjp(h, st.copy(), wl.dtime, adj, cfg, col_status=status)
        s = status.cpu().numpy()
        assert s[3] & abi.COL_ADJ_UNSUPPORTED
        assert np.all((np.delete(s, 3) & (abi.COL_ADJ_UNSUPPORTED | abi.COL_TAPE_FULL)) == 0)
    finally:
        h.close()


def test_vjp_requires_reserved_tape():
    h = api.Handle(synth.clm5_varpar())
    try:
        wl, G, I = _workload(32, 1)
        st = wl.state.to_device()
        adj = adjoint.StepAdjointBuffers(st)
        with pytest.raises(api.CLMGBError):
            api.column_step_vjp(h, st, wl.dtime, adj)
    finally:
        h.close()


class _LinearSeed:
    """A fixed random linear functional of every step's outputs: temperatures, liquid
    water, ice, t_grnd, t_h2osfc and qcharge all carry adjoint."""

    def __init__(self, st0, nsteps, seed):
        rng = np.random.default_rng(seed)
        shp = tuple(st0["t_soisno"].shape)
        nc = st0.nc
        t = lambda *s: torch.from_numpy(rng.normal(size=s)).cuda()  # noqa: E731
        self.w = [dict(t=t(*shp), l=t(*shp), i=t(*shp), g=t(nc), h=t(nc), q=t(nc)) for _ in range(nsteps)]

    def seed(self, t, adj):
        w = self.w[t]
        adj.lam_t_soisno += w["t"]
        adj.lam_h2osoi_liq += w["l"]
        adj.lam_h2osoi_ice += w["i"]
        adj.lam_t_grnd += w["g"]
        adj.lam_t_h2osfc += w["h"]
        adj.lam_qcharge.copy_(w["q"])


def _adjoint_arrays(adj):
    out = {k: getattr(adj, k).clone() for k in ("lam_t_soisno", "lam_h2osoi_liq", "lam_h2osoi_ice", "lam_t_grnd",
                                                 "lam_t_h2osfc")}
    out.update({"grad_" + p: adj.grad[p].clone() for p in adjoint.PARAMS})
    return out


def _traj_method(h, wl, G, I, nsteps, cfg, method):
    def forcing(t, st):
        api.synth_forcing(h, st, G[t], I[t])
    return adjoint.Trajectory(h, nsteps, wl.dtime, forcing, cfg, snow_method=method,
                              forcing_reverse=adjoint.synth_forcing_reverse)


@pytest.mark.parametrize("cfg_id,method,bc", [(1, abi.SNOW_JORDAN1991, abi.BC_FLUX),
                                              (1, abi.SNOW_STURM1997, abi.BC_FLUX),
                                              (2, abi.SNOW_JORDAN1991, abi.BC_FLUX),
                                              (1, abi.SNOW_JORDAN1991, abi.BC_WATERTABLE),
                                              (2, abi.SNOW_JORDAN1991, abi.BC_ZERO_FLUX)])
def test_closed_form_step_adjoint_matches_recorded(handle, cfg_id, method, bc):
    """The hand-written reverse of the whole step (soil_temperature! stage by stage,
    fractions, impedance, substeps) and the recording kernel differentiate the same
    arithmetic: every input adjoint and parameter gradient agrees to rounding, per
    column relative to the column's largest entry of that quantity; for both snow
    conductivity methods and the free-drainage, water-table and zero-flux lower
    boundaries."""
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = bc
    nsteps = 4
    wl, G, I = _workload_cfg(cfg_id, 512, nsteps, seed=31 + cfg_id)
    traj = _traj_method(handle, wl, G, I, nsteps, cfg, method)
    st0 = wl.state.to_device()
    if bc == abi.BC_WATERTABLE:
        st0["zwt"][::2] += 1.5     # water table below the soil column: drainage to it is active
    lin = _LinearSeed(st0, nsteps, 7 + cfg_id)
    out, stat = {}, {}
    try:
        for mode in (abi.ADJ_ST_CLOSED_FORM, abi.ADJ_ST_RECORDED):
            handle.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, mode)
            status = torch.zeros(st0.nc, dtype=torch.int32, device="cuda")
            adj = adjoint.multistep_reverse(traj, st0.copy(), lin.seed, None, checkpoint_every=2, col_status=status)
            out[mode] = _adjoint_arrays(adj)
            stat[mode] = status.cpu().numpy()
    finally:
        handle.set_option(abi.OPT_ADJ_SOIL_TEMPERATURE, abi.ADJ_ST_CLOSED_FORM)
    assert np.all((stat[abi.ADJ_ST_CLOSED_FORM] & abi.COL_TAPE_FULL) == 0)
    assert np.all((stat[abi.ADJ_ST_RECORDED] & abi.COL_TAPE_FULL) == 0)
    ok = (stat[abi.ADJ_ST_CLOSED_FORM] & abi.COL_ADJ_UNSUPPORTED) == 0
    assert ok.mean() > 0.5
    worst = 0.0
    for k in out[abi.ADJ_ST_CLOSED_FORM]:
        a = out[abi.ADJ_ST_CLOSED_FORM][k].cpu().numpy()
        b = out[abi.ADJ_ST_RECORDED][k].cpu().numpy()
        assert np.isfinite(a).all(), k
        if a.ndim == 1:
            a, b = a[None, :], b[None, :]
        scale = np.max(np.abs(b), axis=0)
        rel = np.max(np.abs(a - b), axis=0) / np.maximum(scale, 1e-300)
        rel = rel[ok & (scale > 0)]
        if rel.size:
            print("%s: max rel diff %.3g" % (k, rel.max()))
            worst = max(worst, rel.max())
    assert worst < 1e-9, worst


def test_substep_log_gives_the_same_bits(handle):
    """The reverse reading the substep log of the recomputed forward, running the
    substep loop itself (no log), or mixing both (a log too small for some columns)
    gives the same bits, with and without the soil_temperature! records."""
    cfg = _cfg_flux()
    nsteps = 6
    wl, G, I = _workload(384, nsteps, seed=808)
    traj = _traj(handle, wl, G, I, nsteps, cfg)
    st0 = wl.state.to_device()
    lin = _LinearSeed(st0, nsteps, 3)
    res = {}
    for cap, stlog in ((0, False), (24, True), (24, False), (2, True)):
        adj = adjoint.multistep_reverse(traj, st0.copy(), lin.seed, None, checkpoint_every=3, log_cap=cap,
                                        log_soil_temperature=stlog)
        res[cap, stlog] = _adjoint_arrays(adj)
    for key in ((24, True), (24, False), (2, True)):
        for k in res[0, False]:
            assert torch.equal(res[0, False][k], res[key][k]), (key, k)


def test_logged_step_is_the_production_step(handle):
    cfg = _cfg_flux()
    wl, G, I = _workload(600, 3, seed=99)
    a = wl.state.to_device()
    b = a.copy()
    log = api.SubstepLog(a.nc, 16)
    for t in range(3):
        api.synth_forcing(handle, a, G[t], I[t])
        api.column_step(handle, a, wl.dtime, cfg)
        api.synth_forcing(handle, b, G[t], I[t])
        api.column_step_logged(handle, b, wl.dtime, log, cfg)
        torch.cuda.synchronize()
        for k in a.arrays:
            assert torch.equal(a[k], b[k]), "step %d field %s" % (t, k)
        cnt = log.count.cpu().numpy()
        hyd = b["mask_hydrology"].cpu().numpy() != 0
        assert np.all(cnt[hyd] >= 1) and np.all(cnt[~hyd] == -1)
        # the log's final block holds the solve's outputs
        stride = abi.log_stride(log.cap)
        rec = log.rec.view(a.nc, stride)
        fin = rec[:, log.cap * abi.LOG_REC:]
        nl = int(b["col_nbedrock"].min())
        j0 = a.vp.nlevsno
        hydt = torch.from_numpy(hyd).cuda()
        assert torch.equal(fin[hydt, :nl].T.contiguous(), b["h2osoi_liq"][j0:j0 + nl][:, hydt])
        assert torch.equal(fin[hydt, 3 * abi.MAX_NLEVSOI], b["qcharge"][hydt])
        # the soil_temperature! record: the state the call left (the Richards solve
        # changes neither temperature, ice, fact nor t_grnd), the band size and status
        srec = log.st_rec.view(a.nc, abi.LOG_ST_STRIDE)
        act = torch.from_numpy(b["mask_nolakec"].cpu().numpy() != 0).cuda()
        snl = b["col_snl"].cpu().numpy()
        nw = a.vp.nlevsno + a.vp.nlevgrnd
        nL = abi.MAX_NLEVSNO + abi.MAX_NLEVGRND
        assert torch.equal(srec[act, 2], b["t_grnd"][act]) and torch.equal(srec[act, 3], b["t_h2osfc"][act])
        assert torch.all(srec[act, 1] == 0)
        for c in np.nonzero(act.cpu().numpy())[0][::7]:
            jt = int(snl[c]) + j0          # 0-based top level
            for off, k in ((4, "t_soisno"), (4 + 2 * nL, "h2osoi_ice"), (4 + 3 * nL, "fact")):
                assert torch.equal(srec[c, off + jt:off + nw], b[k][jt:nw, c]), (t, c, k)
            assert int(srec[c, 0]) == nw - jt + 1          # snow + ground levels + the surface-water row


@pytest.mark.parametrize("nsteps,min_share", [(1, 0.18), (48, 0.38)])
def test_calibration_gradient_every_entry_by_batched_differences(handle, nsteps, min_share):
    """Every one of the 80 parameter entries (watsat, bsw, sucsat, hksat of 20 levels)
    of 64 columns, each with its own step: the perturbed copies are extra columns of one
    batched forward run (64 x 80 entries x 7 step sizes x 2 signs), so every entry gets
    central differences at h = 1e-6, 3e-6, ..., 3e-4, 1e-3 relative.  An entry is resolved
    at the smallest h whose quotient agrees with the next larger one to 1e-4 relative
    (quotients across a kink of a clamp drift slowly with h, by 1e-4 to 1e-3 between
    neighbouring step sizes, and are left out),
    where neither pair of runs moves a discrete decision (substep counts, melt flags)
    and the loss changes by at least 1e5 times what one ulp of every observation y_t
    moves it (sum_t 2 |y_t - target_t| ulp(y_t): a column close to its target has a
    small loss whose own ulps say nothing about the noise of its quotients); a resolved
    entry must match the adjoint to 1e-3 relative.  Levels below a column's bedrock take no part in the solve: their
    adjoint and every quotient must be exactly zero.  Reports the shares."""
    cfg = _cfg_flux()
    nc0 = 64
    wl, G, I = _workload(nc0, nsteps, seed=4242)
    traj = _traj(handle, wl, G, I, nsteps, cfg)
    st0 = wl.state.to_device()
    pert = wl.state.copy()
    adjoint.perturb_parameters(pert, np.random.default_rng(9))
    tl = adjoint.CalibrationLoss(st0, wl.dtime)
    _params_and_decisions(traj, pert.to_device(), tl, nsteps)
    target = torch.stack(tl.y)                                   # [nsteps, nc0]
    loss = adjoint.CalibrationLoss(st0, wl.dtime, target)
    adj = adjoint.multistep_reverse(traj, st0.copy(), loss.seed, loss.observe, checkpoint_every=8)
    params = adjoint.PARAMS
    nsoi = wl.state.vp.nlevsoi
    gr = np.stack([adj.grad[p].cpu().numpy() for p in params])   # [4, nsoi, nc0]
    rels = np.array([1e-6, 3e-6, 1e-5, 3e-5, 1e-4, 3e-4, 1e-3])
    K, E = len(rels), len(params) * nsoi
    # column layout of the batch: the nc0 base columns, then for each (entry, step, sign)
    # a block of nc0 copies
    nrep = nc0 + E * K * 2 * nc0
    base_of = np.tile(np.arange(nc0), nrep // nc0)
    host = wl.state.subset(base_of)
    theta0 = {p: host[p].copy() for p in params}
    blk = 1
    for e in range(E):
        p, j = params[e // nsoi], e % nsoi
        for k in range(K):
            for sgn in (1.0, -1.0):
                sl = slice(blk * nc0, (blk + 1) * nc0)
                host[p][j, sl] = theta0[p][j, sl] * (1.0 + sgn * rels[k])
                blk += 1
    st = host.to_device()
    bo = torch.from_numpy(base_of).cuda()
    Gr, Ir = G[:, bo].contiguous(), I[:, bo].contiguous()
    trajr = _traj(handle, wl, Gr, Ir, nsteps, cfg)
    lossr = adjoint.CalibrationLoss(st, wl.dtime, target[:, bo].contiguous())
    same = torch.ones(nrep, dtype=torch.bool, device="cuda")
    for t in range(nsteps):
        trajr.step(t, st)
        lossr.observe(t, st)
        ns, im = st["num_substeps"], st["imelt"]
        same &= (ns == ns[bo]) & (im == im[:, bo]).all(0)
    L = lossr.per_column().cpu().numpy()
    same = same.cpu().numpy()
    Lr = L[nc0:].reshape(E, K, 2, nc0)
    okr = same[nc0:].reshape(E, K, 2, nc0).all(2)                # [E, K, nc0]
    h = rels[None, :, None] * np.abs(np.stack([theta0[params[e // nsoi]][e % nsoi, :nc0]
                                                for e in range(E)]))[:, None, :]
    fd = (Lr[:, :, 0] - Lr[:, :, 1]) / (2.0 * h)                 # [E, K, nc0]
    dl = np.abs(Lr[:, :, 0] - Lr[:, :, 1])
    g = gr.reshape(E, nc0)
    Y = torch.stack(lossr.y)[:, :nc0].cpu().numpy()
    Rz = Y - target.cpu().numpy()
    conditioned = np.abs(Rz).max(0) >= 1e-6 * np.abs(Y).max(0)
    noise = (2.0 * np.abs(Rz) * np.abs(Y)).sum(0) * 2.0 ** -52     # loss change per ulp of every y_t
    resolved = np.zeros((E, nc0), dtype=bool)
    checked_fd = np.zeros((E, nc0))
    for k in range(K - 1):
        agree = (okr[:, k] & okr[:, k + 1] & (dl[:, k] >= 1e5 * noise[None, :]) &
                 (np.abs(fd[:, k] - fd[:, k + 1]) <= 1e-4 * np.abs(fd[:, k])))
        new = agree & ~resolved
        checked_fd[new] = fd[:, k][new]
        resolved |= agree
    resolved &= conditioned[None, :]
    zero = (g == 0.0)
    nb = wl.state["col_nbedrock"][:nc0]
    below = np.array([[e % nsoi + 1 > nb[c] for c in range(nc0)] for e in range(E)])
    assert np.all(g[below] == 0.0) and np.all(fd.transpose(1, 0, 2)[:, below] == 0.0)
    rel_err = np.abs(g - checked_fd) / np.maximum(np.abs(checked_fd), 1e-300)
    bad = resolved & (rel_err > 1e-3)
    if bad.any():
        lines = []
        for e, c in np.argwhere(bad)[:6]:
            lines.append("%s[%d] col %d adj %.10e fd %s ok %s dl/noise %s" % (
                params[e // nsoi], e % nsoi + 1, c, g[e, c], np.array2string(fd[e, :, c], precision=10),
                okr[e, :, c], np.array2string(dl[e, :, c] / noise[c], precision=2)))
        raise AssertionError("%d entries off:\n" % bad.sum() + "\n".join(lines))
    live = ~zero & conditioned[None, :]
    share = resolved[live].mean()
    print("every entry, %d steps: %d of %d nonzero entries resolved (%.1f%%), %d below bedrock (zero), "
          "max rel err %.2e" % (nsteps, resolved[live].sum(), live.sum(), 100 * share, below.sum(),
                                rel_err[resolved].max() if resolved.any() else 0.0))
    assert share >= min_share, share
