"""GPU tests of the warm-start perceptron's kernels against the numpy reference
(tests/mlp_reference.py, the same bf16 rounding points; products summed in fp32 on
the GPU), of training, and of the warm-started solve."""
import numpy as np
import pytest

import mlp_reference as R
from clmgb import abi, api, mlp, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def h():
    assert torch.cuda.is_available()
    hd = api.Handle(synth.clm5_varpar())
    yield hd
    hd.close()


def _bf(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda().to(torch.bfloat16)


def _f(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("K,N", [(64, 128), (128, 128), (128, 32), (32, 128)])
def test_linear_matches_reference(h, K, N):
    rng = np.random.default_rng(K + N)
    M = 1000
    X = R.bf16(rng.normal(size=(M, K)).astype(np.float32))
    W = R.bf16(rng.normal(0, 0.2, (N, K)).astype(np.float32))
    b = rng.normal(0, 0.1, N).astype(np.float32)
    Z = torch.empty((M, N), dtype=torch.float32, device="cuda")
    Y = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    import ctypes as C
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    Xd, Wd, bd = _bf(X), _bf(W), _f(b)
    api.check(h.lib.clmgb_mlp_linear(h.h, M, N, K, p(Xd), K, p(Wd), p(bd), 1, p(Z), N, p(Y), N,
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream)), "linear")
    Zr = X.astype(np.float64) @ W.astype(np.float64).T + b
    z = Z.cpu().numpy()
    assert np.max(np.abs(z - Zr)) <= 2e-5 * np.max(np.abs(Zr)) + 1e-6
    y = Y.float().cpu().numpy()
    yr = R.bf16(R.silu(z.astype(np.float64)).astype(np.float32))
    assert np.max(np.abs(y - yr)) <= 1e-2 * np.max(np.abs(yr))


def test_training_gradients_match_reference(h):
    rng = np.random.default_rng(7)
    model = mlp.WarmStartMLP(h, seed=3)
    W = [w.cpu().numpy() for w in model.w]
    b = [x.cpu().numpy() for x in model.b]
    M = 512
    X = R.bf16(rng.normal(size=(M, R.IN)).astype(np.float32))
    T = rng.normal(size=(M, R.OUTP)).astype(np.float32)
    T[:, R.OUT:] = 0.0
    Y, acts = model.forward(_bf(X), keep=True)
    l, dY = model.loss(Y, _f(T))
    dW, db = model.gradients(acts, dY)
    Yr, acts_r = R.forward(X, W, b)
    Lr, dYr = R.loss_and_dy(Yr, T)
    assert abs(float(l) - Lr) <= 1e-3 * Lr
    dWr, dbr = R.backward(acts_r, dYr, W)
    for li in range(3):
        g = dW[li].cpu().numpy()
        err = np.max(np.abs(g - dWr[li])) / np.max(np.abs(dWr[li]))
        assert err < 2e-2, (li, err)
        gb = db[li].cpu().numpy()
        errb = np.max(np.abs(gb - dbr[li])) / max(np.max(np.abs(dbr[li])), 1e-12)
        assert errb < 2e-2, (li, errb)
    assert float(dW[2][R.OUT:].abs().max()) == 0.0


def test_training_reduces_loss(h):
    """Fit a smooth function of the inputs: the loss falls by a large factor."""
    rng = np.random.default_rng(11)
    n = 16384
    F = rng.normal(size=(n, R.IN)).astype(np.float32)
    T = np.zeros((n, R.OUTP), dtype=np.float32)
    T[:, 0] = 2.0 + np.tanh(F[:, 0] + 0.5 * F[:, 1] * F[:, 2])
    T[:, 1:R.OUT] = 0.01 * np.sin(F[:, 3:3 + R.OUT - 1])
    model = mlp.WarmStartMLP(h, seed=1)
    hist = model.train(_f(F), _f(T), epochs=10, batch=512, lr=3e-3)
    assert hist[-1] < 0.25 * hist[0], hist


def _cfg():
    cfg = abi.SwmConfig.clm5_default()
    return cfg


def test_warm_solve_with_full_step_proposal_is_the_plain_solve(h):
    wl = synth.make_workload(2, nc=2048, seed=5, nsteps=2)
    st = wl.state.to_device()
    G, I = wl.forcing(0)
    api.synth_forcing(h, st, torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda())
    api.soil_temperature(h, st, wl.dtime)
    api.set_soil_water_fractions(h, st)
    a, b = st.copy(), st.copy()
    api.soil_water(h, a, wl.dtime, _cfg())
    dt = torch.full((st.nc,), wl.dtime, dtype=torch.float64, device="cuda")
    mlp.soil_water_warm(h, b, wl.dtime, dt, _cfg())
    for k in ("h2osoi_liq", "qcharge", "num_substeps", "smp_l", "hk_l"):
        assert torch.equal(a[k], b[k]), k


def test_warm_solve_conserves_water_and_meets_tolerance(h):
    """Any proposal: the solve conserves water exactly like the plain one and stays
    within the accepted-substep tolerance of it."""
    wl = synth.make_workload(2, nc=4096, seed=6, nsteps=1)
    st = wl.state.to_device()
    G, I = wl.forcing(0)
    api.synth_forcing(h, st, torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda())
    api.soil_temperature(h, st, wl.dtime)
    api.set_soil_water_fractions(h, st)
    a, b = st.copy(), st.copy()
    api.soil_water(h, a, wl.dtime, _cfg())
    rng = np.random.default_rng(2)
    k = torch.from_numpy(rng.integers(0, 7, st.nc)).cuda()
    dt = wl.dtime / (2.0 ** k.double())
    mlp.soil_water_warm(h, b, wl.dtime, dt, _cfg())
    joff = st.vp.nlevsno
    lv = slice(joff, joff + st.vp.nlevsoi)
    w0 = st["h2osoi_liq"][lv].sum(0)
    sink = st["qflx_rootsoi"][:st.vp.nlevsoi].sum(0)
    for s in (a, b):
        dw = s["h2osoi_liq"][lv].sum(0) - w0
        budget = (st["qflx_infl"] - s["qcharge"] - sink) * wl.dtime
        assert float((dw - budget).abs().max()) <= 1e-8 * float(w0.abs().max())
    # both solves are within the accepted-substep tolerance: the water of each level
    # differs by far less than the 0.1 mm local error bound times the substep count
    d = (a["h2osoi_liq"][lv] - b["h2osoi_liq"][lv]).abs().max()
    assert float(d) < 0.1 * float(torch.maximum(a["num_substeps"], b["num_substeps"]).max())


def test_samples_record_consistent_labels(h):
    wl = synth.make_workload(2, nc=1024, seed=8, nsteps=1)
    st = wl.state.to_device()
    G, I = wl.forcing_block(range(1))
    F, T = mlp.generate_samples(h, st, torch.from_numpy(G).cuda(), torch.from_numpy(I).cuda(), 1, wl.dtime,
                                per_column=3)
    assert F.shape[0] >= st.nc            # at least the first substep of every column
    k = T[:, 0].cpu().numpy()
    assert np.all((k >= 0) & (k <= 12)) and np.all(k == np.round(k))
    rem = F[:, 62].cpu().numpy()
    assert np.all((rem > 0) & (rem <= 1.0))
    assert np.isfinite(F.cpu().numpy()).all() and np.isfinite(T.cpu().numpy()).all()
