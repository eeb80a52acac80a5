"""GPU parity of the reverse-mode rules of the linear solves (enzyme_rules.jl:80-107,
160-201) through the C ABI, against the oracle's restatement: no transcendental is
involved, so the results must match bit for bit.  The golden 9-level system of
test_enzyme_smoke.jl:194-248 is checked to the reference's own tolerances too.
"""
import numpy as np
import pytest

from clmgb import api, synth
from fixtures import golden, random_band_system
from oracle import oracle as orc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

G = golden()


@pytest.fixture(scope="module")
def h():
    assert torch.cuda.is_available()
    hd = api.Handle(synth.clm5_varpar())
    yield hd
    hd.close()


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_tridiagonal_adjoint_golden(h):
    g = G["tridiag_adjoint9"]
    n, jtop = g["n"], g["jtop"]
    a0, b0, c0, r0, w = (np.array(g[k], dtype=np.float64) for k in ("a", "b", "c", "r", "w"))
    u = orc.tridiagonal_solve(a0, b0, c0, r0, jtop, n)
    ub = np.zeros(n)
    ub[jtop - 1:] = w[jtop - 1:]
    ref = orc.tridiagonal_adjoint(u, a0, b0, c0, ub.copy(), jtop, n)
    col = lambda x: _dev(np.asarray(x, dtype=np.float64).reshape(n, 1))  # noqa: E731
    ubar = col(ub)
    bars = [col(np.zeros(n)) for _ in range(4)]
    api.tridiagonal_adjoint(h, col(u), col(a0), col(b0), col(c0), ubar, *bars,
                            _dev(np.array([jtop], dtype=np.int64)), _dev(np.ones(1, dtype=np.uint8)))
    got = [x.cpu().numpy()[:, 0] for x in bars]
    for k in range(4):
        assert np.array_equal(got[k], ref[k]), "abcr"[k]
    assert np.all(ubar.cpu().numpy() == 0.0)
    assert np.all(got[0][:jtop] == 0.0) and got[2][n - 1] == 0.0


def test_tridiagonal_adjoint_bit_exact_vs_oracle(h):
    rng = np.random.default_rng(3)
    nlevs, ncols = 25, 4111
    a = rng.uniform(-0.6, 0.6, (nlevs, ncols))
    c = rng.uniform(-0.6, 0.6, (nlevs, ncols))
    b = rng.uniform(2.0, 3.5, (nlevs, ncols))
    r = rng.normal(size=(nlevs, ncols))
    jtop = rng.integers(1, 8, ncols).astype(np.int64)
    mask = (rng.random(ncols) < 0.9).astype(np.uint8)
    u = np.zeros((nlevs, ncols))
    orc.tridiagonal_multi(u, a, b, c, r, jtop, mask)
    ubar = rng.normal(size=(nlevs, ncols))
    bars = [rng.normal(size=(nlevs, ncols)) for _ in range(4)]
    ref_ub = ubar.copy()
    ref_bars = [x.copy() for x in bars]
    orc.tridiagonal_adjoint_multi(u, a, b, c, ref_ub, *ref_bars, jtop, mask)
    d_ub = _dev(ubar)
    d_bars = [_dev(x) for x in bars]
    api.tridiagonal_adjoint(h, *[_dev(x) for x in (u, a, b, c)], d_ub, *d_bars, _dev(jtop), _dev(mask))
    assert np.array_equal(d_ub.cpu().numpy(), ref_ub)
    for k in range(4):
        assert np.array_equal(d_bars[k].cpu().numpy(), ref_bars[k]), "abcr"[k]


@pytest.mark.parametrize("kl", [1, 2])
def test_band_factor_and_adjoint_bit_exact_vs_oracle(h, kl):
    rng = np.random.default_rng(21 + kl)
    nc, nlev = 4099, 38
    nb, W = 2 * kl + 1, 3 * kl + 1
    bm, rv = random_band_system(nc, nlev, kl, kl, rng, pivot_frac=0.25)
    jtop = rng.integers(1, 14, nc).astype(np.int64)
    jbot = np.full(nc, nlev, dtype=np.int64)
    jbot[::7] = rng.integers(20, nlev + 1, len(jbot[::7]))
    mask = (rng.random(nc) < 0.95).astype(np.uint8)
    tv_ref = np.full((nlev, nc), -7.0)
    orc.batched_band_solve(tv_ref, bm, rv, jtop, jbot, mask, kl, kl, -1)
    dm = [_dev(x) for x in (bm, rv, jtop, jbot, mask)]
    tv = _dev(np.full((nlev, nc), -7.0))
    lu = torch.zeros((nlev, W, nc), dtype=torch.float64, device="cuda")
    piv = torch.zeros((nlev, nc), dtype=torch.uint8, device="cuda")
    api.batched_band_solve_factor(h, tv, *dm, lu, piv, kl, kl, -1)
    assert np.array_equal(tv.cpu().numpy(), tv_ref)
    tbar = rng.normal(size=(nlev, nc))
    bbar = rng.normal(size=(nlev, nb, nc))
    rbar = rng.normal(size=(nlev, nc))
    ref_t, ref_b, ref_r = tbar.copy(), bbar.copy(), rbar.copy()
    orc.batched_band_solve_adjoint(tv_ref, ref_t, bm, ref_b, ref_r, jtop, jbot, mask, kl, kl, -1)
    d_t, d_b, d_r = _dev(tbar), _dev(bbar), _dev(rbar)
    api.batched_band_solve_adjoint(h, tv, d_t, lu, piv, d_b, d_r, dm[2], dm[3], dm[4], kl, kl, -1)
    assert np.array_equal(d_t.cpu().numpy(), ref_t)
    assert np.array_equal(d_r.cpu().numpy(), ref_r), "max %g" % np.max(np.abs(d_r.cpu().numpy() - ref_r))
    assert np.array_equal(d_b.cpu().numpy(), ref_b), "max %g" % np.max(np.abs(d_b.cpu().numpy() - ref_b))
    # the pivoting systems did exchange rows
    assert int((piv.cpu().numpy() != 0).sum()) > 0
