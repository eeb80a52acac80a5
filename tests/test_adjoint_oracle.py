"""Oracle restatements of the reverse-mode rules of the linear solves
(enzyme_rules.jl:80-107 band_solve!, :160-201 tridiagonal_solve!), pinned against
the reference's own adjoint test (test_enzyme_smoke.jl:194-248): the fixed 9-level
system with jtop = 3, every band checked against an exact forward-mode derivative
(here complex-step, which like ForwardDiff is exact to rounding) to 1e-10 and
against central finite differences (h = 1e-6*max(|v|,1)) to 1e-6, and the entries
the solve never reads carry exactly zero gradient.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_cases.json")))


def thomas(a, b, c, r, jtop, n):
    """tridiagonal_solve! (tridiagonal.jl:35-63) in generic arithmetic (complex-step)."""
    dt = np.result_type(a, b, c, r)
    cp = np.zeros(n + 1, dtype=dt)
    dp = np.zeros(n + 1, dtype=dt)
    u = np.zeros(n, dtype=dt)
    j = jtop
    cp[j] = c[j - 1] / b[j - 1]
    dp[j] = r[j - 1] / b[j - 1]
    for jj in range(j + 1, n + 1):
        den = b[jj - 1] - a[jj - 1] * cp[jj - 1]
        cp[jj] = c[jj - 1] / den
        dp[jj] = (r[jj - 1] - a[jj - 1] * dp[jj - 1]) / den
    u[n - 1] = dp[n]
    for jj in range(n - 1, j - 1, -1):
        u[jj - 1] = dp[jj] - cp[jj] * u[jj]
    return u


def relerr(x, y):
    return np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-12)


def complex_step_grad(f, v0):
    g = np.zeros_like(v0)
    h = 1e-30
    for i in range(len(v0)):
        v = v0.astype(np.complex128)
        v[i] += 1j * h
        g[i] = f(v).imag / h
    return g


def central_fd_grad(f, v0):
    g = np.zeros_like(v0)
    for i in range(len(v0)):
        h = 1e-6 * max(abs(v0[i]), 1.0)
        vp = v0.copy(); vp[i] += h
        vm = v0.copy(); vm[i] -= h
        g[i] = (f(vp) - f(vm)) / (2 * h)
    return g


def test_tridiagonal_adjoint_golden_9_level():
    g = GOLD["tridiag_adjoint9"]
    n, jtop = g["n"], g["jtop"]
    a0, b0, c0, r0, w = (np.array(g[k], dtype=np.float64) for k in ("a", "b", "c", "r", "w"))

    def obj(a, b, c, r):
        u = thomas(a, b, c, r, jtop, n)
        return np.sum(w[jtop - 1:] * u[jtop - 1:])

    u = oracle.tridiagonal_solve(a0, b0, c0, r0, jtop, n)
    ubar = np.zeros(n)
    ubar[jtop - 1:] = w[jtop - 1:]
    da, db, dc, dr = oracle.tridiagonal_adjoint(u, a0, b0, c0, ubar, jtop, n)
    assert np.all(ubar[jtop - 1:] == 0.0)   # the output adjoint is consumed
    args = [a0, b0, c0, r0]
    for k, (name, e) in enumerate(zip("abcr", (da, db, dc, dr))):
        def fk(v, k=k):
            x = list(args)
            x[k] = v
            return obj(*x)
        exact = complex_step_grad(fk, args[k])
        fd = central_fd_grad(fk, args[k])
        assert np.all(np.isfinite(e))
        assert relerr(e, exact) < g["tol_vs_exact"], name
        assert relerr(e, fd) < g["tol_vs_fd"], name
    assert np.all(da[:jtop] == 0.0)
    assert dc[n - 1] == 0.0


def test_tridiagonal_adjoint_multi_matches_single():
    rng = np.random.default_rng(11)
    nlevs, ncols = 12, 37
    a = rng.uniform(-0.5, 0.5, (nlevs, ncols))
    c = rng.uniform(-0.5, 0.5, (nlevs, ncols))
    b = rng.uniform(2.0, 3.0, (nlevs, ncols))
    r = rng.normal(size=(nlevs, ncols))
    jtop = rng.integers(1, nlevs + 1, ncols).astype(np.int64)
    mask = (rng.random(ncols) < 0.9).astype(np.uint8)
    u = np.zeros((nlevs, ncols))
    for col in range(ncols):
        u[:, col] = oracle.tridiagonal_solve(a[:, col], b[:, col], c[:, col], r[:, col], int(jtop[col]), nlevs)
    ubar = rng.normal(size=(nlevs, ncols))
    bars = [rng.normal(size=(nlevs, ncols)) for _ in range(4)]
    ub2 = ubar.copy()
    bars2 = [x.copy() for x in bars]
    oracle.tridiagonal_adjoint_multi(u, a, b, c, ub2, *bars2, jtop, mask)
    for col in range(ncols):
        if not mask[col]:
            assert np.array_equal(ub2[:, col], ubar[:, col])
            continue
        ub = ubar[:, col].copy()
        d = oracle.tridiagonal_adjoint(u[:, col], a[:, col], b[:, col], c[:, col], ub, int(jtop[col]), nlevs)
        assert np.array_equal(ub2[:, col], ub)
        for k in range(4):
            assert np.array_equal(bars2[k][:, col], bars[k][:, col] + d[k])


def dense_from_bands(bm, jt, n, kl, ku, col=0, dtype=np.float64):
    A = np.zeros((n, n), dtype=dtype)
    for j in range(1, n + 1):
        for i in range(max(1, j - kl), min(n, j + ku) + 1):
            A[i - 1, j - 1] = bm[jt + i - 2, (i - j) + kl, col]
    return A


def ge_solve(A, x):
    """Partial-pivoting GE (band_diagonal.jl:87-170) in generic arithmetic."""
    A = A.copy()
    x = x.copy()
    n = len(x)
    for k in range(n - 1):
        p = k + int(np.argmax(np.abs(A[k:, k].real)))
        if abs(A[p, k].real) <= abs(A[k, k].real):
            p = k
        if p != k:
            A[[k, p]] = A[[p, k]]
            x[[k, p]] = x[[p, k]]
        for i in range(k + 1, n):
            f = A[i, k] / A[k, k]
            A[i, k:] = A[i, k:] - f * A[k, k:]
            x[i] = x[i] - f * x[k]
    for i in range(n - 1, -1, -1):
        x[i] = (x[i] - A[i, i + 1:] @ x[i + 1:]) / A[i, i]
    return x


@pytest.mark.parametrize("pivot", [False, True])
def test_band_adjoint_vs_complex_step(pivot):
    rng = np.random.default_rng(5 + pivot)
    kl = ku = 2
    nb = kl + ku + 1
    nlev, ncols = 14, 4
    bm = rng.uniform(-1.0, 1.0, (nlev, nb, ncols))
    if not pivot:
        bm[:, kl, :] += 6.0      # diagonally dominant: no row exchange
    else:
        bm[:, kl, :] *= 0.05     # weak diagonal: pivoting fires
    rv = rng.normal(size=(nlev, ncols))
    jtop = np.array([0, 2, 1, 5], dtype=np.int64)
    jbot = np.array([13, 13, 9, 12], dtype=np.int64)
    mask = np.ones(ncols, dtype=np.uint8)
    tv = np.zeros((nlev, ncols))
    oracle.batched_band_solve(tv, bm, rv, jtop, jbot, mask, kl, ku, 0)
    w = rng.normal(size=(nlev, ncols))
    tbar = w.copy()
    bbar = np.zeros_like(bm)
    rbar = np.zeros_like(rv)
    oracle.batched_band_solve_adjoint(tv, tbar, bm, bbar, rbar, jtop, jbot, mask, kl, ku, 0)
    for col in range(ncols):
        jt = int(jtop[col]) + 1
        n = int(jbot[col] - jtop[col] + 1)
        rows = slice(jt - 1, jt - 1 + n)
        assert np.all(tbar[rows, col] == 0.0)

        def obj_r(rvec):
            return np.sum(w[rows, col] * ge_solve(dense_from_bands(bm, jt, n, kl, ku, col, rvec.dtype), rvec))
        gr = complex_step_grad(obj_r, rv[rows, col])
        assert relerr(rbar[rows, col], gr) < 1e-10
        # the matrix gradient on every band entry the forward reads
        flat = []
        for j in range(1, n + 1):
            for i in range(max(1, j - kl), min(n, j + ku) + 1):
                flat.append((jt + i - 2, (i - j) + kl))
        v0 = np.array([bm[lv, bd, col] for lv, bd in flat])

        def obj_b(v):
            bmc = bm[:, :, col:col + 1].astype(v.dtype)
            for (lv, bd), x in zip(flat, v):
                bmc[lv, bd, 0] = x
            A = dense_from_bands(bmc, jt, n, kl, ku, 0, v.dtype)
            return np.sum(w[rows, col] * ge_solve(A, rv[rows, col].astype(v.dtype)))
        gb = complex_step_grad(obj_b, v0)
        e = np.array([bbar[lv, bd, col] for lv, bd in flat])
        assert relerr(e, gb) < 1e-10
        # band entries outside the system get nothing
        touched = np.zeros((nlev, nb), dtype=bool)
        for lv, bd in flat:
            touched[lv, bd] = True
        assert np.all(bbar[:, :, col][~touched] == 0.0)


def test_complex_step_moisture_form_matches_oracle():
    """The complex-step restatement used as the exact derivative reference reproduces
    the oracle's moisture-form solve (real part) on the no-frost workload, where the
    soil-temperature step leaves the water alone."""
    from adjoint_reference import moisture_form
    from clmgb import abi, synth
    wl = synth.make_workload(0, nc=48, seed=31, nsteps=1)
    st = wl.state
    G, I = wl.forcing(0)
    synth.apply_forcing_host(st, G, I)
    cfg = abi.SwmConfig.clm5_default()
    cfg.lower_boundary_condition = abi.BC_FLUX
    ref = st.copy()
    oracle.soil_water_fractions(ref)
    oracle.soil_water(ref, wl.dtime, cfg)
    joff = st.vp.nlevsno
    worst = 0.0
    for c in range(st.nc):
        nl = int(st["col_nbedrock"][c])
        lv = slice(joff, joff + nl)
        liq, qc, _ = moisture_form(st["h2osoi_liq"][lv, c], st["dz"][lv, c], st["z"][lv, c],
                                   st["watsat"][:nl, c], st["bsw"][:nl, c], st["sucsat"][:nl, c],
                                   st["hksat"][:nl, c], np.ones(nl), st["qflx_infl"][c],
                                   st["qflx_rootsoi"][:nl, c], wl.dtime, cfg, "flux")
        worst = max(worst, np.max(np.abs(liq.real - ref["h2osoi_liq"][lv, c]) / np.abs(ref["h2osoi_liq"][lv, c])))
        assert abs(qc.real - ref["qcharge"][c]) <= 1e-9 * max(abs(ref["qcharge"][c]), 1e-12)
        assert np.all(liq.imag == 0.0)
    assert worst < 1e-9, worst
