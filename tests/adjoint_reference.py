"""Complex-step reference derivatives of the moisture-form Richards solve (TEST
INFRASTRUCTURE ONLY).

A numpy restatement of _soilwm_moisture_form_kernel! (soil_water_movement.jl:1250-
1489) that runs in complex arithmetic: with a parameter perturbed by i*h (h = 1e-30)
the imaginary part of the result divided by h is its derivative, exact to rounding
(no subtraction, so no cancellation).  Discrete decisions (clamps, accept/reject,
substep doubling) are taken on real parts, as the solver takes them on values, so
the reference differentiates the same branch the adjoint differentiates.  The
tridiagonal system is solved densely (numpy.linalg.solve): the derivative of the
solution does not depend on how the system is solved.
"""
import numpy as np


def _clamp(x, lo, hi):
    if x.real > hi:
        return complex(hi)
    if x.real < lo:
        return complex(lo)
    return x


def moisture_form(liq, dz, z, watsat, bsw, sucsat, hksat, imp, qflx_infl, qflx_rootsoi, dtime, cfg,
                  lower_bc):
    """One call for one column; arrays over layers 1..nlayers.  Returns (liq, qcharge,
    attempts).  Complex inputs propagate through; decisions use real parts."""
    nl = len(liq)
    liq = np.asarray(liq, dtype=complex).copy()
    dtsub, dtdone, qc, nsub = dtime, 0.0, 0.0 + 0j, 0
    dtdz_of = lambda dts: dts / (1000.0 * dz)  # noqa: E731
    while True:
        nsub += 1
        # hydraulic properties and fluxes from the current water (:1274-1378)
        s2 = np.empty(nl, complex)
        for j in range(nl):
            vwc = (liq[j] if liq[j].real >= 1e-6 else complex(1e-6)) / (dz[j] * 1000.0)
            s2[j] = _clamp(vwc / watsat[j], 0.01, 1.0)
        hk = np.empty(nl, complex)
        dhkdw = np.empty(nl, complex)
        smp = np.empty(nl, complex)
        dsmpdw = np.empty(nl, complex)
        for j in range(nl):
            s1 = s2[j] if j == nl - 1 else 0.5 * (s2[j] + s2[j + 1])
            s1 = _clamp(s1, 0.01, 1.0)
            hk[j] = imp[j] * hksat[j] * s1 ** (2.0 * bsw[j] + 3.0)
            dhkdw[j] = (2.0 * bsw[j] + 3.0) * hk[j] / s1
            smp[j] = -sucsat[j] * s2[j] ** (-bsw[j])
            dsmpdw[j] = (-bsw[j] * smp[j] / s2[j]) / watsat[j]
        qout = np.zeros(nl, complex)
        d1 = np.zeros(nl, complex)
        d2 = np.zeros(nl, complex)
        for j in range(nl - 1):
            k1 = 0.5 * dhkdw[j] / watsat[j]
            k2 = 0.5 * dhkdw[j] / watsat[j + 1]
            num = smp[j + 1] - smp[j]
            den = 1000.0 * (z[j + 1] - z[j])
            qout[j] = -hk[j] * num / den + hk[j]
            d1[j] = (hk[j] * dsmpdw[j] - k1 * num) / den + k1
            d2[j] = (-hk[j] * dsmpdw[j + 1] - k2 * num) / den + k2
        if lower_bc == "flux":
            qout[nl - 1] = hk[nl - 1]
            d1[nl - 1] = dhkdw[nl - 1] / watsat[nl - 1]
        qin = np.zeros(nl, complex)
        i0 = np.zeros(nl, complex)
        i1 = np.zeros(nl, complex)
        qin[1:] = qout[:-1]
        i0[1:] = d1[:-1]
        i1[1:] = d2[:-1]
        qin[0] = qflx_infl
        fnet = qin - qout - qflx_rootsoi
        while True:
            dtdz = dtdz_of(dtsub)
            A = np.zeros((nl, nl), complex)
            for j in range(nl):
                A[j, j] = -1.0 - (-i1[j] + d1[j]) * dtdz[j]
                if j > 0:
                    A[j, j - 1] = i0[j] * dtdz[j]
                if j < nl - 1:
                    A[j, j + 1] = -d2[j] * dtdz[j]
            dwat = np.linalg.solve(A, -fnet * dtdz)
            # error estimate (:1440-1457), inexpensive flux form
            err = np.max(np.abs(fnet.real - dwat.real / dtdz) * dtsub * 0.5)
            if err > cfg.xTolerUpper and dtsub > cfg.dtmin:
                dtsub = max(dtsub / 2.0, cfg.dtmin)
                nsub += 1
                continue
            break
        liq = liq + dwat * (1000.0 * dz)
        if lower_bc == "flux":
            qct = hk[nl - 1] + dhkdw[nl - 1] * dwat[nl - 1]
        else:
            qct = 0.0
        qc = qc + qct * (dtsub / dtime)
        dtdone += dtsub
        if abs(dtime - dtdone) < cfg.verySmall:
            return liq, qc, nsub
        nd = dtsub * 2.0 if err < cfg.xTolerLower else dtsub
        dtsub = min(nd, dtime - dtdone)


def complex_step(f, x0, i, h=1e-30):
    """d f / d x_i at x0 (f maps a complex vector to a complex scalar)."""
    x = np.asarray(x0, dtype=complex).copy()
    x[i] += 1j * h
    return f(x).imag / h
