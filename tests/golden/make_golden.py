"""Writes tests/golden/reference_cases.json: the known-answer fixtures of CLM.jl's
own test suite for this path, transcribed from its test files (cited per case).

CLM.jl is Julia and cannot run here, so these are the reference's hand-built inputs
and analytic answers (x = 1:n solutions, [1,1,1], impedance powers, conservation
identities), not outputs captured from a run.  Run:  python tests/golden/make_golden.py
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def penta(n):
    # test_band_diagonal.jl:52-89 (n=5) and :114-139 (n=6): diag 10, +-1 off -2, +-2 off -1
    A = np.diag(np.full(n, 10.0)) + np.diag(np.full(n - 1, -2.0), -1) + np.diag(np.full(n - 1, -2.0), 1) \
        + np.diag(np.full(n - 2, -1.0), -2) + np.diag(np.full(n - 2, -1.0), 2)
    return A


def tri(n, d, o):
    return np.diag(np.full(n, d)) + np.diag(np.full(n - 1, o), -1) + np.diag(np.full(n - 1, o), 1)


def band_case(A, x, jtop, nlevs, kl, ku, tol, src):
    n = A.shape[0]
    nband = kl + ku + 1
    rhs = A @ x
    bm = np.zeros((nband, nlevs))
    r = np.zeros(nlevs)
    for i in range(n):
        lev = jtop - 1 + i
        r[lev] = rhs[i]
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            band = (i - j) + kl  # 0-based: band 1 = A[i, i+ku]
            bm[band, lev] = A[i, j]
    return dict(bmatrix=bm.tolist(), rvector=r.tolist(), x_exact=x.tolist(), jtop=jtop,
                jbot=jtop + n - 1, nlevs=nlevs, kl=kl, ku=ku, atol=tol, source=src)


def main():
    cases = {}
    cases["band_penta5"] = band_case(penta(5), np.arange(1.0, 6.0), 1, 5, 2, 2, 1e-10,
                                     "test/test_band_diagonal.jl:52-89")
    cases["band_penta6"] = band_case(penta(6), np.arange(1.0, 7.0), 1, 6, 2, 2, 1e-10,
                                     "test/test_band_diagonal.jl:114-139")
    cases["band_tri4"] = band_case(tri(4, 4.0, -1.0), np.array([1.0, 2.0, 3.0, 4.0]), 1, 4, 1, 1, 1e-12,
                                   "test/test_band_diagonal.jl:6-49")
    cases["band_partial"] = band_case(tri(4, 5.0, -1.0), np.array([2.0, 4.0, 6.0, 8.0]), 3, 8, 1, 1, 1e-12,
                                      "test/test_band_diagonal.jl:174-202")
    cases["tridiag_3x3"] = dict(a=[0.0, -1.0, -1.0], b=[2.0, 2.0, 2.0], c=[-1.0, -1.0, 0.0],
                                r=[1.0, 0.0, 1.0], jtop=1, u=[1.0, 1.0, 1.0], atol=1e-12,
                                source="test/test_tridiagonal.jl:6-16")
    cases["tridiag_identity"] = dict(a=[0.0] * 5, b=[1.0] * 5, c=[0.0] * 5, r=[1.0, 2.0, 3.0, 4.0, 5.0],
                                     jtop=1, u=[1.0, 2.0, 3.0, 4.0, 5.0], atol=1e-14,
                                     source="test/test_tridiagonal.jl:18-28")
    cases["tridiag_partial"] = dict(a=[0.0, 0.0, 0.0, -1.0, -1.0], b=[1.0, 1.0, 2.0, 2.0, 2.0],
                                    c=[0.0, 0.0, -1.0, -1.0, 0.0], r=[0.0, 0.0, 1.0, 0.0, 1.0], jtop=3,
                                    u=[None, None, 1.0, 1.0, 1.0], atol=1e-12,
                                    source="test/test_tridiagonal.jl:30-45")
    coeff = 1.0e-6 * 3600.0 / (0.1 ** 2)
    cases["tridiag_residual"] = dict(a=[0.0] + [-coeff] * 9, b=[1.0 + 2.0 * coeff] * 10,
                                     c=[-coeff] * 9 + [0.0], r=[300.0 - 2.0 * j for j in range(1, 11)],
                                     jtop=1, atol=1e-10, source="test/test_tridiagonal.jl:47-68")
    cases["tridiag_col_3x3"] = dict(a=[0.0, -1.0, -1.0], b=[2.0, 2.0, 2.0], c=[-1.0, -1.0, 0.0],
                                    r=[1.0, 0.0, 1.0], jtop=1, lbj=1, ubj=3, u=[1.0, 1.0, 1.0], atol=1e-12,
                                    source="test/test_soil_water_movement.jl:95-118")
    cases["tridiag_col_jtop"] = dict(a=[0.0, 0.0, -1.0, -1.0], b=[1.0, 2.0, 2.0, 2.0], c=[0.0, -1.0, -1.0, 0.0],
                                     r=[0.0, 1.0, 0.0, 1.0], jtop=2, lbj=1, ubj=4, atol=1e-12,
                                     source="test/test_soil_water_movement.jl:120-134")
    # test/test_enzyme_smoke.jl:194-248 — fixed 9-level system, jtop=3, objective sum(w .* u)
    cases["tridiag_adjoint9"] = dict(
        n=9, jtop=3,
        a=[0.0, 0.0, 0.0, 0.31, -0.22, 0.44, -0.17, 0.28, -0.39],
        b=[3.4, 3.1, 3.9, 3.2, 3.7, 3.3, 3.5, 3.8, 3.6],
        c=[-0.25, 0.33, -0.41, 0.19, -0.29, 0.37, -0.21, 0.24, 0.0],
        r=[0.7, -1.2, 0.4, 1.9, -0.6, 0.3, -1.1, 0.8, 0.2],
        w=[0.9, -0.4, 1.3, 0.2, -1.7, 0.6, 0.5, -0.8, 1.1],
        tol_vs_exact=1e-10, tol_vs_fd=1e-6, source="test/test_enzyme_smoke.jl:194-248")
    cases["ice_impedance"] = dict(values=[[0.0, 6.0, 1.0], [1.0, 6.0, 1.0e-6], [0.5, 6.0, 10.0 ** -3.0],
                                          [0.5, 4.0, 10.0 ** -2.0]],
                                  source="test/test_soil_water_movement.jl:76-88")
    cases["swm_config_defaults"] = dict(dtmin=60.0, verySmall=1.0e-8, xTolerUpper=1.0e-1, xTolerLower=1.0e-2,
                                        expensive=42, inexpensive=1, flux_calculation=1, e_ice=6.0,
                                        source="test/test_soil_water_movement.jl:18-31")
    # test/test_soil_water_movement.jl:272-336
    cases["moisture_form_conservation"] = dict(nc=12, nlev=10, nlevsno=5, dtime=1800.0, dz=0.05,
                                               watsat=0.45, hksat=0.02, bsw=5.0, sucsat=100.0,
                                               qflx_infl=1.0e-5, liq_profile="(0.30+0.01*j)*watsat*dz*1000",
                                               rtol=1e-10, source="test/test_soil_water_movement.jl:272-336")
    # test/test_soil_temperature.jl:1-226 (setup_soil_column!)
    cases["soiltemp_fixture"] = dict(nlevsno=5, nlevgrnd=10, nlevurb=5, nlevmaxurbgrnd=10, nlevsoi=8, nc=4,
                                     t=280.0, liq=5.0, watsat=0.45, bsw=5.0, sucsat=100.0, tkmg=2.0,
                                     tkdry=0.25, csol=2.0e6, emg=0.97, dlrad=50.0, cgrnd=5.0, sh=10.0,
                                     sabg=100.0, sabg_soil=100.0, sabg_snow=0.0, sabg_lyr_top=100.0,
                                     source="test/test_soil_temperature.jl:41-226")
    cases["phase_change_melt"] = dict(j=2, ice=5.0, liq=2.0, dT=2.0, dtime=1800.0, dhsdT=-5.0,
                                      source="test/test_soil_temperature.jl:566-599")
    cases["phase_change_mass"] = dict(layers=[[4.0, 1.0, 3.0], [0.0, 6.0, -3.0], [7.0, 0.0, -1.0],
                                              [0.0, 0.0, -1.0], [0.5, 0.05, 0.5]],
                                      atol=1e-12, rtol=1e-12, dtime=1800.0, dhsdT=-5.0,
                                      source="test/test_soil_temperature.jl:613-666")
    cases["phase_change_h2osfc_depth"] = dict(snl=-1, ice0=40.0, snow_depth=0.10, frac_sno_eff=1.0,
                                              frac_h2osfc=0.5, h2osfc=20.0, dT=-1.0, fact0=1.0, c_h2osfc=0.0,
                                              dtime=1800.0, dhsdT=-1000.0,
                                              source="test/test_soil_temperature.jl:498-532")
    with open(os.path.join(HERE, "reference_cases.json"), "w") as fh:
        json.dump(cases, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
