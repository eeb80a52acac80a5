// adjoint_richards.cuh — closed-form reverse of one accepted substep of the
// moisture-form Richards solve, shared by the recording and the hand-written step
// adjoints.  ws, bb, suc, ks: the hydraulic parameters watsat, bsw, sucsat, hksat of
// levels 1..nl (1-based arrays).
#pragma once
#include "clmgb_device.cuh"

namespace clmgb {

// ---------------------------------------------------------------------------
// Closed-form reverse of one accepted substep of the moisture-form solve
// (soil_water_movement.jl:1274-1483).  The substep's values are recomputed from its
// starting water (the clamps and decisions with the production arithmetic; the
// derivative coefficients with reciprocals, and s^a as exp(a log s) from the logs
// the parameter derivatives need anyway), then its adjoint is formed section by
// section, last to first:
//   update    liq' = liq + dwat*1000 dz,  qc += qcT*dtsub/dtime
//   solve     A dwat = rmx (tridiagonal): lambda = A^-T dwat_bar by the same Thomas
//             sweep on the transposed bands (the tridiagonal_solve! rule,
//             enzyme_rules.jl:160-201), rmx_bar = lambda, band_bar = -lambda dwat^T
//   assembly  amx = dqidw0 dt_dz, bmx = -1 - (-dqidw1 + dqodw1) dt_dz,
//             cmx = -dqodw2 dt_dz, rmx = -fnet dt_dz
//   fluxes    qout, dqodw1, dqodw2 of each interface and the lower boundary
//   hydraulics  hk = imp ksat s1^(2b+3), dhkdw, smp = -sucsat s^-b, dsmpdw, with
//             the clamps of s and s1 passing the derivative only where the value
//             was not clamped (the branch Julia's max/min took).
// The parameter and impedance adjoints accumulate in RichardsBar across substeps.
// ---------------------------------------------------------------------------
struct RichardsBar {
  double ws[MAXSOI + 1], b[MAXSOI + 1], suc[MAXSOI + 1], ks[MAXSOI + 1], imp[MAXSOI + 1];
};

static __device__ __noinline__ void mf_substep_reverse(const Dims& D, const clmgb_soilwater_fields& f,
                                                const clmgb_swm_config& cfg, double dtime, int64_t c, int nl,
                                                const double* dzv, const double* imp, const double* ws,
                                                const double* bb, const double* suc, const double* ks,
                                                double dtsub, const double* liq, double* lamL, double lamQ,
                                                RichardsBar& R) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno, joff_zi = D.nlevsno + 1, nlevsoi = D.nlevsoi;
  const int lower_bc = cfg.lower_boundary_condition;
  // ---- forward values ----
  double s[MAXSOI + 2], s0[MAXSOI + 2], s1c[MAXSOI + 2], e[MAXSOI + 2], P[MAXSOI + 2], Q[MAXSOI + 2];
  double hk[MAXSOI + 2], dhkdw[MAXSOI + 2], smp[MAXSOI + 2], dsmpds[MAXSOI + 2], dsmpdw[MAXSOI + 2];
  bool lpass[MAXSOI + 2], spass[MAXSOI + 2], s1pass[MAXSOI + 2];
  double rws[MAXSOI + 2], rs[MAXSOI + 2], rs1[MAXSOI + 2], Ls[MAXSOI + 2], L1[MAXSOI + 2], rden[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) {
    lpass[j] = liq[j] >= 1.0e-6;         // Julia max(liq, 1e-6) took liq
    const double vwc = jl_max(liq[j], 1.0e-6) / (dzv[j] * DENH2O);
    s0[j] = vwc / ws[j];
    double sv = jl_min(s0[j], 1.0);
    sv = jl_max(0.01, sv);
    s[j] = sv;
    spass[j] = s0[j] <= 1.0 && s0[j] > 0.01;
    rws[j] = 1.0 / ws[j];
    rs[j] = 1.0 / sv;
    Ls[j] = ::cm_log(sv);
  }
  for (int j = 1; j <= nl; j++) {
    const double s1r = (j == nl) ? s[j] : 0.5 * (s[j] + s[j + 1]);
    double sv = jl_min(s1r, 1.0);
    sv = jl_max(0.01, sv);
    s1c[j] = sv;
    s1pass[j] = s1r <= 1.0 && s1r > 0.01;
    rs1[j] = 1.0 / sv;
    L1[j] = ::cm_log(sv);
    e[j] = 2.0 * bb[j] + 3.0;
    P[j] = ::cm_exp(e[j] * L1[j]);          // s1^e as a derivative coefficient
    hk[j] = imp[j] * ks[j] * P[j];
    dhkdw[j] = e[j] * hk[j] * rs1[j];
    Q[j] = ::cm_exp(-bb[j] * Ls[j]);
    smp[j] = -suc[j] * Q[j];
    dsmpds[j] = -bb[j] * smp[j] * rs[j];
    dsmpdw[j] = dsmpds[j] * rws[j];
  }
  double qout[MAXSOI + 2], d1[MAXSOI + 2], d2[MAXSOI + 2], den[MAXSOI + 2], num[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) { qout[j] = 0.0; d1[j] = 0.0; d2[j] = 0.0; }
  for (int j = 1; j <= nl - 1; j++) {
    const double dk1 = 0.5 * dhkdw[j] * rws[j];
    const double dk2 = 0.5 * dhkdw[j] * rws[j + 1];
    num[j] = smp[j + 1] - smp[j];
    den[j] = M_TO_MM * (LVc(f.z, c, joff + j + 1, ld) - LVc(f.z, c, joff + j, ld));
    rden[j] = 1.0 / den[j];
    qout[j] = -hk[j] * num[j] * rden[j] + hk[j];
    d1[j] = (hk[j] * dsmpdw[j] - dk1 * num[j]) * rden[j] + dk1;
    d2[j] = (-hk[j] * dsmpdw[j + 1] - dk2 * num[j]) * rden[j] + dk2;
  }
  bool wt_active = false;
  if (lower_bc == CLMGB_BC_WATERTABLE) {
    int jwt = nlevsoi;
    for (int jj = 1; jj <= nlevsoi; jj++) {
      if (f.zwt[c] <= LVc(f.zi, c, joff_zi + jj, ld)) { jwt = jj - 1; break; }
    }
    if (nl <= jwt) {
      wt_active = true;
      const double dk1l = dhkdw[nl] * rws[nl];
      num[nl] = -smp[nl];
      den[nl] = M_TO_MM * (f.zwt[c] - LVc(f.z, c, joff + nl, ld));
      rden[nl] = 1.0 / den[nl];
      qout[nl] = -hk[nl] * num[nl] * rden[nl] + hk[nl];
      d1[nl] = (hk[nl] * dsmpdw[nl] - dk1l * num[nl]) * rden[nl] + dk1l;
    }
  } else if (lower_bc == CLMGB_BC_FLUX) {
    qout[nl] = hk[nl];
    d1[nl] = dhkdw[nl] * rws[nl];
  }
  double dtdz[MAXSOI + 2], amx[MAXSOI + 2], bmx[MAXSOI + 2], cmx[MAXSOI + 2], dwat[MAXSOI + 2], gam[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) {
    const double qin = j == 1 ? f.qflx_infl[c] : qout[j - 1];
    const double i0 = j == 1 ? 0.0 : d1[j - 1];
    const double i1 = j == 1 ? 0.0 : d2[j - 1];
    const double fnet = qin - qout[j] - LVc(f.qflx_rootsoi, c, j, ld);
    dtdz[j] = dtsub / (M_TO_MM * dzv[j]);
    amx[j] = i0 * dtdz[j];
    bmx[j] = -1.0 - (-i1 + d1[j]) * dtdz[j];
    cmx[j] = j == nl ? 0.0 : -d2[j] * dtdz[j];
    dwat[j] = -fnet * dtdz[j];     // right-hand side, solved in place below
  }
  {
    double bet = bmx[1];
    if (abs_lt(bet, 1.0e-30)) bet = 1.0e-30;
    double rbet = 1.0 / bet;
    dwat[1] = dwat[1] * rbet;
    for (int j = 2; j <= nl; j++) {
      gam[j] = cmx[j - 1] * rbet;
      bet = bmx[j] - amx[j] * gam[j];
      if (abs_lt(bet, 1.0e-30)) bet = copysign(1.0e-30, bet == 0.0 ? 1.0 : bet);
      rbet = 1.0 / bet;
      dwat[j] = (dwat[j] - amx[j] * dwat[j - 1]) * rbet;
    }
    for (int j = nl - 1; j >= 1; j--) dwat[j] = dwat[j] - gam[j + 1] * dwat[j + 1];
  }
  // ---- reverse: update and drainage ----
  double g[MAXSOI + 2], hkb[MAXSOI + 2], dhkdwb[MAXSOI + 2], qoutb[MAXSOI + 2], d1b[MAXSOI + 2], d2b[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) {
    g[j] = lamL[j] * (M_TO_MM * dzv[j]);
    hkb[j] = 0.0; dhkdwb[j] = 0.0; qoutb[j] = 0.0; d1b[j] = 0.0; d2b[j] = 0.0;
  }
  const double cq = lamQ * (dtsub / dtime);
  if (lower_bc == CLMGB_BC_FLUX) {
    hkb[nl] += cq;
    dhkdwb[nl] += cq * dwat[nl];
    g[nl] += cq * dhkdw[nl];
  } else if (lower_bc != CLMGB_BC_ZERO_FLUX) {
    qoutb[nl] += cq;
    d1b[nl] += cq * dwat[nl];
    g[nl] += cq * d1[nl];
  }
  // ---- reverse: the tridiagonal solve (transposed Thomas sweep) ----
  double lam[MAXSOI + 2];
  {
    double cp[MAXSOI + 2];
    // A^T: sub_j = cmx[j-1], diag bmx[j], super_j = amx[j+1]
    const double rb1 = 1.0 / bmx[1];
    cp[1] = (nl > 1 ? amx[2] : 0.0) * rb1;
    lam[1] = g[1] * rb1;
    for (int j = 2; j <= nl; j++) {
      const double sub = cmx[j - 1];
      const double rdn = 1.0 / (bmx[j] - sub * cp[j - 1]);
      cp[j] = (j < nl ? amx[j + 1] : 0.0) * rdn;
      lam[j] = (g[j] - sub * lam[j - 1]) * rdn;
    }
    for (int j = nl - 1; j >= 1; j--) lam[j] = lam[j] - cp[j] * lam[j + 1];
  }
  // ---- reverse: assembly ----
  for (int j = 1; j <= nl; j++) {
    const double bmxb = -lam[j] * dwat[j];
    const double fnetb = -lam[j] * dtdz[j];
    // fnet_j = qin_j - qout_j - rootsoi_j ; qin_j = qout_{j-1} (j > 1)
    qoutb[j] -= fnetb;
    if (j > 1) {
      qoutb[j - 1] += fnetb;
      d1b[j - 1] += (-lam[j] * dwat[j - 1]) * dtdz[j];   // amx = dqidw0 dt_dz, dqidw0_j = dqodw1_{j-1}
      d2b[j - 1] += bmxb * dtdz[j];                       // bmx: -(-dqidw1) dt_dz, dqidw1_j = dqodw2_{j-1}
    }
    d1b[j] -= bmxb * dtdz[j];
    if (j < nl) d2b[j] -= (-lam[j] * dwat[j + 1]) * dtdz[j];
  }
  // ---- reverse: fluxes ----
  double smpb[MAXSOI + 2], dsmpdwb[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) { smpb[j] = 0.0; dsmpdwb[j] = 0.0; }
  double wsb[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) wsb[j] = 0.0;
  if (lower_bc == CLMGB_BC_FLUX) {
    hkb[nl] += qoutb[nl];
    dhkdwb[nl] += d1b[nl] * rws[nl];
    wsb[nl] -= d1b[nl] * d1[nl] * rws[nl];
  } else if (wt_active) {
    const double dk1l = dhkdw[nl] * rws[nl];
    double numb = qoutb[nl] * (-hk[nl] * rden[nl]);
    hkb[nl] += qoutb[nl] * (1.0 - num[nl] * rden[nl]);
    hkb[nl] += d1b[nl] * dsmpdw[nl] * rden[nl];
    dsmpdwb[nl] += d1b[nl] * hk[nl] * rden[nl];
    const double dk1lb = d1b[nl] * (1.0 - num[nl] * rden[nl]);
    numb += d1b[nl] * (-dk1l * rden[nl]);
    smpb[nl] -= numb;
    dhkdwb[nl] += dk1lb * rws[nl];
    wsb[nl] -= dk1lb * dk1l * rws[nl];
  }
  for (int j = 1; j <= nl - 1; j++) {
    const double dk1 = 0.5 * dhkdw[j] * rws[j];
    const double dk2 = 0.5 * dhkdw[j] * rws[j + 1];
    const double r = 1.0 - num[j] * rden[j];
    hkb[j] += qoutb[j] * r + d1b[j] * dsmpdw[j] * rden[j] - d2b[j] * dsmpdw[j + 1] * rden[j];
    double numb = -qoutb[j] * hk[j] * rden[j] - d1b[j] * dk1 * rden[j] - d2b[j] * dk2 * rden[j];
    dsmpdwb[j] += d1b[j] * hk[j] * rden[j];
    dsmpdwb[j + 1] -= d2b[j] * hk[j] * rden[j];
    const double dk1b = d1b[j] * r, dk2b = d2b[j] * r;
    smpb[j + 1] += numb;
    smpb[j] -= numb;
    dhkdwb[j] += 0.5 * dk1b * rws[j] + 0.5 * dk2b * rws[j + 1];
    wsb[j] -= dk1b * dk1 * rws[j];
    wsb[j + 1] -= dk2b * dk2 * rws[j + 1];
  }
  // ---- reverse: hydraulic properties ----
  double sb[MAXSOI + 2];
  for (int j = 1; j <= nl; j++) sb[j] = 0.0;
  for (int j = 1; j <= nl; j++) {
    const double dsb = dsmpdwb[j] * rws[j];
    wsb[j] -= dsmpdwb[j] * dsmpdw[j] * rws[j];
    R.b[j] += dsb * (-smp[j] * rs[j]);
    smpb[j] += dsb * (-bb[j] * rs[j]);
    sb[j] += dsb * (-dsmpds[j] * rs[j]);
    R.suc[j] += smpb[j] * (-Q[j]);
    const double Qb = smpb[j] * (-suc[j]);
    sb[j] += Qb * (-bb[j]) * Q[j] * rs[j];
    if (Qb != 0.0) R.b[j] += Qb * Q[j] * (-Ls[j]);
    double eb = dhkdwb[j] * hk[j] * rs1[j];
    hkb[j] += dhkdwb[j] * e[j] * rs1[j];
    double s1cb = dhkdwb[j] * (-dhkdw[j] * rs1[j]);
    R.imp[j] += hkb[j] * ks[j] * P[j];
    R.ks[j] += hkb[j] * imp[j] * P[j];
    const double Pb = hkb[j] * imp[j] * ks[j];
    s1cb += Pb * e[j] * P[j] * rs1[j];
    if (Pb != 0.0) eb += Pb * P[j] * L1[j];
    R.b[j] += 2.0 * eb;
    if (s1pass[j]) {
      if (j == nl) {
        sb[j] += s1cb;
      } else {
        sb[j] += 0.5 * s1cb;
        sb[j + 1] += 0.5 * s1cb;
      }
    }
  }
  for (int j = 1; j <= nl; j++) {
    double lb = lamL[j];
    if (spass[j]) {
      const double vwcb = sb[j] * rws[j];
      wsb[j] -= sb[j] * s0[j] * rws[j];
      if (lpass[j]) lb += vwcb / (dzv[j] * DENH2O);
    }
    lamL[j] = lb;
    R.ws[j] += wsb[j];
  }
}

}  // namespace clmgb
