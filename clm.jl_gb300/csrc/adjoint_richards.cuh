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

// The forward values are kept as sixteen level arrays (the saturation powers and logs,
// the reciprocals, the band and the two sweeps); every other forward quantity is
// formed again from them where the reverse needs it, by the same expression.  The
// reverse is one downward sweep that finishes the transposed back substitution, the
// assembly, the fluxes and the hydraulic properties level by level, with the adjoints
// of the levels still open (at most three) in registers: at level j, interface j's
// adjoints are complete once level j's assembly is reversed, level j+1's hydraulic
// adjoints once interface j is, and level j+2's saturation adjoint once level j+1's
// hydraulics are.
struct MfAcc {
  double smpb, dsmpdwb, hkb, dhkdwb, sb, wsb;
};
__device__ __forceinline__ void mf_acc_zero(MfAcc& a) { a.smpb = a.dsmpdwb = a.hkb = a.dhkdwb = a.sb = a.wsb = 0.0; }

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
  double P[MAXSOI + 2], Q[MAXSOI + 2], Ls[MAXSOI + 2], L1[MAXSOI + 2];
  double rs[MAXSOI + 2], rs1[MAXSOI + 2], rws[MAXSOI + 2], s0[MAXSOI + 2], rden[MAXSOI + 2];
  double dtdz[MAXSOI + 2], amx[MAXSOI + 2], bmx[MAXSOI + 2], cmx[MAXSOI + 2], gc[MAXSOI + 2];
  double dwat[MAXSOI + 2], lam[MAXSOI + 2];
  uint32_t lpass = 0, spass = 0, s1pass = 0;          // bit j: Julia's max/min took the unclamped value
  // saturation of level j (:1283-1287)
  auto saturation = [&](int j) -> double {
    const double vwc = jl_max(liq[j], 1.0e-6) / (dzv[j] * DENH2O);
    s0[j] = vwc / ws[j];
    double sv = jl_min(s0[j], 1.0);
    sv = jl_max(0.01, sv);
    if (liq[j] >= 1.0e-6) lpass |= 1u << j;
    if (s0[j] <= 1.0 && s0[j] > 0.01) spass |= 1u << j;
    return sv;
  };
  // hydraulic properties (:1288-1308), powers as exp(a log s) from the logs the
  // parameter derivatives need anyway
  double s_n = saturation(1);
  for (int j = 1; j <= nl; j++) {
    const double sj = s_n;
    if (j < nl) s_n = saturation(j + 1);
    rws[j] = 1.0 / ws[j];
    rs[j] = 1.0 / sj;
    Ls[j] = ::cm_log(sj);
    const double s1r = (j == nl) ? sj : 0.5 * (sj + s_n);
    double sv = jl_min(s1r, 1.0);
    sv = jl_max(0.01, sv);
    if (s1r <= 1.0 && s1r > 0.01) s1pass |= 1u << j;
    rs1[j] = 1.0 / sv;
    L1[j] = ::cm_log(sv);
    P[j] = ::cm_exp((2.0 * bb[j] + 3.0) * L1[j]);
    Q[j] = ::cm_exp(-bb[j] * Ls[j]);
  }
  struct Hyd { double e, hk, dhkdw, smp, dsmpds, dsmpdw; };
  auto hyd = [&](int j) -> Hyd {
    Hyd h;
    h.e = 2.0 * bb[j] + 3.0;
    h.hk = imp[j] * ks[j] * P[j];
    h.dhkdw = h.e * h.hk * rs1[j];
    h.smp = -suc[j] * Q[j];
    h.dsmpds = -bb[j] * h.smp * rs[j];
    h.dsmpdw = h.dsmpds * rws[j];
    return h;
  };
  // the water-table boundary is active when the bottom level lies above the table
  bool wt_active = false;
  if (lower_bc == CLMGB_BC_WATERTABLE) {
    int jwt = nlevsoi;
    for (int jj = 1; jj <= nlevsoi; jj++) {
      if (f.zwt[c] <= LVc(f.zi, c, joff_zi + jj, ld)) { jwt = jj - 1; break; }
    }
    wt_active = nl <= jwt;
  }
  // fluxes (:1310-1378), the band (:1380-1412) and the forward Thomas sweep, level by level
  double qout_p = 0.0, d1_p = 0.0, d2_p = 0.0;          // interface j-1
  double d1_nl = 0.0;
  double rbet = 0.0;
  Hyd hn = hyd(1);
  for (int j = 1; j <= nl; j++) {
    const Hyd hj = hn;
    double qo = 0.0, d1 = 0.0, d2 = 0.0;
    if (j < nl) {
      hn = hyd(j + 1);
      const double dk1 = 0.5 * hj.dhkdw * rws[j];
      const double dk2 = 0.5 * hj.dhkdw * rws[j + 1];
      const double num = hn.smp - hj.smp;
      rden[j] = 1.0 / (M_TO_MM * (LVc(f.z, c, joff + j + 1, ld) - LVc(f.z, c, joff + j, ld)));
      qo = -hj.hk * num * rden[j] + hj.hk;
      d1 = (hj.hk * hj.dsmpdw - dk1 * num) * rden[j] + dk1;
      d2 = (-hj.hk * hn.dsmpdw - dk2 * num) * rden[j] + dk2;
    } else if (wt_active) {
      const double dk1l = hj.dhkdw * rws[nl];
      const double num = -hj.smp;
      rden[nl] = 1.0 / (M_TO_MM * (f.zwt[c] - LVc(f.z, c, joff + nl, ld)));
      qo = -hj.hk * num * rden[nl] + hj.hk;
      d1 = (hj.hk * hj.dsmpdw - dk1l * num) * rden[nl] + dk1l;
    } else if (lower_bc == CLMGB_BC_FLUX) {
      qo = hj.hk;
      d1 = hj.dhkdw * rws[nl];
    }
    if (j == nl) d1_nl = d1;
    const double qin = j == 1 ? f.qflx_infl[c] : qout_p;
    const double i0 = j == 1 ? 0.0 : d1_p;
    const double i1 = j == 1 ? 0.0 : d2_p;
    const double fnet = qin - qo - LVc(f.qflx_rootsoi, c, j, ld);
    dtdz[j] = dtsub / (M_TO_MM * dzv[j]);
    amx[j] = i0 * dtdz[j];
    bmx[j] = -1.0 - (-i1 + d1) * dtdz[j];
    cmx[j] = j == nl ? 0.0 : -d2 * dtdz[j];
    const double rhs = -fnet * dtdz[j];
    if (j == 1) {
      double bet = bmx[1];
      if (abs_lt(bet, 1.0e-30)) bet = 1.0e-30;
      rbet = 1.0 / bet;
      dwat[1] = rhs * rbet;
    } else {
      gc[j] = cmx[j - 1] * rbet;
      double bet = bmx[j] - amx[j] * gc[j];
      if (abs_lt(bet, 1.0e-30)) bet = copysign(1.0e-30, bet == 0.0 ? 1.0 : bet);
      rbet = 1.0 / bet;
      dwat[j] = (rhs - amx[j] * dwat[j - 1]) * rbet;
    }
    qout_p = qo;
    d1_p = d1;
    d2_p = d2;
  }
  for (int j = nl - 1; j >= 1; j--) dwat[j] = dwat[j] - gc[j + 1] * dwat[j + 1];
  // ---- reverse: update and drainage ----
  MfAcc a0, a1, a2;                                       // levels j, j+1, j+2
  mf_acc_zero(a0);
  mf_acc_zero(a1);
  mf_acc_zero(a2);
  double QB = 0.0, D1B = 0.0, D2B = 0.0;                 // interface j, carried from level j+1
  const double cq = lamQ * (dtsub / dtime);
  double gnl = 0.0;
  if (lower_bc == CLMGB_BC_FLUX) {
    a0.hkb += cq;
    a0.dhkdwb += cq * dwat[nl];
    gnl = cq * hyd(nl).dhkdw;
  } else if (lower_bc != CLMGB_BC_ZERO_FLUX) {
    QB += cq;
    D1B += cq * dwat[nl];
    gnl = cq * d1_nl;
  }
  // ---- reverse: the tridiagonal solve, forward sweep on the transposed bands ----
  // A^T: sub_j = cmx[j-1], diag bmx[j], super_j = amx[j+1]; gc now holds cp
  {
    const double rb1 = 1.0 / bmx[1];
    gc[1] = (nl > 1 ? amx[2] : 0.0) * rb1;
    lam[1] = (lamL[1] * (M_TO_MM * dzv[1]) + (nl == 1 ? gnl : 0.0)) * rb1;
    for (int j = 2; j <= nl; j++) {
      const double sub = cmx[j - 1];
      const double rdn = 1.0 / (bmx[j] - sub * gc[j - 1]);
      gc[j] = (j < nl ? amx[j + 1] : 0.0) * rdn;
      const double gj = lamL[j] * (M_TO_MM * dzv[j]) + (j == nl ? gnl : 0.0);
      lam[j] = (gj - sub * lam[j - 1]) * rdn;
    }
  }
  // ---- reverse: one downward sweep (back substitution, assembly, fluxes, hydraulics) ----
  double lam_n = 0.0;                                     // lambda of level j+1
  for (int j = nl; j >= -1; j--) {
    if (j >= 1) {
      const double lj = (j == nl) ? lam[nl] : lam[j] - gc[j] * lam_n;
      lam_n = lj;
      // assembly (:1380-1412) of level j
      const double bmxb = -lj * dwat[j];
      const double fnetb = -lj * dtdz[j];
      QB -= fnetb;
      D1B -= bmxb * dtdz[j];
      if (j < nl) D2B -= (-lj * dwat[j + 1]) * dtdz[j];
      // the contributions of level j to interface j-1: fnet_j = qout_{j-1} - ...,
      // amx_j = dqodw1_{j-1} dt_dz, bmx_j = -(-dqodw2_{j-1}) dt_dz
      double QBn = 0.0, D1Bn = 0.0, D2Bn = 0.0;
      if (j > 1) {
        QBn = fnetb;
        D1Bn = (-lj * dwat[j - 1]) * dtdz[j];
        D2Bn = bmxb * dtdz[j];
      }
      // interface j (complete)
      const Hyd hj = hyd(j);
      if (j < nl) {
        const Hyd hn2 = hyd(j + 1);
        const double dk1 = 0.5 * hj.dhkdw * rws[j];
        const double dk2 = 0.5 * hj.dhkdw * rws[j + 1];
        const double num = hn2.smp - hj.smp;
        const double r = 1.0 - num * rden[j];
        a0.hkb += QB * r + D1B * hj.dsmpdw * rden[j] - D2B * hn2.dsmpdw * rden[j];
        const double numb = -QB * hj.hk * rden[j] - D1B * dk1 * rden[j] - D2B * dk2 * rden[j];
        a0.dsmpdwb += D1B * hj.hk * rden[j];
        a1.dsmpdwb -= D2B * hj.hk * rden[j];
        const double dk1b = D1B * r, dk2b = D2B * r;
        a1.smpb += numb;
        a0.smpb -= numb;
        a0.dhkdwb += 0.5 * dk1b * rws[j] + 0.5 * dk2b * rws[j + 1];
        a0.wsb -= dk1b * dk1 * rws[j];
        a1.wsb -= dk2b * dk2 * rws[j + 1];
      } else if (lower_bc == CLMGB_BC_FLUX) {
        a0.hkb += QB;
        a0.dhkdwb += D1B * rws[nl];
        a0.wsb -= D1B * d1_nl * rws[nl];
      } else if (wt_active) {
        const double dk1l = hj.dhkdw * rws[nl];
        const double num = -hj.smp;
        double numb = QB * (-hj.hk * rden[nl]);
        a0.hkb += QB * (1.0 - num * rden[nl]);
        a0.hkb += D1B * hj.dsmpdw * rden[nl];
        a0.dsmpdwb += D1B * hj.hk * rden[nl];
        const double dk1lb = D1B * (1.0 - num * rden[nl]);
        numb += D1B * (-dk1l * rden[nl]);
        a0.smpb -= numb;
        a0.dhkdwb += dk1lb * rws[nl];
        a0.wsb -= dk1lb * dk1l * rws[nl];
      }
      QB = QBn;
      D1B = D1Bn;
      D2B = D2Bn;
    }
    // hydraulic properties of level m = j+1 (:1288-1308)
    const int m = j + 1;
    if (m >= 1 && m <= nl) {
      const Hyd h = hyd(m);
      MfAcc& A = a1;
      const double dsb = A.dsmpdwb * rws[m];
      A.wsb -= A.dsmpdwb * h.dsmpdw * rws[m];
      R.b[m] += dsb * (-h.smp * rs[m]);
      A.smpb += dsb * (-bb[m] * rs[m]);
      A.sb += dsb * (-h.dsmpds * rs[m]);
      R.suc[m] += A.smpb * (-Q[m]);
      const double Qb = A.smpb * (-suc[m]);
      A.sb += Qb * (-bb[m]) * Q[m] * rs[m];
      if (Qb != 0.0) R.b[m] += Qb * Q[m] * (-Ls[m]);
      double eb = A.dhkdwb * h.hk * rs1[m];
      A.hkb += A.dhkdwb * h.e * rs1[m];
      double s1cb = A.dhkdwb * (-h.dhkdw * rs1[m]);
      R.imp[m] += A.hkb * ks[m] * P[m];
      R.ks[m] += A.hkb * imp[m] * P[m];
      const double Pb = A.hkb * imp[m] * ks[m];
      s1cb += Pb * h.e * P[m] * rs1[m];
      if (Pb != 0.0) eb += Pb * P[m] * L1[m];
      R.b[m] += 2.0 * eb;
      if ((s1pass >> m) & 1u) {
        if (m == nl) {
          A.sb += s1cb;
        } else {
          A.sb += 0.5 * s1cb;
          a2.sb += 0.5 * s1cb;
        }
      }
    }
    // saturation and the water of level k = j+2 (:1283-1287)
    const int k = j + 2;
    if (k >= 1 && k <= nl) {
      double lb = lamL[k];
      if ((spass >> k) & 1u) {
        const double vwcb = a2.sb * rws[k];
        a2.wsb -= a2.sb * s0[k] * rws[k];
        if ((lpass >> k) & 1u) lb += jl_div(vwcb, dzv[k] * DENH2O);
      }
      lamL[k] = lb;
      R.ws[k] += a2.wsb;
    }
    a2 = a1;
    a1 = a0;
    mf_acc_zero(a0);
  }
}

}  // namespace clmgb
