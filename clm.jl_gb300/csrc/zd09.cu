// zd09.cu — soilwater_zengdecker2009! (soil_water_movement.jl:1616-1764), the
// Zeng & Decker (2009) soil water method: equilibrium water content and matric
// potential from the water-table depth, one implicit tridiagonal solve over the
// soil layers plus an aquifer layer, aquifer recharge and the water deficit.
//
// The reference runs ten kernels over [nc, nlevsoi(+1)] scratch matrices with a
// synchronisation between each.  Every one of them is per column, so here one
// thread runs them all for its column in the reference's order, with the scratch
// rows in registers/local memory: _soilwm_mm_icefrac_kernel! (:97-127),
// _soilwm_zwtmm_kernel! (:143-150), _soilwm_jwt_vwczwt_kernel! (:289-327),
// _soilwm_voleq_zq_kernel! (:171-205), _soilwm_voleq_zq_aqu_kernel! (:346-366),
// _soilwm_hk_smp_kernel! (:223-270), _soilwm_aqu_zmm_kernel! (:385-397),
// _soilwm_tridiag_assemble_kernel! (:430-539), _tridiag_multi_kernel!
// (tridiagonal.jl:86-127), _soilwm_renew_qcharge_kernel! (:561-605),
// _soilwm_deficit_kernel! (:621-635).  smooth_min/max/ifelse are exact for Float64
// (smooth_ad.jl:91-149, 253-256); ^ is Julia's Float64 pow (cm_pow).
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int ZD_BLOCK = 128;
constexpr int ZN = MAXSOI + 3;     // soil layers + the aquifer layer, 1-based

__device__ void zd09_col(const Dims& D, const clmgb_zd09_fields& f, double e_ice, double dtime, int64_t c) {
  const int64_t ld = D.ldc;
  const int nlevsoi = D.nlevsoi, nlevgrnd = D.nlevgrnd;
  const int joff = D.nlevsno, joff_zi = D.nlevsno + 1;
  const double sdamp = 0.0;
  double zmm[ZN], dzmm[ZN], zimm[ZN + 1], icef[ZN], vwc_liq[ZN], vol_eq[ZN], zq[ZN];
  double hk[ZN], dhkdw[ZN], smp[ZN], dsmpdw[ZN], imped[ZN];
  double qin[ZN], qout[ZN], dqidw0[ZN], dqidw1[ZN], dqodw1[ZN], dqodw2[ZN];
  double amx[ZN], bmx[ZN], cmx[ZN], rmx[ZN], dwat2[ZN];
  for (int j = 1; j <= nlevsoi + 1; j++) {
    zmm[j] = 0.0; dzmm[j] = 0.0; vol_eq[j] = 0.0; zq[j] = 0.0;
    qin[j] = 0.0; qout[j] = 0.0; dqidw0[j] = 0.0; dqidw1[j] = 0.0; dqodw1[j] = 0.0; dqodw2[j] = 0.0;
    amx[j] = 0.0; bmx[j] = 0.0; cmx[j] = 0.0; rmx[j] = 0.0;
  }
  // ---- geometry in mm, ice and liquid volume fractions ----
  for (int j = 1; j <= nlevsoi; j++) {
    zmm[j] = LVc(f.z, c, joff + j, ld) * 1.0e3;
    dzmm[j] = LVc(f.dz, c, joff + j, ld) * 1.0e3;
    zimm[j + 1] = LVc(f.zi, c, joff_zi + j, ld) * 1.0e3;
    const double ws = LVc(f.watsat, c, j, ld);
    const double dzj = LVc(f.dz, c, joff + j, ld);
    const double vol_ice = jl_min(ws, LVc(f.h2osoi_ice, c, joff + j, ld) / (dzj * DENICE));
    icef[j] = jl_min(1.0, vol_ice / ws);
    LV(f.icefrac, c, j, ld) = icef[j];
    vwc_liq[j] = jl_max(LV(f.h2osoi_liq, c, joff + j, ld), 1.0e-6) / (dzj * DENH2O);
  }
  // ---- water table in mm ----
  zimm[1] = 0.0;
  const double zwtmm = f.zwt[c] * 1.0e3;
  // ---- layer above the water table, water content at the water table ----
  int jwt = nlevsoi;
  for (int j = 1; j <= nlevsoi; j++) {
    if (f.zwt[c] <= LVc(f.zi, c, joff_zi + j, ld)) {
      jwt = j - 1;
      break;
    }
  }
  double vwc_zwt = LVc(f.watsat, c, nlevsoi, ld);
  if (LVc(f.t_soisno, c, joff + jwt + 1, ld) < TFRZ) {
    double v = vwc_liq[nlevsoi];
    for (int j = nlevsoi; j <= nlevgrnd; j++) {
      if (f.zwt[c] <= LVc(f.zi, c, joff_zi + j, ld)) {
        const double t = LVc(f.t_soisno, c, joff + j, ld);
        double smp1 = HFUS * (TFRZ - t) / (GRAV * t) * 1000.0;
        smp1 = jl_max(LVc(f.sucsat, c, nlevsoi, ld), smp1);
        v = LVc(f.watsat, c, nlevsoi, ld) *
            cm_pow(smp1 / LVc(f.sucsat, c, nlevsoi, ld), -1.0 / LVc(f.bsw, c, nlevsoi, ld));
        v = jl_min(v, 0.5 * (LVc(f.watsat, c, nlevsoi, ld) + LVc(f.h2osoi_vol, c, nlevsoi, ld)));
        break;
      }
    }
    vwc_zwt = v;
  }
  // ---- equilibrium water content and matric potential ----
  const double smpmin = f.smpmin[c];
  for (int j = 1; j <= nlevsoi; j++) {
    const double zimm_jm1 = zimm[j], zimm_j = zimm[j + 1];
    const double ws = LVc(f.watsat, c, j, ld), suc = LVc(f.sucsat, c, j, ld), b = LVc(f.bsw, c, j, ld);
    const double zwt = zwtmm;
    const double onem1b = 1.0 - 1.0 / b;
    if (zwt <= zimm_jm1) {
      vol_eq[j] = ws;
    } else if (zwt < zimm_j && zwt > zimm_jm1) {
      const double tempi = 1.0;
      const double temp0 = cm_pow((suc + zwt - zimm_jm1) / suc, onem1b);
      const double voleq1 = -suc * ws / onem1b / (zwt - zimm_jm1) * (tempi - temp0);
      double v = (voleq1 * (zwt - zimm_jm1) + ws * (zimm_j - zwt)) / (zimm_j - zimm_jm1);
      v = jl_min(ws, v);
      vol_eq[j] = jl_max(v, 0.0);
    } else {
      const double tempi = cm_pow((suc + zwt - zimm_j) / suc, onem1b);
      const double temp0 = cm_pow((suc + zwt - zimm_jm1) / suc, onem1b);
      double v = -suc * ws / onem1b / (zimm_j - zimm_jm1) * (tempi - temp0);
      v = jl_max(v, 0.0);
      vol_eq[j] = jl_min(ws, v);
    }
    const double zqv = -suc * cm_pow(jl_max(vol_eq[j] / ws, 0.01), -b);
    zq[j] = jl_max(smpmin, zqv);
  }
  // aquifer layer when the water table is below the soil column
  if (jwt == nlevsoi) {
    const int j = nlevsoi;
    const double suc = LVc(f.sucsat, c, j, ld), ws = LVc(f.watsat, c, j, ld), b = LVc(f.bsw, c, j, ld);
    const double zwt = zwtmm;
    const double zimm_j = zimm[j + 1];
    const double onem1b = 1.0 - 1.0 / b;
    const double tempi = 1.0;
    const double temp0 = cm_pow((suc + zwt - zimm_j) / suc, onem1b);
    double v = -suc * ws / onem1b / (zwt - zimm_j) * (tempi - temp0);
    v = jl_max(v, 0.0);
    v = jl_min(ws, v);
    vol_eq[j + 1] = v;
    const double zqv = -suc * cm_pow(jl_max(v / ws, 0.01), -b);
    zq[j + 1] = jl_max(smpmin, zqv);
  }
  // ---- hydraulic conductivity, matric potential and their derivatives ----
  for (int j = 1; j <= nlevsoi; j++) {
    const int jp1 = min(nlevsoi, j + 1);
    const double b = LVc(f.bsw, c, j, ld);
    const double wsj = LVc(f.watsat, c, j, ld), wsp = LVc(f.watsat, c, jp1, ld);
    double s1 = 0.5 * (vwc_liq[j] + vwc_liq[jp1]) / (0.5 * (wsj + wsp));
    s1 = jl_min(1.0, s1);
    const double s2 = LVc(f.hksat, c, j, ld) * cm_pow(s1, 2.0 * b + 2.0);
    const double imp = cm_pow(10.0, -e_ice * (0.5 * (icef[j] + icef[jp1])));
    imped[j] = imp;
    hk[j] = imp * s1 * s2;
    dhkdw[j] = imp * (2.0 * b + 3.0) * s2 * (1.0 / (wsj + wsp));
    double s_node = jl_max(vwc_liq[j] / wsj, 0.01);
    s_node = jl_min(1.0, s_node);
    double smpv = -LVc(f.sucsat, c, j, ld) * cm_pow(s_node, -b);
    smpv = jl_max(smpmin, smpv);
    smp[j] = smpv;
    dsmpdw[j] = -b * smpv / vwc_liq[j];
    LV(f.smp_l, c, j, ld) = smpv;
    LV(f.hk_l, c, j, ld) = hk[j];
  }
  // ---- aquifer layer geometry ----
  zmm[nlevsoi + 1] = 0.5 * (1.0e3 * f.zwt[c] + zmm[nlevsoi]);
  if (jwt < nlevsoi) dzmm[nlevsoi + 1] = dzmm[nlevsoi];
  else dzmm[nlevsoi + 1] = 1.0e3 * f.zwt[c] - zmm[nlevsoi];
  // ---- tridiagonal system ----
  {
    const int j = 1;
    qin[j] = f.qflx_infl[c];
    const double den = zmm[j + 1] - zmm[j];
    const double dzq = zq[j + 1] - zq[j];
    const double num = (smp[j + 1] - smp[j]) - dzq;
    qout[j] = -hk[j] * num / den;
    dqodw1[j] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
    dqodw2[j] = -(hk[j] * dsmpdw[j + 1] + num * dhkdw[j]) / den;
    rmx[j] = qin[j] - qout[j] - LVc(f.qflx_rootsoi, c, j, ld);
    amx[j] = 0.0;
    bmx[j] = dzmm[j] * (sdamp + 1.0 / dtime) + dqodw1[j];
    cmx[j] = dqodw2[j];
  }
  for (int j = 2; j <= nlevsoi - 1; j++) {
    double den = zmm[j] - zmm[j - 1];
    double dzq = zq[j] - zq[j - 1];
    double num = (smp[j] - smp[j - 1]) - dzq;
    qin[j] = -hk[j - 1] * num / den;
    dqidw0[j] = -(-hk[j - 1] * dsmpdw[j - 1] + num * dhkdw[j - 1]) / den;
    dqidw1[j] = -(hk[j - 1] * dsmpdw[j] + num * dhkdw[j - 1]) / den;
    den = zmm[j + 1] - zmm[j];
    dzq = zq[j + 1] - zq[j];
    num = (smp[j + 1] - smp[j]) - dzq;
    qout[j] = -hk[j] * num / den;
    dqodw1[j] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
    dqodw2[j] = -(hk[j] * dsmpdw[j + 1] + num * dhkdw[j]) / den;
    rmx[j] = qin[j] - qout[j] - LVc(f.qflx_rootsoi, c, j, ld);
    amx[j] = -dqidw0[j];
    bmx[j] = dzmm[j] / dtime - dqidw1[j] + dqodw1[j];
    cmx[j] = dqodw2[j];
  }
  {
    const int j = nlevsoi;
    if (j > jwt) {   // the water table is in the soil column
      const double den = zmm[j] - zmm[j - 1];
      const double dzq = zq[j] - zq[j - 1];
      const double num = (smp[j] - smp[j - 1]) - dzq;
      qin[j] = -hk[j - 1] * num / den;
      dqidw0[j] = -(-hk[j - 1] * dsmpdw[j - 1] + num * dhkdw[j - 1]) / den;
      dqidw1[j] = -(hk[j - 1] * dsmpdw[j] + num * dhkdw[j - 1]) / den;
      qout[j] = 0.0;
      dqodw1[j] = 0.0;
      rmx[j] = qin[j] - qout[j] - LVc(f.qflx_rootsoi, c, j, ld);
      amx[j] = -dqidw0[j];
      bmx[j] = dzmm[j] / dtime - dqidw1[j] + dqodw1[j];
      cmx[j] = 0.0;
      // aquifer layer: hydrologically inactive
      rmx[j + 1] = 0.0;
      amx[j + 1] = 0.0;
      bmx[j + 1] = dzmm[j + 1] / dtime;
      cmx[j + 1] = 0.0;
    } else {         // the water table is below the soil column
      const double wsj = LVc(f.watsat, c, j, ld);
      double s_node = jl_max(0.5 * ((vwc_zwt + vwc_liq[j]) / wsj), 0.01);
      s_node = jl_min(1.0, s_node);
      double smp1 = -LVc(f.sucsat, c, j, ld) * cm_pow(s_node, -LVc(f.bsw, c, j, ld));
      smp1 = jl_max(smpmin, smp1);
      const double dsmpdw1 = -LVc(f.bsw, c, j, ld) * smp1 / (s_node * wsj);
      double den = zmm[j] - zmm[j - 1];
      double dzq = zq[j] - zq[j - 1];
      double num = (smp[j] - smp[j - 1]) - dzq;
      qin[j] = -hk[j - 1] * num / den;
      dqidw0[j] = -(-hk[j - 1] * dsmpdw[j - 1] + num * dhkdw[j - 1]) / den;
      dqidw1[j] = -(hk[j - 1] * dsmpdw[j] + num * dhkdw[j - 1]) / den;
      den = zmm[j + 1] - zmm[j];
      dzq = zq[j + 1] - zq[j];
      num = (smp1 - smp[j]) - dzq;
      qout[j] = -hk[j] * num / den;
      dqodw1[j] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
      dqodw2[j] = -(hk[j] * dsmpdw1 + num * dhkdw[j]) / den;
      rmx[j] = qin[j] - qout[j] - LVc(f.qflx_rootsoi, c, j, ld);
      amx[j] = -dqidw0[j];
      bmx[j] = dzmm[j] / dtime - dqidw1[j] + dqodw1[j];
      cmx[j] = dqodw2[j];
      // aquifer layer
      qin[j + 1] = qout[j];
      dqidw0[j + 1] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
      dqidw1[j + 1] = -(hk[j] * dsmpdw1 + num * dhkdw[j]) / den;
      qout[j + 1] = 0.0;
      dqodw1[j + 1] = 0.0;
      rmx[j + 1] = qin[j + 1] - qout[j + 1];
      amx[j + 1] = -dqidw0[j + 1];
      bmx[j + 1] = dzmm[j + 1] / dtime - dqidw1[j + 1] + dqodw1[j + 1];
      cmx[j + 1] = 0.0;
    }
  }
  // ---- tridiagonal_multi! over the soil layers and the aquifer layer (jtop = 1) ----
  {
    const int n = nlevsoi + 1;
    double cpv[ZN];
    double bet = bmx[1];
    if (abs_lt(bet, 1.0e-30)) bet = 1.0e-30;
    double cp_prev = cmx[1] / bet;
    double dp_prev = rmx[1] / bet;
    cpv[1] = cp_prev;
    dwat2[1] = dp_prev;
    for (int jj = 2; jj <= n; jj++) {
      double denom = bmx[jj] - amx[jj] * cp_prev;
      if (abs_lt(denom, 1.0e-30)) denom = copysign(1.0e-30, denom == 0.0 ? 1.0 : denom);
      cp_prev = cmx[jj] / denom;
      dp_prev = (rmx[jj] - amx[jj] * dp_prev) / denom;
      cpv[jj] = cp_prev;
      dwat2[jj] = dp_prev;
    }
    double u_next = dp_prev;
    dwat2[n] = u_next;
    for (int jj = n - 1; jj >= 1; jj--) {
      u_next = dwat2[jj] - cpv[jj] * u_next;
      dwat2[jj] = u_next;
    }
  }
  // ---- renew the liquid water, aquifer recharge ----
  for (int j = 1; j <= nlevsoi; j++) LV(f.h2osoi_liq, c, joff + j, ld) = LV(f.h2osoi_liq, c, joff + j, ld) + dwat2[j] * dzmm[j];
  double qc;
  if (jwt < nlevsoi) {
    const int jw = jwt;
    const double wh_zwt = 0.0;
    const double s_node = jl_max(LVc(f.h2osoi_vol, c, jw + 1, ld) / LVc(f.watsat, c, jw + 1, ld), 0.01);
    const double s1 = jl_min(1.0, s_node);
    const double ka = imped[jw + 1] * LVc(f.hksat, c, jw + 1, ld) * cm_pow(s1, 2.0 * LVc(f.bsw, c, jw + 1, ld) + 3.0);
    const int jm = jw > 1 ? jw : 1;
    const double smp1 = jl_max(smpmin, smp[jm]);
    const double wh = smp1 - zq[jm];
    if (jw == 0) qc = -ka * (wh_zwt - wh) / ((f.zwt[c] + 1.0e-3) * 1000.0);
    else qc = -ka * (wh_zwt - wh) / ((f.zwt[c] - LVc(f.z, c, joff + jw, ld)) * 1000.0 * 2.0);
    qc = jl_max(-10.0 / dtime, qc);
    qc = jl_min(10.0 / dtime, qc);
  } else {
    qc = dwat2[nlevsoi + 1] * dzmm[nlevsoi + 1] / dtime;
  }
  f.qcharge[c] = qc;
  // ---- water deficit ----
  double acc = 0.0;
  for (int j = 1; j <= nlevsoi; j++) {
    const double l = LV(f.h2osoi_liq, c, joff + j, ld);
    acc = acc + (l >= 0.0 ? 0.0 : -l);
  }
  f.qflx_deficit[c] = acc;
}

__global__ void __launch_bounds__(ZD_BLOCK)
k_zd09(Dims D, int64_t nc, clmgb_zd09_fields f, double e_ice, double dtime) {
  const int64_t c = (int64_t)blockIdx.x * ZD_BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_hydrology[c]) return;
  zd09_col(D, f, e_ice, dtime, c);
}

}  // namespace

cudaError_t launch_zd09(const Dims& D, int64_t nc, const clmgb_zd09_fields& f, double e_ice, double dtime,
                        cudaStream_t s) {
  k_zd09<<<(unsigned int)((nc + ZD_BLOCK - 1) / ZD_BLOCK), ZD_BLOCK, 0, s>>>(D, nc, f, e_ice, dtime);
  return cudaGetLastError();
}

}  // namespace clmgb
