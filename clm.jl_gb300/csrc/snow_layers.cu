// snow_layers.cu — the snow layer dynamics of clm_drv_core! after the soil solve
// (clm_driver.jl:2146-2200): compaction, combination of thin layers, division of thick
// ones, zeroing of the emptied levels and the rebuilt snow filter.  They make the
// snow-layer count snl of the next step.
//
// Each routine is a per-column sequence over at most nlevsno (<= 12) snow levels with
// loop-carried state (the overburden, the layer shifts, the top-down split), so one
// thread owns one column: it loads the column's snow levels into on-chip arrays once,
// runs the selected routines in the driver's order on them, and stores them once.  The
// arithmetic is the reference's, expression by expression, so the results are its bits.
#include <cfloat>

#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int SL_BLOCK = 64;
constexpr int NAER = 8;                 // bcphi, bcpho, ocphi, ocpho, dst1..dst4
constexpr double LSADZ = 0.03;          // snow_hydrology.jl:130
constexpr int64_t ISTDLAK = 5;          // landunit_varcon.jl:11

// Layer thresholds of init_snow_layers! (snow_hydrology.jl:2357-2377); the deepest
// level never divides.
struct SnowThresh {
  double dzmin[MAXSNO], dzmax_l[MAXSNO], dzmax_u[MAXSNO];
};

// The snow levels of one column, index jj-1 for CLM.jl's combined level jj = 1..nlevsno.
struct SnowCol {
  double dz[MAXSNO], z[MAXSNO], zi[MAXSNO + 1], t[MAXSNO], ice[MAXSNO], liq[MAXSNO], rds[MAXSNO];
  double aer[NAER][MAXSNO];
  double liq1, ice1;                     // soil level 1
};

// combo_scalar (snow_hydrology.jl:1960-2000): two elements merged, heat conserved
__device__ __forceinline__ void combo(double& dz, double& wliq, double& wice, double& t, double dz2, double wliq2,
                                      double wice2, double t2) {
  const double dzc = dz + dz2;
  const double wicec = wice + wice2;
  const double wliqc = wliq + wliq2;
  const double h = (CPICE * wice + CPLIQ * wliq) * (t - TFRZ) + HFUS * wliq;
  const double h2 = (CPICE * wice2 + CPLIQ * wliq2) * (t2 - TFRZ) + HFUS * wliq2;
  const double hc = h + h2;
  const double denom = CPICE * wicec + CPLIQ * wliqc;
  t = denom > 0.0 ? TFRZ + (hc - HFUS * wliqc) / denom : TFRZ;
  dz = dzc;
  wliq = wliqc;
  wice = wicec;
}

// Julia's clamp(x, lo, hi) (NaN passes through)
__device__ __forceinline__ double jl_clamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

// mass_weighted_snow_radius (snow_hydrology.jl:2021-2031)
__device__ __forceinline__ double mass_weighted_radius(double rds1, double rds2, double swtot, double zwtot,
                                                       double rmin, double rmax) {
  const double total = swtot + zwtot;
  const double r = total > 0.0 ? (rds2 * swtot + rds1 * zwtot) / total : 0.5 * (rds1 + rds2);
  return jl_clamp(r, rmin, rmax);
}

// snow_compaction! for one column (_snowhyd_compaction_kernel!, :1203-1326)
__device__ void compaction(const clmgb_snowlayer_fields& f, const clmgb_snowlayer_config& P, SnowCol& S, int64_t c,
                           int64_t snl, int ns, int64_t ld, double dtime) {
  constexpr double C3 = 2.777e-6, C4 = 0.04, C5 = 2.0;
  const double fsno = f.frac_sno[c];
  double burden = 0.0, zpseudo = 0.0;
  bool mobile = true;
  for (int j = -ns + 1; j <= 0; j++) {
    if (j < snl + 1) continue;
    const int k = j + ns - 1;
    const double ice = S.ice[k], liq = S.liq[k];
    const double wx = ice + liq;
    const double voidf = 1.0 - (ice / DENICE + liq / DENH2O) / (fsno * S.dz[k]);
    if (voidf > 0.001 && ice > 0.1) {
      const double bi = ice / (fsno * S.dz[k]);
      const double fi = ice / wx;
      const double td = TFRZ - S.t[k];
      const double dexpf = cm_exp(-C4 * td);
      // destructive metamorphism
      double ddz1 = -C3 * dexpf;
      if (bi > P.upplim_destruct_metamorph) ddz1 = ddz1 * cm_exp(-46.0e-3 * (bi - P.upplim_destruct_metamorph));
      if (liq > 0.01 * S.dz[k] * fsno) ddz1 = ddz1 * C5;                   // liquid water
      // overburden (:1412-1418 Anderson 1976, :1437-1448 Vionnet 2012)
      double ddz2;
      if (P.overburden_method == CLMGB_OVERBURDEN_ANDERSON1976) {
        ddz2 = -(burden + wx / 2.0) * cm_exp(-P.overburden_compress_tfactor * td - 23.0e-3 * bi) / P.eta0_anderson;
      } else {
        const double f1 = 1.0 / (1.0 + 60.0 * liq / (DENH2O * S.dz[k]));
        const double eta = f1 * 4.0 * (bi / P.ceta) * cm_exp(0.1 * td + 0.023 * bi) * P.eta0_vionnet;
        ddz2 = -(burden + wx / 2.0) / eta;
      }
      // melt
      double ddz3 = 0.0;
      if (LVc(f.imelt, c, k + 1, ld) == 1) {
        const int64_t l = f.col_landunit[c] - 1;
        if (P.use_subgrid_fluxes && !f.lun_lakpoi[l] && !f.lun_urbpoi[l]) {
          const double swe_old = LVc(f.swe_old, c, k + 1, ld);
          ddz3 = jl_max(0.0, jl_min(1.0, (swe_old - wx) / wx));
          if ((swe_old - wx) > 0.0) {
            double wsum = 0.0;
            for (int j2 = (int)snl + 1; j2 <= 0; j2++) wsum += S.liq[j2 + ns - 1] + S.ice[j2 + ns - 1];
            // FracSnowDuringMelt (Swenson and Lawrence 2012)
            const double lim = jl_min(f.int_snow[c], P.int_snow_max);
            double fsno_melt;
            if (lim > 0.0) {
              const double smr = jl_min(1.0, wsum / lim);
              fsno_melt = 1.0 - cm_pow(cm_acos(jl_min(1.0, 2.0 * smr - 1.0)) / CM_PI_HI, f.n_melt[c]);
            } else {
              fsno_melt = 1.0;
            }
            if ((fsno_melt + f.frac_h2osfc[c]) > 1.0) fsno_melt = 1.0 - f.frac_h2osfc[c];
            ddz3 = ddz3 - jl_max(0.0, (fsno_melt - fsno) / fsno);
          }
          ddz3 = -1.0 / dtime * ddz3;
        } else {
          const double fio = LVc(f.frac_iceold, c, k + 1, ld);
          ddz3 = -1.0 / dtime * jl_max(0.0, (fio - fi) / fio);
        }
      }
      // wind drift (:1466-1500), carried down the pack
      double ddz4 = 0.0;
      if (P.wind_dependent_snow_density && mobile) {
        const double fw = f.forc_wind[f.col_gridcell[c] - 1];
        const double frho = 1.25 - 0.0042 * (jl_max(P.rho_min, bi) - P.rho_min);
        const double mo = 0.34 * (-0.583 * P.drift_gs - 0.833 * 1.0 + 0.833) + 0.66 * frho;
        double si = -2.868 * cm_exp(-0.085 * fw) + 1.0 + mo;
        if (si > 0.0) {
          si = jl_min(si, 3.25);
          double zp = zpseudo + 0.5 * S.dz[k] * (3.25 - si);
          const double gamma_drift = si * cm_exp(-zp / 0.1);
          const double tau_inverse = gamma_drift / P.tau_ref;
          ddz4 = -jl_max(0.0, P.rho_max - bi) * tau_inverse;
          zp = zp + 0.5 * S.dz[k] * (3.25 - si);
          zpseudo = zp;
        } else {
          mobile = false;
        }
      }
      const double pdzdtc = ddz1 + ddz2 + ddz3 + ddz4;
      S.dz[k] = jl_max(S.dz[k] * (1.0 + pdzdtc * dtime), (ice / DENICE + liq / DENH2O) / fsno);
    } else {
      mobile = false;
    }
    burden = burden + wx;
  }
}

__device__ __forceinline__ void copy_level(SnowCol& S, int to, int from) {
  S.liq[to] = S.liq[from];
  S.ice[to] = S.ice[from];
  S.t[to] = S.t[from];
  S.dz[to] = S.dz[from];
  for (int a = 0; a < NAER; a++) S.aer[a][to] = S.aer[a][from];
  S.rds[to] = S.rds[from];
}

__device__ __forceinline__ void reset_depths(SnowCol& S, int64_t snl, int ns) {
  for (int jl = 0; jl >= -ns + 1; jl--) {
    if (jl < snl + 1) continue;
    const int k = jl + ns - 1;              // zi[k + 1] is the interface below level k
    S.z[k] = S.zi[k + 1] - 0.5 * S.dz[k];
    S.zi[k] = S.zi[k + 1] - S.dz[k];
  }
}

// combine_snow_layers! for one column (_snowhyd_combine_kernel!, :1584-1874); the
// default (non-smoothed) triggers
__device__ void combine(const clmgb_snowlayer_fields& f, const SnowThresh& T, SnowCol& S, int64_t c, int64_t& snl,
                        int ns, double dtime, double& frac_sno, double& frac_sno_eff, double& int_snow,
                        double& h2osno_no_layers, bool& wrote_h2osno, double& snow_depth, double& qsl) {
  const int64_t l = f.col_landunit[c] - 1;
  const int64_t ltype = f.lun_itype[l];
  const bool soil_below = ltype == ISTSOIL || f.lun_urbpoi[l] || ltype == ISTCROP;
  qsl = 0.0;
  // remove thin layers with very little ice
  const int64_t msn_old = snl;
  for (int64_t j = msn_old + 1; j <= 0; j++) {
    const int k = (int)j + ns - 1;
    if (!(S.ice[k] <= 0.01)) continue;
    if (j < 0 || soil_below) {
      if (k + 1 < ns) {
        S.liq[k + 1] += S.liq[k];
        S.ice[k + 1] += S.ice[k];
      } else {                              // the level below is soil level 1
        S.liq1 += S.liq[k];
        S.ice1 += S.ice[k];
      }
    }
    if (j == 0) qsl = (S.liq[k] + S.ice[k]) / dtime;
    if (j < 0) {
      S.dz[k + 1] += S.dz[k];
      for (int a = 0; a < NAER; a++) S.aer[a][k + 1] += S.aer[a][k];
    }
    if (j > snl + 1 && snl < -1)
      for (int64_t i = j; i >= snl + 2; i--) copy_level(S, (int)i + ns - 1, (int)i + ns - 2);
    snl = snl + 1;
  }
  // snow depth and total water
  double depth = 0.0, h2osno_total = 0.0;
  for (int64_t jl = snl + 1; jl <= 0; jl++) {
    const int k = (int)jl + ns - 1;
    depth += S.dz[k];
    h2osno_total += S.ice[k] + S.liq[k];
  }
  snow_depth = depth;
  if (snow_depth > 0.0) {
    const bool gone = (ltype == ISTDLAK && snow_depth < T.dzmin[0] + LSADZ) ||
                      (ltype != ISTDLAK && (frac_sno_eff * snow_depth < T.dzmin[0] ||
                                            h2osno_total / (frac_sno_eff * snow_depth) < 50.0));
    if (gone) {
      double zwice = 0.0, zwliq = 0.0;
      for (int64_t jl = snl + 1; jl <= 0; jl++) {
        zwice += S.ice[(int)jl + ns - 1];
        zwliq += S.liq[(int)jl + ns - 1];
      }
      h2osno_no_layers = zwice;
      wrote_h2osno = true;
      if (soil_below) S.liq1 += zwliq;
      snl = 0;
      h2osno_total = h2osno_no_layers;
      for (int a = 0; a < NAER; a++)
        for (int k = 0; k < ns; k++) S.aer[a][k] = 0.0;
      if (h2osno_no_layers <= 0.0) snow_depth = 0.0;
    }
  }
  if (h2osno_total <= 0.0) {
    snow_depth = 0.0;
    frac_sno = 0.0;
    frac_sno_eff = 0.0;
    int_snow = 0.0;
  }
  // combine thin layers with a neighbour
  if (snl < -1) {
    int mssi = 0;
    for (int64_t i = snl + 1; i <= 0; i++) {
      const int ki = (int)i + ns - 1;
      const bool thin = (frac_sno_eff * S.dz[ki] < T.dzmin[mssi]) ||
                        ((S.ice[ki] + S.liq[ki]) / (frac_sno_eff * S.dz[ki]) < 50.0);
      if (!thin) {
        mssi = mssi + 1;
        continue;
      }
      int64_t neibor;
      if (i == snl + 1) neibor = i + 1;
      else if (i == 0) neibor = i - 1;
      else {
        neibor = i + 1;
        if ((S.dz[ki - 1] + S.dz[ki]) < (S.dz[ki + 1] + S.dz[ki])) neibor = i - 1;
      }
      const int64_t j_keep = neibor > i ? neibor : i;
      const int64_t l_rm = neibor > i ? i : neibor;
      const int kk = (int)j_keep + ns - 1, kr = (int)l_rm + ns - 1;
      for (int a = 0; a < NAER; a++) S.aer[a][kk] += S.aer[a][kr];
      const double total_mass = S.liq[kk] + S.ice[kk] + S.liq[kr] + S.ice[kr];
      if (total_mass > 0.0)
        S.rds[kk] = (S.rds[kk] * (S.liq[kk] + S.ice[kk]) + S.rds[kr] * (S.liq[kr] + S.ice[kr])) / total_mass;
      combo(S.dz[kk], S.liq[kk], S.ice[kk], S.t[kk], S.dz[kr], S.liq[kr], S.ice[kr], S.t[kr]);
      if (j_keep - 1 > snl + 1)
        for (int64_t m = j_keep - 1; m >= snl + 2; m--) copy_level(S, (int)m + ns - 1, (int)m + ns - 2);
      snl = snl + 1;
      if (snl >= -1) break;
    }
  }
  reset_depths(S, snl, ns);
}

// divide_snow_layers! for one column (_snowhyd_divide_kernel!, :2057-2237): the pack
// copied top-down (k = 0 is the top layer), split where thicker than allowed, copied back
__device__ void divide(const clmgb_snowlayer_config& P, const SnowThresh& T, SnowCol& S, int64_t& snl, int ns,
                       double frac_sno) {
  double dzs[MAXSNO], swi[MAXSNO], swl[MAXSNO], ts[MAXSNO], rd[MAXSNO], ma[NAER][MAXSNO];
  for (int k = 0; k < ns; k++) {
    dzs[k] = swi[k] = swl[k] = ts[k] = rd[k] = 0.0;
    for (int a = 0; a < NAER; a++) ma[a][k] = 0.0;
  }
  int msno = (int)(snl < 0 ? -snl : snl);
  const bool lake = P.is_lake != 0;
  for (int k = 0; k < msno; k++) {
    const int jj = k + 1 + (int)snl + ns - 1;   // level k+1 from the top
    dzs[k] = lake ? S.dz[jj] : frac_sno * S.dz[jj];
    swi[k] = S.ice[jj];
    swl[k] = S.liq[jj];
    ts[k] = S.t[jj];
    for (int a = 0; a < NAER; a++) ma[a][k] = S.aer[a][jj];
    rd[k] = S.rds[jj];
  }
  const double rmin = P.snw_rds_min, rmax = P.snw_rds_max;
  for (int k = 0; k < msno && k < ns - 1; k++) {
    if (k == msno - 1) {                         // bottom layer
      const double off = lake ? 2.0 * LSADZ : 0.0;
      if (dzs[k] > T.dzmax_l[k] + off) {
        msno += 1;
        dzs[k] /= 2.0;
        dzs[k + 1] = dzs[k];
        swi[k] /= 2.0;
        swi[k + 1] = swi[k];
        swl[k] /= 2.0;
        swl[k + 1] = swl[k];
        if (k == 0) {
          ts[k + 1] = ts[k];
        } else {
          const double dtdz = (ts[k - 1] - ts[k]) / ((dzs[k - 1] + 2.0 * dzs[k]) / 2.0);
          const double cand1 = ts[k] - dtdz * dzs[k] / 2.0;
          const double cand0 = ts[k] + dtdz * dzs[k] / 2.0;
          const double w = (TFRZ - cand1 >= 0.0) ? 1.0 : 0.0;     // smooth_heaviside on Float64
          ts[k + 1] = w * cand1 + (1.0 - w) * ts[k];
          ts[k] = w * cand0 + (1.0 - w) * ts[k];
        }
        for (int a = 0; a < NAER; a++) {
          ma[a][k] /= 2.0;
          ma[a][k + 1] = ma[a][k];
        }
        rd[k + 1] = rd[k];
      }
    }
    if (k < msno - 1) {                          // layers below exist
      const double off = lake ? LSADZ : 0.0;
      if (dzs[k] > T.dzmax_u[k] + off) {
        const double drr = dzs[k] - T.dzmax_u[k] - off;
        const double propor = drr / dzs[k];
        const double zwice = propor * swi[k];
        const double zwliq = propor * swl[k];
        double zm[NAER];
        for (int a = 0; a < NAER; a++) zm[a] = propor * ma[a][k];
        const double keep = (T.dzmax_u[k] + off) / dzs[k];
        swi[k] *= keep;
        swl[k] *= keep;
        for (int a = 0; a < NAER; a++) ma[a][k] *= keep;
        dzs[k] = T.dzmax_u[k] + off;
        for (int a = 0; a < NAER; a++) ma[a][k + 1] += zm[a];
        rd[k + 1] = mass_weighted_radius(rd[k], rd[k + 1], swl[k + 1] + swi[k + 1], zwliq + zwice, rmin, rmax);
        combo(dzs[k + 1], swl[k + 1], swi[k + 1], ts[k + 1], drr, zwliq, zwice, ts[k]);
      }
    }
  }
  snl = -msno;
  for (int jl = -ns + 1; jl <= 0; jl++) {
    if (jl < snl + 1) continue;
    const int kk = jl + ns - 1, k = (int)(jl - snl) - 1;
    S.dz[kk] = lake ? dzs[k] : dzs[k] / frac_sno;
    S.ice[kk] = swi[k];
    S.liq[kk] = swl[k];
    S.t[kk] = ts[k];
    for (int a = 0; a < NAER; a++) S.aer[a][kk] = ma[a][k];
    S.rds[kk] = rd[k];
  }
  reset_depths(S, snl, ns);
}

__global__ void __launch_bounds__(SL_BLOCK)
k_snow_layers(int64_t nc, int64_t nl, int ns, int64_t ld, clmgb_snowlayer_fields f, clmgb_snowlayer_config P,
              SnowThresh T, uint32_t stages, double dtime, uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * SL_BLOCK + threadIdx.x;
  if (c >= nc) return;
  constexpr uint32_t LAYERS = CLMGB_SL_COMPACTION | CLMGB_SL_COMBINE | CLMGB_SL_DIVIDE | CLMGB_SL_ZERO_EMPTY;
  if ((stages & LAYERS) && f.mask_snow[c]) {
    int64_t snl = f.col_snl[c];
    uint32_t bad = 0;
    if (snl > 0 || snl < -ns) bad = CLMGB_COL_LEVEL_RANGE;
    if (stages & (CLMGB_SL_COMPACTION | CLMGB_SL_COMBINE)) {
      const int64_t l = f.col_landunit[c];
      if (l < 1 || l > nl) bad |= CLMGB_COL_PATCH_RANGE;
    }
    if ((stages & CLMGB_SL_COMPACTION) && P.wind_dependent_snow_density) {
      const int64_t g = f.col_gridcell[c];
      if (g < 1 || g > P.ng) bad |= CLMGB_COL_PATCH_RANGE;
    }
    if (bad) {
      if (dev_status) atomicOr(dev_status, bad);
    } else {
      // the arrays the selected stages read and write
      const bool geom = stages & (CLMGB_SL_COMBINE | CLMGB_SL_DIVIDE | CLMGB_SL_ZERO_EMPTY);
      const bool grain = stages & (CLMGB_SL_COMBINE | CLMGB_SL_DIVIDE);
      const bool soil1 = stages & CLMGB_SL_COMBINE;
      SnowCol S;
      for (int k = 0; k < ns; k++) {
        S.dz[k] = LV(f.dz, c, k + 1, ld);
        S.t[k] = LV(f.t_soisno, c, k + 1, ld);
        S.ice[k] = LV(f.h2osoi_ice, c, k + 1, ld);
        S.liq[k] = LV(f.h2osoi_liq, c, k + 1, ld);
        if (geom) {
          S.z[k] = LV(f.z, c, k + 1, ld);
          S.zi[k] = LV(f.zi, c, k + 1, ld);
        }
        if (grain) {
          S.rds[k] = LV(f.snw_rds, c, k + 1, ld);
          S.aer[0][k] = LV(f.mss_bcphi, c, k + 1, ld);
          S.aer[1][k] = LV(f.mss_bcpho, c, k + 1, ld);
          S.aer[2][k] = LV(f.mss_ocphi, c, k + 1, ld);
          S.aer[3][k] = LV(f.mss_ocpho, c, k + 1, ld);
          S.aer[4][k] = LV(f.mss_dst1, c, k + 1, ld);
          S.aer[5][k] = LV(f.mss_dst2, c, k + 1, ld);
          S.aer[6][k] = LV(f.mss_dst3, c, k + 1, ld);
          S.aer[7][k] = LV(f.mss_dst4, c, k + 1, ld);
        }
      }
      if (geom) S.zi[ns] = LV(f.zi, c, ns + 1, ld);
      if (soil1) {
        S.liq1 = LV(f.h2osoi_liq, c, ns + 1, ld);
        S.ice1 = LV(f.h2osoi_ice, c, ns + 1, ld);
      }

      if (stages & CLMGB_SL_COMPACTION) compaction(f, P, S, c, snl, ns, ld, dtime);

      double frac_sno = grain ? f.frac_sno[c] : 0.0;
      if (stages & CLMGB_SL_COMBINE) {
        double fse = f.frac_sno_eff[c], isn = f.int_snow[c], h2n = 0.0, depth = 0.0, qsl = 0.0;
        bool wrote_h2n = false;
        const double fs0 = frac_sno, fse0 = fse, isn0 = isn;
        combine(f, T, S, c, snl, ns, dtime, frac_sno, fse, isn, h2n, wrote_h2n, depth, qsl);
        f.snow_depth[c] = depth;
        f.qflx_sl_top_soil[c] = qsl;
        if (wrote_h2n) f.h2osno_no_layers[c] = h2n;
        if (frac_sno != fs0 || fse != fse0 || isn != isn0) {
          f.frac_sno[c] = frac_sno;
          f.frac_sno_eff[c] = fse;
          f.int_snow[c] = isn;
        }
      }
      if (stages & CLMGB_SL_DIVIDE) divide(P, T, S, snl, ns, frac_sno);
      if ((stages & CLMGB_SL_ZERO_EMPTY) && snl > -ns) {
        for (int k = 0; k < ns; k++) {
          if (k + 1 - ns > snl) continue;          // level j = k + 1 - ns is below snl + 1
          S.ice[k] = S.liq[k] = S.t[k] = S.dz[k] = S.z[k] = S.zi[k] = 0.0;
        }
      }

      for (int k = 0; k < ns; k++) {
        LV(f.dz, c, k + 1, ld) = S.dz[k];
        if (!geom) continue;
        LV(f.z, c, k + 1, ld) = S.z[k];
        LV(f.zi, c, k + 1, ld) = S.zi[k];
        LV(f.t_soisno, c, k + 1, ld) = S.t[k];
        LV(f.h2osoi_ice, c, k + 1, ld) = S.ice[k];
        LV(f.h2osoi_liq, c, k + 1, ld) = S.liq[k];
        if (!grain) continue;
        LV(f.snw_rds, c, k + 1, ld) = S.rds[k];
        LV(f.mss_bcphi, c, k + 1, ld) = S.aer[0][k];
        LV(f.mss_bcpho, c, k + 1, ld) = S.aer[1][k];
        LV(f.mss_ocphi, c, k + 1, ld) = S.aer[2][k];
        LV(f.mss_ocpho, c, k + 1, ld) = S.aer[3][k];
        LV(f.mss_dst1, c, k + 1, ld) = S.aer[4][k];
        LV(f.mss_dst2, c, k + 1, ld) = S.aer[5][k];
        LV(f.mss_dst3, c, k + 1, ld) = S.aer[6][k];
        LV(f.mss_dst4, c, k + 1, ld) = S.aer[7][k];
      }
      if (soil1) {
        LV(f.h2osoi_liq, c, ns + 1, ld) = S.liq1;
        LV(f.h2osoi_ice, c, ns + 1, ld) = S.ice1;
      }
      f.col_snl[c] = snl;
    }
  }
  // build_snow_filter! (:2488-2510)
  if (stages & CLMGB_SL_FILTER) {
    const bool nolake = f.mask_nolakec[c];
    const int64_t snl = f.col_snl[c];
    f.mask_snow[c] = nolake && snl < 0;
    f.mask_nosnow[c] = nolake && snl >= 0;
  }
}

}  // namespace

cudaError_t launch_snow_layers(const Dims& D, int64_t nc, int64_t nl, const clmgb_snowlayer_fields& f,
                               const clmgb_snowlayer_config& P, uint32_t stages, double dtime, uint32_t* dev_status,
                               cudaStream_t s) {
  // init_snow_layers!'s thresholds (snow_hydrology.jl:2357-2377)
  SnowThresh T;
  const int ns = D.nlevsno;
  for (int k = 0; k < MAXSNO; k++) T.dzmin[k] = T.dzmax_l[k] = T.dzmax_u[k] = 0.0;
  T.dzmin[0] = P.dzmin_1;
  T.dzmax_l[0] = P.dzmax_l_1;
  T.dzmax_u[0] = P.dzmax_u_1;
  if (ns >= 2) {
    T.dzmin[1] = P.dzmin_2;
    T.dzmax_l[1] = P.dzmax_l_2;
    T.dzmax_u[1] = P.dzmax_u_2;
  }
  for (int j = 3; j <= ns; j++) {
    T.dzmin[j - 1] = T.dzmax_u[j - 2] * 0.5;
    T.dzmax_u[j - 1] = 2.0 * T.dzmax_u[j - 2] + 0.01;
    T.dzmax_l[j - 1] = T.dzmax_u[j - 1] + T.dzmax_l[j - 2];
    if (j == ns) T.dzmax_u[j - 1] = T.dzmax_l[j - 1] = DBL_MAX;
  }
  k_snow_layers<<<(unsigned int)((nc + SL_BLOCK - 1) / SL_BLOCK), SL_BLOCK, 0, s>>>(nc, nl, ns, D.ldc, f, P, T, stages,
                                                                                    dtime, dev_status);
  return cudaGetLastError();
}

}  // namespace clmgb
