// lake.cu — lake_temperature! (lake_temperature.jl:1016-1295): the temperatures of the
// snow, lake-water and soil levels of lake columns, with the lake's eddy diffusivity,
// penetrating solar radiation, phase change and convective mixing.
//
// The reference runs ~25 kernels over (column), (column, level) and (patch) ranges; none
// couples columns (each lake column has one patch), so one thread owns one lake column
// through the whole sequence.  The column's lake, snow and soil state is read into
// on-chip arrays once, the Crank-Nicolson system over the extended column (snow, lake,
// soil: up to nlevsno + nlevlak + nlevgrnd levels) is assembled and solved there, and the
// state is written back once.  Expressions keep the reference's operation order.
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int LK_BLOCK = 64;
constexpr int MAXK = CLMGB_MAX_NLEVLAK;
constexpr int MAXX = MAXL + MAXK + 2;          // extended column, 1-based
constexpr double BETAVIS = 0.0, ZA_LAKE = 0.6, TDMAX = 277.0, N2MIN = 7.5e-5;
constexpr double VKC = 0.4, GRAV = 9.80616, TKAIR = 0.023, TKICE = 2.290, TKWAT = 0.57, CNFAC = 0.5;
constexpr double THK_BEDROCK = 3.0, CSOL_BEDROCK = 2.0e6;

// One lake column's state: level arrays 1-based as in CLM.jl (jj = 1..nlevsno+nlevgrnd
// for snow and soil, j = 1..nlevlak for the lake).
struct LakeCol {
  double t[MAXL + 1], liq[MAXL + 1], ice[MAXL + 1], dz[MAXL + 1], z[MAXL + 1], zi[MAXL + 2];
  double tl[MAXK + 1], fi[MAXK + 1], dzl[MAXK + 1], zl[MAXK + 1];
};

__device__ __forceinline__ double lake_density(double icefrac, double t) {
  return (1.0 - icefrac) * 1000.0 * (1.0 - 1.9549e-05 * cm_pow(fabs(t - TDMAX), 1.68)) + icefrac * DENICE;
}

// soil_therm_prop_lake! (:39-192): interface conductivity tk, heat capacity cv and the
// top soil level's conductivity
__device__ void therm_prop(const clmgb_lake_fields& f, const LakeCol& S, int64_t c, int64_t ld, int ns, int ngr,
                           int nsoi, int64_t snl, double* tk, double* cv, double& tktopsoillay) {
  double thk[MAXL + 2];
  for (int jj = 1; jj <= ns + ngr + 1; jj++) thk[jj] = 0.0;
  for (int jj = 1; jj <= ns + ngr; jj++) {
    const int j = jj - ns;
    if (j >= 1 && j <= nsoi) {
      const double ws = LVc(f.watsat, c, j, ld);
      double satw = 1.0;
      const double fl = S.liq[jj] / (S.ice[jj] + S.liq[jj]);
      double dke, dksat;
      if (S.t[jj] >= TFRZ) {
        dke = jl_max(0.0, cm_log10(satw) + 1.0);
        dksat = LVc(f.tksatu, c, j, ld);
      } else {
        dke = satw;
        dksat = LVc(f.tkmg, c, j, ld) * cm_pow(0.249, fl * ws) * cm_pow(2.29, ws);
      }
      thk[jj] = dke * dksat + (1.0 - dke) * LVc(f.tkdry, c, j, ld);
      satw = (S.liq[jj] / DENH2O + S.ice[jj] / DENICE) / (S.dz[jj] * ws);
      if (satw > 1.0) {
        const double xicevol = (satw - 1.0) * ws;
        thk[jj] = (thk[jj] + xicevol * TKICE) / (1.0 + xicevol) / (1.0 + xicevol);
      }
    } else if (j > nsoi) {
      thk[jj] = THK_BEDROCK;
    }
    if (snl + 1 < 1 && j >= snl + 1 && j <= 0) {           // snow (Jordan 1991)
      const double bw = (S.ice[jj] + S.liq[jj]) / S.dz[jj];
      thk[jj] = TKAIR + (7.75e-5 * bw + 1.105e-6 * bw * bw) * (TKICE - TKAIR);
    }
  }
  for (int jj = 1; jj <= ns + ngr; jj++) {
    const int j = jj - ns;
    if (j >= snl + 1 && j <= ngr - 1 && j != 0) {
      tk[jj] = thk[jj] * thk[jj + 1] * (S.z[jj + 1] - S.z[jj]) /
               (thk[jj] * (S.z[jj + 1] - S.zi[jj + 1]) + thk[jj + 1] * (S.zi[jj + 1] - S.z[jj]));
    } else if (j == 0 && j >= snl + 1) {
      tk[jj] = thk[jj];
    } else if (j == ngr) {
      tk[jj] = 0.0;
    }
    if (j == 1) tktopsoillay = thk[jj];
  }
  for (int j = 1; j <= ngr; j++) {
    const int jj = j + ns;
    cv[jj] = LVc(f.csol, c, j, ld) * (1.0 - LVc(f.watsat, c, j, ld)) * S.dz[jj] + (S.ice[jj] * CPICE + S.liq[jj] * CPLIQ);
    if (j > nsoi) cv[jj] = CSOL_BEDROCK * S.dz[jj];
  }
  for (int jj = 1; jj <= ns; jj++)
    if (snl + 1 < 1 && jj - ns >= snl + 1) cv[jj] = CPLIQ * S.liq[jj] + CPICE * S.ice[jj];
}

__device__ __forceinline__ double h2osno_total(const LakeCol& S, double h2osno_no_layers, int ns, int64_t snl) {
  double tot = h2osno_no_layers;
  for (int jj = 1; jj <= ns; jj++)
    if (jj - ns >= snl + 1) tot += S.ice[jj] + S.liq[jj];
  return tot;
}

// convective mixing of lake levels lo..hi (:787-894): heat and ice redistributed with
// the ice on top
__device__ void mix(LakeCol& S, double* rhow, int lo, int hi, double cwat, double cice_eff) {
  double qav = 0.0, nav = 0.0, iceav = 0.0;
  for (int i = lo; i <= hi; i++) {
    qav += S.dzl[i] * (S.tl[i] - TFRZ) * ((1.0 - S.fi[i]) * cwat + S.fi[i] * cice_eff);
    iceav += S.fi[i] * S.dzl[i];
    nav += S.dzl[i];
  }
  qav /= nav;
  iceav /= nav;
  double tav_froz = 0.0, tav_unfr = 0.0;
  if (qav > 0.0) tav_unfr = qav / ((1.0 - iceav) * cwat);
  else if (qav < 0.0) tav_froz = qav / (iceav * cice_eff);
  double zsum = 0.0;
  for (int i = lo; i <= hi; i++) {
    if ((zsum + S.dzl[i]) / nav <= iceav) {
      S.fi[i] = 1.0;
      S.tl[i] = tav_froz + TFRZ;
    } else if (zsum / nav < iceav) {
      S.fi[i] = (iceav * nav - zsum) / S.dzl[i];
      S.tl[i] = (S.fi[i] * tav_froz * cice_eff + (1.0 - S.fi[i]) * tav_unfr * cwat) /
                    (S.fi[i] * cice_eff + (1.0 - S.fi[i]) * cwat) + TFRZ;
    } else {
      S.fi[i] = 0.0;
      S.tl[i] = tav_unfr + TFRZ;
    }
    zsum += S.dzl[i];
    rhow[i] = lake_density(S.fi[i], S.tl[i]);
  }
}

__global__ void __launch_bounds__(LK_BLOCK)
k_lake_temperature(Dims D, int64_t nc, clmgb_lake_fields f, clmgb_lake_config P, double dtime,
                   uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * LK_BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_lakec[c]) return;
  const int ns = D.nlevsno, ngr = D.nlevgrnd, nsoi = D.nlevsoi, nlak = P.nlevlak;
  const int64_t ld = D.ldc, ldp = D.ldp;
  const int64_t p = f.col_patchi[c] - 1;
  const int64_t snl = f.col_snl[c];
  if (p < 0 || p >= D.np || f.patch_column[p] != c + 1) {
    if (dev_status) atomicOr(dev_status, CLMGB_COL_PATCH_RANGE);
    return;
  }
  if (snl > 0 || snl < -ns) {
    if (dev_status) atomicOr(dev_status, CLMGB_COL_LEVEL_RANGE);
    return;
  }
  const int ntot = ns + nlak + ngr;
  const bool pact = f.mask_lakep[p] != 0;
  const bool puddling = P.lakepuddling != 0, no_ed = P.lake_no_ed != 0, lch4 = P.use_lch4 != 0;
  const double p0 = 1.0, cwat = CPLIQ * DENH2O, cice_eff = CPICE * DENH2O, cfus = HFUS * DENH2O;
  const double tkice_eff = TKICE * DENICE / DENH2O, km = TKWAT / cwat;

  LakeCol S;
  for (int jj = 1; jj <= ns + ngr; jj++) {
    S.t[jj] = LV(f.t_soisno, c, jj, ld);
    S.liq[jj] = LV(f.h2osoi_liq, c, jj, ld);
    S.ice[jj] = LV(f.h2osoi_ice, c, jj, ld);
    S.dz[jj] = LVc(f.dz, c, jj, ld);
    S.z[jj] = LVc(f.z, c, jj, ld);
    S.zi[jj] = LVc(f.zi, c, jj, ld);
  }
  S.zi[ns + ngr + 1] = LVc(f.zi, c, ns + ngr + 1, ld);
  for (int j = 1; j <= nlak; j++) {
    S.tl[j] = LV(f.t_lake, c, j, ld);
    S.fi[j] = LV(f.lake_icefrac, c, j, ld);
    S.dzl[j] = LVc(f.dz_lake, c, j, ld);
    S.zl[j] = LVc(f.z_lake, c, j, ld);
  }
  double h2osno_nl = f.h2osno_no_layers[c], snow_depth = f.snow_depth[c];

  // prior ice fraction of the snow levels (:406-415)
  for (int jj = 1; jj <= ns; jj++)
    if (jj - ns >= snl + 1) LV(f.frac_iceold, c, jj, ld) = S.ice[jj] / (S.liq[jj] + S.ice[jj]);
  // ground heat flux and the NIR fraction of absorbed solar (:419-432)
  double fin = 0.0, beta = f.betaprime[c];
  if (pact) {
    fin = f.eflx_gnet[p];
    double sabg_nir = f.fsds_nir_d[p] + f.fsds_nir_i[p] - f.fsr_nir_d[p] - f.fsr_nir_i[p];
    sabg_nir = jl_min(sabg_nir, f.sabg[p]);
    beta = sabg_nir / jl_max(1.0e-5, f.sabg[p]);
    beta = beta + (1.0 - beta) * BETAVIS;
    f.betaprime[c] = beta;
  }
  // density, eddy diffusivity and conductivity of the lake levels (:434-527)
  double rhow[MAXK + 1], kme[MAXK + 1], tk_lake[MAXK + 1], phi[MAXK + 1], cv_lake[MAXK + 1];
  for (int j = 1; j <= nlak; j++) {
    rhow[j] = lake_density(S.fi[j], S.tl[j]);
    kme[j] = tk_lake[j] = phi[j] = 0.0;
  }
  const bool warm = f.t_grnd[c] > TFRZ && S.tl[1] > TFRZ && snl == 0;
  const double wsc = f.ws[c], ksc = f.ks[c], depth = f.lakedepth[c];
  bool frzn = false;
  for (int j = 1; j <= nlak - 1; j++) {
    const double drhodz = (rhow[j + 1] - rhow[j]) / (S.zl[j + 1] - S.zl[j]);
    const double n2 = GRAV / rhow[j] * drhodz;
    const double vz = VKC * S.zl[j];
    const double num = 40.0 * n2 * (vz * vz);
    const double den = jl_max((wsc * wsc) * cm_exp(-2.0 * ksc * S.zl[j]), 1.0e-10);
    const double ri = (-1.0 + sqrt(jl_max(1.0 + num / den, 0.0))) / 20.0;
    if (puddling && j == 1) frzn = false;
    if (warm && (!puddling || (S.fi[j] == 0.0 && !frzn))) {
      const double ke = VKC * wsc * S.zl[j] / p0 * cm_exp(-ksc * S.zl[j]) / (1.0 + 37.0 * ri * ri);
      kme[j] = km + ke;
      if (!no_ed) kme[j] = kme[j] + 1.039e-8 * cm_pow(jl_max(n2, N2MIN), -0.43);
      if (depth >= P.deepmixing_depthcrit) kme[j] = kme[j] * P.deepmixing_mixfact;
      tk_lake[j] = kme[j] * cwat;
    } else {
      kme[j] = km;
      if (!no_ed) {
        kme[j] = kme[j] + 1.039e-8 * cm_pow(jl_max(n2, N2MIN), -0.43);
        if (depth >= P.deepmixing_depthcrit) kme[j] = kme[j] * P.deepmixing_mixfact;
        tk_lake[j] = kme[j] * cwat * tkice_eff / ((1.0 - S.fi[j]) * tkice_eff + kme[j] * cwat * S.fi[j]);
      } else {
        tk_lake[j] = TKWAT * tkice_eff / ((1.0 - S.fi[j]) * tkice_eff + TKWAT * S.fi[j]);
      }
      if (puddling) frzn = true;
    }
  }
  kme[nlak] = kme[nlak - 1];
  if (warm && (!puddling || (S.fi[nlak] == 0.0 && !frzn)))
    tk_lake[nlak] = tk_lake[nlak - 1];
  else if (!no_ed)
    tk_lake[nlak] = kme[nlak] * cwat * tkice_eff / ((1.0 - S.fi[nlak]) * tkice_eff + kme[nlak] * cwat * S.fi[nlak]);
  else
    tk_lake[nlak] = TKWAT * tkice_eff / ((1.0 - S.fi[nlak]) * tkice_eff + TKWAT * S.fi[nlak]);
  f.savedtke1[c] = kme[1] * cwat;
  const int64_t jtop = snl + 1;

  // solar radiation absorbed in each lake level (:533-565); under snow the top level
  // takes sabg_lyr[p, 1], as the reference indexes it
  double phi_soil = 0.0;
  if (pact) {
    const double sabg = f.sabg[p];
    const double eta = f.etal[c] > 0.0 ? f.etal[c] : 1.1925 * cm_pow(jl_max(depth, 1.0), -0.424);
    for (int j = 1; j <= nlak; j++) {
      const double zin = S.zl[j] - 0.5 * S.dzl[j];
      const double zout = S.zl[j] + 0.5 * S.dzl[j];
      const double rsfin = cm_exp(-eta * jl_max(zin - ZA_LAKE, 0.0));
      const double rsfout = cm_exp(-eta * jl_max(zout - ZA_LAKE, 0.0));
      double phidum;
      if (warm) {
        phidum = (rsfin - rsfout) * sabg * (1.0 - beta);
        if (j == nlak) phi_soil = rsfout * sabg * (1.0 - beta);
      } else if (j == 1 && snl == 0) {
        phidum = sabg * (1.0 - beta);
      } else if (j == 1) {
        phidum = LVc(f.sabg_lyr, p, 1, ldp);
      } else {
        phidum = 0.0;
        if (j == nlak) phi_soil = 0.0;
      }
      phi[j] = phidum;
    }
  }
  // heat capacities and conductivities, and the energy before (:567-613)
  for (int j = 1; j <= nlak; j++) cv_lake[j] = S.dzl[j] * (cwat * (1.0 - S.fi[j]) + cice_eff * S.fi[j]);
  double tk[MAXL + 2], cv[MAXL + 2];
  for (int jj = 0; jj <= ns + ngr + 1; jj++) tk[jj] = cv[jj] = 0.0;
  double tktopsoillay = 0.0;
  therm_prop(f, S, c, ld, ns, ngr, nsoi, snl, tk, cv, tktopsoillay);
  double ocvts = 0.0;
  for (int j = 1; j <= nlak; j++) ocvts += cv_lake[j] * (S.tl[j] - TFRZ) + cfus * S.dzl[j] * (1.0 - S.fi[j]);
  double hsn = h2osno_total(S, h2osno_nl, ns, snl);
  for (int j = -ns + 1; j <= ngr; j++) {
    const int jj = j + ns;
    if (j < jtop) continue;
    ocvts += cv[jj] * (S.t[jj] - TFRZ) + HFUS * S.liq[jj];
    if (j == 1 && hsn > 0.0 && j == jtop) ocvts -= hsn * HFUS;
  }

  // the extended column: snow, lake, soil (:615-665)
  double zx[MAXX], cvx[MAXX], phix[MAXX], tx[MAXX], tkix[MAXX], fnx[MAXX], factx[MAXX];
  for (int ji = 0; ji <= ntot + 1; ji++) zx[ji] = cvx[ji] = phix[ji] = tx[ji] = tkix[ji] = fnx[ji] = factx[ji] = 0.0;
  for (int je = (int)jtop; je <= nlak + ngr; je++) {
    const int ji = je + ns;
    if (je < 1) {
      zx[ji] = S.z[ji];
      cvx[ji] = cv[ji];
      phix[ji] = (je == jtop || !pact) ? 0.0 : LVc(f.sabg_lyr, p, je + ns, ldp);
      tx[ji] = S.t[ji];
    } else if (je <= nlak) {
      zx[ji] = S.zl[je];
      cvx[ji] = cv_lake[je];
      phix[ji] = phi[je];
      tx[ji] = S.tl[je];
    } else {
      const int jpjj = je - nlak + ns;
      zx[ji] = zx[nlak + ns] + S.dzl[nlak] / 2.0 + S.z[jpjj];
      cvx[ji] = cv[jpjj];
      phix[ji] = je == nlak + 1 ? phi_soil : 0.0;
      tx[ji] = S.t[jpjj];
    }
  }
  // interface conductivities (:673-703)
  for (int je = (int)jtop; je <= nlak + ngr; je++) {
    const int ji = je + ns;
    if (je < 0) {
      tkix[ji] = tk[ji];
    } else if (je == 0) {
      const double dzp = zx[ji + 1] - zx[ji];
      tkix[ji] = tk_lake[1] * tk[ji] * dzp / (tk[ji] * S.zl[1] + tk_lake[1] * (-S.z[ji]));
    } else if (je < nlak) {
      tkix[ji] = (tk_lake[je] * tk_lake[je + 1] * (S.dzl[je + 1] + S.dzl[je])) /
                 (tk_lake[je] * S.dzl[je + 1] + tk_lake[je + 1] * S.dzl[je]);
    } else if (je == nlak) {
      const double dzp = zx[ji + 1] - zx[ji];
      tkix[ji] = tktopsoillay * tk_lake[je] * dzp / (tktopsoillay * S.dzl[je] / 2.0 + tk_lake[je] * S.z[1 + ns]);
    } else {
      tkix[ji] = tk[je - nlak + ns];
    }
  }
  // Crank-Nicolson system (:705-755) and its Thomas solve (tridiagonal.jl:86-127)
  for (int je = (int)jtop; je <= nlak + ngr; je++) {
    const int ji = je + ns;
    factx[ji] = dtime / cvx[ji];
    fnx[ji] = je < nlak + ngr ? tkix[ji] * (tx[ji + 1] - tx[ji]) / (zx[ji + 1] - zx[ji]) : 0.0;
  }
  const double omc = 1.0 - CNFAC;
  const int j0 = (int)jtop + ns;
  double cpv[MAXX], dpv[MAXX];
  const double tiny = 1e-30;
  double cpp = 0.0, dpp = 0.0;
  for (int ji = j0; ji <= ntot; ji++) {
    const int je = ji - ns;
    double av, bv, cvv, rv;
    if (je == jtop) {
      const double dzp = zx[ji + 1] - zx[ji];
      av = 0.0;
      bv = 1.0 + omc * factx[ji] * tkix[ji] / dzp;
      cvv = -omc * factx[ji] * tkix[ji] / dzp;
      rv = tx[ji] + factx[ji] * (fin + phix[ji] + CNFAC * fnx[ji]);
    } else if (je < nlak + ngr) {
      const double dzm = zx[ji] - zx[ji - 1], dzp = zx[ji + 1] - zx[ji];
      av = -omc * factx[ji] * tkix[ji - 1] / dzm;
      bv = 1.0 + omc * factx[ji] * (tkix[ji] / dzp + tkix[ji - 1] / dzm);
      cvv = -omc * factx[ji] * tkix[ji] / dzp;
      rv = tx[ji] + CNFAC * factx[ji] * (fnx[ji] - fnx[ji - 1]) + factx[ji] * phix[ji];
    } else {
      const double dzm = zx[ji] - zx[ji - 1];
      av = -omc * factx[ji] * tkix[ji - 1] / dzm;
      bv = 1.0 + omc * factx[ji] * tkix[ji - 1] / dzm;
      cvv = 0.0;
      rv = tx[ji] - CNFAC * factx[ji] * fnx[ji - 1];
    }
    if (ji == j0) {
      double bet = bv;
      if (fabs(bet) < tiny) bet = tiny;
      cpp = cvv / bet;
      dpp = rv / bet;
    } else {
      double denom = bv - av * cpp;
      if (fabs(denom) < tiny) denom = copysign(tiny, denom == 0.0 ? 1.0 : denom);
      cpp = cvv / denom;
      dpp = (rv - av * dpp) / denom;
    }
    cpv[ji] = cpp;
    dpv[ji] = dpp;
  }
  double un = dpp;
  tx[ntot] = un;
  for (int ji = ntot - 1; ji >= j0; ji--) {
    un = dpv[ji] - cpv[ji] * un;
    tx[ji] = un;
  }
  for (int je = (int)jtop; je <= nlak + ngr; je++) {
    const int ji = je + ns;
    if (je < 1) S.t[ji] = tx[ji];
    else if (je <= nlak) S.tl[je] = tx[ji];
    else S.t[je - nlak + ns] = tx[ji];
  }

  // phase_change_lake! (:204-314)
  {
    const double small = 1.0e-12;
    double qsm = 0.0, qsd = 0.0, qsf = 0.0;
    for (int jj = 1; jj <= ns; jj++) {
      LV(f.qflx_snomelt_lyr, c, jj, ld) = 0.0;
      LV(f.qflx_snofrz_lyr, c, jj, ld) = 0.0;
      LV(f.imelt, c, jj, ld) = 0;
    }
    if (h2osno_nl > 0.0 && S.tl[1] > TFRZ) {                 // unresolved snow on warm water
      const double heatavail = (S.tl[1] - TFRZ) * cv_lake[1];
      const double melt = jl_min(h2osno_nl, heatavail / HFUS);
      const double heatrem = jl_max(heatavail - melt * HFUS, 0.0);
      S.tl[1] = TFRZ + heatrem / cv_lake[1];
      snow_depth = snow_depth * (1.0 - melt / h2osno_nl);
      h2osno_nl = h2osno_nl - melt;
      qsm += melt / dtime;
      qsd += melt / dtime;
      if (h2osno_nl < small) h2osno_nl = 0.0;
      if (snow_depth < small) snow_depth = 0.0;
    }
    for (int j = 1; j <= nlak; j++) {
      bool dophase = false;
      double heatavail = 0.0, melt = 0.0, heatrem = 0.0;
      if (S.tl[j] > TFRZ && S.fi[j] > 0.0) {
        dophase = true;
        heatavail = (S.tl[j] - TFRZ) * cv_lake[j];
        melt = jl_min(S.fi[j] * DENH2O * S.dzl[j], heatavail / HFUS);
        heatrem = jl_max(heatavail - melt * HFUS, 0.0);
      } else if (S.tl[j] < TFRZ && S.fi[j] < 1.0) {
        dophase = true;
        heatavail = (S.tl[j] - TFRZ) * cv_lake[j];
        melt = jl_max(-(1.0 - S.fi[j]) * DENH2O * S.dzl[j], heatavail / HFUS);
        heatrem = jl_min(heatavail - melt * HFUS, 0.0);
      }
      if (dophase) {
        S.fi[j] = S.fi[j] - melt / (DENH2O * S.dzl[j]);
        cv_lake[j] = cv_lake[j] + melt * (CPLIQ - CPICE);
        S.tl[j] = TFRZ + heatrem / cv_lake[j];
        if (S.fi[j] > 1.0 - small) S.fi[j] = 1.0;
        if (S.fi[j] < small) S.fi[j] = 0.0;
      }
    }
    for (int j = (int)snl + 1; j <= ngr; j++) {
      const int jj = j + ns;
      bool dophase = false;
      double heatavail = 0.0, melt = 0.0, heatrem = 0.0;
      if (S.t[jj] > TFRZ && S.ice[jj] > 0.0) {
        dophase = true;
        heatavail = (S.t[jj] - TFRZ) * cv[jj];
        melt = jl_min(S.ice[jj], heatavail / HFUS);
        heatrem = jl_max(heatavail - melt * HFUS, 0.0);
        if (j <= 0) {
          LV(f.imelt, c, jj, ld) = 1;
          const double q = melt / dtime;
          LV(f.qflx_snomelt_lyr, c, jj, ld) = q;
          qsm += q;
        }
      } else if (S.t[jj] < TFRZ && S.liq[jj] > 0.0) {
        dophase = true;
        heatavail = (S.t[jj] - TFRZ) * cv[jj];
        melt = jl_max(-S.liq[jj], heatavail / HFUS);
        heatrem = jl_min(heatavail - melt * HFUS, 0.0);
        if (j <= 0) {
          LV(f.imelt, c, jj, ld) = 2;
          const double q = -melt / dtime;
          LV(f.qflx_snofrz_lyr, c, jj, ld) = q;
          qsf += q;
        }
      }
      if (dophase) {
        S.ice[jj] = S.ice[jj] - melt;
        S.liq[jj] = S.liq[jj] + melt;
        cv[jj] = cv[jj] + melt * (CPLIQ - CPICE);
        S.t[jj] = TFRZ + heatrem / cv[jj];
        if (S.ice[jj] < small) S.ice[jj] = 0.0;
        if (S.liq[jj] < small) S.liq[jj] = 0.0;
      }
    }
    f.qflx_snomelt[c] = qsm;
    f.qflx_snofrz[c] = qsf;
    f.qflx_snow_drain[c] = qsd;
    f.eflx_snomelt[c] = qsm * HFUS;
  }

  // convective mixing, top down then bottom up (:1204-1241, :787-894)
  for (int j = 1; j <= nlak; j++) rhow[j] = lake_density(S.fi[j], S.tl[j]);
  bool puddle = false;
  if (puddling) {
    double icesum = 0.0;
    for (int j = 1; j <= nlak; j++) icesum = icesum + S.fi[j] * S.dz[j + ns];
    puddle = icesum >= P.lake_puddle_thick;
  }
  const bool mixing = !puddling || !puddle;
  int jconvect = 0, jconvectbot = nlak + 1;
  for (int j = 1; j <= nlak - 2; j++) {
    if (!(mixing && (rhow[j] > rhow[j + 1] || (S.fi[j] < 1.0 && S.fi[j + 1] > 0.0)))) continue;
    jconvect = j + 1;
    mix(S, rhow, 1, j + 1, cwat, cice_eff);
  }
  const int jb = nlak - 1;
  const bool bottomconvect = mixing && (rhow[jb] > rhow[jb + 1] || (S.fi[jb] < 1.0 && S.fi[jb + 1] > 0.0));
  for (int j = nlak - 1; j >= 1; j--) {
    if (!(bottomconvect && mixing && (rhow[j] > rhow[j + 1] || (S.fi[j] < 1.0 && S.fi[j + 1] > 0.0)))) continue;
    jconvectbot = j;
    mix(S, rhow, j, nlak, cwat, cice_eff);
  }
  if (lch4) {                                              // lake resistance to CH4 (:902-921)
    double lr = 0.0;
    for (int j = 1; j <= nlak; j++)
      if (j > jconvect && j < jconvectbot) lr += S.dzl[j] / kme[j];
    f.lakeresist[c] = lr;
    double gc = 1.0 / (lr + f.lake_raw[c]);
    if (S.fi[1] > 0.1) gc = 0.0;
    f.grnd_ch4_cond[c] = gc;
  }

  // energy after, and the conservation check (:923-983)
  for (int j = 1; j <= nlak; j++) cv_lake[j] = S.dzl[j] * (cwat * (1.0 - S.fi[j]) + cice_eff * S.fi[j]);
  therm_prop(f, S, c, ld, ns, ngr, nsoi, snl, tk, cv, tktopsoillay);
  double ncvts = 0.0;
  for (int j = 1; j <= nlak; j++) {
    ncvts += cv_lake[j] * (S.tl[j] - TFRZ) + cfus * S.dzl[j] * (1.0 - S.fi[j]);
    fin += phi[j];
  }
  hsn = h2osno_total(S, h2osno_nl, ns, snl);
  for (int j = -ns + 1; j <= ngr; j++) {
    const int jj = j + ns;
    if (j >= jtop) {
      ncvts += cv[jj] * (S.t[jj] - TFRZ) + HFUS * S.liq[jj];
      if (j < 1) fin += phix[j + ns];
      if (j == 1 && hsn > 0.0 && j == jtop) ncvts -= hsn * HFUS;
    }
    if (j == 1) fin += phi_soil;
  }
  if (pact) {
    double err = (ncvts - ocvts) / dtime - fin;
    if (fabs(err) < 0.10) {
      f.eflx_sh_tot[p] -= err;
      f.eflx_sh_grnd[p] -= err;
      f.eflx_soil_grnd[p] += err;
      f.eflx_gnet[p] += err;
      err = 0.0;
    }
    f.errsoi_col[c] = err;
  }
  double thick = 0.0;
  for (int j = 1; j <= nlak; j++) thick += S.fi[j] * S.dzl[j] * DENH2O / DENICE;
  f.lake_icefracsurf[c] = S.fi[1];
  f.lake_icethick[c] = thick;

  // state back
  for (int jj = 1; jj <= ns + ngr; jj++) {
    LV(f.t_soisno, c, jj, ld) = S.t[jj];
    LV(f.h2osoi_liq, c, jj, ld) = S.liq[jj];
    LV(f.h2osoi_ice, c, jj, ld) = S.ice[jj];
  }
  for (int j = 1; j <= nlak; j++) {
    LV(f.t_lake, c, j, ld) = S.tl[j];
    LV(f.lake_icefrac, c, j, ld) = S.fi[j];
  }
  f.h2osno_no_layers[c] = h2osno_nl;
  f.snow_depth[c] = snow_depth;
}

}  // namespace

cudaError_t launch_lake_temperature(const Dims& D, int64_t nc, const clmgb_lake_fields& f, const clmgb_lake_config& P,
                                    double dtime, uint32_t* dev_status, cudaStream_t s) {
  k_lake_temperature<<<(unsigned int)((nc + LK_BLOCK - 1) / LK_BLOCK), LK_BLOCK, 0, s>>>(D, nc, f, P, dtime,
                                                                                         dev_status);
  return cudaGetLastError();
}

}  // namespace clmgb
