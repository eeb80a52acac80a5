// adjoint_closed.cu — reverse of one column step written out by hand (no tape).
//
// The recording kernel (adjoint_step.cu) differentiates soil_temperature! by
// replaying it through a recording scalar and sweeping the tape.  This kernel runs
// the production arithmetic on plain values (soil_temperature_col with a per-thread
// state accessor, so the forward is the production step bit for bit) and then
// applies the transpose of every stage's derivative, last stage first:
//
//   t_grnd        tg = fse ts + (1-fse-fh) t1 + fh th, or (1-fh) t1 + fh th
//                 (_tgrnd_kernel!, soil_temperature.jl:224-247)
//   phase change  per level: the melt/freeze decision, hm, xm, the new ice and
//                 liquid water and the temperature correction
//                 (_phase_change_beta_kernel!, :1929-2230)
//   band solve    lambda = A^-T xbar from the factors the forward kept,
//                 rbar = lambda, Abar = -lambda x^T (band_solve! rule,
//                 enzyme_rules.jl:80-107)
//   assembly      the rows of set_rhs_vec! / set_matrix! (:1365-1748)
//   heat flux     fn, the ground heat flux sums dhsdT, hs_soil, hs_h2osfc,
//                 hs_top_snow (:1200-1263, :1271-1319)
//   capacity      fact = dtime/cv (top layer with the CAPR factor), cv (:599-942)
//   conductivity  interface tk, tk_h2osfc, layer thk (Johansen for soil, Jordan or
//                 Sturm for snow) (:647-776)
//
// The Richards substeps are reversed by mf_substep_reverse (adjoint_richards.cuh,
// shared with the recording kernel); set_soil_water_fractions! and the ice
// impedance are reversed here in closed form.  Every decision (branch, clamp,
// pivot) is the forward's; the derivative of a Julia max/min passes to the
// argument it returned (the constant when a tie returned it), as in the recording
// kernel, so both kernels differentiate the same piecewise function.
//
// Elementwise stages keep their local partial derivatives from the forward sweep
// (thk and fact with respect to liquid water, ice and watsat; the interface
// conductivity with respect to its two layers), so the reverse is a few
// multiply-adds per level.
//
// With a substep log (clmgb_substep_log, written by clmgb_column_step_logged) the
// Richards forward is not run again: its accepted substeps' starting water comes
// from the log, and so do the solve's outputs.  Without one (or for a column the
// log could not hold) the substep loop runs on values here, keeping the same
// checkpoints in the reserved per-slot storage.
#include "adjoint_richards.cuh"
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

constexpr int CF_BLOCK = 64;

// The factorisation of the column's band system: lu/x/piv point at the thread's own
// storage (soil_temperature! run here) or at the column's soil_temperature! record.
struct CfBand {
  int n;
  const double* lu;
  const double* x;
  const uint8_t* piv;
  double lu_s[MAXROWS * 7];
  double x_s[MAXROWS];
  uint8_t piv_s[MAXROWS];
};

// The column's active state in per-thread storage, values only.
struct CfState {
  typedef double S;
  double t[MAXL + 2], liq[MAXL + 2], ice[MAXL + 2], fact[MAXL + 2];
  double icefrac[MAXSOI + 2];
  double tg, th, qc, forc;
  const double *ws, *bs, *suc, *ks;
  int64_t c, ld;
  CfBand* band;
  __device__ __forceinline__ double& T(int jj) { return t[jj]; }
  __device__ __forceinline__ double& Liq(int jj) { return liq[jj]; }
  __device__ __forceinline__ double& Ice(int jj) { return ice[jj]; }
  __device__ __forceinline__ double& Fact(int jj) { return fact[jj]; }
  __device__ __forceinline__ double& Icefrac(int j) { return icefrac[j]; }
  __device__ __forceinline__ double& Tgrnd() { return tg; }
  __device__ __forceinline__ double& Th2osfc() { return th; }
  __device__ __forceinline__ double& Qcharge() { return qc; }
  __device__ __forceinline__ double ForcLwrad() const { return forc; }
  __device__ __forceinline__ double Watsat(int j) const { return LVc(ws, c, j, ld); }
  __device__ __forceinline__ double Bsw(int j) const { return LVc(bs, c, j, ld); }
  __device__ __forceinline__ double Sucsat(int j) const { return LVc(suc, c, j, ld); }
  __device__ __forceinline__ double Hksat(int j) const { return LVc(ks, c, j, ld); }
  // the production factorisation, keeping the factors, pivots and solution
  __device__ __forceinline__ void band_solve(double* ab, double* x, int n) {
    band_lu_factor_solve<2, 2>(ab, x, band->piv_s, n);
    band->n = n;
    for (int k = 0; k < n * 7; k++) band->lu_s[k] = ab[k];
    for (int r = 0; r < n; r++) band->x_s[r] = x[r];
    band->lu = band->lu_s;
    band->x = band->x_s;
    band->piv = band->piv_s;
  }
};

__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}

// ---------------------------------------------------------------------------
// Phase change of one level (snow or soil), reversed.  T0: the temperature the
// band solve left, wice0/wliq0: ice and liquid water before the phase change,
// fct: the level's fact.  In: the adjoints of the level's temperature, liquid
// water and ice after the phase change.  Out (accumulated): the adjoints of T0,
// wice0, wliq0, fct, dhsdT and the level's watsat, bsw, sucsat (supercooled water).
// Columns with excess ice or snow without layers are flagged by the caller; their
// branches are not taken here.
// ---------------------------------------------------------------------------
struct PcLevelIn {
  int j, jtop;
  double T0, wice0, wliq0, fct, dhsdT, fse, fh, dtime;
  bool sc_type;
  double ws, bs, suc, dz;
};

__device__ __noinline__ void phase_change_level_reverse(const PcLevelIn& in, double Tpc_b, double liqpc_b,
                                                        double icepc_b, double& T0_b, double& ice0_b,
                                                        double& liq0_b, double& fct_b, double& dhsdT_b,
                                                        double& ws_b, double& bs_b, double& suc_b) {
  const int j = in.j, jtop = in.jtop;
  const double T0 = in.T0, wice0 = in.wice0, wliq0 = in.wliq0, fct = in.fct, dhsdT = in.dhsdT;
  const double fse = in.fse, fh = in.fh, dtime = in.dtime;
  const double wmass0 = wice0 + wliq0 + 0.0;
  // ---- the melt / freeze decision (:1990-2040) ----
  int im = 0;
  double tinc = 0.0;
  bool sc_on = false;
  double sc = 0.0, P = 0.0, r = 0.0, e = 0.0, q = 0.0, g = 0.0;
  if (j <= 0) {
    if (wice0 > 0.0 && T0 > TFRZ) {
      im = 1;
      tinc = TFRZ - T0;
    } else if (wliq0 > 0.0 && T0 < TFRZ) {
      im = 2;
      tinc = TFRZ - T0;
    }
  } else {
    double T = T0;
    if (wice0 > 0.0 && T0 > TFRZ) {
      im = 1;
      tinc = TFRZ - T0;
      T = TFRZ;
    }
    if (in.sc_type && T < TFRZ) {
      sc_on = true;
      q = HFUS * (TFRZ - T) / (GRAV * T);
      g = GRAV * T;
      const double smp = q * 1000.0;
      r = smp / in.suc;
      e = -1.0 / in.bs;
      P = cm_pow(r, e);
      sc = in.ws * P;
      sc *= in.dz * 1000.0;
    }
    if (wliq0 > sc && T < TFRZ) {
      im = 2;
      tinc = TFRZ - T;
    }
  }
  if (im == 0) {
    T0_b += Tpc_b;
    liq0_b += liqpc_b;
    ice0_b += icepc_b;
    return;
  }
  // ---- hm (:2060-2085) ----
  double hm;
  if (j == jtop) {
    if (j > 0) hm = dhsdT * tinc - tinc / fct;
    else hm = fse * (dhsdT * tinc - tinc / fct);
    if (j == 1 && fh != 0.0) hm -= fh * dhsdT * tinc;
  } else if (j == 1) {
    hm = (1.0 - fse - fh) * dhsdT * tinc - tinc / fct;
  } else {
    if (j < 1) hm = -fse * tinc / fct;
    else hm = -tinc / fct;
  }
  if ((im == 1 && hm < 0.0) || (im == 2 && hm > 0.0)) im = 0;
  if (im == 0 || !(fabs(hm) > 0.0)) {
    // the temperature was set to freezing (a constant); the water is unchanged
    liq0_b += liqpc_b;
    ice0_b += icepc_b;
    return;
  }
  // ---- new ice and liquid water (:2090-2140) ----
  const double xm = jl_div(hm * dtime, HFUS);
  double ice = wice0, heatr = 0.0;
  int kind = 0;   // 0 ice unchanged, 1 wice0 - xm, 2 constant, 3 wmass0, 4 wmass0 - sc
  if (xm > 0.0) {
    const double v = wice0 - xm;
    ice = jl_max(0.0, v);
    kind = same_bits(ice, 0.0) ? 2 : 1;
    heatr = hm - jl_div(HFUS * (wice0 - ice), dtime);
  } else if (xm < 0.0) {
    if (j <= 0) {
      const double a = wmass0, b = wice0 - xm;
      ice = jl_min(a, b);
      kind = same_bits(ice, a) ? 3 : 1;
    } else {
      if (wmass0 - 0.0 < sc) {
        ice = 0.0;
        kind = 2;
      } else {
        const double a = wmass0 - 0.0 - sc, b = wice0 - xm;
        ice = jl_min(a, b);
        kind = same_bits(ice, a) ? 4 : 1;
      }
    }
    heatr = hm - jl_div(HFUS * (wice0 - ice), dtime);
  }
  const double liqv = wmass0 - ice - 0.0;
  const double liq = jl_max(0.0, liqv);
  const bool liq_pass = !same_bits(liq, 0.0);
  // ---- reverse (derivative coefficients with reciprocals) ----
  double heatr_b = 0.0, hm_b = 0.0, xm_b = 0.0, ice_b = icepc_b, wmass0_b = 0.0, wice0_b = 0.0, sc_b = 0.0;
  double tinc_b = 0.0;
  const double rf = 1.0 / fct;
  if (fabs(heatr) > 0.0 && !(j <= 0 && liq * ice > 0.0)) {
    // temperature correction (:2145-2165); the level starts from freezing
    if (j == 1) {
      const double k = (j == jtop) ? (1.0 - fh) : (1.0 - fse - fh);
      const double rden = 1.0 / (1.0 - k * fct * dhsdT);
      const double incr = fct * heatr * rden;
      const double N_b = Tpc_b * rden, den_b = -Tpc_b * incr * rden;
      fct_b += N_b * heatr - den_b * k * dhsdT;
      heatr_b += N_b * fct;
      dhsdT_b += -den_b * k * fct;
    } else if (j == jtop) {      // top snow layer
      if (fse > 0.0) {
        const double rfse = 1.0 / fse;
        const double rden = 1.0 / (1.0 - fct * dhsdT);
        const double incr = fct * rfse * heatr * rden;
        const double N_b = Tpc_b * rden, den_b = -Tpc_b * incr * rden;
        fct_b += N_b * heatr * rfse - den_b * dhsdT;
        heatr_b += N_b * fct * rfse;
        dhsdT_b += -den_b * fct;
      }
    } else if (j > 0) {
      fct_b += Tpc_b * heatr;
      heatr_b += Tpc_b * fct;
    } else if (fse > 0.0) {
      const double rfse = 1.0 / fse;
      fct_b += Tpc_b * heatr * rfse;
      heatr_b += Tpc_b * fct * rfse;
    }
  }
  if (liq_pass) {
    wmass0_b += liqpc_b;
    ice_b -= liqpc_b;
  }
  if (xm != 0.0) {
    hm_b += heatr_b;
    const double d_b = -heatr_b * HFUS * (1.0 / dtime);
    wice0_b += d_b;
    ice_b -= d_b;
  }
  switch (kind) {
    case 0: wice0_b += ice_b; break;
    case 1: wice0_b += ice_b; xm_b -= ice_b; break;
    case 3: wmass0_b += ice_b; break;
    case 4: wmass0_b += ice_b; sc_b -= ice_b; break;
    default: break;
  }
  hm_b += xm_b * dtime * (1.0 / HFUS);
  // hm
  if (j == jtop) {
    const double hb = (j > 0) ? hm_b : hm_b * fse;
    dhsdT_b += hb * tinc;
    tinc_b += hb * dhsdT - hb * rf;
    fct_b += hb * tinc * rf * rf;
    if (j == 1 && fh != 0.0) {
      dhsdT_b -= hm_b * fh * tinc;
      tinc_b -= hm_b * fh * dhsdT;
    }
  } else if (j == 1) {
    const double k = 1.0 - fse - fh;
    dhsdT_b += hm_b * k * tinc;
    tinc_b += hm_b * k * dhsdT - hm_b * rf;
    fct_b += hm_b * tinc * rf * rf;
  } else {
    const double a = (j < 1) ? fse : 1.0;     // hm = -a tinc / fct
    tinc_b -= hm_b * a * rf;
    fct_b += hm_b * a * tinc * rf * rf;
  }
  T0_b -= tinc_b;
  // supercooled water sc = watsat (smp/sucsat)^(-1/bsw) dz 1000, smp = HFUS (TFRZ-T)/(GRAV T) 1000
  if (sc_b != 0.0 && sc_on) {
    const double sc0_b = sc_b * (in.dz * 1000.0);
    ws_b += sc0_b * P;
    const double P_b = sc0_b * in.ws;
    const double rr = 1.0 / r, rsuc = 1.0 / in.suc, rg = 1.0 / g;
    const double r_b = r != 0.0 ? P_b * e * P * rr : 0.0;
    const double e_b = r > 0.0 ? P_b * P * cm_log(r) : 0.0;
    bs_b += e_b * (-e) * (1.0 / in.bs);
    const double smp_b = r_b * rsuc;
    suc_b += r_b * (-r) * rsuc;
    const double q_b = smp_b * 1000.0;
    const double a_b = q_b * rg;
    const double g_b = -q_b * q * rg;
    T0_b += -a_b * HFUS + g_b * GRAV;
  }
  ice0_b += wice0_b + wmass0_b;
  liq0_b += wmass0_b;
}

// ---------------------------------------------------------------------------
// soil_temperature! reversed for column c.  The forward left in V the final state
// and in B the band factors; tin, liq0, ice0, tg0, th0 are the step's inputs.
// Tb, liqb, iceb, tgb, thb hold on entry the adjoints of the quantities after the
// call and on return those of its inputs; forcb and wsb/bsb/sucb accumulate.
// ---------------------------------------------------------------------------
__device__ __noinline__ void soil_temperature_reverse(const Dims& D, const clmgb_soiltemp_fields& f,
                                                      const clmgb_soilwater_fields& fw, int64_t c, double dtime,
                                                      int snow_method, const double* fact, const double* tin,
                                                      const double* liq0, const double* ice0, double tg0, double th0,
                                                      double forc, const CfBand& B, double* Tb, double* liqb,
                                                      double* iceb, double& tgb, double& thb, double& forcb,
                                                      double* wsb, double* bsb, double* sucb) {
  const int64_t ld = D.ldc, ldp = D.ldp;
  const int nlevsno = D.nlevsno, nlevgrnd = D.nlevgrnd;
  const int joff = nlevsno;
  const int nw = nlevsno + nlevgrnd;
  const int64_t snl = f.col_snl[c];
  const int jtop = (int)snl + 1, jjtop = jtop + joff;
  const int64_t l = f.col_landunit[c] - 1;
  const int64_t it = f.col_itype[c];
  const int64_t lit = f.lun_itype[l];
  const bool is_special = (lit == ISTWET || lit == ISTICE);
  const int64_t nbedrock = f.col_nbedrock[c];
  const double fse = f.frac_sno_eff[c];
  const double fh = f.frac_h2osfc[c];
  const double omc = 1.0 - CNFAC;
  const double LN_TKWAT = cm_log(TKWAT), LN_TKICE = cm_log(TKICE);

  double zz[MAXL + 2], rdzp[MAXL + 2];     // rdzp[jj] = 1 / (z[jj+1] - z[jj])
  for (int jj = jjtop; jj <= nw; jj++) zz[jj] = LVc(f.z, c, jj, ld);
  for (int jj = jjtop; jj < nw; jj++) rdzp[jj] = 1.0 / (zz[jj + 1] - zz[jj]);

  // ---- forward values with local partials ----
  // layer conductivity thk and its partials in liquid water, ice and watsat
  double thk[MAXL + 2], tl[MAXL + 2], ti[MAXL + 2], tw[MAXL + 2];
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    double v = 0.0, dl = 0.0, di = 0.0, dw = 0.0;
    if (j >= 1) {
      if (!is_special) {
        if (j > nbedrock) {
          v = THK_BEDROCK;
        } else {
          const double liq = liq0[jj], ice = ice0[jj];
          const double exi = LV(f.excess_ice, c, j, ld);
          const double dzv = LVc(f.dz, c, jj, ld);
          const double ws = LVc(fw.watsat, c, j, ld);
          const double m = dzv * ws;
          const double satw0 = (jl_div(liq, DENH2O) + jl_div(ice, DENICE) + jl_div(exi, DENICE)) / m;
          const double satw = jl_min(1.0, satw0);
          const bool spass = !same_bits(satw, 1.0);
          if (satw > 1.0e-7) {
            double dke, ddke;
            if (tin[jj] >= TFRZ) {
              const double L = cm_log10(satw) + 1.0;
              dke = jl_max(0.0, L);
              ddke = same_bits(dke, 0.0) ? 0.0 : 0.43429448190325182765 * (1.0 / satw);
            } else {
              dke = satw;
              ddke = 1.0;
            }
            // derivative coefficients (reciprocals instead of divisions; TKWAT^a TKICE^b
            // as one exponential)
            const double rm = 1.0 / m, rdz = 1.0 / dzv;
            const double a1 = liq * (1.0 / DENH2O) * rdz;
            const double fl_denom = a1 + (ice + exi) * (1.0 / DENICE) * rdz;
            const double rfd = 1.0 / fl_denom;
            const double fl = a1 * rfd;
            const double tkmg = LVc(f.tkmg, c, j, ld), tkdry = LVc(f.tkdry, c, j, ld);
            const double dksat = tkmg * cm_exp(ws * (fl * LN_TKWAT + (1.0 - fl) * LN_TKICE));
            v = dke * dksat + (1.0 - dke) * tkdry;
            // d satw
            const double sl = spass ? (1.0 / DENH2O) * rm : 0.0;
            const double si = spass ? (1.0 / DENICE) * rm : 0.0;
            const double sw = spass ? -(satw0 * rm) * dzv : 0.0;
            // d dksat / d fl, d ws
            const double kfl = dksat * (LN_TKWAT * ws - LN_TKICE * ws);
            const double kws = dksat * (LN_TKWAT * fl + LN_TKICE * (1.0 - fl));
            const double fll = (1.0 - fl) * rfd * (1.0 / DENH2O) * rdz;
            const double fli = -fl * rfd * (1.0 / DENICE) * rdz;
            const double cdke = (dksat - tkdry) * ddke;
            dl = cdke * sl + dke * kfl * fll;
            di = cdke * si + dke * kfl * fli;
            dw = cdke * sw + dke * kws;
          } else {
            v = LVc(f.tkdry, c, j, ld);
          }
        }
      } else if (lit == ISTICE) {
        v = tin[jj] < TFRZ ? TKICE : TKWAT;
      } else {
        if (j > D.nlevsoi) v = THK_BEDROCK;
        else v = tin[jj] < TFRZ ? TKICE : TKWAT;
      }
    } else {
      const double denom = jl_max(fse, 1.0e-6) * jl_max(LVc(f.dz, c, jj, ld), 1.0e-6);
      const double bwv = (ice0[jj] + liq0[jj]) / denom;
      double dbw;
      if (snow_method == CLMGB_SNOW_JORDAN1991) {
        v = TKAIR + (7.75e-5 * bwv + 1.105e-6 * (bwv * bwv)) * (TKICE - TKAIR);
        dbw = (7.75e-5 + 1.105e-6 * (bwv + bwv)) * (TKICE - TKAIR);
      } else if (bwv <= 156.0) {
        v = 0.023 + 0.234 * (bwv / 1000.0);
        dbw = 0.234 / 1000.0;
      } else {
        v = 0.138 - 1.01 * (bwv / 1000.0) + 3.233 * ((bwv / 1000.0) * (bwv / 1000.0));
        dbw = (-1.01 + 3.233 * (2.0 * (bwv / 1000.0))) / 1000.0;
      }
      dl = dbw / denom;
      di = dbw / denom;
    }
    thk[jj] = v;
    tl[jj] = dl;
    ti[jj] = di;
    tw[jj] = dw;
  }
  // tk_h2osfc from the soil-1 layer conductivity
  double tkh, dtkh;
  {
    const double zh2osfc = 1.0e-3 * (0.5 * f.h2osfc[c]);
    const double z1 = zz[1 + joff];
    const double tk1 = thk[1 + joff];
    const double den = TKWAT * z1 + tk1 * zh2osfc;
    if (den > 0.0) {
      tkh = TKWAT * tk1 * (z1 + zh2osfc) / den;
      dtkh = (TKWAT * (z1 + zh2osfc) - tkh * zh2osfc) / den;
    } else {
      tkh = tk1;
      dtkh = 1.0;
    }
  }
  // interface conductivity and its partials in the two layers
  double tkif[MAXL + 2], da[MAXL + 2], db[MAXL + 2];
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    if (j <= nlevgrnd - 1) {
      const double tkj = thk[jj], tkj1 = thk[jj + 1];
      const double zj = zz[jj], zj1 = zz[jj + 1], zij1 = LVc(f.zi, c, jj + 1, ld);
      const double A = zj1 - zj, Bz = zj1 - zij1, Cz = zij1 - zj;
      const double rden = 1.0 / (tkj * Bz + tkj1 * Cz);
      const double v = tkj * tkj1 * A * rden;
      tkif[jj] = v;
      da[jj] = (tkj1 * A - v * Bz) * rden;
      db[jj] = (tkj * A - v * Cz) * rden;
    } else {
      tkif[jj] = 0.0;
      da[jj] = 0.0;
      db[jj] = 0.0;
    }
  }
  // heat capacity: cv and the partials of fact in liquid water, ice and watsat
  double cl[MAXL + 2], ci[MAXL + 2], cw[MAXL + 2];
  double fn[MAXL + 2];
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    const double dzv = LVc(f.dz, c, jj, ld);
    double cv, dl = 0.0, di = 0.0, dw = 0.0;
    if (j >= 1) {
      if (!is_special) {
        const double ws = LVc(fw.watsat, c, j, ld);
        cv = LVc(f.csol, c, j, ld) * (1.0 - ws) * dzv + (ice0[jj] * CPICE + liq0[jj] * CPLIQ) +
             LV(f.excess_ice, c, j, ld) * CPICE;
        dl = CPLIQ;
        di = CPICE;
        dw = -LVc(f.csol, c, j, ld) * dzv;
      } else {
        cv = ice0[jj] * CPICE + liq0[jj] * CPLIQ;
        dl = CPLIQ;
        di = CPICE;
      }
      if (j > nbedrock) {
        cv = CSOL_BEDROCK * dzv;
        dl = di = dw = 0.0;
      }
      if (j == 1 && f.h2osno_no_layers[c] > 0.0) cv += CPICE * f.h2osno_no_layers[c];
    } else {
      if (fse > 0.0) {
        const double v = (CPLIQ * liq0[jj] + CPICE * ice0[jj]) / fse;
        cv = jl_max(THIN_SFCLAYER, v);
        if (!same_bits(cv, THIN_SFCLAYER)) {
          dl = CPLIQ / fse;
          di = CPICE / fse;
        }
      } else {
        cv = THIN_SFCLAYER;
      }
    }
    const double dfdcv = -fact[jj] / cv;
    cl[jj] = dfdcv * dl;
    ci[jj] = dfdcv * di;
    cw[jj] = dfdcv * dw;
    if (j <= nlevgrnd - 1) fn[jj] = tkif[jj] * (tin[jj + 1] - tin[jj]) * rdzp[jj];
    else fn[jj] = f.eflx_bot[c];
  }
  // ground heat flux sums and their derivative weights
  const double eg = f.emg[c];
  const double htvp = f.htvp[c];
  double dhsdT = 0.0, hs_soil = 0.0, hs_h2osfc = 0.0, hs_top = 0.0;
  double w_set = 0.0, wb_set = 0.0, w_act = 0.0, wb_act = 0.0;
  double sabg_col[MAXSNO + 2];
  for (int k = 0; k <= nlevsno + 1; k++) sabg_col[k] = 0.0;
  {
    const double dlwrad_emit = 4.0 * eg * SB * (tg0 * tg0 * tg0);
    const double lwe_snow = eg * SB * jl_pow4(tin[jjtop]);
    const double lwe_soil = eg * SB * jl_pow4(tin[1 + joff]);
    const double lwe_h2osfc = eg * SB * jl_pow4(th0);
    for (int64_t p1 = f.col_patchi[c]; p1 <= f.col_patchf[c]; p1++) {
      const int64_t p = p1 - 1;
      if (f.patch_column[p] != c + 1 + D.c0) continue;
      double dh_p = 0.0, hsoil_p = 0.0, hh_p = 0.0;
      const bool act = f.mask_nolakep[p] != 0;
      const double cb = (1.0 - (double)f.frac_veg_nosno[p]) * eg;
      const double base = f.dlrad[p] + cb * forc;
      const double wt = f.patch_wtcol[p];
      if (act && !f.lun_urbpoi[f.patch_landunit[p] - 1]) {
        const double dg = -f.cgrnd[p] - dlwrad_emit;
        const double gsoil = f.sabg_soil[p] + base - lwe_soil - (f.eflx_sh_soil[p] + f.qflx_ev_soil[p] * htvp);
        const double gh2o = f.sabg_soil[p] + base - lwe_h2osfc - (f.eflx_sh_h2osfc[p] + f.qflx_ev_h2osfc[p] * htvp);
        if (wt != 0.0) {
          dh_p = dg * wt;
          hsoil_p = gsoil * wt;
          hh_p = gh2o * wt;
          w_set += wt;
          wb_set += wt * cb;
        }
      }
      dhsdT += dh_p; hs_soil += hsoil_p; hs_h2osfc += hh_p;
      if (act) {
        const double sab = LVc(f.sabg_lyr, p, jtop + joff, ldp);
        const double gsnow = sab + base - lwe_snow - (f.eflx_sh_snow[p] + f.qflx_ev_snow[p] * htvp);
        hs_top += gsnow * wt;
        w_act += wt;
        wb_act += wt * cb;
        for (int j = jtop; j <= 1; j++) sabg_col[j + nlevsno] += LVc(f.sabg_lyr, p, j + joff, ldp) * wt;
      }
    }
  }
  double ch, dz_h2osfc;
  if (f.h2osfc[c] > THIN_SFCLAYER && fh > THIN_SFCLAYER) {
    ch = jl_max(THIN_SFCLAYER, CPLIQ * f.h2osfc[c] / fh);
    dz_h2osfc = jl_max(THIN_SFCLAYER, 1.0e-3 * f.h2osfc[c] / fh);
  } else {
    ch = THIN_SFCLAYER;
    dz_h2osfc = THIN_SFCLAYER;
  }
  const int n = B.n;
  const int rsw = -(int)snl;

  // ---- reverse: t_grnd ----
  double Tpc_b[MAXL + 2];
  for (int jj = jjtop; jj <= nw; jj++) Tpc_b[jj] = Tb[jj];
  double thpc_b = thb;                          // t_h2osfc after the call
  if (snl < 0) {
    Tpc_b[jjtop] += fse * tgb;
    Tpc_b[1 + joff] += (fh != 0.0 ? (1.0 - fse - fh) : (1.0 - fse)) * tgb;
    if (fh != 0.0) thpc_b += fh * tgb;
  } else {
    Tpc_b[1 + joff] += (fh != 0.0 ? (1.0 - fh) : 1.0) * tgb;
    if (fh != 0.0) thpc_b += fh * tgb;
  }
  // ---- reverse: phase change ----
  double ts_b[MAXL + 2], fct_b[MAXL + 2], liq_in_b[MAXL + 2], ice_in_b[MAXL + 2];
  double dhsdT_b = 0.0;
  const bool sc_type = (lit == ISTSOIL || lit == ISTCROP || it == ICOL_ROAD_PERV);
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    ts_b[jj] = 0.0;
    fct_b[jj] = 0.0;
    liq_in_b[jj] = 0.0;
    ice_in_b[jj] = 0.0;
    PcLevelIn in;
    in.j = j;
    in.jtop = jtop;
    in.T0 = B.x[j <= 0 ? j - jtop : rsw + j];
    in.wice0 = ice0[jj];
    in.wliq0 = liq0[jj];
    in.fct = fact[jj];
    in.dhsdT = dhsdT;
    in.fse = fse;
    in.fh = fh;
    in.dtime = dtime;
    in.sc_type = sc_type;
    in.ws = j >= 1 ? LVc(fw.watsat, c, j, ld) : 0.0;
    in.bs = j >= 1 ? LVc(fw.bsw, c, j, ld) : 0.0;
    in.suc = j >= 1 ? LVc(fw.sucsat, c, j, ld) : 0.0;
    in.dz = LVc(f.dz, c, jj, ld);
    double wsd = 0.0, bsd = 0.0, sud = 0.0;
    phase_change_level_reverse(in, Tpc_b[jj], liqb[jj], iceb[jj], ts_b[jj], ice_in_b[jj], liq_in_b[jj], fct_b[jj],
                               dhsdT_b, wsd, bsd, sud);
    if (j >= 1) {
      wsb[j] += wsd;
      bsb[j] += bsd;
      sucb[j] += sud;
    }
  }
  // ---- reverse: extraction and the band solve ----
  double w[MAXROWS];
  for (int r = 0; r < n; r++) w[r] = 0.0;
  for (int j = jtop; j <= 0; j++) w[j - jtop] += ts_b[j + joff];
  for (int j = 1; j <= nlevgrnd; j++) w[rsw + j] += ts_b[j + joff];
  if (fh == 0.0) w[rsw + 1] += thpc_b;   // t_h2osfc took the soil-1 temperature
  else w[rsw] += thpc_b;
  band_lu_transpose_solve<2, 2>(B.lu, B.piv, w, n);    // w = lambda
  // Abar[r][col] = -lambda_r x_col
#define ABAR(r, d) ((((r) - 2 + (d)) >= 0 && ((r) - 2 + (d)) < n) ? -w[r] * B.x[(r) - 2 + (d)] : 0.0)
  // ---- reverse: assembly ----
  double tin_b[MAXL + 2], tkif_b[MAXL + 2], fn_b[MAXL + 2];
  for (int jj = jjtop; jj <= nw; jj++) {
    tin_b[jj] = 0.0;
    tkif_b[jj] = 0.0;
    fn_b[jj] = 0.0;
  }
  double hs_top_b = 0.0, hs_soil_b = 0.0, hs_h2osfc_b = 0.0, tkh_b = 0.0, th_b = 0.0;
  for (int j = jtop; j <= 0; j++) {
    const int jj = j + joff;
    const int r = j - jtop;
    const double fc = fact[jj];
    const double rp = rdzp[jj];
    const double lam = w[r];
    tin_b[jj] += lam;
    if (j == jtop) {
      const double inner = hs_top - dhsdT * tin[jj] + CNFAC * fn[jj];
      fct_b[jj] += lam * inner;
      const double ib = lam * fc;
      hs_top_b += ib;
      dhsdT_b -= ib * tin[jj];
      tin_b[jj] -= ib * dhsdT;
      fn_b[jj] += ib * CNFAC;
      const double g2 = ABAR(r, 2);
      fct_b[jj] += g2 * (omc * tkif[jj] * rp - dhsdT);
      tkif_b[jj] += g2 * omc * fc * rp;
      dhsdT_b -= g2 * fc;
    } else {
      fct_b[jj] += lam * (CNFAC * (fn[jj] - fn[jj - 1]) + sabg_col[jj]);
      fn_b[jj] += lam * CNFAC * fc;
      fn_b[jj - 1] -= lam * CNFAC * fc;
      const double rmn = rdzp[jj - 1];
      const double g1 = ABAR(r, 1), g2 = ABAR(r, 2);
      fct_b[jj] += -g1 * omc * tkif[jj - 1] * rmn + g2 * omc * (tkif[jj] * rp + tkif[jj - 1] * rmn);
      tkif_b[jj - 1] += -g1 * omc * fc * rmn + g2 * omc * fc * rmn;
      tkif_b[jj] += g2 * omc * fc * rp;
    }
    const double g = (j != 0) ? ABAR(r, 3) : ABAR(r, 4);
    fct_b[jj] += -g * omc * tkif[jj] * rp;
    tkif_b[jj] += -g * omc * fc * rp;
  }
  {   // surface-water row
    const double rdh = 1.0 / (0.5 * dz_h2osfc + zz[1 + joff]);
    const double dtc = dtime / ch;
    const double t1 = tin[1 + joff];
    const double fnh = tkh * (t1 - th0) * rdh;
    const double lam = w[rsw];
    th_b += lam;
    const double ib = lam * dtc;
    hs_h2osfc_b += ib;
    dhsdT_b -= ib * th0;
    th_b -= ib * dhsdT;
    const double fnh_b = ib * CNFAC;
    const double g2 = ABAR(rsw, 2), g3 = ABAR(rsw, 3);
    tkh_b += g2 * omc * dtc * rdh - g3 * omc * dtc * rdh;
    dhsdT_b -= g2 * dtc;
    tkh_b += fnh_b * (t1 - th0) * rdh;
    const double d_b = fnh_b * tkh * rdh;
    tin_b[1 + joff] += d_b;
    th_b -= d_b;
    (void)fnh;
  }
  for (int j = 1; j <= nlevgrnd; j++) {
    const int jj = j + joff;
    const int r = rsw + j;
    const double fc = fact[jj];
    const double t0 = tin[jj];
    const double lam = w[r];
    tin_b[jj] += lam;
    if (j == jtop) {
      const double rp = rdzp[jj];
      const double inner = hs_top - dhsdT * t0 + CNFAC * fn[jj];
      fct_b[jj] += lam * inner;
      const double ib = lam * fc;
      hs_top_b += ib;
      dhsdT_b -= ib * t0;
      tin_b[jj] -= ib * dhsdT;
      fn_b[jj] += ib * CNFAC;
      const double g2 = ABAR(r, 2), g3 = ABAR(r, 3);
      fct_b[jj] += g2 * (omc * tkif[jj] * rp - dhsdT) - g3 * omc * tkif[jj] * rp;
      tkif_b[jj] += g2 * omc * fc * rp - g3 * omc * fc * rp;
      dhsdT_b -= g2 * fc;
    } else if (j == 1) {
      const double rmn = rdzp[jj - 1];
      const double rp = rdzp[jj];
      const double inner = (1.0 - fse) * (hs_soil - dhsdT * t0) + CNFAC * (fn[jj] - fse * fn[jj - 1]);
      fct_b[jj] += lam * (inner + fse * sabg_col[j + nlevsno]);
      const double ib = lam * fc;
      const double u = ib * (1.0 - fse);
      hs_soil_b += u;
      dhsdT_b -= u * t0;
      tin_b[jj] -= u * dhsdT;
      fn_b[jj] += ib * CNFAC;
      fn_b[jj - 1] -= ib * CNFAC * fse;
      const double g0 = ABAR(r, 0), g2 = ABAR(r, 2), g3 = ABAR(r, 3);
      fct_b[jj] += -g3 * omc * tkif[jj] * rp +
                   g2 * (omc * (tkif[jj] * rp + fse * tkif[jj - 1] * rmn) - (1.0 - fse) * dhsdT) -
                   g0 * fse * omc * tkif[jj - 1] * rmn;
      tkif_b[jj] += -g3 * omc * fc * rp + g2 * omc * fc * rp;
      tkif_b[jj - 1] += g2 * omc * fc * fse * rmn - g0 * fse * omc * fc * rmn;
      dhsdT_b -= g2 * (1.0 - fse) * fc;
    } else if (j <= nlevgrnd - 1) {
      const double rmn = rdzp[jj - 1];
      const double rp = rdzp[jj];
      fct_b[jj] += lam * CNFAC * (fn[jj] - fn[jj - 1]);
      fn_b[jj] += lam * CNFAC * fc;
      fn_b[jj - 1] -= lam * CNFAC * fc;
      const double g1 = ABAR(r, 1), g2 = ABAR(r, 2), g3 = ABAR(r, 3);
      fct_b[jj] += -g3 * omc * tkif[jj] * rp + g2 * omc * (tkif[jj] * rp + tkif[jj - 1] * rmn) -
                   g1 * omc * tkif[jj - 1] * rmn;
      tkif_b[jj] += -g3 * omc * fc * rp + g2 * omc * fc * rp;
      tkif_b[jj - 1] += g2 * omc * fc * rmn - g1 * omc * fc * rmn;
    } else {
      const double rmn = rdzp[jj - 1];
      fct_b[jj] += lam * (-CNFAC * fn[jj - 1] + fn[jj]);
      fn_b[jj - 1] -= lam * CNFAC * fc;
      const double g1 = ABAR(r, 1), g2 = ABAR(r, 2);
      fct_b[jj] += g2 * omc * tkif[jj - 1] * rmn - g1 * omc * tkif[jj - 1] * rmn;
      tkif_b[jj - 1] += g2 * omc * fc * rmn - g1 * omc * fc * rmn;
    }
  }
  if (fh != 0.0) {   // surface-water corrections to soil layer 1
    const int jj = 1 + joff;
    const int r = rsw + 1;
    const double fc = fact[jj];
    const double rdh = 1.0 / (0.5 * dz_h2osfc + zz[1 + joff]);
    const double fnh = tkh * (tin[jj] - th0) * rdh;
    const double lam = w[r];
    // x[r] -= fh fc ((hs_soil - dhsdT t1) + CNFAC fnh)
    const double ib = -lam * fh;
    fct_b[jj] += ib * ((hs_soil - dhsdT * tin[jj]) + CNFAC * fnh);
    hs_soil_b += ib * fc;
    dhsdT_b -= ib * fc * tin[jj];
    tin_b[jj] -= ib * fc * dhsdT;
    const double fnh_b = ib * fc * CNFAC;
    tkh_b += fnh_b * (tin[jj] - th0) * rdh;
    tin_b[jj] += fnh_b * tkh * rdh;
    th_b -= fnh_b * tkh * rdh;
    // ab[r][2] += fh (omc fc tkh / dzm + fc dhsdT); ab[r][1] = -fh omc fc tkh / dzm
    const double g2 = ABAR(r, 2), g1 = ABAR(r, 1);
    fct_b[jj] += g2 * fh * (omc * tkh * rdh + dhsdT) - g1 * fh * omc * tkh * rdh;
    tkh_b += g2 * fh * omc * fc * rdh - g1 * fh * omc * fc * rdh;
    dhsdT_b += g2 * fh * fc;
  }
#undef ABAR
  // ---- reverse: fn ----
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    if (j <= nlevgrnd - 1 && fn_b[jj] != 0.0) {
      const double rz = rdzp[jj];
      tkif_b[jj] += fn_b[jj] * (tin[jj + 1] - tin[jj]) * rz;
      const double d_b = fn_b[jj] * tkif[jj] * rz;
      tin_b[jj + 1] += d_b;
      tin_b[jj] -= d_b;
    }
  }
  // ---- reverse: ground heat flux sums ----
  const double e4 = eg * SB * 4.0;
  tgb = dhsdT_b * (-w_set) * (4.0 * eg * SB) * (3.0 * (tg0 * tg0));
  forcb += (hs_soil_b + hs_h2osfc_b) * wb_set + hs_top_b * wb_act;
  tin_b[1 + joff] += hs_soil_b * (-w_set) * e4 * (tin[1 + joff] * tin[1 + joff] * tin[1 + joff]);
  th_b += hs_h2osfc_b * (-w_set) * e4 * (th0 * th0 * th0);
  tin_b[jjtop] += hs_top_b * (-w_act) * e4 * (tin[jjtop] * tin[jjtop] * tin[jjtop]);
  // ---- reverse: fact (through cv) ----
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    liq_in_b[jj] += fct_b[jj] * cl[jj];
    ice_in_b[jj] += fct_b[jj] * ci[jj];
    if (j >= 1) wsb[j] += fct_b[jj] * cw[jj];
  }
  // ---- reverse: interface conductivity, tk_h2osfc, layer conductivity ----
  double thk_b[MAXL + 2];
  for (int jj = jjtop; jj <= nw; jj++) thk_b[jj] = 0.0;
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    if (j <= nlevgrnd - 1) {
      thk_b[jj] += tkif_b[jj] * da[jj];
      thk_b[jj + 1] += tkif_b[jj] * db[jj];
    }
  }
  thk_b[1 + joff] += tkh_b * dtkh;
  for (int jj = jjtop; jj <= nw; jj++) {
    const int j = jj - nlevsno;
    liq_in_b[jj] += thk_b[jj] * tl[jj];
    ice_in_b[jj] += thk_b[jj] * ti[jj];
    if (j >= 1) wsb[j] += thk_b[jj] * tw[jj];
  }
  // ---- adjoints of the inputs ----
  for (int jj = jjtop; jj <= nw; jj++) {
    Tb[jj] = tin_b[jj];
    liqb[jj] = liq_in_b[jj];
    iceb[jj] = ice_in_b[jj];
  }
  thb = th_b;
}

// ---------------------------------------------------------------------------
// The kernel: one thread per column, columns handed out by a work counter.
// ---------------------------------------------------------------------------
struct CfSub {
  double* sub;
  int maxsub;
  int64_t slots;
};

__device__ __forceinline__ double& cf_sub(const CfSub& S, int64_t slot, int sidx, int j) {
  return S.sub[((slot >> 5) * ((int64_t)S.maxsub * SUB_REC) + (int64_t)sidx * SUB_REC + j) * 32 + (slot & 31)];
}

// 8 blocks of 64 per SM (128 registers): 1,216 resident blocks, so each thread of a
// 65,536-column launch takes one column and no second round of columns trails the
// first (6 blocks at the 168 registers the compiler chose otherwise)
__global__ void __launch_bounds__(CF_BLOCK, 8)
k_column_step_vjp_cf(Dims D, int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw, clmgb_swm_config cfg,
                     double dtime, int snow_method, double* t_ssbef, double* t_h2osfc_bef, clmgb_step_adjoint adj,
                     CfSub S, SubstepLogView lg, unsigned long long* queue, const uint32_t* order,
                     uint32_t* col_status, uint32_t* dev_status) {
  const int64_t ld = D.ldc;
  const int nlevsno = D.nlevsno, nlevgrnd = D.nlevgrnd, nlevsoi = D.nlevsoi;
  const int nlev = nlevsno + D.nlevmax;
  const int nw = nlevsno + nlevgrnd;
  const int joff = nlevsno;
  const int64_t slot = (int64_t)blockIdx.x * CF_BLOCK + threadIdx.x;
  const double LN10 = cm_log(10.0);
  CfBand band;
  for (;;) {
    const int64_t k = (int64_t)atomicAdd(queue, 1ULL);
    if (k >= nc) break;
    const int64_t c = order ? (int64_t)order[k] : k;
    const bool do_t = ft.mask_nolakec[c] != 0, do_w = fw.mask_hydrology[c] != 0;
    if (!do_t && !do_w) {     // the step leaves the column alone: identity
      if (col_status) col_status[c] = 0;
      continue;
    }
    uint32_t st = 0;
    const int64_t snl = ft.col_snl[c];
    if (snl > 0 || snl < -nlevsno) {
      st = CLMGB_COL_LEVEL_RANGE;
      if (col_status) col_status[c] = st;
      if (dev_status) atomicOr(dev_status, st);
      continue;
    }
    const int jjtop = (int)snl + 1 + nlevsno;
    if (ft.frac_h2osfc[c] > 0.0 || ft.h2osno_no_layers[c] > 0.0) st |= CLMGB_COL_ADJ_UNSUPPORTED;
    for (int j = 1; j <= nlevgrnd; j++)
      if (LV(ft.excess_ice, c, j, ld) != 0.0) st |= CLMGB_COL_ADJ_UNSUPPORTED;
    // ---- load the state, keep the inputs ----
    CfState V;
    V.c = c;
    V.ld = ld;
    V.ws = fw.watsat;
    V.bs = fw.bsw;
    V.suc = fw.sucsat;
    V.ks = fw.hksat;
    V.band = &band;
    band.n = 0;
    double tin[MAXL + 2], liq0[MAXL + 2], ice0[MAXL + 2];
    for (int jj = 1; jj <= nlev; jj++) {
      V.t[jj] = LV(ft.t_soisno, c, jj, ld);
      V.liq[jj] = LV(ft.h2osoi_liq, c, jj, ld);
      V.ice[jj] = LV(ft.h2osoi_ice, c, jj, ld);
      tin[jj] = V.t[jj];
      liq0[jj] = V.liq[jj];
      ice0[jj] = V.ice[jj];
    }
    for (int jj = 1; jj <= nw; jj++) V.fact[jj] = LV(ft.fact, c, jj, ld);
    for (int j = 1; j <= nlevsoi; j++) V.icefrac[j] = LV(fw.icefrac, c, j, ld);
    V.tg = ft.t_grnd[c];
    V.th = ft.t_h2osfc[c];
    V.forc = ft.forc_lwrad[c];
    V.qc = fw.qcharge[c];
    const double tg0 = V.tg, th0 = V.th;
    // ---- soil_temperature!: run here, or its record read from the log ----
    bool st_full = false;
    if (do_t) {
      if (t_ssbef)
        for (int jj = 1; jj <= nlev; jj++) LV(t_ssbef, c, jj, ld) = V.t[jj];
      if (t_h2osfc_bef) t_h2osfc_bef[c] = V.th;
      uint32_t s1;
      if (lg.st) {
        const double* rec = lg.st + c * (int64_t)CLMGB_LOG_ST_STRIDE;
        s1 = (uint32_t)rec[ST_STATUS];
        band.n = (int)rec[ST_N];
        band.lu = rec + ST_LU;
        band.x = rec + ST_X;
        band.piv = reinterpret_cast<const uint8_t*>(rec + ST_PIV);
        for (int jj = jjtop; jj <= nlev; jj++) V.t[jj] = rec[ST_T + jj - 1];
        for (int jj = jjtop; jj <= nw; jj++) {
          V.liq[jj] = rec[ST_LIQ + jj - 1];
          V.ice[jj] = rec[ST_ICE + jj - 1];
          V.fact[jj] = rec[ST_FACT + jj - 1];
        }
        V.tg = rec[ST_TG];
        V.th = rec[ST_TH];
      } else {
        s1 = soil_temperature_col(D, ft, c, dtime, snow_method, V);
      }
      st |= s1;
      st_full = !(s1 & (CLMGB_COL_URBAN | CLMGB_COL_PATCH_RANGE | CLMGB_COL_LEVEL_RANGE)) && band.n > 0;
    }
    // ---- set_soil_water_fractions! and soil_water! ----
    MfLane L;
    bool rich = false;
    int nacc = 0;
    const double* logc = nullptr;     // this column's log region, when it holds the solve
    if (do_w) {
      water_fractions_col(D, fw, c, V);
      rich = mf_begin(L, D, fw, cfg, dtime, c, V);
      if (!rich) {
        st |= L.status;
      } else {
        const int32_t cnt = lg.rec ? lg.count[c] : -1;
        if (cnt >= 0 && cnt <= lg.cap) {
          logc = lg.rec + c * lg.stride;
          nacc = cnt;
          const double* fin = logc + (int64_t)lg.cap * SUB_REC;
          uint32_t rs = (uint32_t)fin[3 * MAXSOI + 2];
          for (int j = 1; j <= L.nlayers; j++) {
            V.liq[joff + j] = fin[j - 1];
            LV(fw.smp_l, c, j, ld) = fin[MAXSOI + j - 1];
            LV(fw.hk_l, c, j, ld) = fin[2 * MAXSOI + j - 1];
          }
          V.qc = fin[3 * MAXSOI];
          fw.num_substeps[c] = fin[3 * MAXSOI + 1];
          st |= rs;
        } else {
          bool done = false;
          while (!done) {
            if (L.fresh && nacc < S.maxsub)
              for (int j = 1; j <= L.nlayers; j++) cf_sub(S, slot, nacc, j - 1) = L.liq[j];
            const double dts = L.dtsub, dtd = L.dtdone;
            done = mf_attempt(L, D, fw, cfg, dtime, V);
            if (L.dtdone != dtd) {
              if (nacc < S.maxsub) {
                cf_sub(S, slot, nacc, MAXSOI) = dts;
                cf_sub(S, slot, nacc, MAXSOI + 1) = dtd;
              }
              nacc++;
            }
          }
          st |= mf_end(L, D, fw, V);
          if (nacc > S.maxsub) st |= CLMGB_COL_TAPE_FULL;
        }
      }
    }
    // ---- the final forward state ----
    for (int jj = jjtop; jj <= nlev; jj++) LV(ft.t_soisno, c, jj, ld) = V.t[jj];
    for (int jj = jjtop; jj <= nw; jj++) {
      LV(ft.h2osoi_liq, c, jj, ld) = V.liq[jj];
      LV(ft.h2osoi_ice, c, jj, ld) = V.ice[jj];
      if (do_t) LV(ft.fact, c, jj, ld) = V.fact[jj];
    }
    if (do_w)
      for (int j = 1; j <= nlevsoi; j++) LV(fw.icefrac, c, j, ld) = V.icefrac[j];
    ft.t_grnd[c] = V.tg;
    ft.t_h2osfc[c] = V.th;
    if (do_w) fw.qcharge[c] = V.qc;

    if (!(st & CLMGB_COL_TAPE_FULL)) {
      // ---- seeds: the adjoints of the step's outputs ----
      double Tb[MAXL + 2], liqb[MAXL + 2], iceb[MAXL + 2];
      for (int jj = jjtop; jj <= nw; jj++) {
        Tb[jj] = LV(adj.lam_t_soisno, c, jj, ld);
        liqb[jj] = LV(adj.lam_h2osoi_liq, c, jj, ld);
        iceb[jj] = LV(adj.lam_h2osoi_ice, c, jj, ld);
      }
      double tgb = adj.lam_t_grnd[c], thb = adj.lam_t_h2osfc[c], forcb = 0.0;
      double wsb[MAXGRND + 2], bsb[MAXGRND + 2], sucb[MAXGRND + 2], ksb[MAXSOI + 2];
      for (int j = 1; j <= nlevgrnd; j++) {
        wsb[j] = 0.0;
        bsb[j] = 0.0;
        sucb[j] = 0.0;
      }
      for (int j = 1; j <= nlevsoi; j++) ksb[j] = 0.0;
      // ---- the substeps in reverse ----
      if (rich) {
        const int nl = L.nlayers;
        const double lamQ = adj.lam_qcharge && !qcharge_replaced(D, fw, cfg, c) ? adj.lam_qcharge[c] : 0.0;
        double lamL[MAXSOI + 1], liqs[MAXSOI + 1];
        double wsv[MAXSOI + 2], bbv[MAXSOI + 2], sucv[MAXSOI + 2], ksv[MAXSOI + 2];
        RichardsBar RB;
        for (int j = 1; j <= nl; j++) {
          lamL[j] = liqb[joff + j];
          RB.ws[j] = 0.0; RB.b[j] = 0.0; RB.suc[j] = 0.0; RB.ks[j] = 0.0; RB.imp[j] = 0.0;
          wsv[j] = LV(fw.watsat, c, j, ld);
          bbv[j] = LV(fw.bsw, c, j, ld);
          sucv[j] = LV(fw.sucsat, c, j, ld);
          ksv[j] = LV(fw.hksat, c, j, ld);
        }
        for (int sidx = nacc - 1; sidx >= 0; sidx--) {
          double dts;
          if (logc) {
            const double* rec = logc + (int64_t)sidx * SUB_REC;
            for (int j = 1; j <= nl; j++) liqs[j] = rec[j - 1];
            dts = rec[MAXSOI];
          } else {
            for (int j = 1; j <= nl; j++) liqs[j] = cf_sub(S, slot, sidx, j - 1);
            dts = cf_sub(S, slot, sidx, MAXSOI);
          }
          mf_substep_reverse(D, fw, cfg, dtime, c, nl, L.dzv, L.imp, wsv, bbv, sucv, ksv, dts, liqs, lamL, lamQ, RB);
        }
        for (int j = 1; j <= nl; j++) {
          liqb[joff + j] = lamL[j];
          wsb[j] += RB.ws[j];
          bsb[j] += RB.b[j];
          sucb[j] += RB.suc[j];
          ksb[j] += RB.ks[j];
        }
        // ice impedance 10^(-e_ice icef) and set_soil_water_fractions!
        double icefb[MAXSOI + 2];
        for (int j = 1; j <= nl + 1; j++) icefb[j] = 0.0;
        for (int j = 1; j <= nl; j++) {
          const double ib = -cfg.e_ice * (RB.imp[j] * L.imp[j] * LN10);
          if (j == nl) {
            icefb[j] += ib;
          } else {
            icefb[j] += 0.5 * ib;
            icefb[j + 1] += 0.5 * ib;
          }
        }
        for (int j = 1; j <= nl; j++) {
          if (icefb[j] == 0.0) continue;
          const double exi = LV(ft.excess_ice, c, j, ld);
          const double dz_ext = LVc(fw.dz, c, j + joff, ld) + jl_div(exi, DENICE);
          const double ws = wsv[j];
          const double y = jl_div(V.ice[j + joff] + exi, dz_ext * DENICE);
          const double vol_ice = jl_min(ws, y);
          const double v = jl_div(vol_ice, ws);
          const double icef = jl_min(1.0, v);
          if (same_bits(icef, 1.0)) continue;
          wsb[j] -= icefb[j] * v / ws;
          const double vb = icefb[j] / ws;
          if (same_bits(vol_ice, ws)) wsb[j] += vb;
          else iceb[j + joff] += vb / (dz_ext * DENICE);
        }
      }
      // ---- soil_temperature! in reverse ----
      if (st_full)
        soil_temperature_reverse(D, ft, fw, c, dtime, snow_method, V.fact, tin, liq0, ice0, tg0, th0, V.forc, band,
                                 Tb, liqb, iceb, tgb, thb, forcb, wsb, bsb, sucb);
      // ---- adjoints of the step's inputs ----
      for (int jj = jjtop; jj <= nw; jj++) {
        LV(adj.lam_t_soisno, c, jj, ld) = Tb[jj];
        LV(adj.lam_h2osoi_liq, c, jj, ld) = liqb[jj];
        LV(adj.lam_h2osoi_ice, c, jj, ld) = iceb[jj];
      }
      adj.lam_t_grnd[c] = tgb;
      adj.lam_t_h2osfc[c] = thb;
      if (adj.lam_forc_lwrad) adj.lam_forc_lwrad[c] = forcb;
      for (int j = 1; j <= nlevsoi; j++) {
        if (adj.grad_watsat) LV(adj.grad_watsat, c, j, ld) += wsb[j];
        if (adj.grad_bsw) LV(adj.grad_bsw, c, j, ld) += bsb[j];
        if (adj.grad_sucsat) LV(adj.grad_sucsat, c, j, ld) += sucb[j];
        if (adj.grad_hksat) LV(adj.grad_hksat, c, j, ld) += ksb[j];
      }
    }
    if (col_status) col_status[c] = st;
    if (st && dev_status) atomicOr(dev_status, st);
  }
}

// Work order of the adjoint: the 32 columns a warp runs side by side should take
// the same paths, so columns are handed out sorted (counting sort, descending) on
// a key of the Richards work (accepted substeps from the log, else the previous
// call's attempt count) and the number of snow layers.  Columns the step leaves
// alone sort last.  The order does not change any result.
constexpr int VJP_BINS = 64;
__device__ __forceinline__ int vjp_key(const clmgb_soiltemp_fields& ft, const clmgb_soilwater_fields& fw,
                                       const SubstepLogView& lg, int64_t c) {
  if (!ft.mask_nolakec[c] && !fw.mask_hydrology[c]) return 0;
  int a;
  if (lg.rec) {
    const int32_t n = lg.count[c];
    a = n < 0 ? 0 : (n > lg.cap ? 15 : n);
  } else {
    const double ns = fw.num_substeps[c];
    a = ns > 0.0 ? (ns >= 15.0 ? 15 : (int)ns) : 0;
  }
  if (a > 15) a = 15;
  const int64_t snl = ft.col_snl[c];
  int sb = (int)((-snl + 3) / 4);
  sb = sb < 0 ? 0 : (sb > 3 ? 3 : sb);
  return a * 4 + sb;
}
__global__ void k_vjp_hist(int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw, SubstepLogView lg,
                           unsigned int* bins) {
  __shared__ unsigned int sh[VJP_BINS];
  for (int i = threadIdx.x; i < VJP_BINS; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nc) atomicAdd(&sh[vjp_key(ft, fw, lg, c)], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < VJP_BINS; i += blockDim.x)
    if (sh[i]) atomicAdd(&bins[i], sh[i]);
}
__global__ void k_vjp_scan(unsigned int* bins) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned int run = 0;
  for (int b = VJP_BINS - 1; b >= 0; b--) {
    bins[VJP_BINS + b] = run;
    run += bins[b];
  }
}
__global__ void k_vjp_scatter(int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw, SubstepLogView lg,
                              unsigned int* bins, uint32_t* order) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const unsigned int pos = atomicAdd(&bins[VJP_BINS + vjp_key(ft, fw, lg, c)], 1u);
  order[pos] = (uint32_t)c;
}

int vjp_cf_blocks_per_sm() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_column_step_vjp_cf, CF_BLOCK, 0) != cudaSuccess) nb = 1;
  return nb > 0 ? nb : 1;
}

cudaError_t launch_column_step_vjp_cf(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                      const clmgb_soilwater_fields& fw, const clmgb_swm_config& cfg, double dtime,
                                      int snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                      const clmgb_step_adjoint& adj, const AdjTape& tp, const SubstepLogView& lg,
                                      const QueueScratch& qs, unsigned long long* queue, int grid_blocks,
                                      uint32_t* col_status, uint32_t* dev_status, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const uint32_t* order = nullptr;
  if (qs.capacity >= nc && qs.order && qs.bins && nc < (int64_t)0xffffffffLL) {
    const unsigned g = (unsigned)((nc + 127) / 128);
    if ((e = cudaMemsetAsync(qs.bins, 0, 2 * VJP_BINS * sizeof(unsigned int), s)) != cudaSuccess) return e;
    k_vjp_hist<<<g, 128, 0, s>>>(nc, ft, fw, lg, qs.bins);
    k_vjp_scan<<<1, 32, 0, s>>>(qs.bins);
    k_vjp_scatter<<<g, 128, 0, s>>>(nc, ft, fw, lg, qs.bins, qs.order);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    order = qs.order;
  }
  int64_t blocks = grid_blocks;
  const int64_t max_blocks = tp.slots / CF_BLOCK;
  if (blocks > max_blocks) blocks = max_blocks;
  const int64_t need = (nc + CF_BLOCK - 1) / CF_BLOCK;
  if (blocks > need) blocks = need;
  if (blocks < 1) return cudaErrorInvalidValue;
  CfSub S{tp.sub, (int)tp.maxsub, tp.slots};
  k_column_step_vjp_cf<<<(unsigned int)blocks, CF_BLOCK, 0, s>>>(D, nc, ft, fw, cfg, dtime, snow_method, t_ssbef,
                                                                 t_h2osfc_bef, adj, S, lg, queue, order,
                                                                 col_status, dev_status);
  return cudaGetLastError();
}

}  // namespace clmgb
