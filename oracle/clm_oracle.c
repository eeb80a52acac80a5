/*
 * clm_oracle.c — TEST INFRASTRUCTURE ONLY: the CPU oracle (parity checker) and the
 * timed CPU baseline for the soil/snow column solve.  Nothing in the product links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs do.
 *
 * A plain-C restatement of CLM.jl's Float64 CPU path, kernel by kernel, in the
 * reference's own operation order (compiled with -ffp-contract=off so no a*b+c is
 * fused, as Julia does not fuse without muladd):
 *   soil_temperature!            src/biogeophys/soil_temperature.jl:358-593
 *     _soil_snow_tk_kernel!      :647-716      _soil_tk_interface_kernel! :599-629
 *     _tk_h2osfc_kernel!         :762-776      _soil_cv_kernel!           :781-813
 *     _unresolved_snow_cv_kernel!:842-850      _snow_cv_kernel!           :855-869
 *     _ground_lwrad_emit_kernel! :946-960      _gnet_patch_rural*_kernel! :1003-1044
 *     scatter_add_1d!            src/infrastructure/kernels.jl:166-170
 *     _gnet_snicar_kernel!       :1139-1167    _heat_diff_kernel!         :1271-1319
 *     _h2osfc_thermprop_kernel!  :116-130      set_rhs_vec! kernels       :1365-1542
 *     set_matrix! kernels        :1549-1748    _tvector_init/extract      :133-167
 *     _batched_band_solve_kernel! src/infrastructure/band_diagonal.jl:87-170 (dense GE)
 *     _fn1_kernel!               :170-206      _phase_change_h2osfc_kernel! :1757-1855
 *     _phase_change_beta_kernel! :1929-2230    _tgrnd_kernel!             :224-247
 *     _eflx_fgr_kernel!          :250-269
 *   _soilhyd_water_fractions_kernel!  src/biogeophys/soil_hydrology.jl:110-130
 *   soil_fluxes!                      src/biogeophys/soil_fluxes.jl:19-697
 *   soilwater_zengdecker2009!         src/biogeophys/soil_water_movement.jl:97-635,1616-1764
 *   compute_effec_rootfrac_and_vert_tran_sink!  src/biogeophys/soil_water_plant_sink.jl:48-78,
 *                                     :210-245, :341-451
 *   _soilwm_moisture_form_kernel!     src/biogeophys/soil_water_movement.jl:1250-1489
 *   compute_qcharge! after it         src/biogeophys/soil_water_movement.jl:1153-1215,1575-1598
 *   soil_water!'s use_flexibleCN step src/biogeophys/soil_water_movement.jl:1812-1843
 *   tridiagonal_solve! / _tridiag_multi_kernel!  src/infrastructure/tridiagonal.jl:35-127
 *   tridiagonal_col!                  src/biogeophys/soil_water_movement.jl:736-773
 *   init_soil_properties!             src/infrastructure/cold_start.jl:225-391
 *
 *   surface hydrology (clm_driver.jl:1938-2007), routine by routine:
 *     set_floodc!                     src/biogeophys/soil_hydrology.jl:139-152
 *     saturated_excess_runoff!        src/biogeophys/sat_excess_runoff.jl:246-300,329-365
 *     set_qflx_inputs!                src/biogeophys/soil_hydrology.jl:160-187
 *     infiltration_excess_runoff!     src/biogeophys/infilt_excess_runoff.jl:142-211,241-274
 *     route_infiltration_excess!      src/biogeophys/soil_hydrology.jl:199-225
 *     update_h2osfc!                  src/biogeophys/surface_water.jl:279-520
 *     infiltration!                   src/biogeophys/soil_hydrology.jl:236-243
 *     total_surface_runoff!           src/biogeophys/soil_hydrology.jl:250-301,567-604
 *     update_urban_ponding!           src/biogeophys/soil_hydrology.jl:316-338
 *   snow layer dynamics (clm_driver.jl:2146-2200), routine by routine:
 *     snow_compaction!                src/biogeophys/snow_hydrology.jl:1203-1326,1412-1500
 *     combine_snow_layers!, combo     :1584-1874, :1960-2000
 *     divide_snow_layers!             :2021-2031, :2057-2237
 *     zero_empty_snow_layers!         :2314-2329
 *     build_snow_filter!              :2488-2510
 *   lake_temperature!                 src/biogeophys/lake_temperature.jl:39-1295, kernel by kernel
 *   balance_check! column checks      src/biogeophys/balance_check.jl:723-770, 1124-1160, 1347-1365
 *
 * Transcendentals: the reference uses Julia Base's exp/log/pow/sin (openlibm for
 * log10); this file and the CUDA kernels share clm_math.h's binary64 versions, which
 * are within ~1 ulp of those, so parity at the 1e-10 level is unaffected; decisions
 * that sit within an ulp of a threshold can flip.
 * Integer powers follow Julia's literal_pow: x^2 = x*x, x^3 = x*x*x, and x^4 uses
 * Base.Math.pow_body's compensated squaring (Julia >= 1.10, Project.toml compat).
 * smooth_min/smooth_max are exact min/max for Float64 (smooth_ad.jl:91-149), with
 * Julia's NaN-propagating min/max semantics.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/clmgb.h"
/* Transcendentals: the same table-driven binary64 log/exp/pow as the CUDA kernels
 * (published method, see clm_math.h), so the oracle and the GPU round identically. */
#include "../clm.jl_gb300/csrc/clm_math.h"

/* ---- sensitivity hook (test infrastructure): perturbs the results of the hot path's
 * pow and log10 calls for oracle/perturb_experiment.py, which measures how far one
 * ulp in those functions moves the path's results.  Off (mode 0) unless
 * orc_set_perturbation selects a mode:
 *   1: every result moved by +-1 ulp;
 *   2: a fraction `frac` of the results moved by +-1 ulp (the rate at which two nearly
 *      correctly rounded implementations, such as this one and Julia's, disagree);
 *   3: the results of the previous, single-precision-logarithm library:
 *      exp(y*log(x)) and log(x)/ln(10) in binary64 (errors up to |y log x| ulp).
 * Which results move, and in which direction, is a hash of the arguments, so runs are
 * reproducible whatever the thread schedule. ---- */
static int g_perturb_mode = 0;
static double g_perturb_frac = 0.0;
static unsigned long long g_perturb_salt = 0;
void orc_set_perturbation(int32_t mode, double frac, uint64_t salt)
{
  g_perturb_mode = mode;
  g_perturb_frac = frac;
  g_perturb_salt = salt;
}
static uint64_t perturb_hash(double x, double y)
{
  uint64_t z = cm_as_u64_(x) ^ ((cm_as_u64_(y) << 17) | (cm_as_u64_(y) >> 47)) ^ g_perturb_salt;
  z += 0x9e3779b97f4a7c15ULL;                       /* splitmix64 finaliser */
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static double perturb(double v, double x, double y)
{
  if (!isfinite(v) || v == 0.0) return v;
  const uint64_t h = perturb_hash(x, y);
  if (g_perturb_mode == 2 && (double)(h >> 11) * 0x1p-53 >= g_perturb_frac) return v;
  const uint64_t b = cm_as_u64_(v);
  return cm_as_f64_((h & 1) ? b + 1 : b - 1);
}
static double o_pow(double x, double y)
{
  if (g_perturb_mode == 3) {
    if (x > 0.0 && isfinite(x) && x != 1.0 && y != 0.0 && isfinite(y)) return cm_exp(y * cm_log(x));
    return cm_pow(x, y);
  }
  const double v = cm_pow(x, y);
  return g_perturb_mode ? perturb(v, x, y) : v;
}
static double o_log10(double x)
{
  if (g_perturb_mode == 3) return (x > 0.0 && isfinite(x)) ? cm_log(x) * CM_INVLN10 : cm_log10(x);
  const double v = cm_log10(x);
  return g_perturb_mode ? perturb(v, x, 10.0) : v;
}

/* ---- constants: src/constants/varcon.jl:15-70 ---- */
#define GRAV   9.80616
#define SB     5.67e-8
#define CPLIQ  4188.0
#define CPICE  2117.27
#define HFUS   3.337e5
#define DENH2O 1000.0
#define DENICE 917.0
#define TFRZ   273.15
#define TKAIR  0.023
#define TKICE  2.290
#define TKWAT  0.57
#define CAPR   0.34
#define CNFAC  0.5
#define THK_BEDROCK  3.0
#define CSOL_BEDROCK 2.0e6
#define THIN_SFCLAYER 1.0e-6
#define M_TO_MM 1.0e3
/* landunit / column types: src/constants/landunit_varcon.jl, column_varcon.jl */
#define ISTSOIL 1
#define ISTCROP 2
#define ISTICE  4
#define ISTWET  6
#define ICOL_ROOF 71
#define ICOL_SUNWALL 72
#define ICOL_SHADEWALL 73
#define ICOL_ROAD_IMPERV 74
#define ICOL_ROAD_PERV 75

#define ORC_MAXL 80          /* any CLM level structure (49SL_10m: 12+54) */

/* Julia Base.max / Base.min on Float64: NaN propagates, -0.0 < 0.0. */
static inline double jl_max(double x, double y) {
  if (x != x) return x;
  if (y != y) return y;
  if (x > y) return x;
  if (y > x) return y;
  return signbit(x) ? y : x;
}
static inline double jl_min(double x, double y) {
  if (x != x) return x;
  if (y != y) return y;
  if (x < y) return x;
  if (y < x) return y;
  return signbit(x) ? x : y;
}
/* Julia x^4 for Float64: Base.Math.pow_body(x, 4) — compensated power by squaring. */
static inline double jl_pow4(double x) {
  double xnlo = 0.0, err, x2, x4, lo;
  err = x * 2.0 * xnlo;                 /* n = 4: no odd bit */
  x2 = x * x; xnlo = fma(x, x, -x2); xnlo += err;
  err = x2 * 2.0 * xnlo;                /* n = 2 */
  x4 = x2 * x2; lo = fma(x2, x2, -x4); xnlo = lo + err;
  err = xnlo;                           /* muladd(1.0, xnlo, x4*0.0) */
  if (isfinite(x4) && isfinite(err)) return x4 + err;  /* muladd(x4, 1.0, err) */
  return x4;
}

#define IX(p, c, jj, ld) ((p)[(int64_t)(c) + ((int64_t)(jj) - 1) * (int64_t)(ld)])

/* ===================================================================== */
/* Dense pivoted Gaussian elimination — _batched_band_solve_kernel!       */
/* band_diagonal.jl:87-170, one column.  A is n x n row-major scratch.    */
/* ===================================================================== */
static void dense_band_solve_col(double* tvector_col /* 1-based via offset */, int64_t ldt,
                                 const double* bmatrix, int64_t ldb, int nlev,
                                 const double* rvector, int64_t ldr, int64_t c,
                                 int jt, int n, int kl, int ku)
{
  double A[ORC_MAXL * ORC_MAXL];
  double x[ORC_MAXL];
  const int nband = kl + ku + 1;
  (void)nband;
  for (int j = 1; j <= n; j++)
    for (int i = 1; i <= n; i++) A[(i - 1) * n + (j - 1)] = 0.0;
  for (int j = 1; j <= n; j++) {
    int ilo = j - kl > 1 ? j - kl : 1;
    int ihi = j + ku < n ? j + ku : n;
    for (int i = ilo; i <= ihi; i++) {
      int band = (i - j) + kl + 1;              /* 1-based band */
      int lev = jt + i - 1;                     /* 1-based level */
      A[(i - 1) * n + (j - 1)] = bmatrix[c + (int64_t)(band - 1) * ldb + (int64_t)(lev - 1) * ldb * (kl + ku + 1)];
    }
  }
  for (int i = 1; i <= n; i++) x[i - 1] = rvector[c + (int64_t)(jt + i - 2) * ldr];
#define AA(i, j) A[((i) - 1) * n + ((j) - 1)]
  for (int k = 1; k <= n - 1; k++) {
    int piv = k;
    double maxv = fabs(AA(k, k));
    for (int i = k + 1; i <= n; i++) {
      double v = fabs(AA(i, k));
      if (v > maxv) { maxv = v; piv = i; }
    }
    double akk = AA(piv, k);
    if (piv != k) {
      for (int j = k; j <= n; j++) {
        double akj = AA(k, j), apj = AA(piv, j);
        AA(k, j) = apj; AA(piv, j) = akj;
      }
      double xk = x[k - 1], xp = x[piv - 1];
      x[k - 1] = xp; x[piv - 1] = xk;
    }
    for (int i = k + 1; i <= n; i++) {
      double f = AA(i, k) / akk;
      for (int j = k; j <= n; j++) AA(i, j) = AA(i, j) - f * AA(k, j);
      x[i - 1] = x[i - 1] - f * x[k - 1];
    }
  }
  for (int i = n; i >= 1; i--) {
    double s = x[i - 1];
    for (int j = i + 1; j <= n; j++) s = s - AA(i, j) * x[j - 1];
    x[i - 1] = s / AA(i, i);
  }
#undef AA
  for (int i = 1; i <= n; i++) tvector_col[c + (int64_t)(jt + i - 2) * ldt] = x[i - 1];
  (void)nlev;
}

/* batched_band_solve! (band_diagonal.jl:179-189). bmatrix [ld, nband, nlev]. */
int orc_batched_band_solve(int64_t nc, int64_t ld, int32_t nlev, double* tvector,
                           const double* bmatrix, const double* rvector,
                           const int64_t* jtop, const int64_t* jbot, const uint8_t* mask,
                           int32_t kl, int32_t ku, int32_t nlevsno_off, int32_t nthreads)
{
  if (nlev > ORC_MAXL) return CLMGB_ERR_DIMS;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t c = 0; c < nc; c++) {
    if (!mask[c]) continue;
    int jt = (int)(jtop[c] + nlevsno_off + 1);
    int n = (int)(jbot[c] - jtop[c] + 1);
    if (n > 0) dense_band_solve_col(tvector, ld, bmatrix, ld, nlev, rvector, ld, c, jt, n, kl, ku);
  }
  return 0;
}

/* tridiagonal_solve! (tridiagonal.jl:35-63), single column, no pivot guard. */
void orc_tridiagonal_solve(double* u, const double* a, const double* b, const double* c,
                           const double* r, int32_t jtop, int32_t nlevs)
{
  double cp[ORC_MAXL + 1], dp[ORC_MAXL + 1];
  int j = jtop;
  cp[j] = c[j - 1] / b[j - 1];
  dp[j] = r[j - 1] / b[j - 1];
  for (int jj = j + 1; jj <= nlevs; jj++) {
    double denom = b[jj - 1] - a[jj - 1] * cp[jj - 1];
    cp[jj] = c[jj - 1] / denom;
    dp[jj] = (r[jj - 1] - a[jj - 1] * dp[jj - 1]) / denom;
  }
  u[nlevs - 1] = dp[nlevs];
  for (int jj = nlevs - 1; jj >= j; jj--) u[jj - 1] = dp[jj] - cp[jj] * u[jj];
}

/* _tridiag_multi_kernel! (tridiagonal.jl:86-127): [ld, nlevs] matrices, 1e-30 guard. */
int orc_tridiagonal_multi(int64_t ncols, int64_t ld, int32_t nlevs, double* u,
                          const double* a, const double* b, const double* c, const double* r,
                          const int64_t* jtop, const uint8_t* mask, int32_t nthreads)
{
  if (nlevs > ORC_MAXL) return CLMGB_ERR_DIMS;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t col = 0; col < ncols; col++) {
    if (!mask[col]) continue;
    double cpv[ORC_MAXL + 1], dpv[ORC_MAXL + 1];
    int j = (int)jtop[col];
    const double tiny = 1e-30;
    double bet = IX(b, col, j, ld);
    if (fabs(bet) < tiny) bet = tiny;
    double cp_prev = IX(c, col, j, ld) / bet;
    double dp_prev = IX(r, col, j, ld) / bet;
    cpv[j] = cp_prev; dpv[j] = dp_prev;
    for (int jj = j + 1; jj <= nlevs; jj++) {
      double denom = IX(b, col, jj, ld) - IX(a, col, jj, ld) * cp_prev;
      if (fabs(denom) < tiny) denom = copysign(tiny, denom == 0.0 ? 1.0 : denom);
      cp_prev = IX(c, col, jj, ld) / denom;
      dp_prev = (IX(r, col, jj, ld) - IX(a, col, jj, ld) * dp_prev) / denom;
      cpv[jj] = cp_prev; dpv[jj] = dp_prev;
    }
    double u_next = dp_prev;
    IX(u, col, nlevs, ld) = u_next;
    for (int jj = nlevs - 1; jj >= j; jj--) {
      u_next = dpv[jj] - cpv[jj] * u_next;
      IX(u, col, jj, ld) = u_next;
    }
  }
  return 0;
}

/* tridiagonal_col! (soil_water_movement.jl:736-773), gam form, 1-based arrays via lbj. */
void orc_tridiagonal_col(double* u, const double* a, const double* b, const double* c,
                         const double* r, int32_t jtop, int32_t lbj, int32_t ubj)
{
  double gam[ORC_MAXL + 2];
  for (int j = 0; j < ORC_MAXL + 2; j++) gam[j] = 0.0;
#define V(arr, j) arr[(j) - lbj]
  double bet = V(b, jtop);
  if (fabs(bet) < 1.0e-30) bet = 1.0e-30;
  for (int j = lbj; j <= ubj; j++) {
    if (j >= jtop) {
      if (j == jtop) {
        V(u, j) = V(r, j) / bet;
      } else {
        gam[j - lbj] = V(c, j - 1) / bet;
        bet = V(b, j) - V(a, j) * gam[j - lbj];
        if (fabs(bet) < 1.0e-30) bet = copysign(1.0e-30, bet == 0.0 ? 1.0 : bet);
        V(u, j) = (V(r, j) - V(a, j) * V(u, j - 1)) / bet;
      }
    }
  }
  for (int j = ubj - 1; j >= lbj; j--)
    if (j >= jtop) V(u, j) = V(u, j) - gam[j + 1 - lbj] * V(u, j + 1);
#undef V
}

/* ===================================================================== */
/* Reverse-mode rules of the linear solves (enzyme_rules.jl)             */
/* ===================================================================== */

/* tridiagonal_solve! reverse rule (enzyme_rules.jl:160-201), arrays 1-based through
 * 0-based pointers: lambda = A^-T ubar, solved with tridiagonal_solve! on the
 * transposed bands over jtop..n (sub = c[j-1], diag = b[j], super = a[j+1]);
 * rbar += lambda; bbar -= lambda*u; abar[j] -= lambda[j]*u[j-1] for j > jtop;
 * cbar[j] -= lambda[j]*u[j+1] for j < n; ubar[jtop..n] is consumed (set to 0).
 * abar, bbar, cbar, rbar may be NULL (inactive arguments). */
void orc_tridiagonal_adjoint(const double* u, const double* a, const double* b, const double* c,
                             double* ubar, double* abar, double* bbar, double* cbar, double* rbar,
                             int32_t jtop, int32_t n)
{
  double aT[ORC_MAXL], bT[ORC_MAXL], cT[ORC_MAXL], rT[ORC_MAXL], lam[ORC_MAXL];
  for (int j = 1; j <= n; j++) {
    aT[j - 1] = 0.0; bT[j - 1] = 0.0; cT[j - 1] = 0.0; rT[j - 1] = 0.0; lam[j - 1] = 0.0;
  }
  for (int j = jtop; j <= n; j++) {
    bT[j - 1] = b[j - 1];
    rT[j - 1] = ubar[j - 1];
    if (j > jtop) aT[j - 1] = c[j - 2];
    if (j < n) cT[j - 1] = a[j];
  }
  orc_tridiagonal_solve(lam, aT, bT, cT, rT, jtop, n);
  if (rbar) for (int j = jtop; j <= n; j++) rbar[j - 1] += lam[j - 1];
  if (bbar) for (int j = jtop; j <= n; j++) bbar[j - 1] -= lam[j - 1] * u[j - 1];
  if (abar) for (int j = jtop + 1; j <= n; j++) abar[j - 1] -= lam[j - 1] * u[j - 2];
  if (cbar) for (int j = jtop; j <= n - 1; j++) cbar[j - 1] -= lam[j - 1] * u[j];
  for (int j = jtop; j <= n; j++) ubar[j - 1] = 0.0;
}

/* The same rule over the batched [ld, nlevs] layout of tridiagonal_multi!
 * (tridiagonal.jl:129), one system per masked column from jtop[col] to nlevs. */
int orc_tridiagonal_adjoint_multi(int64_t ncols, int64_t ld, int32_t nlevs, const double* u,
                                  const double* a, const double* b, const double* c, double* ubar,
                                  double* abar, double* bbar, double* cbar, double* rbar,
                                  const int64_t* jtop, const uint8_t* mask, int32_t nthreads)
{
  if (nlevs > ORC_MAXL) return CLMGB_ERR_DIMS;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t col = 0; col < ncols; col++) {
    if (!mask[col]) continue;
    const int j0 = (int)jtop[col];
    if (j0 < 1 || j0 > nlevs) continue;
    double uc[ORC_MAXL], ac[ORC_MAXL], bc[ORC_MAXL], cc[ORC_MAXL], ub[ORC_MAXL];
    double ab_[ORC_MAXL], bb_[ORC_MAXL], cb_[ORC_MAXL], rb_[ORC_MAXL];
    for (int j = 1; j <= nlevs; j++) {
      uc[j - 1] = IX(u, col, j, ld); ac[j - 1] = IX(a, col, j, ld); bc[j - 1] = IX(b, col, j, ld);
      cc[j - 1] = IX(c, col, j, ld); ub[j - 1] = IX(ubar, col, j, ld);
      ab_[j - 1] = abar ? IX(abar, col, j, ld) : 0.0;
      bb_[j - 1] = bbar ? IX(bbar, col, j, ld) : 0.0;
      cb_[j - 1] = cbar ? IX(cbar, col, j, ld) : 0.0;
      rb_[j - 1] = rbar ? IX(rbar, col, j, ld) : 0.0;
    }
    orc_tridiagonal_adjoint(uc, ac, bc, cc, ub, abar ? ab_ : NULL, bbar ? bb_ : NULL, cbar ? cb_ : NULL,
                            rbar ? rb_ : NULL, j0, nlevs);
    for (int j = 1; j <= nlevs; j++) {
      IX(ubar, col, j, ld) = ub[j - 1];
      if (abar) IX(abar, col, j, ld) = ab_[j - 1];
      if (bbar) IX(bbar, col, j, ld) = bb_[j - 1];
      if (cbar) IX(cbar, col, j, ld) = cb_[j - 1];
      if (rbar) IX(rbar, col, j, ld) = rb_[j - 1];
    }
  }
  return 0;
}

/* band_solve! reverse rule (enzyme_rules.jl:80-107) on the batched layout of
 * batched_band_solve! (band_diagonal.jl:179-189; A[i,j] = bmatrix[c, (i-j)+kl+1, jt+i-1]).
 * The rule factorises A with LAPACK gbtrf and solves A^T lambda = xbar with
 * gbtrs('T'); restated here on the dense matrix (entries outside the band are exact
 * zeros, so the in-band arithmetic and its order are those of the banded factors):
 *   factor: for k = 1..n-1 pick the largest |A(i,k)|, i >= k, swap rows k and piv(k),
 *           f_ik = A(i,k)/A(k,k), A(i,j) -= f_ik*A(k,j) for j > k (multipliers of
 *           earlier columns are not permuted: L in product form, as gbtrf keeps it);
 *   U^T w = xbar:  w_i = (xbar_i - sum_{j<i} U(j,i) w_j) / U(i,i), j ascending;
 *   L^T, P^T:      for k = n-1..1: w_k -= sum_{i>k} f_ik w_i (i ascending), swap(w_k, w_piv(k));
 *   rbar += lambda; bmatrix_bar -= lambda_i * x_j on every band entry the forward reads;
 *   xbar is consumed over the solved rows.  bbar and rbar may be NULL. */
int orc_batched_band_solve_adjoint(int64_t nc, int64_t ld, int32_t nlev, const double* tvector,
                                   double* tbar, const double* bmatrix, double* bbar, double* rbar,
                                   const int64_t* jtop, const int64_t* jbot, const uint8_t* mask,
                                   int32_t kl, int32_t ku, int32_t nlevsno_off, int32_t nthreads)
{
  if (nlev > ORC_MAXL) return CLMGB_ERR_DIMS;
  const int nb = kl + ku + 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t c = 0; c < nc; c++) {
    if (!mask[c]) continue;
    const int jt = (int)(jtop[c] + nlevsno_off + 1);
    const int n = (int)(jbot[c] - jtop[c] + 1);
    if (n <= 0) continue;
    double A[ORC_MAXL * ORC_MAXL];
    double w[ORC_MAXL], xs[ORC_MAXL];
    int piv[ORC_MAXL];
#define AA(i, j) A[((i) - 1) * n + ((j) - 1)]
#define BM(bnd, lev) bmatrix[c + (int64_t)((bnd) - 1) * ld + (int64_t)((lev) - 1) * ld * nb]
    for (int i = 1; i <= n; i++)
      for (int j = 1; j <= n; j++) AA(i, j) = 0.0;
    for (int j = 1; j <= n; j++) {
      const int ilo = j - kl > 1 ? j - kl : 1;
      const int ihi = j + ku < n ? j + ku : n;
      for (int i = ilo; i <= ihi; i++) AA(i, j) = BM((i - j) + kl + 1, jt + i - 1);
    }
    for (int k = 1; k <= n - 1; k++) {
      int p = k;
      double maxv = fabs(AA(k, k));
      for (int i = k + 1; i <= n; i++) {
        const double v = fabs(AA(i, k));
        if (v > maxv) { maxv = v; p = i; }
      }
      piv[k - 1] = p;
      if (p != k)
        for (int j = k; j <= n; j++) {
          const double akj = AA(k, j), apj = AA(p, j);
          AA(k, j) = apj; AA(p, j) = akj;
        }
      const double akk = AA(k, k);
      for (int i = k + 1; i <= n; i++) {
        const double f = AA(i, k) / akk;
        for (int j = k + 1; j <= n; j++) AA(i, j) = AA(i, j) - f * AA(k, j);
        AA(i, k) = f;
      }
    }
    for (int i = 1; i <= n; i++) {
      xs[i - 1] = tvector[c + (int64_t)(jt + i - 2) * ld];
      double s = tbar[c + (int64_t)(jt + i - 2) * ld];
      for (int j = 1; j < i; j++) s = s - AA(j, i) * w[j - 1];
      w[i - 1] = s / AA(i, i);
    }
    for (int k = n - 1; k >= 1; k--) {
      double s = w[k - 1];
      for (int i = k + 1; i <= n; i++) s = s - AA(i, k) * w[i - 1];
      w[k - 1] = s;
      const int p = piv[k - 1];
      if (p != k) { const double t = w[k - 1]; w[k - 1] = w[p - 1]; w[p - 1] = t; }
    }
    for (int i = 1; i <= n; i++) {
      const int lev = jt + i - 1;
      if (rbar) rbar[c + (int64_t)(lev - 1) * ld] += w[i - 1];
      tbar[c + (int64_t)(lev - 1) * ld] = 0.0;
    }
    if (bbar)
      for (int j = 1; j <= n; j++) {
        const int ilo = j - kl > 1 ? j - kl : 1;
        const int ihi = j + ku < n ? j + ku : n;
        for (int i = ilo; i <= ihi; i++)
          bbar[c + (int64_t)((i - j) + kl) * ld + (int64_t)(jt + i - 2) * ld * nb] -= w[i - 1] * xs[j - 1];
      }
#undef BM
#undef AA
  }
  return 0;
}

/* ice_impedance (soil_water_movement.jl:722-724). */
double orc_ice_impedance(double icefrac, double e_ice) { return cm_pow(10.0, -e_ice * icefrac); }

/* ===================================================================== */
/* soil_temperature! for one column (non-urban subset).                   */
/* ===================================================================== */
typedef struct {
  const clmgb_varpar* vp;
  const clmgb_bounds* b;
  const clmgb_soiltemp_fields* f;
  double dtime;
  int snow_method;
} st_ctx;

static int col_is_wallroof(int64_t it) { return it == ICOL_SUNWALL || it == ICOL_SHADEWALL || it == ICOL_ROOF; }

/* phase_change_h2osfc kernel body (soil_temperature.jl:1757-1855) for column c. */
static void pc_h2osfc_col(const clmgb_varpar* vp, const clmgb_bounds* bd,
                          const clmgb_soiltemp_fields* f, int64_t c, double dtime,
                          const double* dhsdT)
{
  const int64_t ld = bd->ldc;
  const int joff = vp->nlevsno;
  const int64_t snl = f->col_snl[c];
  double* t = f->t_soisno;
  f->xmf_h2osfc[c] = 0.0;
  f->qflx_h2osfc_to_ice[c] = 0.0;
  f->eflx_h2osfc_to_snow[c] = 0.0;
  if (f->frac_h2osfc[c] > 0.0 && f->t_h2osfc[c] <= TFRZ) {
    double tinc = TFRZ - f->t_h2osfc[c];
    f->t_h2osfc[c] = TFRZ;
    double fh = f->frac_h2osfc[c];
    double ch = f->c_h2osfc[c];
    double hm = fh * (dhsdT[c] * tinc - tinc * ch / dtime);
    double xm = hm * dtime / HFUS;
    double temp1 = f->h2osfc[c] + xm;
    double h2osno_total = f->h2osno_no_layers[c];
    if (snl < 0)
      for (int64_t j = snl + 1; j <= 0; j++)
        h2osno_total += IX(f->h2osoi_ice, c, j + joff, ld) + IX(f->h2osoi_liq, c, j + joff, ld);
    double fs = f->frac_sno_eff[c];
    double z_avg = fs * f->snow_depth[c];
    double rho_avg = z_avg > 0.0 ? jl_min(800.0, h2osno_total / z_avg) : 200.0;
    if (temp1 >= 0.0) {
      f->int_snow[c] -= xm;
      if (snl == 0) f->h2osno_no_layers[c] -= xm;
      else IX(f->h2osoi_ice, c, joff, ld) -= xm;
      h2osno_total -= xm;
      f->h2osfc[c] += xm;
      f->xmf_h2osfc[c] = hm;
      f->qflx_h2osfc_to_ice[c] = -xm / dtime;
      if (fs > 0.0 && snl < 0) f->snow_depth[c] = h2osno_total / (rho_avg * fs);
      else f->snow_depth[c] = h2osno_total / DENICE;
      if (snl == 0) {
        IX(t, c, joff, ld) = f->t_h2osfc[c];
        f->eflx_h2osfc_to_snow[c] = 0.0;
      } else {
        double c1;
        if (snl == -1) c1 = fs * (dtime / IX(f->fact, c, joff, ld) - dhsdT[c] * dtime);
        else c1 = fs / IX(f->fact, c, joff, ld) * dtime;
        double c2 = fh != 0.0 ? (-CPLIQ * xm - fh * dhsdT[c] * dtime) : 0.0;
        IX(t, c, joff, ld) = (c1 * IX(t, c, joff, ld) + c2 * f->t_h2osfc[c]) / (c1 + c2);
        f->eflx_h2osfc_to_snow[c] = (f->t_h2osfc[c] - IX(t, c, joff, ld)) * c2 / dtime;
      }
    } else {
      rho_avg = (h2osno_total * rho_avg + f->h2osfc[c] * DENICE) / (h2osno_total + f->h2osfc[c]);
      f->int_snow[c] += f->h2osfc[c];
      if (snl == 0) f->h2osno_no_layers[c] += f->h2osfc[c];
      else IX(f->h2osoi_ice, c, joff, ld) += f->h2osfc[c];
      h2osno_total += f->h2osfc[c];
      f->qflx_h2osfc_to_ice[c] = f->h2osfc[c] / dtime;
      f->t_h2osfc[c] -= temp1 * HFUS / (dtime * dhsdT[c] - ch);
      f->xmf_h2osfc[c] = hm - fh * temp1 * HFUS / dtime;
      if (snl == 0) {
        IX(t, c, joff, ld) = f->t_h2osfc[c];
      } else {
        double c1;
        if (snl == -1) c1 = fs * (dtime / IX(f->fact, c, joff, ld) - dhsdT[c] * dtime);
        else c1 = fs / IX(f->fact, c, joff, ld) * dtime;
        double c2 = fh != 0.0 ? fh * (ch - dtime * dhsdT[c]) : 0.0;
        IX(t, c, joff, ld) = (c1 * IX(t, c, joff, ld) + c2 * f->t_h2osfc[c]) / (c1 + c2);
        f->t_h2osfc[c] = IX(t, c, joff, ld);
      }
      f->h2osfc[c] = 0.0;
      if (fs > 0.0 && snl < 0) f->snow_depth[c] = h2osno_total / (rho_avg * fs);
      else f->snow_depth[c] = h2osno_total / DENICE;
    }
  }
}

/* phase_change_beta kernel body (soil_temperature.jl:1929-2230), hard (Float64) path. */
static void pc_beta_col(const clmgb_varpar* vp, const clmgb_bounds* bd,
                        const clmgb_soiltemp_fields* f, int64_t c, double dtime,
                        const double* dhsdT)
{
  const int64_t ld = bd->ldc;
  const int nlevsno = vp->nlevsno, nlevgrnd = vp->nlevgrnd, nlevurb = vp->nlevurb;
  const int nlevmaxurbgrnd = vp->nlevmaxurbgrnd;
  const int joff = nlevsno;
  const int64_t snl = f->col_snl[c];
  const int64_t l = f->col_landunit[c] - 1;
  const int64_t it = f->col_itype[c];
  const int64_t lit = f->lun_itype[l];
  const int wallroof = col_is_wallroof(it);
  double hm[ORC_MAXL + 1], xm[ORC_MAXL + 1], xm2[ORC_MAXL + 1], wice0[ORC_MAXL + 1];
  double wliq0[ORC_MAXL + 1], wexice0[ORC_MAXL + 1], wmass0[ORC_MAXL + 1], tinc[ORC_MAXL + 1];
  double supercool[ORC_MAXL + 1];
  for (int k = 0; k <= ORC_MAXL; k++) {
    hm[k] = xm[k] = xm2[k] = wice0[k] = wliq0[k] = wexice0[k] = wmass0[k] = tinc[k] = 0.0;
    supercool[k] = 0.0;
  }
  double* T = f->t_soisno;
  double* ICE = f->h2osoi_ice;
  double* LIQ = f->h2osoi_liq;
  double* EXI = f->excess_ice;
  const double fse = f->frac_sno_eff[c];
  const double fh = f->frac_h2osfc[c];

  f->xmf[c] = 0.0;
  f->qflx_snomelt[c] = 0.0;
  f->qflx_snofrz[c] = 0.0;
  f->qflx_snow_drain[c] = 0.0;

  for (int j = -nlevsno + 1; j <= nlevmaxurbgrnd; j++) {
    int jj = j + joff;
    if (j >= snl + 1) {
      IX(f->imelt, c, jj, ld) = 0;
      hm[jj] = 0.0; xm[jj] = 0.0; xm2[jj] = 0.0;
      wice0[jj] = IX(ICE, c, jj, ld);
      wliq0[jj] = IX(LIQ, c, jj, ld);
      wexice0[jj] = j >= 1 ? IX(EXI, c, j, ld) : 0.0;
      wmass0[jj] = IX(ICE, c, jj, ld) + IX(LIQ, c, jj, ld) + wexice0[jj];
      if (j >= 1) IX(f->exice_subs, c, j, ld) = 0.0;
    }
    if (j <= 0) {
      IX(f->qflx_snomelt_lyr, c, jj, ld) = 0.0;
      IX(f->qflx_snofrz_lyr, c, jj, ld) = 0.0;
    }
  }
  /* snow layers: melting / freezing identification (hard default) */
  for (int j = -nlevsno + 1; j <= 0; j++) {
    int jj = j + joff;
    if (j >= snl + 1) {
      if (IX(ICE, c, jj, ld) > 0.0 && IX(T, c, jj, ld) > TFRZ) {
        IX(f->imelt, c, jj, ld) = 1;
        tinc[jj] = TFRZ - IX(T, c, jj, ld);
        IX(T, c, jj, ld) = TFRZ;
      }
      if (IX(LIQ, c, jj, ld) > 0.0 && IX(T, c, jj, ld) < TFRZ) {
        IX(f->imelt, c, jj, ld) = 2;
        tinc[jj] = TFRZ - IX(T, c, jj, ld);
        IX(T, c, jj, ld) = TFRZ;
      }
    }
  }
  /* soil layers */
  for (int j = 1; j <= nlevmaxurbgrnd; j++) {
    int jj = j + joff;
    supercool[j] = 0.0;
    int active = (!wallroof && j <= nlevgrnd) || (wallroof && j <= nlevurb);
    if (active) {
      if (IX(ICE, c, jj, ld) > 0.0 && IX(T, c, jj, ld) > TFRZ) {
        IX(f->imelt, c, jj, ld) = 1; tinc[jj] = TFRZ - IX(T, c, jj, ld); IX(T, c, jj, ld) = TFRZ;
      }
      if (IX(EXI, c, j, ld) > 0.0 && IX(T, c, jj, ld) > TFRZ) {
        IX(f->imelt, c, jj, ld) = 1; tinc[jj] = TFRZ - IX(T, c, jj, ld); IX(T, c, jj, ld) = TFRZ;
      }
      supercool[j] = 0.0;
      if (lit == ISTSOIL || lit == ISTCROP || it == ICOL_ROAD_PERV) {
        if (IX(T, c, jj, ld) < TFRZ) {
          double tt = IX(T, c, jj, ld);
          double smp = HFUS * (TFRZ - tt) / (GRAV * tt) * 1000.0;
          supercool[j] = IX(f->watsat, c, j, ld) * o_pow(smp / IX(f->sucsat, c, j, ld), -1.0 / IX(f->bsw, c, j, ld));
          supercool[j] *= IX(f->dz, c, jj, ld) * 1000.0;
        }
      }
      if (IX(LIQ, c, jj, ld) > supercool[j] && IX(T, c, jj, ld) < TFRZ) {
        IX(f->imelt, c, jj, ld) = 2; tinc[jj] = TFRZ - IX(T, c, jj, ld); IX(T, c, jj, ld) = TFRZ;
      }
      if (f->h2osno_no_layers[c] > 0.0 && j == 1) {
        if (IX(T, c, jj, ld) > TFRZ) {
          IX(f->imelt, c, jj, ld) = 1; tinc[jj] = TFRZ - IX(T, c, jj, ld); IX(T, c, jj, ld) = TFRZ;
        }
      }
    }
  }
  /* energy surplus / loss and rate of phase change */
  for (int j = -nlevsno + 1; j <= nlevmaxurbgrnd; j++) {
    int jj = j + joff;
    int active = (!wallroof && j <= nlevgrnd) || (wallroof && j <= nlevurb);
    if (!(active && j >= snl + 1)) continue;
    int64_t* im = &IX(f->imelt, c, jj, ld);
    const double fct = IX(f->fact, c, jj, ld);
    if (*im > 0) {
      if (j == snl + 1) {
        if (j > 0) hm[jj] = dhsdT[c] * tinc[jj] - tinc[jj] / fct;
        else hm[jj] = fse * (dhsdT[c] * tinc[jj] - tinc[jj] / fct);
        if (j == 1 && fh != 0.0) hm[jj] -= fh * dhsdT[c] * tinc[jj];
      } else if (j == 1) {
        hm[jj] = (1.0 - fse - fh) * dhsdT[c] * tinc[jj] - tinc[jj] / fct;
      } else {
        if (j < 1) hm[jj] = -fse * tinc[jj] / fct;
        else hm[jj] = -tinc[jj] / fct;
      }
    }
    if (*im == 1 && hm[jj] < 0.0) { hm[jj] = 0.0; *im = 0; }
    if (*im == 2 && hm[jj] > 0.0) { hm[jj] = 0.0; *im = 0; }
    if (*im > 0 && fabs(hm[jj]) > 0.0) {
      xm[jj] = hm[jj] * dtime / HFUS;
      if (j == 1) {
        if (f->h2osno_no_layers[c] > 0.0 && xm[jj] > 0.0) {
          double temp1 = f->h2osno_no_layers[c];
          f->h2osno_no_layers[c] = jl_max(0.0, temp1 - xm[jj]);
          double propor = f->h2osno_no_layers[c] / temp1;
          f->snow_depth[c] = propor * f->snow_depth[c];
          double heatr0 = hm[jj] - HFUS * (temp1 - f->h2osno_no_layers[c]) / dtime;
          if (heatr0 > 0.0) { xm[jj] = heatr0 * dtime / HFUS; hm[jj] = heatr0; }
          else { xm[jj] = 0.0; hm[jj] = 0.0; }
          f->qflx_snomelt[c] = jl_max(0.0, temp1 - f->h2osno_no_layers[c]) / dtime;
          f->xmf[c] = HFUS * f->qflx_snomelt[c];
          f->qflx_snow_drain[c] = f->qflx_snomelt[c];
        }
      }
      double heatr = 0.0;
      if (xm[jj] > 0.0) {
        IX(ICE, c, jj, ld) = jl_max(0.0, wice0[jj] - xm[jj]);
        heatr = hm[jj] - HFUS * (wice0[jj] - IX(ICE, c, jj, ld)) / dtime;
        xm2[jj] = xm[jj] - IX(ICE, c, jj, ld);
        if (IX(ICE, c, jj, ld) == 0.0) {
          if (wexice0[jj] >= 0.0 && xm2[jj] > 0.0 && j >= 2) {
            IX(EXI, c, j, ld) = jl_max(0.0, wexice0[jj] - xm2[jj]);
            heatr = hm[jj] - HFUS * (wexice0[jj] - IX(EXI, c, j, ld) + wice0[jj] - IX(ICE, c, jj, ld)) / dtime;
          }
        }
      } else if (xm[jj] < 0.0) {
        if (j <= 0) {
          IX(ICE, c, jj, ld) = jl_min(wmass0[jj], wice0[jj] - xm[jj]);
        } else {
          if (wmass0[jj] - wexice0[jj] < supercool[j]) IX(ICE, c, jj, ld) = 0.0;
          else IX(ICE, c, jj, ld) = jl_min(wmass0[jj] - wexice0[jj] - supercool[j], wice0[jj] - xm[jj]);
        }
        heatr = hm[jj] - HFUS * (wice0[jj] - IX(ICE, c, jj, ld)) / dtime;
      }
      double ei_val = j >= 1 ? IX(EXI, c, j, ld) : 0.0;
      IX(LIQ, c, jj, ld) = jl_max(0.0, wmass0[jj] - IX(ICE, c, jj, ld) - ei_val);
      if (fabs(heatr) > 0.0) {
        double* tp = &IX(T, c, jj, ld);
        if (j == snl + 1) {
          if (j == 1) {
            *tp += fct * heatr / (1.0 - (1.0 - fh) * fct * dhsdT[c]);
          } else {
            if (fse > 0.0) *tp += (fct / fse) * heatr / (1.0 - fct * dhsdT[c]);
          }
        } else if (j == 1) {
          *tp += fct * heatr / (1.0 - (1.0 - fse - fh) * fct * dhsdT[c]);
        } else {
          if (j > 0) *tp += fct * heatr;
          else if (fse > 0.0) *tp += (fct / fse) * heatr;
        }
        if (j <= 0)
          if (IX(LIQ, c, jj, ld) * IX(ICE, c, jj, ld) > 0.0) *tp = TFRZ;
      }
      if (j >= 1) {
        f->xmf[c] += HFUS * (wice0[jj] - IX(ICE, c, jj, ld)) / dtime +
                     HFUS * (wexice0[jj] - IX(EXI, c, j, ld)) / dtime;
        IX(f->exice_subs, c, j, ld) = jl_max(0.0, (wexice0[jj] - IX(EXI, c, j, ld)) / DENICE);
      } else {
        f->xmf[c] += HFUS * (wice0[jj] - IX(ICE, c, jj, ld)) / dtime;
      }
      if (*im == 1 && j < 1) {
        double q = jl_max(0.0, wice0[jj] - IX(ICE, c, jj, ld)) / dtime;
        IX(f->qflx_snomelt_lyr, c, jj, ld) = q;
        f->qflx_snomelt[c] += q;
        f->snomelt_accum[c] += q * dtime * 1.0e-3;
      }
      if (*im == 2 && j < 1) {
        double q = jl_max(0.0, IX(ICE, c, jj, ld) - wice0[jj]) / dtime;
        IX(f->qflx_snofrz_lyr, c, jj, ld) = q;
        f->qflx_snofrz[c] += q;
      }
    }
  }
  f->eflx_snomelt[c] = f->qflx_snomelt[c] * HFUS;
  if (f->lun_urbpoi[l]) f->eflx_snomelt_u[c] = f->eflx_snomelt[c];
  else if (lit == ISTSOIL || lit == ISTCROP) f->eflx_snomelt_r[c] = f->eflx_snomelt[c];
  (void)wliq0;
}

/* Full soil_temperature! on one non-urban column.  Returns a CLMGB_COL_* bit set. */
static uint32_t soiltemp_col(const st_ctx* X, int64_t c)
{
  const clmgb_varpar* vp = X->vp;
  const clmgb_soiltemp_fields* f = X->f;
  const int64_t ld = X->b->ldc, ldp = X->b->ldp;
  const double dtime = X->dtime;
  const int nlevsno = vp->nlevsno, nlevgrnd = vp->nlevgrnd, nlevsoi = vp->nlevsoi;
  const int nlevmaxurbgrnd = vp->nlevmaxurbgrnd;
  const int joff = nlevsno;
  const int nlev = nlevsno + nlevmaxurbgrnd;
  const int nlev_total = nlevsno + 1 + nlevmaxurbgrnd;
  if (!f->mask_nolakec[c]) return 0;
  const int64_t snl = f->col_snl[c];
  /* the reference indexes its level arrays with snl (a BoundsError outside
   * -nlevsno..0); the column is reported and left untouched, as the kernels do */
  if (snl > 0 || snl < -nlevsno) return CLMGB_COL_LEVEL_RANGE;
  const int64_t l = f->col_landunit[c] - 1;
  const int64_t it = f->col_itype[c];
  const int64_t lit = f->lun_itype[l];
  if (f->lun_urbpoi[l] || col_is_wallroof(it) || it == ICOL_ROAD_IMPERV || it == ICOL_ROAD_PERV)
    return CLMGB_COL_URBAN;

  double tk[ORC_MAXL + 2], cv[ORC_MAXL + 2], fn[ORC_MAXL + 2], fn1[ORC_MAXL + 2];
  for (int k = 0; k < ORC_MAXL + 2; k++) tk[k] = cv[k] = fn[k] = fn1[k] = 0.0;
  double tk_h2osfc = NAN;
  double hs_top = 0.0, hs_soil = 0.0, hs_top_snow = 0.0, hs_h2osfc = 0.0, hs = 0.0;
  double dhsdT_c = 0.0;
  double sabg_lyr_col[ORC_MAXL + 2];
  for (int k = 0; k < ORC_MAXL + 2; k++) sabg_lyr_col[k] = 0.0;
  double fn_h2osfc = 0.0, dz_h2osfc = 0.0;
  /* bmatrix[band][lev], tvector/rvector 1-based over nlev_total */
  double bmat[5][ORC_MAXL + 2];
  double tvec[ORC_MAXL + 2], rvec[ORC_MAXL + 2];
  for (int k = 0; k < ORC_MAXL + 2; k++) {
    for (int bb = 0; bb < 5; bb++) bmat[bb][k] = 0.0;
    tvec[k] = NAN; rvec[k] = NAN;
  }
  double* T = f->t_soisno;
  const double* DZ = f->dz;
  const double* Z = f->z;
  const double* ZI = f->zi;
  double* LIQ = f->h2osoi_liq;
  double* ICE = f->h2osoi_ice;
  const double* EXI = f->excess_ice;
  const int is_special = (lit == ISTWET || lit == ISTICE);
  const int64_t nbedrock = f->col_nbedrock[c];
  const double fse = f->frac_sno_eff[c];
  const double fh = f->frac_h2osfc[c];

  /* ---- soil_therm_prop!: layer conductivity (_soil_snow_tk_kernel!) ---- */
  for (int jj = 1; jj <= nlevsno + nlevgrnd; jj++) {
    int j = jj - nlevsno;
    if (j >= 1) {
      if (!is_special) {
        double liq = IX(LIQ, c, jj, ld), ice = IX(ICE, c, jj, ld), exi = IX(EXI, c, j, ld);
        double dzv = IX(DZ, c, jj, ld), ws = IX(f->watsat, c, j, ld);
        double satw = (liq / DENH2O + ice / DENICE + exi / DENICE) / (dzv * ws);
        satw = jl_min(1.0, satw);
        double thkv;
        if (satw > 1.0e-7) {
          double dke;
          if (IX(T, c, jj, ld) >= TFRZ) dke = jl_max(0.0, o_log10(satw) + 1.0);
          else dke = satw;
          double fl_denom = liq / (DENH2O * dzv) + ice / (DENICE * dzv) + exi / (DENICE * dzv);
          double fl = (liq / (DENH2O * dzv)) / fl_denom;
          double dksat = IX(f->tkmg, c, j, ld) * o_pow(TKWAT, fl * ws) * o_pow(TKICE, (1.0 - fl) * ws);
          thkv = dke * dksat + (1.0 - dke) * IX(f->tkdry, c, j, ld);
        } else {
          thkv = IX(f->tkdry, c, j, ld);
        }
        if (j > nbedrock) thkv = THK_BEDROCK;
        IX(f->thk, c, jj, ld) = thkv;
      } else if (lit == ISTICE) {
        IX(f->thk, c, jj, ld) = IX(T, c, jj, ld) < TFRZ ? TKICE : TKWAT;
      } else if (lit == ISTWET) {
        if (j > nlevsoi) IX(f->thk, c, jj, ld) = THK_BEDROCK;
        else IX(f->thk, c, jj, ld) = IX(T, c, jj, ld) < TFRZ ? TKICE : TKWAT;
      }
    }
    if (snl + 1 < 1 && j >= snl + 1 && j <= 0) {
      double denom = jl_max(fse, 1.0e-6) * jl_max(IX(DZ, c, jj, ld), 1.0e-6);
      double bwv = (IX(ICE, c, jj, ld) + IX(LIQ, c, jj, ld)) / denom;
      IX(f->bw, c, jj, ld) = bwv;
      if (X->snow_method == CLMGB_SNOW_JORDAN1991) {
        IX(f->thk, c, jj, ld) = TKAIR + (7.75e-5 * bwv + 1.105e-6 * (bwv * bwv)) * (TKICE - TKAIR);
      } else {
        if (bwv <= 156.0) IX(f->thk, c, jj, ld) = 0.023 + 0.234 * (bwv / 1000.0);
        else IX(f->thk, c, jj, ld) = 0.138 - 1.01 * (bwv / 1000.0) + 3.233 * ((bwv / 1000.0) * (bwv / 1000.0));
      }
    }
  }
  /* interface conductivity (_soil_tk_interface_kernel!) */
  for (int jj = 1; jj <= nlev; jj++) {
    int j = jj - nlevsno;
    if (j >= snl + 1 && j <= nlevgrnd - 1) {
      double tkj = IX(f->thk, c, jj, ld), tkj1 = IX(f->thk, c, jj + 1, ld);
      double zj = IX(Z, c, jj, ld), zj1 = IX(Z, c, jj + 1, ld), zij1 = IX(ZI, c, jj + 1, ld);
      tk[jj] = tkj * tkj1 * (zj1 - zj) / (tkj * (zj1 - zij1) + tkj1 * (zij1 - zj));
    } else if (j == nlevgrnd) {
      tk[jj] = 0.0;
    }
  }
  /* _tk_h2osfc_kernel! */
  {
    double zh2osfc = 1.0e-3 * (0.5 * f->h2osfc[c]);
    double z1 = IX(Z, c, 1 + joff, ld), tk1 = IX(f->thk, c, 1 + joff, ld);
    double denom = TKWAT * z1 + tk1 * zh2osfc;
    tk_h2osfc = denom > 0.0 ? TKWAT * tk1 * (z1 + zh2osfc) / denom : tk1;
  }
  /* _soil_cv_kernel! */
  for (int j = 1; j <= nlevgrnd; j++) {
    int jj = j + nlevsno;
    double dzv = IX(DZ, c, jj, ld);
    if (!is_special) {
      cv[jj] = IX(f->csol, c, j, ld) * (1.0 - IX(f->watsat, c, j, ld)) * dzv +
               (IX(ICE, c, jj, ld) * CPICE + IX(LIQ, c, jj, ld) * CPLIQ) + IX(EXI, c, j, ld) * CPICE;
      if (j > nbedrock) cv[jj] = CSOL_BEDROCK * dzv;
    } else {
      cv[jj] = IX(ICE, c, jj, ld) * CPICE + IX(LIQ, c, jj, ld) * CPLIQ;
      if (j > nbedrock) cv[jj] = CSOL_BEDROCK * dzv;
    }
  }
  /* _unresolved_snow_cv_kernel! */
  if (f->h2osno_no_layers[c] > 0.0) cv[1 + joff] += CPICE * f->h2osno_no_layers[c];
  /* _snow_cv_kernel! */
  for (int jj = 1; jj <= nlevsno; jj++) {
    int j = jj - nlevsno;
    if (snl + 1 < 1 && j >= snl + 1) {
      if (fse > 0.0)
        cv[jj] = jl_max(THIN_SFCLAYER, (CPLIQ * IX(LIQ, c, jj, ld) + CPICE * IX(ICE, c, jj, ld)) / fse);
      else
        cv[jj] = THIN_SFCLAYER;
    }
  }

  /* ---- compute_ground_heat_flux_and_deriv! ---- */
  const double eg = f->emg[c];
  const double tg = f->t_grnd[c];
  const double lwrad_emit = eg * SB * jl_pow4(tg);
  const double dlwrad_emit = 4.0 * eg * SB * (tg * tg * tg);
  const double lwrad_emit_snow = eg * SB * jl_pow4(IX(T, c, snl + 1 + joff, ld));
  const double lwrad_emit_soil = eg * SB * jl_pow4(IX(T, c, 1 + joff, ld));
  const double lwrad_emit_h2osfc = eg * SB * jl_pow4(f->t_h2osfc[c]);
  const double htvp = f->htvp[c];
  const double forc = f->forc_lwrad[c];
  const int64_t pi = f->col_patchi[c], pf = f->col_patchf[c];
  uint32_t status = 0;
  if (pi < 1 || pf > X->b->np || pf < pi - 1) return CLMGB_COL_PATCH_RANGE;
  /* rural gnet + contributions, scattered in ascending patch order */
  for (int64_t p1 = pi; p1 <= pf; p1++) {
    int64_t p = p1 - 1;
    if (f->patch_column[p] != c + 1) continue;
    double hs_p = 0.0, dh_p = 0.0, hsoil_p = 0.0, hh_p = 0.0;
    if (f->mask_nolakep[p] && !f->lun_urbpoi[f->patch_landunit[p] - 1]) {
      double base = f->dlrad[p] + (1.0 - (double)f->frac_veg_nosno[p]) * eg * forc;
      f->eflx_gnet[p] = f->sabg[p] + base - lwrad_emit - (f->eflx_sh_grnd[p] + f->qflx_evap_soi[p] * htvp);
      f->sabg_chk[p] = fse * f->sabg_snow[p] + (1.0 - fse) * f->sabg_soil[p];
      f->dgnetdT[p] = -f->cgrnd[p] - dlwrad_emit;
      double wt = f->patch_wtcol[p];
      double gsoil = f->sabg_soil[p] + base - lwrad_emit_soil - (f->eflx_sh_soil[p] + f->qflx_ev_soil[p] * htvp);
      double gh2o = f->sabg_soil[p] + base - lwrad_emit_h2osfc - (f->eflx_sh_h2osfc[p] + f->qflx_ev_h2osfc[p] * htvp);
      int wnz = wt != 0.0;
      hs_p = wnz ? f->eflx_gnet[p] * wt : 0.0;
      dh_p = wnz ? f->dgnetdT[p] * wt : 0.0;
      hsoil_p = wnz ? gsoil * wt : 0.0;
      hh_p = wnz ? gh2o * wt : 0.0;
    }
    hs += hs_p; dhsdT_c += dh_p; hs_soil += hsoil_p; hs_h2osfc += hh_p;
  }
  /* SNICAR top-layer flux + per-layer solar */
  for (int64_t p1 = pi; p1 <= pf; p1++) {
    int64_t p = p1 - 1;
    if (f->patch_column[p] != c + 1) continue;
    if (!f->mask_nolakep[p]) continue;
    double wt = f->patch_wtcol[p];
    int64_t lyr_top = snl + 1;
    double base = f->dlrad[p] + (1.0 - (double)f->frac_veg_nosno[p]) * eg * forc;
    double sab = IX(f->sabg_lyr, p, lyr_top + joff, ldp);
    double gtop = sab + base - lwrad_emit - (f->eflx_sh_grnd[p] + f->qflx_evap_soi[p] * htvp);
    hs_top += gtop * wt;
    double gsnow = sab + base - lwrad_emit_snow - (f->eflx_sh_snow[p] + f->qflx_ev_snow[p] * htvp);
    hs_top_snow += gsnow * wt;
    for (int64_t j = lyr_top; j <= 1; j++)
      sabg_lyr_col[j + nlevsno] += IX(f->sabg_lyr, p, j + joff, ldp) * wt;
  }
  (void)hs; (void)hs_top;

  /* ---- compute_heat_diff_flux_and_factor! (_heat_diff_kernel!) ---- */
  for (int jj = 1; jj <= nlev; jj++) {
    int j = jj - nlevsno;
    if (j <= nlevgrnd && j >= snl + 1) {
      double* fc = &IX(f->fact, c, jj, ld);
      if (j == snl + 1) {
        *fc = dtime / cv[jj] * IX(DZ, c, jj, ld) /
              (0.5 * (IX(Z, c, jj, ld) - IX(ZI, c, jj, ld) + CAPR * (IX(Z, c, jj + 1, ld) - IX(ZI, c, jj, ld))));
        fn[jj] = tk[jj] * (IX(T, c, jj + 1, ld) - IX(T, c, jj, ld)) / (IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld));
      } else if (j <= nlevgrnd - 1) {
        *fc = dtime / cv[jj];
        fn[jj] = tk[jj] * (IX(T, c, jj + 1, ld) - IX(T, c, jj, ld)) / (IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld));
      } else if (j == nlevgrnd) {
        *fc = dtime / cv[jj];
        fn[jj] = f->eflx_bot[c];
      }
    }
  }
  /* ---- _h2osfc_thermprop_kernel! ---- */
  if (f->h2osfc[c] > THIN_SFCLAYER && fh > THIN_SFCLAYER) {
    f->c_h2osfc[c] = jl_max(THIN_SFCLAYER, CPLIQ * f->h2osfc[c] / fh);
    dz_h2osfc = jl_max(THIN_SFCLAYER, 1.0e-3 * f->h2osfc[c] / fh);
  } else {
    f->c_h2osfc[c] = THIN_SFCLAYER;
    dz_h2osfc = THIN_SFCLAYER;
  }
  const double ch = f->c_h2osfc[c];
  const double dhsdT = dhsdT_c;

  /* ---- set_rhs_vec! ---- */
  for (int s = 1; s <= nlevsno; s++) {
    int j = s - nlevsno, jj = s;
    double fc = IX(f->fact, c, jj, ld);
    if (j == snl + 1) {
      rvec[s] = IX(T, c, jj, ld) + fc * (hs_top_snow - dhsdT * IX(T, c, jj, ld) + CNFAC * fn[jj]);
    } else if (j > snl + 1) {
      rvec[s] = IX(T, c, jj, ld) + CNFAC * fc * (fn[jj] - fn[jj - 1]);
      rvec[s] += fc * sabg_lyr_col[s];
    }
  }
  {
    double dzm = 0.5 * dz_h2osfc + IX(Z, c, 1 + joff, ld);
    double fnh = tk_h2osfc * (IX(T, c, 1 + joff, ld) - f->t_h2osfc[c]) / dzm;
    fn_h2osfc = fnh;
    rvec[nlevsno + 1] = f->t_h2osfc[c] + (dtime / ch) * (hs_h2osfc - dhsdT * f->t_h2osfc[c] + CNFAC * fnh);
  }
  for (int j = 1; j <= nlevgrnd; j++) {
    int jj = j + nlevsno, rv = j + nlevsno + 1;
    double fc = IX(f->fact, c, jj, ld), tt = IX(T, c, jj, ld);
    if (j == snl + 1) {
      rvec[rv] = tt + fc * (hs_top_snow - dhsdT * tt + CNFAC * fn[jj]);
    } else if (j == 1) {
      rvec[rv] = tt + fc * ((1.0 - fse) * (hs_soil - dhsdT * tt) + CNFAC * (fn[jj] - fse * fn[jj - 1]));
      rvec[rv] += fse * fc * sabg_lyr_col[j + nlevsno];
    } else if (j <= nlevgrnd - 1) {
      rvec[rv] = tt + CNFAC * fc * (fn[jj] - fn[jj - 1]);
    } else if (j == nlevgrnd) {
      rvec[rv] = tt - CNFAC * fc * fn[jj - 1] + fc * fn[jj];
    }
  }
  if (fh != 0.0) {
    int jj = 1 + nlevsno, rv = 1 + nlevsno + 1;
    rvec[rv] -= fh * IX(f->fact, c, jj, ld) * ((hs_soil - dhsdT * IX(T, c, jj, ld)) + CNFAC * fn_h2osfc);
  }

  /* ---- set_matrix! (bmat[band-1][row]) ---- */
  {
    const double omc = 1.0 - CNFAC;
    for (int s = 1; s <= nlevsno; s++) {
      int j = s - nlevsno, jj = s, bm = s;
      if (j >= snl + 1) {
        double fc = IX(f->fact, c, jj, ld);
        double dzp = IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld);
        if (j == snl + 1) {
          bmat[2][bm] = 1.0 + omc * fc * tk[jj] / dzp - fc * dhsdT;
        } else {
          double dzm = IX(Z, c, jj, ld) - IX(Z, c, jj - 1, ld);
          bmat[3][bm] = -omc * fc * tk[jj - 1] / dzm;
          bmat[2][bm] = 1.0 + omc * fc * (tk[jj] / dzp + tk[jj - 1] / dzm);
        }
        if (j != 0) bmat[1][bm] = -omc * fc * tk[jj] / dzp;
        else bmat[0][bm] = -omc * fc * tk[jj] / dzp;
      }
    }
    {
      int ssw = nlevsno + 1;
      double dzm = 0.5 * dz_h2osfc + IX(Z, c, 1 + joff, ld);
      bmat[2][ssw] = 1.0 + omc * (dtime / ch) * tk_h2osfc / dzm - (dtime / ch) * dhsdT;
      bmat[1][ssw] = -omc * (dtime / ch) * tk_h2osfc / dzm;
    }
    for (int j = 1; j <= nlevgrnd; j++) {
      int jj = j + nlevsno, bm = j + nlevsno + 1;
      double fc = IX(f->fact, c, jj, ld);
      if (j == snl + 1) {
        double dzp = IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld);
        bmat[2][bm] = 1.0 + omc * fc * tk[jj] / dzp - fc * dhsdT;
        bmat[1][bm] = -omc * fc * tk[jj] / dzp;
      } else if (j == 1) {
        double dzm = IX(Z, c, jj, ld) - IX(Z, c, jj - 1, ld);
        double dzp = IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld);
        bmat[1][bm] = -omc * fc * tk[jj] / dzp;
        bmat[2][bm] = 1.0 + omc * fc * (tk[jj] / dzp + fse * tk[jj - 1] / dzm) - (1.0 - fse) * fc * dhsdT;
        bmat[4][bm] = -fse * omc * fc * tk[jj - 1] / dzm;
      } else if (j <= nlevgrnd - 1) {
        double dzm = IX(Z, c, jj, ld) - IX(Z, c, jj - 1, ld);
        double dzp = IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld);
        bmat[1][bm] = -omc * fc * tk[jj] / dzp;
        bmat[2][bm] = 1.0 + omc * fc * (tk[jj] / dzp + tk[jj - 1] / dzm);
        bmat[3][bm] = -omc * fc * tk[jj - 1] / dzm;
      } else if (j == nlevgrnd) {
        double dzm = IX(Z, c, jj, ld) - IX(Z, c, jj - 1, ld);
        bmat[2][bm] = 1.0 + omc * fc * tk[jj - 1] / dzm;
        bmat[3][bm] = -omc * fc * tk[jj - 1] / dzm;
      }
    }
    if (fh != 0.0) {
      double dzm = 0.5 * dz_h2osfc + IX(Z, c, 1 + joff, ld);
      int bm = 1 + nlevsno + 1;
      double fc = IX(f->fact, c, 1 + joff, ld);
      bmat[2][bm] += fh * (omc * fc * tk_h2osfc / dzm + fc * dhsdT);
      bmat[3][bm] = -fh * omc * fc * tk_h2osfc / dzm;
    }
  }

  /* ---- _tvector_init_kernel! ---- */
  for (int64_t j = snl + 1; j <= 0; j++) tvec[j - 1 + nlevsno + 1] = IX(T, c, j + joff, ld);
  tvec[nlevsno + 1] = f->t_h2osfc[c];
  for (int j = 1; j <= nlevmaxurbgrnd; j++) tvec[j + nlevsno + 1] = IX(T, c, j + joff, ld);

  /* ---- batched_band_solve! on this column: dense pivoted GE ---- */
  {
    const int kl = 2, ku = 2;
    int jt = (int)(snl + nlevsno + 1);
    int n = (int)(nlevgrnd - snl + 1);
    /* bmatrix as [1 column, 5 bands, nlev_total] so the shared dense routine reads it */
    double bm1[5 * (ORC_MAXL + 2)];
    for (int lev = 1; lev <= nlev_total; lev++)
      for (int bb = 1; bb <= 5; bb++) bm1[(bb - 1) + (lev - 1) * 5] = bmat[bb - 1][lev];
    dense_band_solve_col(tvec + 1, 1, bm1, 1, nlev_total, rvec + 1, 1, 0, jt, n, kl, ku);
  }

  /* ---- _tvector_extract_kernel! ---- */
  for (int64_t j = snl + 1; j <= 0; j++) IX(T, c, j + joff, ld) = tvec[j - 1 + nlevsno + 1];
  for (int j = 1; j <= nlevmaxurbgrnd; j++) IX(T, c, j + joff, ld) = tvec[j + nlevsno + 1];
  if (fh == 0.0) f->t_h2osfc[c] = IX(T, c, 1 + joff, ld);
  else f->t_h2osfc[c] = tvec[nlevsno + 1];

  /* ---- _fn1_kernel! ---- */
  for (int jj = 1; jj <= nlev; jj++) {
    int j = jj - nlevsno;
    if (j >= snl + 1) {
      if (j <= nlevgrnd - 1)
        fn1[jj] = tk[jj] * (IX(T, c, jj + 1, ld) - IX(T, c, jj, ld)) / (IX(Z, c, jj + 1, ld) - IX(Z, c, jj, ld));
      else if (j == nlevgrnd)
        fn1[jj] = 0.0;
    }
  }

  /* ---- phase change ---- */
  double dh_arr[1];
  dh_arr[0] = dhsdT;
  {
    /* the per-column helpers index dhsdT[c]; hand them a pointer offset so [c] is ours */
    const double* dh = dh_arr - c;
    pc_h2osfc_col(vp, X->b, f, c, dtime, dh);
    pc_beta_col(vp, X->b, f, c, dtime, dh);
  }

  /* ---- _tgrnd_kernel! ---- */
  {
    double t1 = IX(T, c, 1 + joff, ld), th = f->t_h2osfc[c];
    if (snl < 0) {
      double ts = IX(T, c, snl + 1 + joff, ld);
      if (fh != 0.0) f->t_grnd[c] = fse * ts + (1.0 - fse - fh) * t1 + fh * th;
      else f->t_grnd[c] = fse * ts + (1.0 - fse) * t1;
    } else {
      if (fh != 0.0) f->t_grnd[c] = (1.0 - fh) * t1 + fh * th;
      else f->t_grnd[c] = t1;
    }
  }
  /* ---- eflx_fgr12 / eflx_fgr (_eflx_fgr_kernel!) ---- */
  f->eflx_fgr12[c] = 0.0;
  {
    const int issoilcrop = (lit == ISTSOIL || lit == ISTCROP);
    for (int j = 1; j <= nlevgrnd; j++) {
      int jj = j + joff;
      if (j == 1) f->eflx_fgr12[c] = -CNFAC * fn[1 + joff] - (1.0 - CNFAC) * fn1[1 + joff];
      if (j > 0 && j < nlevgrnd && issoilcrop)
        IX(f->eflx_fgr, c, j, ld) = -CNFAC * fn[jj] - (1.0 - CNFAC) * fn1[jj];
      else if (j == nlevgrnd && issoilcrop)
        IX(f->eflx_fgr, c, j, ld) = 0.0;
    }
  }
  for (int jj = (int)(snl + 1 + joff); jj <= nlev; jj++)
    if (!isfinite(IX(T, c, jj, ld))) status |= CLMGB_COL_NONFINITE;
  return status;
}

static int check_varpar(const clmgb_varpar* vp)
{
  if (!vp) return CLMGB_ERR_NULL_ARG;
  if (vp->nlevsno < 1 || vp->nlevgrnd < 2 || vp->nlevsoi < 1 || vp->nlevsoi > vp->nlevgrnd)
    return CLMGB_ERR_DIMS;
  if (vp->nlevmaxurbgrnd != vp->nlevgrnd) return CLMGB_ERR_DIMS;
  if (vp->nlevsno + vp->nlevmaxurbgrnd + 1 > ORC_MAXL) return CLMGB_ERR_DIMS;
  return 0;
}

int orc_soil_temperature(const clmgb_varpar* vp, const clmgb_bounds* b,
                         const clmgb_soiltemp_fields* f, double dtime, int32_t snow_method,
                         uint32_t* col_status, int32_t nthreads)
{
  int e = check_varpar(vp);
  if (e) return e;
  st_ctx X = {vp, b, f, dtime, snow_method};
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t c = 0; c < b->nc; c++) {
    uint32_t s = soiltemp_col(&X, c);
    if (col_status) col_status[c] = s;
  }
  return 0;
}

/* Standalone phase_change_h2osfc! / phase_change_beta! (soil_temperature.jl:1857, 2232). */
int orc_phase_change_h2osfc(const clmgb_varpar* vp, const clmgb_bounds* b,
                            const clmgb_soiltemp_fields* f, double dtime, const double* dhsdT)
{
  int e = check_varpar(vp);
  if (e) return e;
  for (int64_t c = 0; c < b->nc; c++)
    if (f->mask_nolakec[c]) pc_h2osfc_col(vp, b, f, c, dtime, dhsdT);
  return 0;
}
int orc_phase_change_beta(const clmgb_varpar* vp, const clmgb_bounds* b,
                          const clmgb_soiltemp_fields* f, double dtime, const double* dhsdT)
{
  int e = check_varpar(vp);
  if (e) return e;
  for (int64_t c = 0; c < b->nc; c++)
    if (f->mask_nolakec[c]) pc_beta_col(vp, b, f, c, dtime, dhsdT);
  return 0;
}

/* ===================================================================== */
/* set_soil_water_fractions! — _soilhyd_water_fractions_kernel!          */
/* ===================================================================== */
static void fractions_col(const clmgb_varpar* vp, const clmgb_bounds* b,
                          const clmgb_soilwater_fields* f, int64_t c)
{
  const int64_t ld = b->ldc;
  const int joff = vp->nlevsno;
  if (!f->mask_hydrology[c]) return;
  for (int j = 1; j <= vp->nlevsoi; j++) {
    double dn = DENICE;
    double dz_ext = IX(f->dz, c, j + joff, ld) + IX(f->excess_ice, c, j, ld) / dn;
    double ws = IX(f->watsat, c, j, ld);
    double vol_ice = jl_min(ws, (IX(f->h2osoi_ice, c, j + joff, ld) + IX(f->excess_ice, c, j, ld)) / (dz_ext * dn));
    IX(f->eff_porosity, c, j, ld) = jl_max(0.01, ws - vol_ice);
    IX(f->icefrac, c, j, ld) = jl_min(1.0, vol_ice / ws);
  }
}

int orc_soil_water_fractions(const clmgb_varpar* vp, const clmgb_bounds* b,
                             const clmgb_soilwater_fields* f, int32_t nthreads)
{
  int e = check_varpar(vp);
  if (e) return e;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t c = 0; c < b->nc; c++) fractions_col(vp, b, f, c);
  return 0;
}

/* ===================================================================== */
/* surface hydrology (clm_driver.jl:1938-2007), one loop per routine      */
/* ===================================================================== */
int orc_surface_hydrology(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_surfhyd_fields* f,
                          const clmgb_surfhyd_config* cfg, uint32_t stages, double dtime)
{
  int e = check_varpar(vp);
  if (e) return e;
  const int64_t nc = b->nc, ld = b->ldc;
  const int top = vp->nlevsno + 1;
  if ((stages & CLMGB_SH_SAT_EXCESS) && cfg->fsat_method != CLMGB_FSAT_TOPMODEL && cfg->fsat_method != CLMGB_FSAT_VIC)
    return -1;
  if ((stages & CLMGB_SH_INFL_EXCESS) && cfg->qinmax_method != CLMGB_QINMAX_NONE &&
      cfg->qinmax_method != CLMGB_QINMAX_HKSAT)
    return -1;
  /* set_floodc! (soil_hydrology.jl:139-152) */
  if (stages & CLMGB_SH_FLOODC)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_nolakec[c]) continue;
      if (f->col_itype[c] != ICOL_SUNWALL && f->col_itype[c] != ICOL_SHADEWALL)
        f->qflx_floodc[c] = f->qflx_floodg[f->col_gridcell[c] - 1];
      else
        f->qflx_floodc[c] = 0.0;
    }
  /* saturated_excess_runoff! (sat_excess_runoff.jl:246-300) */
  if (stages & CLMGB_SH_SAT_EXCESS)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      double fs;
      if (cfg->fsat_method == CLMGB_FSAT_TOPMODEL) {
        if (f->frost_table[c] > f->zwt_perched[c] && f->frost_table[c] <= f->zwt[c])
          fs = f->wtfact[c] * cm_exp(-0.5 * cfg->fff * f->zwt_perched[c]);
        else
          fs = f->wtfact[c] * cm_exp(-0.5 * cfg->fff * f->zwt[c]);
      } else {
        double ex = f->b_infil[c] / (1.0 + f->b_infil[c]);
        fs = 1.0 - cm_pow(1.0 - f->top_moist_limited[c] / f->top_max_moist[c], ex);
      }
      if (cfg->crop_fsat_equals_zero && f->lun_itype[f->col_landunit[c] - 1] == ISTCROP) fs = 0.0;
      if (cfg->hillslope_fsat_equals_zero && f->col_is_hillslope[c] && f->col_active[c] && f->col_cold[c] != -9999)
        fs = 0.0;
      f->fsat[c] = fs;
      double q = fs * f->qflx_rain_plus_snomelt[c];
      f->fcov[c] = fs;
      if (f->col_urbpoi[c]) q = q + f->qflx_floodc[c];
      f->qflx_sat_excess_surf[c] = q;
    }
  /* set_qflx_inputs! (soil_hydrology.jl:160-187) */
  if (stages & CLMGB_SH_QFLX_INPUTS)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      f->qflx_top_soil[c] = f->qflx_rain_plus_snomelt[c] + f->qflx_snow_h2osfc[c] + f->qflx_floodc[c];
      double fsno, qflx_evap;
      if (f->col_snl[c] >= 0) {
        fsno = 0.0;
        qflx_evap = f->qflx_liqevap_from_top_layer[c];
      } else {
        fsno = f->frac_sno_eff[c];
        qflx_evap = f->qflx_ev_soil[c];
      }
      f->qflx_in_soil[c] = (1.0 - f->frac_h2osfc[c]) * (f->qflx_top_soil[c] - f->qflx_sat_excess_surf[c]);
      f->qflx_top_soil_to_h2osfc[c] = f->frac_h2osfc[c] * (f->qflx_top_soil[c] - f->qflx_sat_excess_surf[c]);
      f->qflx_in_soil[c] = f->qflx_in_soil[c] - (1.0 - fsno - f->frac_h2osfc[c]) * qflx_evap;
      f->qflx_top_soil_to_h2osfc[c] = f->qflx_top_soil_to_h2osfc[c] - f->frac_h2osfc[c] * f->qflx_ev_h2osfc[c];
    }
  /* infiltration_excess_runoff! (infilt_excess_runoff.jl:142-211, 241-274) */
  if (stages & CLMGB_SH_INFL_EXCESS) {
    double* qinmax_unsat = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      if (cfg->qinmax_method == CLMGB_QINMAX_NONE) {
        qinmax_unsat[c] = 1.0e200;
      } else {
        double qmin = INFINITY;
        for (int j = 1; j <= 3; j++) {
          double val = cm_pow(10.0, -cfg->e_ice * IX(f->icefrac, c, j, ld)) * IX(f->hksat, c, j, ld);
          if (val < qmin) qmin = val;
        }
        qinmax_unsat[c] = qmin;
      }
    }
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      f->qinmax[c] = (1.0 - f->fsat[c]) * qinmax_unsat[c];
      f->qflx_infl_excess[c] = jl_max(0.0, f->qflx_in_soil[c] - (1.0 - f->frac_h2osfc[c]) * f->qinmax[c]);
    }
    free(qinmax_unsat);
  }
  /* route_infiltration_excess! (soil_hydrology.jl:199-225) */
  if (stages & CLMGB_SH_ROUTE)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      int64_t lt = f->lun_itype[f->col_landunit[c] - 1];
      if (lt == ISTSOIL || lt == ISTCROP) {
        f->qflx_in_soil_limited[c] = f->qflx_in_soil[c] - f->qflx_infl_excess[c];
        if (cfg->h2osfcflag != 0) {
          f->qflx_in_h2osfc[c] = f->qflx_top_soil_to_h2osfc[c] + f->qflx_infl_excess[c];
          f->qflx_infl_excess_surf[c] = 0.0;
        } else {
          f->qflx_in_h2osfc[c] = f->qflx_top_soil_to_h2osfc[c];
          f->qflx_infl_excess_surf[c] = f->qflx_infl_excess[c];
        }
      } else {
        f->qflx_in_soil_limited[c] = f->qflx_in_soil[c];
        f->qflx_in_h2osfc[c] = 0.0;
        f->qflx_infl_excess_surf[c] = 0.0;
      }
    }
  /* update_h2osfc! (surface_water.jl:462-520): its four kernels in turn, with the
   * two scratch vectors it allocates */
  if (stages & CLMGB_SH_UPDATE_H2OSFC) {
    const int flag = cfg->update_h2osfcflag;
    double* qsurf = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
    double* qdrain = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
    for (int64_t c = 0; c < nc; c++) {       /* _surfwat_qflx_surf_kernel! (:279-316) */
      if (!f->mask_hydrology[c]) continue;
      if (flag != 1) {
        qsurf[c] = 0.0;
      } else {
        double frac_infclust;
        if (f->frac_h2osfc_nosnow[c] <= cfg->pc) frac_infclust = 0.0;
        else frac_infclust = cm_pow(f->frac_h2osfc_nosnow[c] - cfg->pc, cfg->mu);
        double q = 0.0;
        if (f->h2osfc[c] > f->h2osfc_thresh[c] && flag != 0) {
          double k_wet = 1.0e-4 * cm_sin(CM_DEG2RAD * f->topo_slope[c]);
          q = k_wet * frac_infclust * (f->h2osfc[c] - f->h2osfc_thresh[c]);
          q = jl_min(q, (f->h2osfc[c] - f->h2osfc_thresh[c]) / dtime);
        }
        if (q < 1.0e-8) q = 0.0;
        qsurf[c] = q;
      }
    }
    for (int64_t c = 0; c < nc; c++) {       /* _surfwat_partial_update_kernel! (:400-414) */
      if (!f->mask_hydrology[c]) continue;
      double h = f->h2osfc[c] + (f->qflx_in_h2osfc[c] - qsurf[c]) * dtime;
      if (fabs(h) < 1.0e-13 * fabs(f->h2osfc[c])) h = 0.0;
      f->h2osfc[c] = h;
    }
    for (int64_t c = 0; c < nc; c++) {       /* _surfwat_qflx_drain_kernel! (:357-374) */
      if (!f->mask_hydrology[c]) continue;
      if (f->h2osfc[c] < 0.0) {
        qdrain[c] = f->h2osfc[c] / dtime;
      } else {
        double q = jl_min(f->frac_h2osfc[c] * f->qinmax[c], f->h2osfc[c] / dtime);
        if (flag == 0) q = jl_max(0.0, f->h2osfc[c] / dtime);
        qdrain[c] = q;
      }
    }
    for (int64_t c = 0; c < nc; c++) {       /* _surfwat_final_update_kernel! (:426-443) */
      if (!f->mask_hydrology[c]) continue;
      double h = f->h2osfc[c] - qdrain[c] * dtime;
      if (fabs(h) < 1.0e-13 * fabs(f->h2osfc[c])) h = 0.0;
      f->h2osfc[c] = h;
      f->qflx_h2osfc_surf[c] = qsurf[c];
      f->qflx_h2osfc_drain[c] = qdrain[c];
    }
    free(qsurf);
    free(qdrain);
  }
  /* infiltration! (soil_hydrology.jl:236-243) */
  if (stages & CLMGB_SH_INFILTRATION)
    for (int64_t c = 0; c < nc; c++)
      if (f->mask_hydrology[c]) f->qflx_infl[c] = f->qflx_in_soil_limited[c] + f->qflx_h2osfc_drain[c];
  /* total_surface_runoff! (soil_hydrology.jl:250-301) */
  if (stages & CLMGB_SH_TOTAL_RUNOFF) {
    for (int64_t c = 0; c < nc; c++)
      if (f->mask_hydrology[c])
        f->qflx_surf[c] = f->qflx_sat_excess_surf[c] + f->qflx_infl_excess_surf[c] + f->qflx_h2osfc_surf[c];
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_urban[c]) continue;
      int64_t it = f->col_itype[c];
      if (it == ICOL_ROOF || it == ICOL_ROAD_IMPERV) {
        if (f->col_snl[c] < 0) {
          f->qflx_surf[c] = jl_max(0.0, f->qflx_rain_plus_snomelt[c]);
        } else {
          f->xs_urban[c] = jl_max(0.0, IX(f->h2osoi_liq, c, top, ld) / dtime + f->qflx_rain_plus_snomelt[c] -
                                           f->qflx_liqevap_from_top_layer[c] - cfg->pondmx_urban / dtime);
          f->qflx_surf[c] = f->xs_urban[c];
        }
        f->qflx_surf[c] = f->qflx_surf[c] + f->qflx_floodc[c];
      } else if (it == ICOL_SUNWALL || it == ICOL_SHADEWALL) {
        f->qflx_surf[c] = 0.0;
      }
    }
  }
  /* update_urban_ponding! (soil_hydrology.jl:316-338) */
  if (stages & CLMGB_SH_URBAN_PONDING)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_urban[c]) continue;
      int64_t it = f->col_itype[c];
      if ((it == ICOL_ROOF || it == ICOL_ROAD_IMPERV) && f->col_snl[c] >= 0) {
        if (f->xs_urban[c] > 0.0)
          IX(f->h2osoi_liq, c, top, ld) = cfg->pondmx_urban;
        else
          IX(f->h2osoi_liq, c, top, ld) = jl_max(0.0, IX(f->h2osoi_liq, c, top, ld) +
                                                          (f->qflx_rain_plus_snomelt[c] - f->qflx_liqevap_from_top_layer[c]) * dtime);
      }
    }
  return 0;
}

/* ===================================================================== */
/* snow layer dynamics (clm_driver.jl:2146-2200), one loop per routine    */
/* ===================================================================== */
#define SNW_LSADZ 0.03
#define SNW_ISTDLAK 5

static void snw_combo(double* dz, double* wliq, double* wice, double* t, double dz2, double wliq2, double wice2,
                      double t2)
{
  double dzc = *dz + dz2, wicec = *wice + wice2, wliqc = *wliq + wliq2;
  double h = (CPICE * *wice + CPLIQ * *wliq) * (*t - TFRZ) + HFUS * *wliq;
  double h2 = (CPICE * wice2 + CPLIQ * wliq2) * (t2 - TFRZ) + HFUS * wliq2;
  double hc = h + h2;
  double denom = CPICE * wicec + CPLIQ * wliqc;
  double tc;
  if (denom > 0.0) tc = TFRZ + (hc - HFUS * wliqc) / denom;
  else tc = TFRZ;
  *dz = dzc;
  *wice = wicec;
  *wliq = wliqc;
  *t = tc;
}

static double snw_radius(double rds1, double rds2, double swtot, double zwtot, double rmin, double rmax)
{
  double total_wt = swtot + zwtot;
  double r = total_wt > 0.0 ? (rds2 * swtot + rds1 * zwtot) / total_wt : 0.5 * (rds1 + rds2);
  return r > rmax ? rmax : (r < rmin ? rmin : r);           /* Julia clamp */
}

int orc_snow_layers(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_snowlayer_fields* f,
                    const clmgb_snowlayer_config* cfg, uint32_t stages, double dtime)
{
  int e = check_varpar(vp);
  if (e) return e;
  const int64_t nc = b->nc, ld = b->ldc;
  const int ns = vp->nlevsno;
  if ((stages & CLMGB_SL_COMPACTION) && cfg->overburden_method != CLMGB_OVERBURDEN_ANDERSON1976 &&
      cfg->overburden_method != CLMGB_OVERBURDEN_VIONNET2012)
    return -1;
  /* init_snow_layers! thresholds (snow_hydrology.jl:2357-2377), 1-based like the reference */
  double dzmin[ORC_MAXL + 1], dzmax_l[ORC_MAXL + 1], dzmax_u[ORC_MAXL + 1];
  memset(dzmin, 0, sizeof dzmin);
  memset(dzmax_l, 0, sizeof dzmax_l);
  memset(dzmax_u, 0, sizeof dzmax_u);
  dzmin[1] = cfg->dzmin_1; dzmax_l[1] = cfg->dzmax_l_1; dzmax_u[1] = cfg->dzmax_u_1;
  dzmin[2] = cfg->dzmin_2; dzmax_l[2] = cfg->dzmax_l_2; dzmax_u[2] = cfg->dzmax_u_2;
  for (int j = 3; j <= ns; j++) {
    dzmin[j] = dzmax_u[j - 1] * 0.5;
    dzmax_u[j] = 2.0 * dzmax_u[j - 1] + 0.01;
    dzmax_l[j] = dzmax_u[j] + dzmax_l[j - 1];
    if (j == ns) { dzmax_u[j] = 1.7976931348623157e308; dzmax_l[j] = 1.7976931348623157e308; }
  }
  double* aer[8] = {f->mss_bcphi, f->mss_bcpho, f->mss_ocphi, f->mss_ocpho,
                    f->mss_dst1, f->mss_dst2, f->mss_dst3, f->mss_dst4};

  /* snow_compaction! (_snowhyd_compaction_kernel!, :1203-1326) */
  if (stages & CLMGB_SL_COMPACTION)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_snow[c]) continue;
      const double c3 = 2.777e-6, c4 = 0.04, c5 = 2.0;
      double burden = 0.0, zpseudo = 0.0;
      int mobile = 1;
      for (int j = -ns + 1; j <= 0; j++) {
        if (!(j >= f->col_snl[c] + 1)) continue;
        int jj = j + ns;
        double wx = IX(f->h2osoi_ice, c, jj, ld) + IX(f->h2osoi_liq, c, jj, ld);
        double voidv = 1.0 - (IX(f->h2osoi_ice, c, jj, ld) / DENICE + IX(f->h2osoi_liq, c, jj, ld) / DENH2O) /
                                 (f->frac_sno[c] * IX(f->dz, c, jj, ld));
        if (voidv > 0.001 && IX(f->h2osoi_ice, c, jj, ld) > 0.1) {
          double bi = IX(f->h2osoi_ice, c, jj, ld) / (f->frac_sno[c] * IX(f->dz, c, jj, ld));
          double fi = IX(f->h2osoi_ice, c, jj, ld) / wx;
          double td = TFRZ - IX(f->t_soisno, c, jj, ld);
          double dexpf = cm_exp(-c4 * td);
          double ddz1 = -c3 * dexpf;
          if (bi > cfg->upplim_destruct_metamorph)
            ddz1 = ddz1 * cm_exp(-46.0e-3 * (bi - cfg->upplim_destruct_metamorph));
          if (IX(f->h2osoi_liq, c, jj, ld) > 0.01 * IX(f->dz, c, jj, ld) * f->frac_sno[c]) ddz1 = ddz1 * c5;
          double ddz2;
          if (cfg->overburden_method == CLMGB_OVERBURDEN_ANDERSON1976) {
            double c2 = 23.0e-3;
            ddz2 = -(burden + wx / 2.0) * cm_exp(-cfg->overburden_compress_tfactor * td - c2 * bi) /
                   cfg->eta0_anderson;
          } else {
            double f1 = 1.0 / (1.0 + 60.0 * IX(f->h2osoi_liq, c, jj, ld) / (DENH2O * IX(f->dz, c, jj, ld)));
            double f2 = 4.0;
            double eta = f1 * f2 * (bi / cfg->ceta) * cm_exp(0.1 * td + 0.023 * bi) * cfg->eta0_vionnet;
            ddz2 = -(burden + wx / 2.0) / eta;
          }
          double ddz3;
          if (IX(f->imelt, c, jj, ld) == 1) {
            int64_t l = f->col_landunit[c] - 1;
            if (cfg->use_subgrid_fluxes && !f->lun_lakpoi[l] && !f->lun_urbpoi[l]) {
              ddz3 = jl_max(0.0, jl_min(1.0, (IX(f->swe_old, c, jj, ld) - wx) / wx));
              if ((IX(f->swe_old, c, jj, ld) - wx) > 0.0) {
                double wsum = 0.0;
                for (int64_t jj2 = f->col_snl[c] + 1; jj2 <= 0; jj2++)
                  wsum += IX(f->h2osoi_liq, c, jj2 + ns, ld) + IX(f->h2osoi_ice, c, jj2 + ns, ld);
                double int_snow_lim = jl_min(f->int_snow[c], cfg->int_snow_max);
                double fsno_melt;
                if (int_snow_lim > 0.0) {
                  double smr = jl_min(1.0, wsum / int_snow_lim);
                  fsno_melt = 1.0 - cm_pow(cm_acos(jl_min(1.0, 2.0 * smr - 1.0)) / 3.14159265358979323846,
                                           f->n_melt[c]);
                } else {
                  fsno_melt = 1.0;
                }
                if ((fsno_melt + f->frac_h2osfc[c]) > 1.0) fsno_melt = 1.0 - f->frac_h2osfc[c];
                ddz3 = ddz3 - jl_max(0.0, (fsno_melt - f->frac_sno[c]) / f->frac_sno[c]);
              }
              ddz3 = -1.0 / dtime * ddz3;
            } else {
              ddz3 = -1.0 / dtime * jl_max(0.0, (IX(f->frac_iceold, c, jj, ld) - fi) / IX(f->frac_iceold, c, jj, ld));
            }
          } else {
            ddz3 = 0.0;
          }
          double ddz4_val = 0.0;
          if (cfg->wind_dependent_snow_density) {
            /* _wind_drift_compaction_dev (:1466-1500) */
            if (mobile) {
              double forc_wind = f->forc_wind[f->col_gridcell[c] - 1], dzj = IX(f->dz, c, jj, ld);
              double Frho = 1.25 - 0.0042 * (jl_max(cfg->rho_min, bi) - cfg->rho_min);
              double MO = 0.34 * (-0.583 * cfg->drift_gs - 0.833 * 1.0 + 0.833) + 0.66 * Frho;
              double SI = -2.868 * cm_exp(-0.085 * forc_wind) + 1.0 + MO;
              if (SI > 0.0) {
                SI = jl_min(SI, 3.25);
                double zp = zpseudo + 0.5 * dzj * (3.25 - SI);
                double gamma_drift = SI * cm_exp(-zp / 0.1);
                double tau_inverse = gamma_drift / cfg->tau_ref;
                ddz4_val = -jl_max(0.0, cfg->rho_max - bi) * tau_inverse;
                zp = zp + 0.5 * dzj * (3.25 - SI);
                zpseudo = zp;
                mobile = 1;
              } else {
                ddz4_val = 0.0;
                mobile = 0;
              }
            } else {
              ddz4_val = 0.0;
              mobile = 0;
            }
          }
          double pdzdtc = ddz1 + ddz2 + ddz3 + ddz4_val;
          IX(f->dz, c, jj, ld) = jl_max(IX(f->dz, c, jj, ld) * (1.0 + pdzdtc * dtime),
                                        (IX(f->h2osoi_ice, c, jj, ld) / DENICE + IX(f->h2osoi_liq, c, jj, ld) / DENH2O) /
                                            f->frac_sno[c]);
        } else {
          mobile = 0;
        }
        burden = burden + wx;
      }
    }

  /* combine_snow_layers! (_snowhyd_combine_kernel!, :1584-1874) */
  if (stages & CLMGB_SL_COMBINE)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_snow[c]) continue;
      int64_t* snl = (int64_t*)&f->col_snl[c];
      f->qflx_sl_top_soil[c] = 0.0;
      int64_t msn_old = *snl;
      int64_t j = msn_old + 1;
      while (j <= 0) {
        int64_t jj = j + ns;
        if (IX(f->h2osoi_ice, c, jj, ld) <= 0.01) {
          int64_t l = f->col_landunit[c] - 1;
          int64_t ltype = f->lun_itype[l];
          if (j < 0 || (ltype == ISTSOIL || f->lun_urbpoi[l] || ltype == ISTCROP)) {
            IX(f->h2osoi_liq, c, jj + 1, ld) += IX(f->h2osoi_liq, c, jj, ld);
            IX(f->h2osoi_ice, c, jj + 1, ld) += IX(f->h2osoi_ice, c, jj, ld);
          }
          if (j == 0) f->qflx_sl_top_soil[c] = (IX(f->h2osoi_liq, c, jj, ld) + IX(f->h2osoi_ice, c, jj, ld)) / dtime;
          if (j < 0) {
            IX(f->dz, c, jj + 1, ld) += IX(f->dz, c, jj, ld);
            for (int a = 0; a < 8; a++) IX(aer[a], c, jj + 1, ld) += IX(aer[a], c, jj, ld);
          }
          if (j > *snl + 1 && *snl < -1)
            for (int64_t i = j; i >= *snl + 2; i--) {
              int64_t ii = i + ns, ia = i - 1 + ns;
              IX(f->h2osoi_liq, c, ii, ld) = IX(f->h2osoi_liq, c, ia, ld);
              IX(f->h2osoi_ice, c, ii, ld) = IX(f->h2osoi_ice, c, ia, ld);
              IX(f->t_soisno, c, ii, ld) = IX(f->t_soisno, c, ia, ld);
              IX(f->dz, c, ii, ld) = IX(f->dz, c, ia, ld);
              for (int a = 0; a < 8; a++) IX(aer[a], c, ii, ld) = IX(aer[a], c, ia, ld);
              IX(f->snw_rds, c, ii, ld) = IX(f->snw_rds, c, ia, ld);
            }
          *snl = *snl + 1;
        }
        j += 1;
      }
      double snow_depth_acc = 0.0, h2osno_total = 0.0;
      for (int64_t jl = *snl + 1; jl <= 0; jl++) {
        snow_depth_acc += IX(f->dz, c, jl + ns, ld);
        h2osno_total += IX(f->h2osoi_ice, c, jl + ns, ld) + IX(f->h2osoi_liq, c, jl + ns, ld);
      }
      f->snow_depth[c] = snow_depth_acc;
      if (f->snow_depth[c] > 0.0) {
        int64_t l = f->col_landunit[c] - 1;
        int64_t ltype = f->lun_itype[l];
        int all_gone = (ltype == SNW_ISTDLAK && f->snow_depth[c] < dzmin[1] + SNW_LSADZ) ||
                       (ltype != SNW_ISTDLAK && (f->frac_sno_eff[c] * f->snow_depth[c] < dzmin[1] ||
                                                 h2osno_total / (f->frac_sno_eff[c] * f->snow_depth[c]) < 50.0));
        if (all_gone) {
          double zwice = 0.0, zwliq = 0.0;
          for (int64_t jl = *snl + 1; jl <= 0; jl++) {
            zwice += IX(f->h2osoi_ice, c, jl + ns, ld);
            zwliq += IX(f->h2osoi_liq, c, jl + ns, ld);
          }
          f->h2osno_no_layers[c] = zwice;
          if (ltype == ISTSOIL || f->lun_urbpoi[l] || ltype == ISTCROP) IX(f->h2osoi_liq, c, ns + 1, ld) += zwliq;
          *snl = 0;
          h2osno_total = f->h2osno_no_layers[c];
          for (int jj = 1; jj <= ns; jj++)
            for (int a = 0; a < 8; a++) IX(aer[a], c, jj, ld) = 0.0;
          if (f->h2osno_no_layers[c] <= 0.0) f->snow_depth[c] = 0.0;
        }
      }
      if (h2osno_total <= 0.0) {
        f->snow_depth[c] = 0.0;
        f->frac_sno[c] = 0.0;
        f->frac_sno_eff[c] = 0.0;
        f->int_snow[c] = 0.0;
      }
      if (*snl < -1) {
        int mssi = 1;
        int64_t i = *snl + 1;
        while (i <= 0) {
          int64_t ji = i + ns;
          int thin = (f->frac_sno_eff[c] * IX(f->dz, c, ji, ld) < dzmin[mssi]) ||
                     ((IX(f->h2osoi_ice, c, ji, ld) + IX(f->h2osoi_liq, c, ji, ld)) /
                          (f->frac_sno_eff[c] * IX(f->dz, c, ji, ld)) < 50.0);
          if (thin) {
            int64_t neibor;
            if (i == *snl + 1) neibor = i + 1;
            else if (i == 0) neibor = i - 1;
            else {
              neibor = i + 1;
              if ((IX(f->dz, c, ji - 1, ld) + IX(f->dz, c, ji, ld)) < (IX(f->dz, c, ji + 1, ld) + IX(f->dz, c, ji, ld)))
                neibor = i - 1;
            }
            int64_t j_keep, l_remove;
            if (neibor > i) { j_keep = neibor; l_remove = i; }
            else { j_keep = i; l_remove = neibor; }
            int64_t jk = j_keep + ns, jr = l_remove + ns;
            for (int a = 0; a < 8; a++) IX(aer[a], c, jk, ld) += IX(aer[a], c, jr, ld);
            double total_mass = IX(f->h2osoi_liq, c, jk, ld) + IX(f->h2osoi_ice, c, jk, ld) +
                                IX(f->h2osoi_liq, c, jr, ld) + IX(f->h2osoi_ice, c, jr, ld);
            if (total_mass > 0.0)
              IX(f->snw_rds, c, jk, ld) =
                  (IX(f->snw_rds, c, jk, ld) * (IX(f->h2osoi_liq, c, jk, ld) + IX(f->h2osoi_ice, c, jk, ld)) +
                   IX(f->snw_rds, c, jr, ld) * (IX(f->h2osoi_liq, c, jr, ld) + IX(f->h2osoi_ice, c, jr, ld))) /
                  total_mass;
            snw_combo(&IX(f->dz, c, jk, ld), &IX(f->h2osoi_liq, c, jk, ld), &IX(f->h2osoi_ice, c, jk, ld),
                      &IX(f->t_soisno, c, jk, ld), IX(f->dz, c, jr, ld), IX(f->h2osoi_liq, c, jr, ld),
                      IX(f->h2osoi_ice, c, jr, ld), IX(f->t_soisno, c, jr, ld));
            if (j_keep - 1 > *snl + 1)
              for (int64_t k = j_keep - 1; k >= *snl + 2; k--) {
                int64_t kk = k + ns, ka = k - 1 + ns;
                IX(f->h2osoi_ice, c, kk, ld) = IX(f->h2osoi_ice, c, ka, ld);
                IX(f->h2osoi_liq, c, kk, ld) = IX(f->h2osoi_liq, c, ka, ld);
                IX(f->t_soisno, c, kk, ld) = IX(f->t_soisno, c, ka, ld);
                IX(f->dz, c, kk, ld) = IX(f->dz, c, ka, ld);
                for (int a = 0; a < 8; a++) IX(aer[a], c, kk, ld) = IX(aer[a], c, ka, ld);
                IX(f->snw_rds, c, kk, ld) = IX(f->snw_rds, c, ka, ld);
              }
            *snl = *snl + 1;
            if (*snl >= -1) break;
          } else {
            mssi = mssi + 1;
          }
          i += 1;
        }
      }
      for (int64_t jl = 0; jl >= -ns + 1; jl--) {
        int64_t jj = jl + ns;
        if (jl >= *snl + 1) {
          IX(f->z, c, jj, ld) = IX(f->zi, c, jj + 1, ld) - 0.5 * IX(f->dz, c, jj, ld);
          IX(f->zi, c, jj, ld) = IX(f->zi, c, jj + 1, ld) - IX(f->dz, c, jj, ld);
        }
      }
    }

  /* divide_snow_layers! (_snowhyd_divide_kernel!, :2057-2237) */
  if (stages & CLMGB_SL_DIVIDE)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_snow[c]) continue;
      double dzsno[ORC_MAXL + 2], swice[ORC_MAXL + 2], swliq[ORC_MAXL + 2], tsno[ORC_MAXL + 2], rds[ORC_MAXL + 2];
      double ma[8][ORC_MAXL + 2];
      memset(dzsno, 0, sizeof dzsno); memset(swice, 0, sizeof swice); memset(swliq, 0, sizeof swliq);
      memset(tsno, 0, sizeof tsno); memset(rds, 0, sizeof rds); memset(ma, 0, sizeof ma);
      const int is_lake = cfg->is_lake != 0;
      int64_t snl = f->col_snl[c];
      int64_t msno = snl < 0 ? -snl : snl;
      for (int64_t k = 1; k <= msno; k++) {
        int64_t jj = (k + snl) + ns;
        dzsno[k] = is_lake ? IX(f->dz, c, jj, ld) : f->frac_sno[c] * IX(f->dz, c, jj, ld);
        swice[k] = IX(f->h2osoi_ice, c, jj, ld);
        swliq[k] = IX(f->h2osoi_liq, c, jj, ld);
        tsno[k] = IX(f->t_soisno, c, jj, ld);
        for (int a = 0; a < 8; a++) ma[a][k] = IX(aer[a], c, jj, ld);
        rds[k] = IX(f->snw_rds, c, jj, ld);
      }
      int64_t k = 1;
      while (k <= msno && k < ns) {
        if (k == msno) {
          double offset = is_lake ? 2.0 * SNW_LSADZ : 0.0;
          if (dzsno[k] > dzmax_l[k] + offset) {
            msno += 1;
            dzsno[k] /= 2.0; dzsno[k + 1] = dzsno[k];
            swice[k] /= 2.0; swice[k + 1] = swice[k];
            swliq[k] /= 2.0; swliq[k + 1] = swliq[k];
            if (k == 1) {
              tsno[k + 1] = tsno[k];
            } else {
              double dtdz = (tsno[k - 1] - tsno[k]) / ((dzsno[k - 1] + 2.0 * dzsno[k]) / 2.0);
              double tsno_kp1_candidate = tsno[k] - dtdz * dzsno[k] / 2.0;
              double tsno_k_candidate = tsno[k] + dtdz * dzsno[k] / 2.0;
              double w_frozen = (TFRZ - tsno_kp1_candidate) >= 0.0 ? 1.0 : 0.0;
              tsno[k + 1] = w_frozen * tsno_kp1_candidate + (1.0 - w_frozen) * tsno[k];
              tsno[k] = w_frozen * tsno_k_candidate + (1.0 - w_frozen) * tsno[k];
            }
            for (int a = 0; a < 8; a++) { ma[a][k] /= 2.0; ma[a][k + 1] = ma[a][k]; }
            rds[k + 1] = rds[k];
          }
        }
        if (k < msno) {
          double offset = is_lake ? SNW_LSADZ : 0.0;
          if (dzsno[k] > dzmax_u[k] + offset) {
            double drr = dzsno[k] - dzmax_u[k] - offset;
            double propor = drr / dzsno[k];
            double zwice = propor * swice[k], zwliq = propor * swliq[k], zm[8];
            for (int a = 0; a < 8; a++) zm[a] = propor * ma[a][k];
            double propor_keep = (dzmax_u[k] + offset) / dzsno[k];
            swice[k] *= propor_keep;
            swliq[k] *= propor_keep;
            for (int a = 0; a < 8; a++) ma[a][k] *= propor_keep;
            dzsno[k] = dzmax_u[k] + offset;
            for (int a = 0; a < 8; a++) ma[a][k + 1] += zm[a];
            rds[k + 1] = snw_radius(rds[k], rds[k + 1], swliq[k + 1] + swice[k + 1], zwliq + zwice,
                                    cfg->snw_rds_min, cfg->snw_rds_max);
            snw_combo(&dzsno[k + 1], &swliq[k + 1], &swice[k + 1], &tsno[k + 1], drr, zwliq, zwice, tsno[k]);
          }
        }
        k += 1;
      }
      f->col_snl[c] = -msno;
      snl = f->col_snl[c];
      for (int64_t jl = -ns + 1; jl <= 0; jl++) {
        int64_t jj = jl + ns;
        if (jl >= snl + 1) {
          int64_t ki = jl - snl;
          IX(f->dz, c, jj, ld) = is_lake ? dzsno[ki] : dzsno[ki] / f->frac_sno[c];
          IX(f->h2osoi_ice, c, jj, ld) = swice[ki];
          IX(f->h2osoi_liq, c, jj, ld) = swliq[ki];
          IX(f->t_soisno, c, jj, ld) = tsno[ki];
          for (int a = 0; a < 8; a++) IX(aer[a], c, jj, ld) = ma[a][ki];
          IX(f->snw_rds, c, jj, ld) = rds[ki];
        }
      }
      for (int64_t jl = 0; jl >= -ns + 1; jl--) {
        int64_t jj = jl + ns;
        if (jl >= snl + 1) {
          IX(f->z, c, jj, ld) = IX(f->zi, c, jj + 1, ld) - 0.5 * IX(f->dz, c, jj, ld);
          IX(f->zi, c, jj, ld) = IX(f->zi, c, jj + 1, ld) - IX(f->dz, c, jj, ld);
        }
      }
    }

  /* zero_empty_snow_layers! (:2314-2329) */
  if (stages & CLMGB_SL_ZERO_EMPTY)
    for (int64_t c = 0; c < nc; c++) {
      if (!f->mask_snow[c]) continue;
      for (int jj = 1; jj <= ns; jj++) {
        int64_t j = jj - ns;
        if (j <= f->col_snl[c] && f->col_snl[c] > -ns) {
          IX(f->h2osoi_ice, c, jj, ld) = 0.0;
          IX(f->h2osoi_liq, c, jj, ld) = 0.0;
          IX(f->t_soisno, c, jj, ld) = 0.0;
          IX(f->dz, c, jj, ld) = 0.0;
          IX(f->z, c, jj, ld) = 0.0;
          IX(f->zi, c, jj, ld) = 0.0;
        }
      }
    }

  /* build_snow_filter! (:2488-2510) */
  if (stages & CLMGB_SL_FILTER)
    for (int64_t c = 0; c < nc; c++) {
      f->mask_snow[c] = 0;
      f->mask_nosnow[c] = 0;
      if (f->mask_nolakec[c]) {
        if (f->col_snl[c] < 0) f->mask_snow[c] = 1;
        else f->mask_nosnow[c] = 1;
      }
    }
  return 0;
}

/* ===================================================================== */
/* lake_temperature! (lake_temperature.jl:1016-1295), kernel by kernel    */
/* ===================================================================== */
#define LK_MAXX (ORC_MAXL + 2 * CLMGB_MAX_NLEVLAK)
#define LK_BETAVIS 0.0
#define LK_ZA 0.6
#define LK_TDMAX 277.0
#define LK_VKC 0.4

/* soil_therm_prop_lake! (:39-192) for column c: tk, cv [1..ns+nlevgrnd] and tktopsoillay */
static void lake_therm_prop(const clmgb_varpar* vp, const clmgb_lake_fields* f, int64_t c, int64_t ld, double* tk,
                            double* cv, double* tktopsoillay)
{
  const int ns = vp->nlevsno, ng = vp->nlevgrnd, nsoi = vp->nlevsoi;
  const int64_t snl = f->col_snl[c];
  double thk[ORC_MAXL + 2];
  memset(thk, 0, sizeof thk);
  for (int jj = 1; jj <= ns + ng; jj++) {           /* _lake_soil_tk_kernel! */
    int j = jj - ns;
    if (j >= 1 && j <= nsoi) {
      double satw = 1.0;
      double fl = IX(f->h2osoi_liq, c, jj, ld) / (IX(f->h2osoi_ice, c, jj, ld) + IX(f->h2osoi_liq, c, jj, ld));
      double dke, dksat;
      if (IX(f->t_soisno, c, jj, ld) >= TFRZ) {
        dke = jl_max(0.0, cm_log10(satw) + 1.0);
        dksat = IX(f->tksatu, c, j, ld);
      } else {
        dke = satw;
        dksat = IX(f->tkmg, c, j, ld) * cm_pow(0.249, fl * IX(f->watsat, c, j, ld)) * cm_pow(2.29, IX(f->watsat, c, j, ld));
      }
      thk[jj] = dke * dksat + (1.0 - dke) * IX(f->tkdry, c, j, ld);
      satw = (IX(f->h2osoi_liq, c, jj, ld) / DENH2O + IX(f->h2osoi_ice, c, jj, ld) / DENICE) /
             (IX(f->dz, c, jj, ld) * IX(f->watsat, c, j, ld));
      if (satw > 1.0) {
        double xicevol = (satw - 1.0) * IX(f->watsat, c, j, ld);
        thk[jj] = (thk[jj] + xicevol * TKICE) / (1.0 + xicevol) / (1.0 + xicevol);
      }
    } else if (j > nsoi) {
      thk[jj] = THK_BEDROCK;
    }
    if (snl + 1 < 1 && j >= snl + 1 && j <= 0) {
      double bw = (IX(f->h2osoi_ice, c, jj, ld) + IX(f->h2osoi_liq, c, jj, ld)) / IX(f->dz, c, jj, ld);
      thk[jj] = TKAIR + (7.75e-5 * bw + 1.105e-6 * bw * bw) * (TKICE - TKAIR);
    }
  }
  for (int jj = 1; jj <= ns + ng; jj++) {           /* _lake_tk_interface_kernel! */
    int j = jj - ns;
    if (j >= snl + 1 && j <= ng - 1 && j != 0) {
      int jj1 = jj + 1;
      tk[jj] = thk[jj] * thk[jj1] * (IX(f->z, c, jj1, ld) - IX(f->z, c, jj, ld)) /
               (thk[jj] * (IX(f->z, c, jj1, ld) - IX(f->zi, c, jj + 1, ld)) +
                thk[jj1] * (IX(f->zi, c, jj + 1, ld) - IX(f->z, c, jj, ld)));
    } else if (j == 0 && j >= snl + 1) {
      tk[jj] = thk[jj];
    } else if (j == ng) {
      tk[jj] = 0.0;
    }
    if (j == 1) *tktopsoillay = thk[jj];
  }
  for (int j = 1; j <= ng; j++) {                   /* _lake_soil_cv_kernel! */
    int jj = j + ns;
    cv[jj] = IX(f->csol, c, j, ld) * (1.0 - IX(f->watsat, c, j, ld)) * IX(f->dz, c, jj, ld) +
             (IX(f->h2osoi_ice, c, jj, ld) * CPICE + IX(f->h2osoi_liq, c, jj, ld) * CPLIQ);
    if (j > nsoi) cv[jj] = CSOL_BEDROCK * IX(f->dz, c, jj, ld);
  }
  for (int jj = 1; jj <= ns; jj++) {                /* _lake_snow_cv_kernel! */
    int j = jj - ns;
    if (snl + 1 < 1 && j >= snl + 1)
      cv[jj] = CPLIQ * IX(f->h2osoi_liq, c, jj, ld) + CPICE * IX(f->h2osoi_ice, c, jj, ld);
  }
}

static double lake_rhow(double icefrac, double t)
{
  return (1.0 - icefrac) * 1000.0 * (1.0 - 1.9549e-05 * cm_pow(fabs(t - LK_TDMAX), 1.68)) + icefrac * DENICE;
}

static double lake_h2osno_total(const clmgb_varpar* vp, const clmgb_lake_fields* f, int64_t c, int64_t ld)
{
  double tot = f->h2osno_no_layers[c];
  for (int jj = 1; jj <= vp->nlevsno; jj++)
    if (jj - vp->nlevsno >= f->col_snl[c] + 1) tot += IX(f->h2osoi_ice, c, jj, ld) + IX(f->h2osoi_liq, c, jj, ld);
  return tot;
}

/* convective mixing of lake levels lo..hi (_lake_top/_bottom_convection_kernel!, :787-894) */
static void lake_mix(const clmgb_lake_fields* f, int64_t c, int64_t ld, int lo, int hi, double* rhow, double cwat,
                     double cice_eff)
{
  double qav = 0.0, nav = 0.0, iceav = 0.0;
  for (int i = lo; i <= hi; i++) {
    qav += IX(f->dz_lake, c, i, ld) * (IX(f->t_lake, c, i, ld) - TFRZ) *
           ((1.0 - IX(f->lake_icefrac, c, i, ld)) * cwat + IX(f->lake_icefrac, c, i, ld) * cice_eff);
    iceav += IX(f->lake_icefrac, c, i, ld) * IX(f->dz_lake, c, i, ld);
    nav += IX(f->dz_lake, c, i, ld);
  }
  qav /= nav;
  iceav /= nav;
  double tav_froz = 0.0, tav_unfr = 0.0;
  if (qav > 0.0) tav_unfr = qav / ((1.0 - iceav) * cwat);
  else if (qav < 0.0) tav_froz = qav / (iceav * cice_eff);
  double zsum = 0.0;
  for (int i = lo; i <= hi; i++) {
    double dzl = IX(f->dz_lake, c, i, ld);
    if ((zsum + dzl) / nav <= iceav) {
      IX(f->lake_icefrac, c, i, ld) = 1.0;
      IX(f->t_lake, c, i, ld) = tav_froz + TFRZ;
    } else if (zsum / nav < iceav) {
      IX(f->lake_icefrac, c, i, ld) = (iceav * nav - zsum) / dzl;
      double fi = IX(f->lake_icefrac, c, i, ld);
      IX(f->t_lake, c, i, ld) = (fi * tav_froz * cice_eff + (1.0 - fi) * tav_unfr * cwat) /
                                    (fi * cice_eff + (1.0 - fi) * cwat) + TFRZ;
    } else {
      IX(f->lake_icefrac, c, i, ld) = 0.0;
      IX(f->t_lake, c, i, ld) = tav_unfr + TFRZ;
    }
    zsum += dzl;
    rhow[i] = lake_rhow(IX(f->lake_icefrac, c, i, ld), IX(f->t_lake, c, i, ld));
  }
}

int orc_lake_temperature(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_lake_fields* f,
                         const clmgb_lake_config* cfg, double dtime)
{
  int e = check_varpar(vp);
  if (e) return e;
  if (cfg->nlevlak < 2 || cfg->nlevlak > CLMGB_MAX_NLEVLAK) return -1;
  const int64_t nc = b->nc, ld = b->ldc, ldp = b->ldp;
  const int ns = vp->nlevsno, ngr = vp->nlevgrnd, nlak = cfg->nlevlak;
  const int ntot = ns + nlak + ngr;
  const double p0 = 1.0, cwat = CPLIQ * DENH2O, cice_eff = CPICE * DENH2O, cfus = HFUS * DENH2O;
  const double tkice_eff = TKICE * DENICE / DENH2O, km = TKWAT / cwat;
  const int puddling = cfg->lakepuddling != 0, no_ed = cfg->lake_no_ed != 0, lch4 = cfg->use_lch4 != 0;
  const double pudz = puddling ? cfg->lake_puddle_thick : 0.0;
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_lakec[c]) continue;
    const int64_t p = f->col_patchi[c] - 1;
    const int pact = f->mask_lakep[p] != 0;
    const int64_t snl = f->col_snl[c];
    double rhow[CLMGB_MAX_NLEVLAK + 1] = {0}, phi[CLMGB_MAX_NLEVLAK + 1] = {0}, kme[CLMGB_MAX_NLEVLAK + 1] = {0};
    double cv_lake[CLMGB_MAX_NLEVLAK + 1] = {0}, tk_lake[CLMGB_MAX_NLEVLAK + 1] = {0};
    double tk[ORC_MAXL + 2] = {0}, cv[ORC_MAXL + 2] = {0}, sabg_lyr_col[ORC_MAXL + 2] = {0};
    double cvx[LK_MAXX] = {0}, tkix[LK_MAXX] = {0}, tx[LK_MAXX] = {0}, phix[LK_MAXX] = {0}, zx[LK_MAXX] = {0};
    double fnx[LK_MAXX] = {0}, factx[LK_MAXX] = {0}, a[LK_MAXX] = {0}, bb[LK_MAXX] = {0}, c1[LK_MAXX] = {0};
    double r[LK_MAXX] = {0};
    double phi_soil = 0.0, fin = 0.0, ocvts = 0.0, ncvts = 0.0, tktopsoillay = 0.0, lhabs = 0.0;
    int jconvect = 0, jconvectbot = nlak + 1, bottomconvect = 0, puddle = 0, frzn = 0;
    /* _lake_init_kernel! */
    if (lch4) f->lakeresist[c] = 0.0;
    /* _lake_prior_ice_kernel! */
    for (int jj = 1; jj <= ns; jj++)
      if (jj - ns >= snl + 1)
        IX(f->frac_iceold, c, jj, ld) =
            IX(f->h2osoi_ice, c, jj, ld) / (IX(f->h2osoi_liq, c, jj, ld) + IX(f->h2osoi_ice, c, jj, ld));
    /* _lake_solar_nir_kernel! */
    if (pact) {
      fin = f->eflx_gnet[p];
      double sabg_nir = f->fsds_nir_d[p] + f->fsds_nir_i[p] - f->fsr_nir_d[p] - f->fsr_nir_i[p];
      sabg_nir = jl_min(sabg_nir, f->sabg[p]);
      f->betaprime[c] = sabg_nir / jl_max(1.0e-5, f->sabg[p]);
      f->betaprime[c] = f->betaprime[c] + (1.0 - f->betaprime[c]) * LK_BETAVIS;
    }
    const double beta = f->betaprime[c];
    /* _lake_density_kernel! */
    for (int j = 1; j <= nlak; j++) rhow[j] = lake_rhow(IX(f->lake_icefrac, c, j, ld), IX(f->t_lake, c, j, ld));
    /* _lake_diffusivity_kernel! (j = 1 .. nlevlak-1, in order) */
    const int warm = f->t_grnd[c] > TFRZ && IX(f->t_lake, c, 1, ld) > TFRZ && snl == 0;
    for (int j = 1; j <= nlak - 1; j++) {
      double zl = IX(f->z_lake, c, j, ld);
      double drhodz = (rhow[j + 1] - rhow[j]) / (IX(f->z_lake, c, j + 1, ld) - zl);
      double n2 = GRAV / rhow[j] * drhodz;
      double vz = LK_VKC * zl;
      double num = 40.0 * n2 * (vz * vz);
      double wsc = f->ws[c];
      double den = jl_max((wsc * wsc) * cm_exp(-2.0 * f->ks[c] * zl), 1.0e-10);
      double ri = (-1.0 + sqrt(jl_max(1.0 + num / den, 0.0))) / 20.0;
      if (puddling && j == 1) frzn = 0;
      double fi = IX(f->lake_icefrac, c, j, ld);
      if (warm && (!puddling || (fi == 0.0 && !frzn))) {
        double ke = LK_VKC * wsc * zl / p0 * cm_exp(-f->ks[c] * zl) / (1.0 + 37.0 * ri * ri);
        kme[j] = km + ke;
        if (!no_ed) {
          double fangkm = 1.039e-8 * cm_pow(jl_max(n2, 7.5e-5), -0.43);
          kme[j] = kme[j] + fangkm;
        }
        if (f->lakedepth[c] >= cfg->deepmixing_depthcrit) kme[j] = kme[j] * cfg->deepmixing_mixfact;
        tk_lake[j] = kme[j] * cwat;
      } else {
        kme[j] = km;
        if (!no_ed) {
          double fangkm = 1.039e-8 * cm_pow(jl_max(n2, 7.5e-5), -0.43);
          kme[j] = kme[j] + fangkm;
          if (f->lakedepth[c] >= cfg->deepmixing_depthcrit) kme[j] = kme[j] * cfg->deepmixing_mixfact;
          tk_lake[j] = kme[j] * cwat * tkice_eff / ((1.0 - fi) * tkice_eff + kme[j] * cwat * fi);
        } else {
          tk_lake[j] = TKWAT * tkice_eff / ((1.0 - fi) * tkice_eff + TKWAT * fi);
        }
        if (puddling) frzn = 1;
      }
    }
    /* _lake_diffusivity_bottom_kernel! */
    {
      int j = nlak;
      double fi = IX(f->lake_icefrac, c, j, ld);
      kme[nlak] = kme[nlak - 1];
      if (warm && (!puddling || (fi == 0.0 && !frzn))) {
        tk_lake[j] = tk_lake[j - 1];
      } else if (!no_ed) {
        tk_lake[j] = kme[j] * cwat * tkice_eff / ((1.0 - fi) * tkice_eff + kme[j] * cwat * fi);
      } else {
        tk_lake[j] = TKWAT * tkice_eff / ((1.0 - fi) * tkice_eff + TKWAT * fi);
      }
      f->savedtke1[c] = kme[1] * cwat;
    }
    const int64_t jtop = snl + 1;
    /* _lake_heat_source_kernel! (the reference reads sabg_lyr[p, 1] for layer 1 under snow) */
    if (pact)
      for (int j = 1; j <= nlak; j++) {
        double eta = f->etal[c] > 0.0 ? f->etal[c] : 1.1925 * cm_pow(jl_max(f->lakedepth[c], 1.0), -0.424);
        double zin = IX(f->z_lake, c, j, ld) - 0.5 * IX(f->dz_lake, c, j, ld);
        double zout = IX(f->z_lake, c, j, ld) + 0.5 * IX(f->dz_lake, c, j, ld);
        double rsfin = cm_exp(-eta * jl_max(zin - LK_ZA, 0.0));
        double rsfout = cm_exp(-eta * jl_max(zout - LK_ZA, 0.0));
        double phidum;
        if (warm) {
          phidum = (rsfin - rsfout) * f->sabg[p] * (1.0 - beta);
          if (j == nlak) phi_soil = rsfout * f->sabg[p] * (1.0 - beta);
        } else if (j == 1 && snl == 0) {
          phidum = f->sabg[p] * (1.0 - beta);
        } else if (j == 1) {
          phidum = IX(f->sabg_lyr, p, j, ldp);
        } else {
          phidum = 0.0;
          if (j == nlak) phi_soil = 0.0;
        }
        phi[j] = phidum;
      }
    /* _lake_cv_lake_kernel!, soil_therm_prop_lake! */
    for (int j = 1; j <= nlak; j++) {
      double fi = IX(f->lake_icefrac, c, j, ld);
      cv_lake[j] = IX(f->dz_lake, c, j, ld) * (cwat * (1.0 - fi) + cice_eff * fi);
    }
    lake_therm_prop(vp, f, c, ld, tk, cv, &tktopsoillay);
    /* _lake_energy_sum_lake_kernel!, _lake_energy_sum_soil_kernel! */
    for (int j = 1; j <= nlak; j++)
      ocvts += cv_lake[j] * (IX(f->t_lake, c, j, ld) - TFRZ) +
               cfus * IX(f->dz_lake, c, j, ld) * (1.0 - IX(f->lake_icefrac, c, j, ld));
    double h2osno_total = lake_h2osno_total(vp, f, c, ld);
    for (int j = -ns + 1; j <= ngr; j++) {
      int jj = j + ns;
      if (j >= jtop) {
        ocvts += cv[jj] * (IX(f->t_soisno, c, jj, ld) - TFRZ) + HFUS * IX(f->h2osoi_liq, c, jj, ld);
        if (j == 1 && h2osno_total > 0.0 && j == jtop) ocvts -= h2osno_total * HFUS;
      }
    }
    /* _lake_solar_transfer_kernel! */
    if (pact)
      for (int jidx = 1; jidx <= ns + 1; jidx++)
        if (jidx - ns >= jtop) sabg_lyr_col[jidx] = IX(f->sabg_lyr, p, jidx, ldp);
    /* _lake_extcol_setup_kernel! */
    for (int je = -ns + 1; je <= nlak + ngr; je++) {
      int ji = je + ns, jj = je + ns;
      if (je < jtop) continue;
      if (je < 1) {
        zx[ji] = IX(f->z, c, jj, ld);
        cvx[ji] = cv[jj];
        phix[ji] = je == jtop ? 0.0 : sabg_lyr_col[je + ns];
        tx[ji] = IX(f->t_soisno, c, jj, ld);
      } else if (je <= nlak) {
        zx[ji] = IX(f->z_lake, c, je, ld);
        cvx[ji] = cv_lake[je];
        phix[ji] = phi[je];
        tx[ji] = IX(f->t_lake, c, je, ld);
      } else {
        int jpjj = je - nlak + ns;
        zx[ji] = zx[nlak + ns] + IX(f->dz_lake, c, nlak, ld) / 2.0 + IX(f->z, c, jpjj, ld);
        cvx[ji] = cv[jpjj];
        phix[ji] = je == nlak + 1 ? phi_soil : 0.0;
        tx[ji] = IX(f->t_soisno, c, jpjj, ld);
      }
    }
    /* _lake_tkix_kernel! */
    for (int ji = 1; ji <= ntot; ji++) {
      int je = ji - ns, jj = je + ns;
      if (je < jtop) continue;
      if (je < 0) {
        tkix[ji] = tk[jj];
      } else if (je == 0) {
        double dzp = zx[ji + 1] - zx[ji];
        tkix[ji] = tk_lake[1] * tk[jj] * dzp / (tk[jj] * IX(f->z_lake, c, 1, ld) + tk_lake[1] * (-IX(f->z, c, jj, ld)));
      } else if (je < nlak) {
        tkix[ji] = (tk_lake[je] * tk_lake[je + 1] * (IX(f->dz_lake, c, je + 1, ld) + IX(f->dz_lake, c, je, ld))) /
                   (tk_lake[je] * IX(f->dz_lake, c, je + 1, ld) + tk_lake[je + 1] * IX(f->dz_lake, c, je, ld));
      } else if (je == nlak) {
        double dzp = zx[ji + 1] - zx[ji];
        tkix[ji] = tktopsoillay * tk_lake[je] * dzp /
                   (tktopsoillay * IX(f->dz_lake, c, je, ld) / 2.0 + tk_lake[je] * IX(f->z, c, 1 + ns, ld));
      } else {
        tkix[ji] = tk[je - nlak + ns];
      }
    }
    /* _lake_tridiag_factors_kernel!, _lake_tridiag_coeffs_kernel! */
    for (int ji = 1; ji <= ntot; ji++) {
      int je = ji - ns;
      if (je < jtop) continue;
      factx[ji] = dtime / cvx[ji];
      fnx[ji] = je < nlak + ngr ? tkix[ji] * (tx[ji + 1] - tx[ji]) / (zx[ji + 1] - zx[ji]) : 0.0;
    }
    const double omc = 1.0 - CNFAC;
    for (int ji = 1; ji <= ntot; ji++) {
      int je = ji - ns;
      if (je < jtop) continue;
      if (je == jtop) {
        double dzp = zx[ji + 1] - zx[ji];
        a[ji] = 0.0;
        bb[ji] = 1.0 + omc * factx[ji] * tkix[ji] / dzp;
        c1[ji] = -omc * factx[ji] * tkix[ji] / dzp;
        r[ji] = tx[ji] + factx[ji] * (fin + phix[ji] + CNFAC * fnx[ji]);
      } else if (je < nlak + ngr) {
        double dzm = zx[ji] - zx[ji - 1], dzp = zx[ji + 1] - zx[ji];
        a[ji] = -omc * factx[ji] * tkix[ji - 1] / dzm;
        bb[ji] = 1.0 + omc * factx[ji] * (tkix[ji] / dzp + tkix[ji - 1] / dzm);
        c1[ji] = -omc * factx[ji] * tkix[ji] / dzp;
        r[ji] = tx[ji] + CNFAC * factx[ji] * (fnx[ji] - fnx[ji - 1]) + factx[ji] * phix[ji];
      } else {
        double dzm = zx[ji] - zx[ji - 1];
        a[ji] = -omc * factx[ji] * tkix[ji - 1] / dzm;
        bb[ji] = 1.0 + omc * factx[ji] * tkix[ji - 1] / dzm;
        c1[ji] = 0.0;
        r[ji] = tx[ji] - CNFAC * factx[ji] * fnx[ji - 1];
      }
    }
    /* tridiagonal_multi! (tridiagonal.jl:86-127) from jtop + nlevsno */
    {
      int j0 = (int)jtop + ns;
      double cp[LK_MAXX], dp[LK_MAXX];
      const double tiny = 1e-30;
      double bet = bb[j0];
      if (fabs(bet) < tiny) bet = tiny;
      double cpp = c1[j0] / bet, dpp = r[j0] / bet;
      cp[j0] = cpp;
      dp[j0] = dpp;
      for (int jj = j0 + 1; jj <= ntot; jj++) {
        double denom = bb[jj] - a[jj] * cpp;
        if (fabs(denom) < tiny) denom = copysign(tiny, denom == 0.0 ? 1.0 : denom);
        cpp = c1[jj] / denom;
        dpp = (r[jj] - a[jj] * dpp) / denom;
        cp[jj] = cpp;
        dp[jj] = dpp;
      }
      double un = dpp;
      tx[ntot] = un;
      for (int jj = ntot - 1; jj >= j0; jj--) {
        un = dp[jj] - cp[jj] * un;
        tx[jj] = un;
      }
    }
    /* _lake_unpack_kernel! */
    for (int ji = 1; ji <= ntot; ji++) {
      int je = ji - ns;
      if (je < jtop) continue;
      if (je < 1) IX(f->t_soisno, c, je + ns, ld) = tx[ji];
      else if (je <= nlak) IX(f->t_lake, c, je, ld) = tx[ji];
      else IX(f->t_soisno, c, je - nlak + ns, ld) = tx[ji];
    }
    /* phase_change_lake! (_phase_change_lake_water_kernel!, _soil_kernel!, :204-314) */
    {
      const double small = 1.0e-12;
      double qsm = 0.0, qsd = 0.0, lh = 0.0, qsf = 0.0;
      for (int jj = 1; jj <= ns; jj++) {
        IX(f->qflx_snomelt_lyr, c, jj, ld) = 0.0;
        IX(f->qflx_snofrz_lyr, c, jj, ld) = 0.0;
        IX(f->imelt, c, jj, ld) = 0;
      }
      if (f->h2osno_no_layers[c] > 0.0 && IX(f->t_lake, c, 1, ld) > TFRZ) {
        double heatavail = (IX(f->t_lake, c, 1, ld) - TFRZ) * cv_lake[1];
        double melt = jl_min(f->h2osno_no_layers[c], heatavail / HFUS);
        double heatrem = jl_max(heatavail - melt * HFUS, 0.0);
        IX(f->t_lake, c, 1, ld) = TFRZ + heatrem / cv_lake[1];
        f->snow_depth[c] = f->snow_depth[c] * (1.0 - melt / f->h2osno_no_layers[c]);
        f->h2osno_no_layers[c] = f->h2osno_no_layers[c] - melt;
        lh += melt * HFUS;
        qsm += melt / dtime;
        qsd += melt / dtime;
        if (f->h2osno_no_layers[c] < small) f->h2osno_no_layers[c] = 0.0;
        if (f->snow_depth[c] < small) f->snow_depth[c] = 0.0;
      }
      for (int j = 1; j <= nlak; j++) {
        int dophase = 0;
        double heatavail = 0.0, melt = 0.0, heatrem = 0.0;
        double tl = IX(f->t_lake, c, j, ld), fi = IX(f->lake_icefrac, c, j, ld), dzl = IX(f->dz_lake, c, j, ld);
        if (tl > TFRZ && fi > 0.0) {
          dophase = 1;
          heatavail = (tl - TFRZ) * cv_lake[j];
          melt = jl_min(fi * DENH2O * dzl, heatavail / HFUS);
          heatrem = jl_max(heatavail - melt * HFUS, 0.0);
        } else if (tl < TFRZ && fi < 1.0) {
          dophase = 1;
          heatavail = (tl - TFRZ) * cv_lake[j];
          melt = jl_max(-(1.0 - fi) * DENH2O * dzl, heatavail / HFUS);
          heatrem = jl_min(heatavail - melt * HFUS, 0.0);
        }
        if (dophase) {
          IX(f->lake_icefrac, c, j, ld) = fi - melt / (DENH2O * dzl);
          lh += melt * HFUS;
          cv_lake[j] = cv_lake[j] + melt * (CPLIQ - CPICE);
          IX(f->t_lake, c, j, ld) = TFRZ + heatrem / cv_lake[j];
          if (IX(f->lake_icefrac, c, j, ld) > 1.0 - small) IX(f->lake_icefrac, c, j, ld) = 1.0;
          if (IX(f->lake_icefrac, c, j, ld) < small) IX(f->lake_icefrac, c, j, ld) = 0.0;
        }
      }
      for (int j = -ns + 1; j <= ngr; j++) {
        int jj = j + ns;
        if (j < snl + 1) continue;
        int dophase = 0;
        double heatavail = 0.0, melt = 0.0, heatrem = 0.0;
        double t = IX(f->t_soisno, c, jj, ld);
        if (t > TFRZ && IX(f->h2osoi_ice, c, jj, ld) > 0.0) {
          dophase = 1;
          heatavail = (t - TFRZ) * cv[jj];
          melt = jl_min(IX(f->h2osoi_ice, c, jj, ld), heatavail / HFUS);
          heatrem = jl_max(heatavail - melt * HFUS, 0.0);
          if (j <= 0) {
            IX(f->imelt, c, jj, ld) = 1;
            IX(f->qflx_snomelt_lyr, c, jj, ld) = melt / dtime;
            qsm += IX(f->qflx_snomelt_lyr, c, jj, ld);
          }
        } else if (t < TFRZ && IX(f->h2osoi_liq, c, jj, ld) > 0.0) {
          dophase = 1;
          heatavail = (t - TFRZ) * cv[jj];
          melt = jl_max(-IX(f->h2osoi_liq, c, jj, ld), heatavail / HFUS);
          heatrem = jl_min(heatavail - melt * HFUS, 0.0);
          if (j <= 0) {
            IX(f->imelt, c, jj, ld) = 2;
            IX(f->qflx_snofrz_lyr, c, jj, ld) = -melt / dtime;
            qsf += IX(f->qflx_snofrz_lyr, c, jj, ld);
          }
        }
        if (dophase) {
          IX(f->h2osoi_ice, c, jj, ld) = IX(f->h2osoi_ice, c, jj, ld) - melt;
          IX(f->h2osoi_liq, c, jj, ld) = IX(f->h2osoi_liq, c, jj, ld) + melt;
          lh += melt * HFUS;
          cv[jj] = cv[jj] + melt * (CPLIQ - CPICE);
          IX(f->t_soisno, c, jj, ld) = TFRZ + heatrem / cv[jj];
          if (IX(f->h2osoi_ice, c, jj, ld) < small) IX(f->h2osoi_ice, c, jj, ld) = 0.0;
          if (IX(f->h2osoi_liq, c, jj, ld) < small) IX(f->h2osoi_liq, c, jj, ld) = 0.0;
        }
      }
      lhabs = lh;
      f->qflx_snomelt[c] = qsm;
      f->qflx_snofrz[c] = qsf;
      f->qflx_snow_drain[c] = qsd;
      f->eflx_snomelt[c] = qsm * HFUS;
    }
    (void)lhabs;
    /* convective mixing: density, puddling, top-down then bottom-up (:1204-1241) */
    for (int j = 1; j <= nlak; j++) rhow[j] = lake_rhow(IX(f->lake_icefrac, c, j, ld), IX(f->t_lake, c, j, ld));
    if (puddling) {
      double icesum = 0.0;
      for (int j = 1; j <= nlak; j++) icesum = icesum + IX(f->lake_icefrac, c, j, ld) * IX(f->dz, c, j + ns, ld);
      puddle = icesum >= pudz;
    }
    for (int j = 1; j <= nlak - 2; j++) {
      int doconv = (!puddling || !puddle) &&
                   (rhow[j] > rhow[j + 1] ||
                    (IX(f->lake_icefrac, c, j, ld) < 1.0 && IX(f->lake_icefrac, c, j + 1, ld) > 0.0));
      if (!doconv) continue;
      if (lch4) jconvect = j + 1;
      lake_mix(f, c, ld, 1, j + 1, rhow, cwat, cice_eff);
    }
    {
      int jb = nlak - 1;
      if ((!puddling || !puddle) &&
          (rhow[jb] > rhow[jb + 1] || (IX(f->lake_icefrac, c, jb, ld) < 1.0 && IX(f->lake_icefrac, c, jb + 1, ld) > 0.0)))
        bottomconvect = 1;
    }
    for (int j = nlak - 1; j >= 1; j--) {
      int doconv = bottomconvect && (!puddling || !puddle) &&
                   (rhow[j] > rhow[j + 1] ||
                    (IX(f->lake_icefrac, c, j, ld) < 1.0 && IX(f->lake_icefrac, c, j + 1, ld) > 0.0));
      if (!doconv) continue;
      if (lch4) jconvectbot = j;
      lake_mix(f, c, ld, j, nlak, rhow, cwat, cice_eff);
    }
    /* _lake_ch4_kernel! */
    if (lch4) {
      double lr = f->lakeresist[c];
      for (int j = 1; j <= nlak; j++)
        if (j > jconvect && j < jconvectbot) lr += IX(f->dz_lake, c, j, ld) / kme[j];
      f->lakeresist[c] = lr;
      double gc = 1.0 / (lr + f->lake_raw[c]);
      if (IX(f->lake_icefrac, c, 1, ld) > 0.1) gc = 0.0;
      f->grnd_ch4_cond[c] = gc;
    }
    /* re-evaluated properties and the energy after (:1250-1267) */
    for (int j = 1; j <= nlak; j++) {
      double fi = IX(f->lake_icefrac, c, j, ld);
      cv_lake[j] = IX(f->dz_lake, c, j, ld) * (cwat * (1.0 - fi) + cice_eff * fi);
    }
    lake_therm_prop(vp, f, c, ld, tk, cv, &tktopsoillay);
    for (int j = 1; j <= nlak; j++) {
      ncvts += cv_lake[j] * (IX(f->t_lake, c, j, ld) - TFRZ) +
               cfus * IX(f->dz_lake, c, j, ld) * (1.0 - IX(f->lake_icefrac, c, j, ld));
      fin += phi[j];
    }
    h2osno_total = lake_h2osno_total(vp, f, c, ld);
    for (int j = -ns + 1; j <= ngr; j++) {
      int jj = j + ns;
      if (j >= jtop) {
        ncvts += cv[jj] * (IX(f->t_soisno, c, jj, ld) - TFRZ) + HFUS * IX(f->h2osoi_liq, c, jj, ld);
        if (j < 1) fin += phix[j + ns];
        if (j == 1 && h2osno_total > 0.0 && j == jtop) ncvts -= h2osno_total * HFUS;
      }
      if (j == 1) fin += phi_soil;
    }
    /* _lake_energy_conservation_kernel!, _lake_icethick_kernel! */
    if (pact) {
      double err = (ncvts - ocvts) / dtime - fin;
      if (fabs(err) < 0.10) {
        f->eflx_sh_tot[p] -= err;
        f->eflx_sh_grnd[p] -= err;
        f->eflx_soil_grnd[p] += err;
        f->eflx_gnet[p] += err;
        err = 0.0;
      }
      f->errsoi_col[c] = err;
    }
    double thick = 0.0;
    for (int j = 1; j <= nlak; j++) {
      if (j == 1) f->lake_icefracsurf[c] = IX(f->lake_icefrac, c, 1, ld);
      thick += IX(f->lake_icefrac, c, j, ld) * IX(f->dz_lake, c, j, ld) * DENH2O / DENICE;
    }
    f->lake_icethick[c] = thick;
  }
  return 0;
}

/* ===================================================================== */
/* balance_check!'s column checks (balance_check.jl:723-770, 1124-1365)  */
/* ===================================================================== */
int orc_balance_check_columns(const clmgb_bounds* b, const clmgb_colbalance_fields* f, double dtime,
                              clmgb_balance_report* rep)
{
  const int64_t nc = b->nc;
  memset(rep, 0, sizeof(*rep));
  /* _bc_forc_rainsnow_kernel!, _bc_errh2o_col_kernel! */
  for (int64_t c = 0; c < nc; c++) {
    double rain = f->forc_rain[c], snow = f->forc_snow[c];
    if (f->col_itype[c] == ICOL_SUNWALL || f->col_itype[c] == ICOL_SHADEWALL) rain = snow = 0.0;
    if (f->col_active[c])
      f->errh2o[c] = f->endwb[c] - f->begwb[c] -
                     (rain + snow + f->qflx_flood[c] + f->qflx_sfc_irrig[c] + f->qflx_glcice_dyn_water_flux[c] -
                      f->qflx_evap_tot[c] - f->qflx_surf[c] - f->qflx_qrgwl[c] - f->qflx_drain[c] -
                      f->qflx_drain_perched[c] - f->qflx_ice_runoff[c] - f->qflx_snwcp_discarded_liq[c] -
                      f->qflx_snwcp_discarded_ice[c]) * dtime;
    else
      f->errh2o[c] = 0.0;
  }
  if (nc == 0) return 0;
  /* the scans: first non-finite, then maximum(abs.(...)) and its first index, where a
   * NaN is the maximum (Julia's findmax) */
  double m = -1.0;
  int64_t im = 0;
  for (int64_t c = 0; c < nc; c++) {
    double a = fabs(f->errh2o[c]);
    if (!isfinite(f->errh2o[c]) && !rep->errh2o_nonfinite) rep->errh2o_nonfinite = c + 1;
    if (isnan(m)) continue;
    if (isnan(a) || a > m) { m = a; im = c + 1; }
  }
  rep->errh2o_max = m;
  rep->errh2o_index = im;
  if (m > 1.0e-9) rep->flags |= CLMGB_BAL_H2O_WARN;
  if (m > 1.0e-5) rep->flags |= CLMGB_BAL_H2O_ERROR;
  if (rep->errh2o_nonfinite) rep->flags |= CLMGB_BAL_H2O_NONFINITE;
  if (f->errsoi) {
    double ms = -1.0;
    int64_t is = 0;
    for (int64_t c = 0; c < nc; c++) {
      double a = f->col_active[c] ? fabs(f->errsoi[c]) : 0.0;
      if (isnan(ms)) continue;
      if (isnan(a) || a > ms) { ms = a; is = c + 1; }
    }
    rep->errsoi_max = ms;
    rep->errsoi_index = is;
    if (ms > 1.0e-5) rep->flags |= CLMGB_BAL_SOI_WARN;
    if (ms > 1.0e-4) rep->flags |= CLMGB_BAL_SOI_ERROR;
  }
  return 0;
}

/* ===================================================================== */
/* soil_fluxes! (soil_fluxes.jl:553-697), loop by loop                    */
/* ===================================================================== */
int orc_soil_fluxes(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_soilflux_fields* f, double dtime)
{
  int e = check_varpar(vp);
  if (e) return e;
  const int64_t nc = b->nc, np = b->np, ld = b->ldc;
  const int nlevsno = vp->nlevsno;
  const double hvap = 2.501e6, sb = 5.67e-8;
  double* tinc = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  double* t_grnd0 = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  double* lwrad_del = (double*)calloc((size_t)(np > 0 ? np : 1), sizeof(double));
  /* _soilflux_tinc_kernel! (:19-41) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_nolakec[c]) continue;
    int64_t snl = f->col_snl[c];
    if (snl < 0)
      t_grnd0[c] = f->frac_sno_eff[c] * IX(f->t_ssbef, c, snl + 1 + nlevsno, ld) +
                   (1.0 - f->frac_sno_eff[c] - f->frac_h2osfc[c]) * IX(f->t_ssbef, c, 1 + nlevsno, ld) +
                   f->frac_h2osfc[c] * f->t_h2osfc_bef[c];
    else
      t_grnd0[c] = (1.0 - f->frac_h2osfc[c]) * IX(f->t_ssbef, c, 1 + nlevsno, ld) + f->frac_h2osfc[c] * f->t_h2osfc_bef[c];
    tinc[c] = f->t_grnd[c] - t_grnd0[c];
  }
  /* _soilflux_correct_kernel! (:51-76) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_nolakep[p]) continue;
    int64_t c = f->patch_column[p] - 1, l = f->patch_landunit[p] - 1;
    f->eflx_sh_grnd[p] += tinc[c] * f->cgrnds[p];
    f->qflx_evap_soi[p] += tinc[c] * f->cgrndl[p];
    if (f->lun_urbpoi[l]) {
      f->qflx_ev_soil[p] = 0.0;
      f->qflx_ev_h2osfc[p] = 0.0;
      f->qflx_ev_snow[p] = f->qflx_evap_soi[p];
    } else {
      f->qflx_ev_snow[p] += tinc[c] * f->cgrndl[p];
      f->qflx_ev_soil[p] += tinc[c] * f->cgrndl[p];
      f->qflx_ev_h2osfc[p] += tinc[c] * f->cgrndl[p];
    }
  }
  /* _soilflux_partition_kernel! (:181-240) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_nolakep[p]) continue;
    int64_t c = f->patch_column[p] - 1, l = f->patch_landunit[p] - 1;
    int64_t jj = f->col_snl[c] + 1 + nlevsno;
    f->qflx_liqevap_from_top_layer[p] = 0.0;
    f->qflx_solidevap_from_top_layer[p] = 0.0;
    f->qflx_soliddew_to_top_layer[p] = 0.0;
    f->qflx_liqdew_to_top_layer[p] = 0.0;
    double liq = IX(f->h2osoi_liq, c, jj, ld), ice = IX(f->h2osoi_ice, c, jj, ld);
    double ev = f->lun_urbpoi[l] ? f->qflx_evap_soi[p] : f->qflx_ev_snow[p];
    if (ev >= 0.0) {
      if ((liq + ice) > 0.0) f->qflx_liqevap_from_top_layer[p] = jl_max(ev * (liq / (liq + ice)), 0.0);
      else f->qflx_liqevap_from_top_layer[p] = 0.0;
      f->qflx_solidevap_from_top_layer[p] = ev - f->qflx_liqevap_from_top_layer[p];
    } else {
      if (f->t_grnd[c] < TFRZ) f->qflx_soliddew_to_top_layer[p] = fabs(ev);
      else f->qflx_liqdew_to_top_layer[p] = fabs(ev);
    }
  }
  /* _soilflux_evaplimit_kernel! (:242-300) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_nolakep[p]) continue;
    int64_t c = f->patch_column[p] - 1, l = f->patch_landunit[p] - 1;
    int64_t j = f->col_snl[c] + 1, jj = j + nlevsno;
    double liq = IX(f->h2osoi_liq, c, jj, ld), ice = IX(f->h2osoi_ice, c, jj, ld);
    double fse = f->frac_sno_eff[c];
    if (j < 1) {
      double lim = (ice + liq) / (fse * dtime);
      if (f->qflx_ev_snow[p] > lim) {
        double dem = f->qflx_ev_snow[p];
        f->qflx_ev_snow[p] = lim;
        f->qflx_evap_soi[p] -= fse * (dem - lim);
        f->qflx_liqevap_from_top_layer[p] = jl_max(liq / (fse * dtime), 0.0);
        f->qflx_solidevap_from_top_layer[p] = jl_max(ice / (fse * dtime), 0.0);
        f->eflx_sh_grnd[p] += fse * (dem - lim) * f->htvp[c];
      }
    }
    if (f->lun_urbpoi[l] && f->col_itype[c] != ICOL_ROAD_PERV && j == 1) {
      double lim = (ice + liq) / dtime;
      if (f->qflx_evap_soi[p] > lim) {
        double dem = f->qflx_evap_soi[p];
        f->qflx_evap_soi[p] = lim;
        f->qflx_ev_snow[p] = f->qflx_evap_soi[p];
        f->qflx_liqevap_from_top_layer[p] = jl_max(liq / dtime, 0.0);
        f->qflx_solidevap_from_top_layer[p] = jl_max(ice / dtime, 0.0);
        f->eflx_sh_grnd[p] += (dem - lim) * f->htvp[c];
      }
    }
    if (j == 1 && f->frac_h2osfc[c] < 1.0) {
      double lim = ice / (dtime * (1.0 - f->frac_h2osfc[c]));
      if (f->qflx_solidevap_from_top_layer[p] >= lim) {
        double dem = f->qflx_solidevap_from_top_layer[p];
        f->qflx_solidevap_from_top_layer[p] = lim;
        f->qflx_liqevap_from_top_layer[p] += (dem - lim);
      }
    }
  }
  /* _soilflux_totals_kernel! (:303-378) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_nolakep[p]) continue;
    int64_t c = f->patch_column[p] - 1, l = f->patch_landunit[p] - 1;
    int64_t lit = f->lun_itype[l];
    double fse = f->frac_sno_eff[c], fh = f->frac_h2osfc[c], emg = f->emg[c], tg0 = t_grnd0[c];
    if (!f->lun_urbpoi[l]) {
      double lw = fse * jl_pow4(IX(f->t_ssbef, c, f->col_snl[c] + 1 + nlevsno, ld)) +
                  (1.0 - fse - fh) * jl_pow4(IX(f->t_ssbef, c, 1 + nlevsno, ld)) + fh * jl_pow4(f->t_h2osfc_bef[c]);
      f->eflx_soil_grnd[p] = ((1.0 - fse) * f->sabg_soil[p] + fse * f->sabg_snow[p]) + f->dlrad[p] +
                             (1.0 - (double)f->frac_veg_nosno[p]) * emg * f->forc_lwrad[c] - emg * sb * lw -
                             emg * sb * (tg0 * tg0 * tg0) * (4.0 * tinc[c]) -
                             (f->eflx_sh_grnd[p] + f->qflx_evap_soi[p] * f->htvp[c]);
      if (lit == ISTSOIL || lit == ISTCROP) f->eflx_soil_grnd_r[p] = f->eflx_soil_grnd[p];
    } else {
      lwrad_del[p] = 4.0 * emg * sb * (tg0 * tg0 * tg0) * tinc[c];
      f->eflx_soil_grnd[p] = f->sabg[p] + f->dlrad[p] - f->eflx_lwrad_net[p] - lwrad_del[p] -
                             (f->eflx_sh_grnd[p] + f->qflx_evap_soi[p] * f->htvp[c] + f->qflx_tran_veg[p] * hvap) +
                             f->eflx_wasteheat[p] + f->eflx_heat_from_ac[p] + f->eflx_traffic[p] + f->eflx_ventilation[p];
      f->eflx_soil_grnd_u[p] = f->eflx_soil_grnd[p];
    }
    f->eflx_sh_tot[p] = f->eflx_sh_veg[p] + f->eflx_sh_grnd[p];
    if (!f->lun_urbpoi[l]) f->eflx_sh_tot[p] += f->eflx_sh_stem[p];
    f->qflx_evap_tot[p] = f->qflx_evap_veg[p] + f->qflx_evap_soi[p];
    f->eflx_lh_tot[p] = hvap * f->qflx_evap_veg[p] + f->htvp[c] * f->qflx_evap_soi[p];
    if (lit == ISTSOIL || lit == ISTCROP) {
      f->eflx_lh_tot_r[p] = f->eflx_lh_tot[p];
      f->eflx_sh_tot_r[p] = f->eflx_sh_tot[p];
    } else if (f->lun_urbpoi[l]) {
      f->eflx_lh_tot_u[p] = f->eflx_lh_tot[p];
      f->eflx_sh_tot_u[p] = f->eflx_sh_tot[p];
    }
    f->qflx_evap_can[p] = f->qflx_evap_veg[p] - f->qflx_tran_veg[p];
    f->eflx_lh_vege[p] = (f->qflx_evap_veg[p] - f->qflx_tran_veg[p]) * hvap;
    f->eflx_lh_vegt[p] = f->qflx_tran_veg[p] * hvap;
    f->eflx_lh_grnd[p] = f->qflx_evap_soi[p] * f->htvp[c];
  }
  /* _soilflux_errsoi_base_kernel! (:380-407) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_nolakep[p]) continue;
    int64_t c = f->patch_column[p] - 1;
    f->errsoi_patch[p] = f->eflx_soil_grnd[p] - f->xmf[c] - f->xmf_h2osfc[c] -
                         f->frac_h2osfc[c] * (f->t_h2osfc[c] - f->t_h2osfc_bef[c]) * (f->c_h2osfc[c] / dtime);
    f->errsoi_patch[p] += f->eflx_h2osfc_to_snow[c];
    if (col_is_wallroof(f->col_itype[c])) f->errsoi_patch[p] += f->eflx_building_heat_errsoi[c];
  }
  /* _soilflux_errsoi_layers_kernel! (:425-453): non-urban then urban */
  for (int pass = 0; pass < 2; pass++) {
    const uint8_t* mask = pass == 0 ? f->mask_nolakep : f->mask_urbanp;
    int jmax = pass == 0 ? vp->nlevgrnd : vp->nlevurb;
    for (int64_t p = 0; p < np; p++) {
      if (!mask[p]) continue;
      int64_t c = f->patch_column[p] - 1;
      int wr = col_is_wallroof(f->col_itype[c]);
      if ((pass == 1) != (wr != 0)) continue;
      for (int jf = -nlevsno + 1; jf <= jmax; jf++) {
        int jl = jf + nlevsno;
        if (jf >= f->col_snl[c] + 1 && jf < 1)
          f->errsoi_patch[p] -= f->frac_sno_eff[c] * (IX(f->t_soisno, c, jl, ld) - IX(f->t_ssbef, c, jl, ld)) / IX(f->fact, c, jl, ld);
        if (jf >= 1)
          f->errsoi_patch[p] -= (IX(f->t_soisno, c, jl, ld) - IX(f->t_ssbef, c, jl, ld)) / IX(f->fact, c, jl, ld);
      }
    }
  }
  /* _soilflux_lwrad_kernel! (:455-497) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_nolakep[p]) continue;
    int64_t c = f->patch_column[p] - 1, l = f->patch_landunit[p] - 1;
    int64_t lit = f->lun_itype[l];
    double fse = f->frac_sno_eff[c], fh = f->frac_h2osfc[c], emg = f->emg[c], tg0 = t_grnd0[c];
    double fvn = (double)f->frac_veg_nosno[p];
    if (!f->lun_urbpoi[l]) {
      double lw = fse * jl_pow4(IX(f->t_ssbef, c, f->col_snl[c] + 1 + nlevsno, ld)) +
                  (1.0 - fse - fh) * jl_pow4(IX(f->t_ssbef, c, 1 + nlevsno, ld)) + fh * jl_pow4(f->t_h2osfc_bef[c]);
      f->eflx_lwrad_out[p] = f->ulrad[p] + (1.0 - fvn) * (1.0 - emg) * f->forc_lwrad[c] + (1.0 - fvn) * emg * sb * lw +
                             4.0 * emg * sb * (tg0 * tg0 * tg0) * tinc[c];
      if (fvn == 0.0) f->t_skin[p] = sqrt(sqrt(lw));
      f->eflx_lwrad_net[p] = f->eflx_lwrad_out[p] - f->forc_lwrad[c];
      if (lit == ISTSOIL || lit == ISTCROP) {
        f->eflx_lwrad_net_r[p] = f->eflx_lwrad_out[p] - f->forc_lwrad[c];
        f->eflx_lwrad_out_r[p] = f->eflx_lwrad_out[p];
      }
    } else {
      f->eflx_lwrad_out[p] += lwrad_del[p];
      f->eflx_lwrad_net[p] += lwrad_del[p];
      f->eflx_lwrad_net_u[p] += lwrad_del[p];
      f->eflx_lwrad_out_u[p] = f->eflx_lwrad_out[p];
    }
  }
  /* _soilflux_errsoi_zero_kernel! and _p2c_kernel! (:499-524), in patch order */
  for (int64_t c = 0; c < nc; c++)
    if (f->mask_nolakec[c]) f->errsoi_col[c] = 0.0;
  for (int64_t p = 0; p < np; p++) {
    int64_t c = f->patch_column[p] - 1;
    if (c >= 0 && f->mask_nolakec[c] && f->col_patchi[c] <= p + 1 && p + 1 <= f->col_patchf[c])
      f->errsoi_col[c] += f->errsoi_patch[p] * f->patch_wtcol[p];
  }
  /* _soilflux_urban_tskin_kernel! (:526-534) */
  for (int64_t p = 0; p < np; p++) {
    if (!f->mask_urbanp[p]) continue;
    int64_t c = f->patch_column[p] - 1;
    f->t_skin[p] = IX(f->t_soisno, c, f->col_snl[c] + 1 + nlevsno, ld);
  }
  free(tinc);
  free(t_grnd0);
  free(lwrad_del);
  return 0;
}

/* ===================================================================== */
/* soilwater_zengdecker2009! (soil_water_movement.jl:1616-1764): the ten  */
/* stages as the reference runs them, each over every column, with       */
/* [nc, nlevsoi+1] scratch matrices (SC(a, c, j) = a[c*n1 + j], j 1-based) */
/* ===================================================================== */
#define SC(a, c, j) ((a)[(int64_t)(c) * n1 + (j)])

int orc_soil_water_zd09(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_zd09_fields* f,
                        double e_ice, double dtime)
{
  int e = check_varpar(vp);
  if (e) return e;
  const int64_t nc = b->nc, ld = b->ldc;
  const int nlevsoi = vp->nlevsoi, nlevgrnd = vp->nlevgrnd, joff = vp->nlevsno, joff_zi = vp->nlevsno + 1;
  const int64_t n1 = nlevsoi + 3;
  const double sdamp = 0.0;
  enum { ZMM, DZMM, ZIMM, ICEF, VWC, VOLEQ, ZQ, HK, DHKDW, SMP, DSMPDW, IMPED, QIN, QOUT, DQIDW0, DQIDW1,
         DQODW1, DQODW2, AMX, BMX, CMX, RMX, DWAT2, CP, NMAT };
  double* M[NMAT];
  for (int k = 0; k < NMAT; k++) M[k] = (double*)calloc((size_t)(nc > 0 ? nc : 1) * n1, sizeof(double));
  double* zwtmm = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  double* vwc_zwt = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  int* jwt = (int*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(int));
  /* _soilwm_mm_icefrac_kernel! (:97-127) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    for (int j = 1; j <= nlevsoi; j++) {
      SC(M[ZMM], c, j) = IX(f->z, c, joff + j, ld) * 1.0e3;
      SC(M[DZMM], c, j) = IX(f->dz, c, joff + j, ld) * 1.0e3;
      SC(M[ZIMM], c, j + 1) = IX(f->zi, c, joff_zi + j, ld) * 1.0e3;
      double vol_ice = jl_min(IX(f->watsat, c, j, ld), IX(f->h2osoi_ice, c, joff + j, ld) / (IX(f->dz, c, joff + j, ld) * DENICE));
      SC(M[ICEF], c, j) = jl_min(1.0, vol_ice / IX(f->watsat, c, j, ld));
      IX(f->icefrac, c, j, ld) = SC(M[ICEF], c, j);
      SC(M[VWC], c, j) = jl_max(IX(f->h2osoi_liq, c, joff + j, ld), 1.0e-6) / (IX(f->dz, c, joff + j, ld) * DENH2O);
    }
  }
  /* _soilwm_zwtmm_kernel! (:143-150) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    SC(M[ZIMM], c, 1) = 0.0;
    zwtmm[c] = f->zwt[c] * 1.0e3;
  }
  /* _soilwm_jwt_vwczwt_kernel! (:289-327) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    int jw = nlevsoi;
    for (int j = 1; j <= nlevsoi; j++)
      if (f->zwt[c] <= IX(f->zi, c, joff_zi + j, ld)) { jw = j - 1; break; }
    jwt[c] = jw;
    vwc_zwt[c] = IX(f->watsat, c, nlevsoi, ld);
    if (IX(f->t_soisno, c, joff + jw + 1, ld) < TFRZ) {
      double v = SC(M[VWC], c, nlevsoi);
      for (int j = nlevsoi; j <= nlevgrnd; j++) {
        if (f->zwt[c] <= IX(f->zi, c, joff_zi + j, ld)) {
          double t = IX(f->t_soisno, c, joff + j, ld);
          double smp1 = HFUS * (TFRZ - t) / (GRAV * t) * 1000.0;
          smp1 = jl_max(IX(f->sucsat, c, nlevsoi, ld), smp1);
          v = IX(f->watsat, c, nlevsoi, ld) * cm_pow(smp1 / IX(f->sucsat, c, nlevsoi, ld), -1.0 / IX(f->bsw, c, nlevsoi, ld));
          v = jl_min(v, 0.5 * (IX(f->watsat, c, nlevsoi, ld) + IX(f->h2osoi_vol, c, nlevsoi, ld)));
          break;
        }
      }
      vwc_zwt[c] = v;
    }
  }
  /* _soilwm_voleq_zq_kernel! (:171-205) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    for (int j = 1; j <= nlevsoi; j++) {
      double zm1 = SC(M[ZIMM], c, j), zj = SC(M[ZIMM], c, j + 1);
      double ws = IX(f->watsat, c, j, ld), suc = IX(f->sucsat, c, j, ld), bb = IX(f->bsw, c, j, ld);
      double zwt = zwtmm[c], onem1b = 1.0 - 1.0 / bb, v;
      if (zwt <= zm1) {
        SC(M[VOLEQ], c, j) = ws;
      } else if (zwt < zj && zwt > zm1) {
        double temp0 = cm_pow((suc + zwt - zm1) / suc, onem1b);
        double voleq1 = -suc * ws / onem1b / (zwt - zm1) * (1.0 - temp0);
        v = (voleq1 * (zwt - zm1) + ws * (zj - zwt)) / (zj - zm1);
        v = jl_min(ws, v);
        SC(M[VOLEQ], c, j) = jl_max(v, 0.0);
      } else {
        double tempi = cm_pow((suc + zwt - zj) / suc, onem1b);
        double temp0 = cm_pow((suc + zwt - zm1) / suc, onem1b);
        v = -suc * ws / onem1b / (zj - zm1) * (tempi - temp0);
        v = jl_max(v, 0.0);
        SC(M[VOLEQ], c, j) = jl_min(ws, v);
      }
      double zqv = -suc * cm_pow(jl_max(SC(M[VOLEQ], c, j) / ws, 0.01), -bb);
      SC(M[ZQ], c, j) = jl_max(f->smpmin[c], zqv);
    }
  }
  /* _soilwm_voleq_zq_aqu_kernel! (:346-366) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c] || jwt[c] != nlevsoi) continue;
    int j = nlevsoi;
    double suc = IX(f->sucsat, c, j, ld), ws = IX(f->watsat, c, j, ld), bb = IX(f->bsw, c, j, ld);
    double zwt = zwtmm[c], zj = SC(M[ZIMM], c, j + 1), onem1b = 1.0 - 1.0 / bb;
    double temp0 = cm_pow((suc + zwt - zj) / suc, onem1b);
    double v = -suc * ws / onem1b / (zwt - zj) * (1.0 - temp0);
    v = jl_max(v, 0.0);
    v = jl_min(ws, v);
    SC(M[VOLEQ], c, j + 1) = v;
    double zqv = -suc * cm_pow(jl_max(v / ws, 0.01), -bb);
    SC(M[ZQ], c, j + 1) = jl_max(f->smpmin[c], zqv);
  }
  /* _soilwm_hk_smp_kernel! (:223-270) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    for (int j = 1; j <= nlevsoi; j++) {
      int jp1 = j + 1 < nlevsoi ? j + 1 : nlevsoi;
      double bb = IX(f->bsw, c, j, ld);
      double s1 = 0.5 * (SC(M[VWC], c, j) + SC(M[VWC], c, jp1)) / (0.5 * (IX(f->watsat, c, j, ld) + IX(f->watsat, c, jp1, ld)));
      s1 = jl_min(1.0, s1);
      double s2 = IX(f->hksat, c, j, ld) * cm_pow(s1, 2.0 * bb + 2.0);
      double imp = cm_pow(10.0, -e_ice * (0.5 * (SC(M[ICEF], c, j) + SC(M[ICEF], c, jp1))));
      SC(M[IMPED], c, j) = imp;
      SC(M[HK], c, j) = imp * s1 * s2;
      SC(M[DHKDW], c, j) = imp * (2.0 * bb + 3.0) * s2 * (1.0 / (IX(f->watsat, c, j, ld) + IX(f->watsat, c, jp1, ld)));
      double s_node = jl_max(SC(M[VWC], c, j) / IX(f->watsat, c, j, ld), 0.01);
      s_node = jl_min(1.0, s_node);
      double smpv = -IX(f->sucsat, c, j, ld) * cm_pow(s_node, -bb);
      smpv = jl_max(f->smpmin[c], smpv);
      SC(M[SMP], c, j) = smpv;
      SC(M[DSMPDW], c, j) = -bb * smpv / SC(M[VWC], c, j);
      IX(f->smp_l, c, j, ld) = smpv;
      IX(f->hk_l, c, j, ld) = SC(M[HK], c, j);
    }
  }
  /* _soilwm_aqu_zmm_kernel! (:385-397) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    SC(M[ZMM], c, nlevsoi + 1) = 0.5 * (1.0e3 * f->zwt[c] + SC(M[ZMM], c, nlevsoi));
    if (jwt[c] < nlevsoi) SC(M[DZMM], c, nlevsoi + 1) = SC(M[DZMM], c, nlevsoi);
    else SC(M[DZMM], c, nlevsoi + 1) = 1.0e3 * f->zwt[c] - SC(M[ZMM], c, nlevsoi);
  }
  /* _soilwm_tridiag_assemble_kernel! (:430-539) */
#define A_(k, j) SC(M[k], c, j)
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    double den, dzq, num;
    int j = 1;
    A_(QIN, j) = f->qflx_infl[c];
    den = A_(ZMM, j + 1) - A_(ZMM, j);
    dzq = A_(ZQ, j + 1) - A_(ZQ, j);
    num = (A_(SMP, j + 1) - A_(SMP, j)) - dzq;
    A_(QOUT, j) = -A_(HK, j) * num / den;
    A_(DQODW1, j) = -(-A_(HK, j) * A_(DSMPDW, j) + num * A_(DHKDW, j)) / den;
    A_(DQODW2, j) = -(A_(HK, j) * A_(DSMPDW, j + 1) + num * A_(DHKDW, j)) / den;
    A_(RMX, j) = A_(QIN, j) - A_(QOUT, j) - IX(f->qflx_rootsoi, c, j, ld);
    A_(AMX, j) = 0.0;
    A_(BMX, j) = A_(DZMM, j) * (sdamp + 1.0 / dtime) + A_(DQODW1, j);
    A_(CMX, j) = A_(DQODW2, j);
    for (j = 2; j <= nlevsoi - 1; j++) {
      den = A_(ZMM, j) - A_(ZMM, j - 1);
      dzq = A_(ZQ, j) - A_(ZQ, j - 1);
      num = (A_(SMP, j) - A_(SMP, j - 1)) - dzq;
      A_(QIN, j) = -A_(HK, j - 1) * num / den;
      A_(DQIDW0, j) = -(-A_(HK, j - 1) * A_(DSMPDW, j - 1) + num * A_(DHKDW, j - 1)) / den;
      A_(DQIDW1, j) = -(A_(HK, j - 1) * A_(DSMPDW, j) + num * A_(DHKDW, j - 1)) / den;
      den = A_(ZMM, j + 1) - A_(ZMM, j);
      dzq = A_(ZQ, j + 1) - A_(ZQ, j);
      num = (A_(SMP, j + 1) - A_(SMP, j)) - dzq;
      A_(QOUT, j) = -A_(HK, j) * num / den;
      A_(DQODW1, j) = -(-A_(HK, j) * A_(DSMPDW, j) + num * A_(DHKDW, j)) / den;
      A_(DQODW2, j) = -(A_(HK, j) * A_(DSMPDW, j + 1) + num * A_(DHKDW, j)) / den;
      A_(RMX, j) = A_(QIN, j) - A_(QOUT, j) - IX(f->qflx_rootsoi, c, j, ld);
      A_(AMX, j) = -A_(DQIDW0, j);
      A_(BMX, j) = A_(DZMM, j) / dtime - A_(DQIDW1, j) + A_(DQODW1, j);
      A_(CMX, j) = A_(DQODW2, j);
    }
    j = nlevsoi;
    if (j > jwt[c]) {
      den = A_(ZMM, j) - A_(ZMM, j - 1);
      dzq = A_(ZQ, j) - A_(ZQ, j - 1);
      num = (A_(SMP, j) - A_(SMP, j - 1)) - dzq;
      A_(QIN, j) = -A_(HK, j - 1) * num / den;
      A_(DQIDW0, j) = -(-A_(HK, j - 1) * A_(DSMPDW, j - 1) + num * A_(DHKDW, j - 1)) / den;
      A_(DQIDW1, j) = -(A_(HK, j - 1) * A_(DSMPDW, j) + num * A_(DHKDW, j - 1)) / den;
      A_(QOUT, j) = 0.0;
      A_(DQODW1, j) = 0.0;
      A_(RMX, j) = A_(QIN, j) - A_(QOUT, j) - IX(f->qflx_rootsoi, c, j, ld);
      A_(AMX, j) = -A_(DQIDW0, j);
      A_(BMX, j) = A_(DZMM, j) / dtime - A_(DQIDW1, j) + A_(DQODW1, j);
      A_(CMX, j) = 0.0;
      A_(RMX, j + 1) = 0.0;
      A_(AMX, j + 1) = 0.0;
      A_(BMX, j + 1) = A_(DZMM, j + 1) / dtime;
      A_(CMX, j + 1) = 0.0;
    } else {
      double ws = IX(f->watsat, c, j, ld);
      double s_node = jl_max(0.5 * ((vwc_zwt[c] + A_(VWC, j)) / ws), 0.01);
      s_node = jl_min(1.0, s_node);
      double smp1 = -IX(f->sucsat, c, j, ld) * cm_pow(s_node, -IX(f->bsw, c, j, ld));
      smp1 = jl_max(f->smpmin[c], smp1);
      double dsmpdw1 = -IX(f->bsw, c, j, ld) * smp1 / (s_node * ws);
      den = A_(ZMM, j) - A_(ZMM, j - 1);
      dzq = A_(ZQ, j) - A_(ZQ, j - 1);
      num = (A_(SMP, j) - A_(SMP, j - 1)) - dzq;
      A_(QIN, j) = -A_(HK, j - 1) * num / den;
      A_(DQIDW0, j) = -(-A_(HK, j - 1) * A_(DSMPDW, j - 1) + num * A_(DHKDW, j - 1)) / den;
      A_(DQIDW1, j) = -(A_(HK, j - 1) * A_(DSMPDW, j) + num * A_(DHKDW, j - 1)) / den;
      den = A_(ZMM, j + 1) - A_(ZMM, j);
      dzq = A_(ZQ, j + 1) - A_(ZQ, j);
      num = (smp1 - A_(SMP, j)) - dzq;
      A_(QOUT, j) = -A_(HK, j) * num / den;
      A_(DQODW1, j) = -(-A_(HK, j) * A_(DSMPDW, j) + num * A_(DHKDW, j)) / den;
      A_(DQODW2, j) = -(A_(HK, j) * dsmpdw1 + num * A_(DHKDW, j)) / den;
      A_(RMX, j) = A_(QIN, j) - A_(QOUT, j) - IX(f->qflx_rootsoi, c, j, ld);
      A_(AMX, j) = -A_(DQIDW0, j);
      A_(BMX, j) = A_(DZMM, j) / dtime - A_(DQIDW1, j) + A_(DQODW1, j);
      A_(CMX, j) = A_(DQODW2, j);
      A_(QIN, j + 1) = A_(QOUT, j);
      A_(DQIDW0, j + 1) = -(-A_(HK, j) * A_(DSMPDW, j) + num * A_(DHKDW, j)) / den;
      A_(DQIDW1, j + 1) = -(A_(HK, j) * dsmpdw1 + num * A_(DHKDW, j)) / den;
      A_(QOUT, j + 1) = 0.0;
      A_(DQODW1, j + 1) = 0.0;
      A_(RMX, j + 1) = A_(QIN, j + 1) - A_(QOUT, j + 1);
      A_(AMX, j + 1) = -A_(DQIDW0, j + 1);
      A_(BMX, j + 1) = A_(DZMM, j + 1) / dtime - A_(DQIDW1, j + 1) + A_(DQODW1, j + 1);
      A_(CMX, j + 1) = 0.0;
    }
  }
  /* tridiagonal_multi! (tridiagonal.jl:86-127), jtop = 1, nlevs = nlevsoi + 1 */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    int n = nlevsoi + 1;
    double bet = A_(BMX, 1);
    if (fabs(bet) < 1.0e-30) bet = 1.0e-30;
    double cp_prev = A_(CMX, 1) / bet, dp_prev = A_(RMX, 1) / bet;
    A_(CP, 1) = cp_prev;
    A_(DWAT2, 1) = dp_prev;
    for (int jj = 2; jj <= n; jj++) {
      double denom = A_(BMX, jj) - A_(AMX, jj) * cp_prev;
      if (fabs(denom) < 1.0e-30) denom = copysign(1.0e-30, denom == 0.0 ? 1.0 : denom);
      cp_prev = A_(CMX, jj) / denom;
      dp_prev = (A_(RMX, jj) - A_(AMX, jj) * dp_prev) / denom;
      A_(CP, jj) = cp_prev;
      A_(DWAT2, jj) = dp_prev;
    }
    double u_next = dp_prev;
    A_(DWAT2, n) = u_next;
    for (int jj = n - 1; jj >= 1; jj--) {
      u_next = A_(DWAT2, jj) - A_(CP, jj) * u_next;
      A_(DWAT2, jj) = u_next;
    }
  }
  /* _soilwm_renew_qcharge_kernel! (:561-605) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    for (int j = 1; j <= nlevsoi; j++)
      IX(f->h2osoi_liq, c, joff + j, ld) = IX(f->h2osoi_liq, c, joff + j, ld) + A_(DWAT2, j) * A_(DZMM, j);
    int jw = jwt[c];
    if (jw < nlevsoi) {
      double wh_zwt = 0.0;
      double s_node = jl_max(IX(f->h2osoi_vol, c, jw + 1, ld) / IX(f->watsat, c, jw + 1, ld), 0.01);
      double s1 = jl_min(1.0, s_node);
      double ka = A_(IMPED, jw + 1) * IX(f->hksat, c, jw + 1, ld) * cm_pow(s1, 2.0 * IX(f->bsw, c, jw + 1, ld) + 3.0);
      int jm = jw > 1 ? jw : 1;
      double smp1 = jl_max(f->smpmin[c], A_(SMP, jm));
      double wh = smp1 - A_(ZQ, jm);
      if (jw == 0) f->qcharge[c] = -ka * (wh_zwt - wh) / ((f->zwt[c] + 1.0e-3) * 1000.0);
      else f->qcharge[c] = -ka * (wh_zwt - wh) / ((f->zwt[c] - IX(f->z, c, joff + jw, ld)) * 1000.0 * 2.0);
      f->qcharge[c] = jl_max(-10.0 / dtime, f->qcharge[c]);
      f->qcharge[c] = jl_min(10.0 / dtime, f->qcharge[c]);
    } else {
      f->qcharge[c] = A_(DWAT2, nlevsoi + 1) * A_(DZMM, nlevsoi + 1) / dtime;
    }
  }
#undef A_
  /* _soilwm_deficit_kernel! (:621-635) */
  for (int64_t c = 0; c < nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    double acc = 0.0;
    for (int j = 1; j <= nlevsoi; j++) {
      double l = IX(f->h2osoi_liq, c, joff + j, ld);
      acc = acc + (l >= 0.0 ? 0.0 : -l);
    }
    f->qflx_deficit[c] = acc;
  }
  for (int k = 0; k < NMAT; k++) free(M[k]);
  free(zwtmm);
  free(vwc_zwt);
  free(jwt);
  return 0;
}
#undef SC

/* ===================================================================== */
/* compute_effec_rootfrac_and_vert_tran_sink! (soil_water_plant_sink.jl)  */
/* ===================================================================== */
/* _plantsink_default_kernel! (:48-78) over one filter */
static void rootsink_default_filter(const clmgb_varpar* vp, const clmgb_bounds* b,
                                    const clmgb_rootsink_fields* f, const int64_t* filt, int64_t n)
{
  for (int64_t i = 0; i < n; i++) {
    const int64_t c = filt[i];
    const int64_t p_lo = f->col_patchi[c] - 1, p_hi = f->col_patchi[c] + f->col_npatches[c] - 2;
    double temp_c = 0.0;
    for (int64_t p = p_lo; p <= p_hi; p++)
      if (f->patch_active[p]) temp_c += f->qflx_tran_veg_patch[p] * f->patch_wtcol[p];
    for (int j = 1; j <= vp->nlevsoi; j++) {
      double acc = 0.0;
      for (int64_t p = p_lo; p <= p_hi; p++)
        if (f->patch_active[p]) acc += IX(f->rootr_patch, p, j, b->ldp) * f->qflx_tran_veg_patch[p] * f->patch_wtcol[p];
      if (temp_c != 0.0) acc /= temp_c;
      IX(f->rootr_col, c, j, b->ldc) = acc;
      IX(f->qflx_rootsoi_col, c, j, b->ldc) = acc * f->qflx_tran_veg_col[c];
    }
  }
}

/* _plantsink_hydstress_kernel! (:210-245) over one filter, root_idx = 4 */
static void rootsink_hydstress_filter(const clmgb_varpar* vp, const clmgb_bounds* b,
                                      const clmgb_rootsink_fields* f, const int64_t* filt, int64_t n)
{
  for (int64_t i = 0; i < n; i++) {
    const int64_t c = filt[i];
    const int64_t p_lo = f->col_patchi[c] - 1, p_hi = f->col_patchi[c] + f->col_npatches[c] - 2;
    f->qflx_phs_neg_col[c] = 0.0;
    for (int j = 1; j <= vp->nlevsoi; j++) {
      const double grav2 = IX(f->z, c, j + vp->nlevsno, b->ldc) * 1000.0;
      double temp_c = 0.0;
      for (int64_t p = p_lo; p <= p_hi; p++) {
        if (j == 1) f->qflx_hydr_redist_patch[p] = 0.0;
        if (f->patch_active[p] && f->frac_veg_nosno[p] > 0) {
          if (f->patch_wtcol[p] > 0.0) {
            const double patchflux = IX(f->k_soil_root_patch, p, j, b->ldp) *
                (IX(f->smp_l, c, j, b->ldc) - IX(f->vegwp_patch, p, 4, b->ldp) - grav2);
            if (patchflux < 0.0) f->qflx_hydr_redist_patch[p] += patchflux;
            temp_c += patchflux * f->patch_wtcol[p];
          }
        }
      }
      IX(f->qflx_rootsoi_col, c, j, b->ldc) = temp_c;
      if (temp_c < 0.0) f->qflx_phs_neg_col[c] += temp_c;
    }
  }
}

/* the wrapper (:341-451): three filters in order; returns 1 when the filter counts do
 * not add up to the hydrology columns (the reference's error) */
int orc_rootsink(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_rootsink_fields* f,
                 int32_t use_hydrstress)
{
  int e = check_varpar(vp);
  if (e) return e;
  int64_t* filt = (int64_t*)calloc((size_t)(b->nc > 0 ? b->nc : 1), sizeof(int64_t));
  int64_t n, total = 0, nhyd = 0;
  for (int64_t c = 0; c < b->nc; c++) nhyd += f->mask_hydrology[c] ? 1 : 0;
  /* 1) pervious roads */
  n = 0;
  for (int64_t c = 0; c < b->nc; c++)
    if (f->mask_hydrology[c] && f->col_itype[c] == ICOL_ROAD_PERV) filt[n++] = c;
  total += n;
  rootsink_default_filter(vp, b, f, filt, n);   /* hydstress_roads is the same algorithm */
  /* 2) neither pervious road nor natural vegetation */
  n = 0;
  for (int64_t c = 0; c < b->nc; c++)
    if (f->mask_hydrology[c] && f->col_itype[c] != ICOL_ROAD_PERV &&
        f->lun_itype[f->col_landunit[c] - 1] != ISTSOIL) filt[n++] = c;
  total += n;
  if (use_hydrstress) rootsink_hydstress_filter(vp, b, f, filt, n);
  else rootsink_default_filter(vp, b, f, filt, n);
  /* 3) natural vegetation */
  n = 0;
  for (int64_t c = 0; c < b->nc; c++)
    if (f->mask_hydrology[c] && f->lun_itype[f->col_landunit[c] - 1] == ISTSOIL) filt[n++] = c;
  total += n;
  if (use_hydrstress) rootsink_hydstress_filter(vp, b, f, filt, n);
  else rootsink_default_filter(vp, b, f, filt, n);
  free(filt);
  return total != nhyd ? 1 : 0;
}

/* ===================================================================== */
/* _soilwm_moisture_form_kernel! (soil_water_movement.jl:1250-1489)       */
/* ===================================================================== */
typedef struct {
  double hk, smp, dhkdw, dsmpdw, imped, s2, vwc_liq, dt_dz, qin, qout;
  double dqidw0, dqidw1, dqodw1, dqodw2, dwat, amx, bmx, cmx, rmx, gam, fluxNet0, fluxNet1;
} mf_row;

/* Optional capture of the last attempt's scratch rows for golden tests. */
typedef struct {
  double* qin;   /* [ld, nlevsoi] */
  double* qout;  /* [ld, nlevsoi] */
} orc_mf_capture;

#define MF_ATTEMPT_CAP 100000

static uint32_t moisture_form_col(const clmgb_varpar* vp, const clmgb_bounds* b,
                                  const clmgb_soilwater_fields* f, const clmgb_swm_config* cfg,
                                  double dtime, int64_t c, const orc_mf_capture* cap)
{
  const int64_t ld = b->ldc;
  const int joff = vp->nlevsno, joff_zi = vp->nlevsno + 1, nlevsoi = vp->nlevsoi;
  if (!f->mask_hydrology[c]) return 0;
  const int nlayers = (int)f->col_nbedrock[c];
  if (nlayers < 1 || nlayers > nlevsoi) return CLMGB_COL_LEVEL_RANGE;
  mf_row R[ORC_MAXL + 2];
  memset(R, 0, sizeof(R));
  const double denh2o = DENH2O, m_to_mm = M_TO_MM;
  const double e_ice = cfg->e_ice, dtmin = cfg->dtmin, xtu = cfg->xTolerUpper, xtl = cfg->xTolerLower;
  const double verysmall = cfg->verySmall;
  const int expensive = (cfg->flux_calculation == 42);
  const int lower_bc = cfg->lower_boundary_condition;
  int nsubstep = 0;
  double dtsub = dtime, dtdone = 0.0, qc = 0.0;
  uint32_t status = 0;
  for (;;) {
    nsubstep += 1;
    if (nsubstep > MF_ATTEMPT_CAP) { status |= CLMGB_COL_SUBSTEP_CAP; break; }
    for (int j = 1; j <= nlayers; j++) {
      R[j].vwc_liq = jl_max(IX(f->h2osoi_liq, c, joff + j, ld), 1.0e-6) / (IX(f->dz, c, joff + j, ld) * denh2o);
      R[j].dt_dz = dtsub / (m_to_mm * IX(f->dz, c, joff + j, ld));
    }
    for (int j = 1; j <= nlayers; j++) {
      double s = R[j].vwc_liq / IX(f->watsat, c, j, ld);
      s = jl_min(s, 1.0); s = jl_max(0.01, s);
      R[j].s2 = s;
    }
    for (int j = 1; j <= nlayers; j++) {
      double s1, imp;
      if (j == nlayers) {
        s1 = R[j].s2;
        imp = o_pow(10.0, -e_ice * IX(f->icefrac, c, j, ld));
      } else {
        s1 = 0.5 * (R[j].s2 + R[j + 1].s2);
        imp = o_pow(10.0, -e_ice * (0.5 * (IX(f->icefrac, c, j, ld) + IX(f->icefrac, c, j + 1, ld))));
      }
      R[j].imped = imp;
      s1 = jl_min(s1, 1.0); s1 = jl_max(0.01, s1);
      double bb = IX(f->bsw, c, j, ld);
      double hkv = imp * IX(f->hksat, c, j, ld) * o_pow(s1, 2.0 * bb + 3.0);
      double dhkds = (2.0 * bb + 3.0) * hkv / s1;
      double sn = R[j].s2;
      double smpv = -IX(f->sucsat, c, j, ld) * o_pow(sn, -bb);
      double dsmpds = -bb * smpv / sn;
      R[j].hk = hkv; R[j].smp = smpv; R[j].dhkdw = dhkds;
      R[j].dsmpdw = dsmpds / IX(f->watsat, c, j, ld);
      IX(f->smp_l, c, j, ld) = smpv;
      IX(f->hk_l, c, j, ld) = hkv;
    }
    for (int j = 1; j <= nlayers; j++) {
      R[j].qin = 0.0; R[j].qout = 0.0;
      R[j].dqidw0 = 0.0; R[j].dqidw1 = 0.0; R[j].dqodw1 = 0.0; R[j].dqodw2 = 0.0;
    }
    for (int j = 1; j <= nlayers - 1; j++) {
      double dhkds1 = 0.5 * R[j].dhkdw / IX(f->watsat, c, j, ld);
      double dhkds2 = 0.5 * R[j].dhkdw / IX(f->watsat, c, j + 1, ld);
      double num = R[j + 1].smp - R[j].smp;
      double den = m_to_mm * (IX(f->z, c, joff + j + 1, ld) - IX(f->z, c, joff + j, ld));
      R[j].qout = -R[j].hk * num / den + R[j].hk;
      R[j].dqodw1 = (R[j].hk * R[j].dsmpdw - dhkds1 * num) / den + dhkds1;
      R[j].dqodw2 = (-R[j].hk * R[j + 1].dsmpdw - dhkds2 * num) / den + dhkds2;
    }
    {
      int j = nlayers;
      if (lower_bc == CLMGB_BC_WATERTABLE) {
        int jwt = nlevsoi;
        for (int jj = 1; jj <= nlevsoi; jj++) {
          if (f->zwt[c] <= IX(f->zi, c, joff_zi + jj, ld)) { jwt = jj - 1; break; }
        }
        if (j > jwt) {
          R[j].qout = 0.0; R[j].dqodw1 = 0.0; R[j].dqodw2 = 0.0;
        } else {
          double dhkds1l = R[j].dhkdw / IX(f->watsat, c, j, ld);
          double num = -R[j].smp;
          double den = m_to_mm * (f->zwt[c] - IX(f->z, c, joff + j, ld));
          R[j].qout = -R[j].hk * num / den + R[j].hk;
          R[j].dqodw1 = (R[j].hk * R[j].dsmpdw - dhkds1l * num) / den + dhkds1l;
          R[j].dqodw2 = 0.0;
        }
      } else if (lower_bc == CLMGB_BC_FLUX) {
        R[j].qout = R[j].hk;
        R[j].dqodw1 = R[j].dhkdw / IX(f->watsat, c, j, ld);
      } else {
        R[j].qout = 0.0;
        R[j].dqodw1 = 0.0;
      }
    }
    for (int j = 2; j <= nlayers; j++) {
      R[j].qin = R[j - 1].qout;
      R[j].dqidw0 = R[j - 1].dqodw1;
      R[j].dqidw1 = R[j - 1].dqodw2;
    }
    R[1].qin = f->qflx_infl[c];
    R[1].dqidw1 = 0.0;
    for (int j = 1; j <= nlayers; j++) {
      double fluxNet = R[j].qin - R[j].qout - IX(f->qflx_rootsoi, c, j, ld);
      R[j].rmx = -fluxNet * R[j].dt_dz;
    }
    R[1].amx = 0.0;
    R[1].bmx = -1.0 - (-R[1].dqidw1 + R[1].dqodw1) * R[1].dt_dz;
    R[1].cmx = -R[1].dqodw2 * R[1].dt_dz;
    for (int j = 2; j <= nlayers - 1; j++) {
      R[j].amx = R[j].dqidw0 * R[j].dt_dz;
      R[j].bmx = -1.0 - (-R[j].dqidw1 + R[j].dqodw1) * R[j].dt_dz;
      R[j].cmx = -R[j].dqodw2 * R[j].dt_dz;
    }
    R[nlayers].amx = R[nlayers].dqidw0 * R[nlayers].dt_dz;
    R[nlayers].bmx = -1.0 - (-R[nlayers].dqidw1 + R[nlayers].dqodw1) * R[nlayers].dt_dz;
    R[nlayers].cmx = 0.0;
    {
      double bet = R[1].bmx;
      if (fabs(bet) < 1.0e-30) bet = 1.0e-30;
      double dwat_prev = R[1].rmx / bet;
      R[1].dwat = dwat_prev;
      for (int j = 2; j <= nlayers; j++) {
        R[j].gam = R[j - 1].cmx / bet;
        bet = R[j].bmx - R[j].amx * R[j].gam;
        if (fabs(bet) < 1.0e-30) bet = copysign(1.0e-30, bet == 0.0 ? 1.0 : bet);
        dwat_prev = (R[j].rmx - R[j].amx * dwat_prev) / bet;
        R[j].dwat = dwat_prev;
      }
      double dwat_next = dwat_prev;
      for (int j = nlayers - 1; j >= 1; j--) {
        dwat_next = R[j].dwat - R[j + 1].gam * dwat_next;
        R[j].dwat = dwat_next;
      }
    }
    double errorMax = 0.0;
    for (int j = 1; j <= nlayers; j++) {
      if (expensive) {
        double qin_test = j == 1 ? R[j].qin + R[j].dqidw1 * R[j].dwat
                                 : R[j].qin + R[j].dqidw0 * R[j - 1].dwat + R[j].dqidw1 * R[j].dwat;
        double qout_test = j == nlayers ? R[j].qout + R[j].dqodw1 * R[j].dwat
                                        : R[j].qout + R[j].dqodw1 * R[j].dwat + R[j].dqodw2 * R[j + 1].dwat;
        R[j].fluxNet0 = qin_test - qout_test - IX(f->qflx_rootsoi, c, j, ld);
      } else {
        R[j].fluxNet0 = R[j].dwat / R[j].dt_dz;
      }
      R[j].fluxNet1 = R[j].qin - R[j].qout - IX(f->qflx_rootsoi, c, j, ld);
    }
    for (int j = 1; j <= nlayers; j++) {
      double ev = fabs(R[j].fluxNet1 - R[j].fluxNet0) * dtsub * 0.5;
      errorMax = jl_max(errorMax, ev);
    }
    if (errorMax > xtu && dtsub > dtmin) {
      dtsub = jl_max(dtsub / 2.0, dtmin);
      continue;
    }
    for (int j = 1; j <= nlayers; j++)
      IX(f->h2osoi_liq, c, joff + j, ld) = IX(f->h2osoi_liq, c, joff + j, ld) + R[j].dwat * (m_to_mm * IX(f->dz, c, joff + j, ld));
    double qcTemp;
    if (lower_bc == CLMGB_BC_FLUX) qcTemp = R[nlayers].hk + R[nlayers].dhkdw * R[nlayers].dwat;
    else if (lower_bc == CLMGB_BC_ZERO_FLUX) qcTemp = 0.0;
    else qcTemp = R[nlayers].qout + R[nlayers].dqodw1 * R[nlayers].dwat;
    qc += qcTemp * (dtsub / dtime);
    dtdone += dtsub;
    if (fabs(dtime - dtdone) < verysmall) break;
    if (errorMax < xtl) dtsub = dtsub * 2.0;
    dtsub = jl_min(dtsub, dtime - dtdone);
  }
  f->qcharge[c] = qc;
  f->num_substeps[c] = (double)nsubstep;
  if (cap) {
    for (int j = 1; j <= nlayers; j++) {
      IX(cap->qin, c, j, ld) = R[j].qin;
      IX(cap->qout, c, j, ld) = R[j].qout;
    }
  }
  for (int j = 1; j <= nlayers; j++)
    if (!isfinite(IX(f->h2osoi_liq, c, joff + j, ld))) status |= CLMGB_COL_NONFINITE;
  return status;
}

/* ===================================================================== */
/* The reference's scalar helpers of the moisture form, restated on one   */
/* column's vectors (1-based j = index j-1 here):                         */
/*   compute_RHS_moisture_form! (soil_water_movement.jl:1080-1102)        */
/*   compute_LHS_moisture_form! (soil_water_movement.jl:1109-1140)        */
/* The solve restates the same expressions fused into its attempt.        */
/* ===================================================================== */
void orc_compute_rhs_moisture_form(int32_t nlayers, const double* vert_trans_sink, const double* vwc_liq,
                                   const double* qin, const double* qout, const double* dt_dz, double* rmx)
{
  (void)vwc_liq;
  for (int j = 0; j < nlayers; j++) rmx[j] = 0.0;
  for (int j = 0; j < nlayers; j++) {
    const double fluxNet = qin[j] - qout[j] - vert_trans_sink[j];
    rmx[j] = -fluxNet * dt_dz[j];
  }
}

void orc_compute_lhs_moisture_form(int32_t nlayers, const double* dt_dz, const double* dqidw0,
                                   const double* dqidw1, const double* dqodw1, const double* dqodw2,
                                   double* amx, double* bmx, double* cmx)
{
  for (int j = 0; j < nlayers; j++) amx[j] = bmx[j] = cmx[j] = 0.0;
  amx[0] = 0.0;
  bmx[0] = -1.0 - (-dqidw1[0] + dqodw1[0]) * dt_dz[0];
  cmx[0] = -dqodw2[0] * dt_dz[0];
  for (int j = 1; j < nlayers - 1; j++) {
    amx[j] = dqidw0[j] * dt_dz[j];
    bmx[j] = -1.0 - (-dqidw1[j] + dqodw1[j]) * dt_dz[j];
    cmx[j] = -dqodw2[j] * dt_dz[j];
  }
  const int j = nlayers - 1;
  amx[j] = dqidw0[j] * dt_dz[j];
  bmx[j] = -1.0 - (-dqidw1[j] + dqodw1[j]) * dt_dz[j];
  cmx[j] = 0.0;
}

/* ===================================================================== */
/* compute_qcharge! (soil_water_movement.jl:1153-1215) as                */
/* soilwater_moisture_form! calls it after the solve when                */
/* use_aquifer_layer(cfg) (:1575-1598): dwat, smp and imped are freshly  */
/* zeroed rows, vwc_liq = smooth_max(h2osoi_liq, 1e-6)/(dz*DENH2O) on    */
/* levels 1..min(nbedrock, nlevsoi) and zero below (:1583-1590).         */
/* ===================================================================== */
static void compute_qcharge_col(const clmgb_varpar* vp, const clmgb_bounds* b,
                                const clmgb_soilwater_fields* f, double dtime, int64_t c)
{
  const int64_t ld = b->ldc;
  const int nlevsoi = vp->nlevsoi, joff = vp->nlevsno, joff_zi = vp->nlevsno + 1;
  if (!f->mask_hydrology[c]) return;
  const int nlayers = (int)f->col_nbedrock[c];
  if (nlayers < 1 || nlayers > nlevsoi) return;   /* not solved: CLMGB_COL_LEVEL_RANGE */
  /* the rows the wrapper builds (:1580-1590) */
  double dwat[ORC_MAXL + 2], smp[ORC_MAXL + 2], imped[ORC_MAXL + 2], vwc[ORC_MAXL + 2];
  for (int j = 1; j <= nlevsoi; j++) { dwat[j] = 0.0; smp[j] = 0.0; imped[j] = 0.0; vwc[j] = 0.0; }
  (void)dwat;
  const int jlast = nlayers < nlevsoi ? nlayers : nlevsoi;
  for (int j = 1; j <= jlast; j++)
    vwc[j] = jl_max(IX(f->h2osoi_liq, c, joff + j, ld), 1.0e-6) / (IX(f->dz, c, joff + j, ld) * DENH2O);
  /* index of the layer above the water table (:1177-1184) */
  int jwt = nlevsoi;
  for (int j = 1; j <= nlevsoi; j++) {
    if (f->zwt[c] <= IX(f->zi, c, joff_zi + j, ld)) { jwt = j - 1; break; }
  }
  if (jwt < nlevsoi) {
    const double wh_zwt = -IX(f->sucsat, c, jwt + 1, ld) - f->zwt[c] * M_TO_MM;
    double s1 = jl_max(vwc[jwt + 1] / IX(f->watsat, c, jwt + 1, ld), 0.01);
    s1 = jl_min(1.0, s1);
    /* soil_hk! of the Clapp-Hornberger curve (swrc_clapp_hornberg.jl:43-55) */
    const double bsw = IX(f->bsw, c, jwt + 1, ld);
    const double ka = imped[jwt + 1] * IX(f->hksat, c, jwt + 1, ld) * cm_pow(s1, 2.0 * bsw + 3.0);
    const int jm = jwt > 1 ? jwt : 1;
    const double smp1 = jl_max(f->smpmin[c], smp[jm]);
    const double wh = smp1 - IX(f->z, c, joff + jm, ld) * M_TO_MM;
    double q;
    if (jwt == 0)
      q = -ka * (wh_zwt - wh) / ((f->zwt[c] + 1.0e-3) * M_TO_MM);
    else
      q = -ka * (wh_zwt - wh) / ((f->zwt[c] - IX(f->z, c, joff + jwt, ld)) * M_TO_MM * 2.0);
    q = jl_max(-10.0 / dtime, q);
    q = jl_min(10.0 / dtime, q);
    f->qcharge[c] = q;
  }
}

/* ===================================================================== */
/* The use_flexibleCN branch of soil_water! (soil_water_movement.jl:     */
/* 1812-1843), loop by loop as the reference writes it (levels outer,    */
/* columns inner); smooth_ifelse on Float64 is the exact branch          */
/* (smooth_ad.jl:253-257).                                               */
/* ===================================================================== */
int orc_soil_water_flexible_cn(const clmgb_varpar* vp, const clmgb_bounds* b, const clmgb_flexcn_fields* f)
{
  const int64_t ld = b->ldc;
  const int nlevsoi = vp->nlevsoi, joff = vp->nlevsno;
  const double watmin = 0.001;
  for (int j = 1; j <= nlevsoi - 1; j++) {
    for (int64_t c = 0; c < b->nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      const double l = IX(f->h2osoi_liq, c, joff + j, ld);
      const double xs = l >= 0.0 ? 0.0 : watmin - l;
      IX(f->h2osoi_liq, c, joff + j, ld) = l + xs;
      IX(f->h2osoi_liq, c, joff + j + 1, ld) = IX(f->h2osoi_liq, c, joff + j + 1, ld) - xs;
    }
  }
  for (int64_t c = 0; c < b->nc; c++) {
    if (!f->mask_hydrology[c]) continue;
    const double l = IX(f->h2osoi_liq, c, joff + nlevsoi, ld);
    const double xs = (l - watmin) >= 0.0 ? 0.0 : watmin - l;
    IX(f->h2osoi_liq, c, joff + nlevsoi, ld) = l + xs;
    f->wa[c] = f->wa[c] - xs;
  }
  for (int j = 1; j <= nlevsoi; j++) {
    for (int64_t c = 0; c < b->nc; c++) {
      if (!f->mask_hydrology[c]) continue;
      const double dzv = IX(f->dz, c, joff + j, ld);
      IX(f->h2osoi_vol, c, j, ld) = IX(f->h2osoi_liq, c, joff + j, ld) / (dzv * DENH2O) +
                                    IX(f->h2osoi_ice, c, joff + j, ld) / (dzv * DENICE);
    }
  }
  return 0;
}

/* soilwater_moisture_form! (soil_water_movement.jl:1532-1601): the solve, then
 * compute_qcharge! under the water-table lower boundary. */
int orc_soil_water(const clmgb_varpar* vp, const clmgb_bounds* b,
                   const clmgb_soilwater_fields* f, const clmgb_swm_config* cfg, double dtime,
                   uint32_t* col_status, double* cap_qin, double* cap_qout, int32_t nthreads)
{
  int e = check_varpar(vp);
  if (e) return e;
  if (cfg->soilwater_movement_method != CLMGB_MOISTURE_FORM) return CLMGB_ERR_UNSUPPORTED;
  if (cfg->upper_boundary_condition != CLMGB_BC_FLUX) return CLMGB_ERR_CONFIG;
  if (!(cfg->lower_boundary_condition == CLMGB_BC_WATERTABLE ||
        cfg->lower_boundary_condition == CLMGB_BC_FLUX ||
        cfg->lower_boundary_condition == CLMGB_BC_ZERO_FLUX)) return CLMGB_ERR_CONFIG;
  orc_mf_capture capv = {cap_qin, cap_qout};
  const orc_mf_capture* cap = (cap_qin && cap_qout) ? &capv : NULL;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t c = 0; c < b->nc; c++) {
    uint32_t s = moisture_form_col(vp, b, f, cfg, dtime, c, cap);
    if (col_status) col_status[c] = s;
    if (cfg->lower_boundary_condition == CLMGB_BC_WATERTABLE) compute_qcharge_col(vp, b, f, dtime, c);
  }
  return 0;
}

/* ===================================================================== */
/* Synthetic multi-step driver: the per-step forcing a test or benchmark  */
/* applies before the path (the upstream radiation/infiltration modules   */
/* are out of scope), then the path in the driver's order.                */
/*   per column, per step t:                                              */
/*     sabg = sabg_soil = sabg_snow = G[t]; sabg_lyr = 0 except the top   */
/*     active layer (snl+1) = G[t]; forc_lwrad = SB * t_grnd^4;           */
/*     qflx_infl = I[t]; t_ssbef = t_soisno; t_h2osfc_bef = t_h2osfc;     */
/*     soil_temperature!, set_soil_water_fractions!, soil_water!.         */
/* G and I are [nsteps, nc] row-major with row stride gstride (0 = the    */
/* same row every step).                                                  */
/* ===================================================================== */
void orc_apply_forcing_col(const clmgb_varpar* vp, const clmgb_bounds* b,
                           const clmgb_soiltemp_fields* ft, const clmgb_soilwater_fields* fw,
                           int64_t c, double G, double I)
{
  const int64_t ldp = b->ldp;
  const int nlevsno = vp->nlevsno;
  double* sabg = (double*)ft->sabg;
  double* sabg_soil = (double*)ft->sabg_soil;
  double* sabg_snow = (double*)ft->sabg_snow;
  double* sabg_lyr = (double*)ft->sabg_lyr;
  for (int64_t p1 = ft->col_patchi[c]; p1 <= ft->col_patchf[c]; p1++) {
    int64_t p = p1 - 1;
    sabg[p] = G; sabg_soil[p] = G; sabg_snow[p] = G;
    for (int k = 1; k <= nlevsno + 1; k++) IX(sabg_lyr, p, k, ldp) = 0.0;
    if (ft->col_snl[c] <= 0 && ft->col_snl[c] >= -nlevsno) IX(sabg_lyr, p, ft->col_snl[c] + 1 + nlevsno, ldp) = G;
  }
  ((double*)ft->forc_lwrad)[c] = SB * jl_pow4(ft->t_grnd[c]);
  ((double*)fw->qflx_infl)[c] = I;
}

int orc_run_steps(const clmgb_varpar* vp, const clmgb_bounds* b,
                  const clmgb_soiltemp_fields* ft, const clmgb_soilwater_fields* fw,
                  const clmgb_swm_config* cfg, double dtime, int32_t snow_method,
                  int32_t nsteps, const double* G, const double* I, int64_t gstride,
                  double* t_ssbef, double* t_h2osfc_bef, uint32_t* col_status,
                  int32_t nthreads)
{
  int e = check_varpar(vp);
  if (e) return e;
  st_ctx X = {vp, b, ft, dtime, snow_method};
  const int64_t ld = b->ldc;
  const int L = vp->nlevsno + vp->nlevmaxurbgrnd;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int64_t c = 0; c < b->nc; c++) {
    uint32_t s = 0;
    for (int32_t t = 0; t < nsteps; t++) {
      if (ft->mask_nolakec[c]) {
        orc_apply_forcing_col(vp, b, ft, fw, c, G[t * gstride + c], I[t * gstride + c]);
        if (t_ssbef)
          for (int jj = 1; jj <= L; jj++) IX(t_ssbef, c, jj, ld) = IX(ft->t_soisno, c, jj, ld);
        if (t_h2osfc_bef) t_h2osfc_bef[c] = ft->t_h2osfc[c];
      }
      s |= soiltemp_col(&X, c);
      fractions_col(vp, b, fw, c);
      s |= moisture_form_col(vp, b, fw, cfg, dtime, c, NULL);
      if (cfg->lower_boundary_condition == CLMGB_BC_WATERTABLE) compute_qcharge_col(vp, b, fw, dtime, c);
    }
    if (col_status) col_status[c] = s;
  }
  return 0;
}

/* ===================================================================== */
/* init_soil_properties! (cold_start.jl:225-391), per column and level,   */
/* with the SoilStateParams defaults (types/soil_state.jl:19-35).         */
/* Inputs sand/clay [%], om_frac (organic fraction after om_frac_sf and   */
/* the 130 kg/m3 normalisation), zsoi [m]; outputs per level.             */
/* ===================================================================== */
void orc_init_soil_properties(int64_t n, const double* sand_in, const double* clay_in,
                              const double* om_in, const double* zsoi,
                              double* watsat, double* bsw, double* sucsat, double* hksat,
                              double* tkmg, double* tkdry, double* csol)
{
  const double tkd_sand = 8.8, tkd_clay = 2.92, tkd_om = 0.05, tkm_om = 0.25;
  const double csol_sand = 2.128, csol_clay = 2.385, csol_om = 2.5, pd = 2700.0;
  const double bsw_sf = 1.0, hksat_sf = 1.0, sucsat_sf = 1.0, watsat_sf = 1.0;
  for (int64_t i = 0; i < n; i++) {
    double sand = sand_in[i], clay = clay_in[i], om_frac = om_in[i];
    double watsat_mineral = 0.489 - 0.00126 * sand;
    double bsw_mineral = 2.91 + 0.159 * clay;
    double sucsat_mineral = 10.0 * cm_pow(10.0, 1.88 - 0.0131 * sand);
    double xksat_mineral = 0.0070556 * cm_pow(10.0, -0.884 + 0.0153 * sand);
    double zsapric = 0.5;
    double depth_ratio = zsoi[i] / zsapric;
    double watsat_organic = jl_max(0.93 - 0.1 * depth_ratio, 0.83);
    double bsw_organic = jl_min(2.7 + 9.3 * depth_ratio, 12.0);
    double sucsat_organic = jl_min(10.3 - 0.2 * depth_ratio, 10.1);
    double xksat_organic = jl_max(0.28 - 0.2799 * depth_ratio, xksat_mineral);
    double watsat_val = jl_min(watsat_sf * ((1.0 - om_frac) * watsat_mineral + om_frac * watsat_organic), 0.93);
    double bsw_val = bsw_sf * ((1.0 - om_frac) * bsw_mineral + om_frac * bsw_organic);
    double sucsat_val = sucsat_sf * ((1.0 - om_frac) * sucsat_mineral + om_frac * sucsat_organic);
    double om_hksat = xksat_organic;
    double pcalpha = 0.5, pcbeta = 0.139, perc_frac;
    if (om_frac > pcalpha) {
      double perc_norm = cm_pow(1.0 - pcalpha, -pcbeta);
      perc_frac = perc_norm * cm_pow(om_frac - pcalpha, pcbeta);
    } else {
      perc_frac = 0.0;
    }
    double uncon_frac = (1.0 - om_frac) + (1.0 - perc_frac) * om_frac;
    double uncon_hksat;
    if (uncon_frac > 0.0)
      uncon_hksat = uncon_frac / ((1.0 - om_frac) / xksat_mineral + ((1.0 - perc_frac) * om_frac) / om_hksat);
    else
      uncon_hksat = 0.0;
    double hksat_val = hksat_sf * (uncon_frac * uncon_hksat + (perc_frac * om_frac) * om_hksat);
    watsat[i] = watsat_val; bsw[i] = bsw_val; sucsat[i] = sucsat_val; hksat[i] = hksat_val;
    double bd = (1.0 - watsat_mineral) * pd;
    double sc = sand + clay;
    double tkm = sc > 0.0 ? (1.0 - om_frac) * (tkd_sand * sand + tkd_clay * clay) / sc + tkm_om * om_frac : tkm_om;
    tkmg[i] = cm_pow(tkm, 1.0 - watsat_val);
    tkdry[i] = ((0.135 * bd + 64.7) / (pd - 0.947 * bd)) * (1.0 - om_frac) + tkd_om * om_frac;
    double csol_min = sc > 0.0 ? (csol_sand * 1.0e6 * sand + csol_clay * 1.0e6 * clay) / sc : csol_om * 1.0e6;
    csol[i] = (1.0 - om_frac) * csol_min + csol_om * 1.0e6 * om_frac;
  }
}

int orc_abi_version(void) { return CLMGB_ABI_VERSION; }

/* Shared transcendentals, exported for the accuracy and GPU bit-parity tests. */
double orc_cm_log(double x) { return cm_log(x); }
double orc_cm_exp(double x) { return cm_exp(x); }
double orc_cm_pow(double x, double y) { return cm_pow(x, y); }
double orc_cm_log10(double x) { return cm_log10(x); }
double orc_cm_sin(double x) { return cm_sin(x); }
double orc_cm_acos(double x) { return cm_acos(x); }
/* The integer-pipe division the GPU kernels use, over n pairs (for the test that it is
 * the IEEE quotient). */
void orc_cm_div_n(int64_t n, const double* x, const double* y, double* out) {
  for (int64_t i = 0; i < n; i++) out[i] = cm_div(x[i], y[i]);
}
