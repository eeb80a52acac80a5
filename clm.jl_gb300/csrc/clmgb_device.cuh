// clmgb_device.cuh — per-column device code of the GB300 soil/snow column solve.
//
// One CUDA thread owns one column.  Every field is read in CLM.jl's own layout
// (Julia column-major [nc, nlev]: element (c, jj) at c + (jj-1)*ldc), so the 32
// threads of a warp touch 32 consecutive doubles of a level: every load and store
// is a fully coalesced 256-byte transaction with no staging.
//
// Arithmetic follows the reference's Float64 expressions operation by operation
// (this file is compiled with --fmad=false so a*b+c is never fused, as in Julia),
// and the transcendentals come from clm_math.h, which the CPU oracle shares: the
// GPU and the oracle produce the same bits.  Citations are to CLM.jl source files.
#pragma once
#include <stdint.h>
#include <math.h>
#include "../../include/clmgb.h"
#include "clm_math.h"

namespace clmgb {

// ---- constants: src/constants/varcon.jl:15-70 ----
constexpr double GRAV = 9.80616;
constexpr double SB = 5.67e-8;
constexpr double CPLIQ = 4188.0;
constexpr double CPICE = 2117.27;
constexpr double HFUS = 3.337e5;
constexpr double DENH2O = 1000.0;
constexpr double DENICE = 917.0;
constexpr double TFRZ = 273.15;
constexpr double TKAIR = 0.023;
constexpr double TKICE = 2.290;
constexpr double TKWAT = 0.57;
constexpr double CAPR = 0.34;
constexpr double CNFAC = 0.5;
constexpr double THK_BEDROCK = 3.0;
constexpr double CSOL_BEDROCK = 2.0e6;
constexpr double THIN_SFCLAYER = 1.0e-6;
constexpr double M_TO_MM = 1.0e3;
// landunit / column types: src/constants/landunit_varcon.jl, column_varcon.jl
constexpr int64_t ISTSOIL = 1, ISTCROP = 2, ISTICE = 4, ISTWET = 6;
constexpr int64_t ICOL_ROOF = 71, ICOL_SUNWALL = 72, ICOL_SHADEWALL = 73;
constexpr int64_t ICOL_ROAD_IMPERV = 74, ICOL_ROAD_PERV = 75;

// compile-time level capacities of the per-thread arrays
constexpr int MAXSNO = CLMGB_MAX_NLEVSNO;
constexpr int MAXGRND = CLMGB_MAX_NLEVGRND;
constexpr int MAXL = MAXSNO + MAXGRND;       // snow + ground levels
constexpr int MAXROWS = MAXL + 1;            // + the surface-water row of the band system
constexpr int MAXSOI = CLMGB_MAX_NLEVSOI;
constexpr int MF_ATTEMPT_CAP = 4096;         // safety cap on Richards substep attempts
// polls of a deferred column's list slot before the drain gives it back (richards_coop.cuh)
constexpr int DEFER_POLL_LIMIT = 1 << 20;

struct Dims {
  int nlevsno, nlevgrnd, nlevsoi, nlevurb, nlevmax;
  int64_t ldc, ldp, np;
  int64_t c0 = 0;    // global index of the call's first column (patch_column holds global indices)
  int attempt_cap = MF_ATTEMPT_CAP;   // Richards attempts after which a column stops (CLMGB_COL_SUBSTEP_CAP)
  int st_block = 320;                 // threads per block of the soil-temperature kernels (CLMGB_OPT_ST_BLOCK)
};

// Julia Base.max / Base.min on Float64 (NaN propagates, -0.0 < 0.0).  They only
// select one argument, so they are done on the integer pipes: the bit pattern
// mapped to a two's-complement key orders doubles exactly (-0.0 below +0.0), and
// NaN is recognised from its bits.  No FP64 instruction is spent on them.
__device__ __forceinline__ long long ord_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool isnan_bits(double x) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
__device__ __forceinline__ double jl_max(double x, double y) {
  if (isnan_bits(x)) return x;
  if (isnan_bits(y)) return y;
  return ord_key(x) >= ord_key(y) ? x : y;
}
__device__ __forceinline__ double jl_min(double x, double y) {
  if (isnan_bits(x)) return x;
  if (isnan_bits(y)) return y;
  return ord_key(x) <= ord_key(y) ? x : y;
}
// Julia's Float64 x / y (IEEE, round to nearest), formed on the integer pipes.  On
// GB300 an FP64 instruction holds its sub-partition's FP64 unit for about 64 cycles,
// and the column kernels are bound by that unit; cm_div (clm_math.h) forms the
// correctly rounded quotient of normal operands with 64-bit integer arithmetic
// instead (measured: 141 against 70 G divisions/s alone, and next to FP64 work it
// costs almost nothing, since it runs on the otherwise idle integer pipes).  A zero x
// over a finite nonzero y, common in this solve (the ice of unfrozen levels, the
// excess ice, the phase-change heat of levels that neither melt nor freeze, the band
// system's zero sub-diagonal), is the zero with the xor of the signs, from the bits;
// the hardware division is 2.6x slower than usual there (27 against 70 G/s).  Every
// other case (subnormal, infinite or NaN operands, quotients outside the normal range)
// is the hardware division.  The result is always the IEEE quotient.
// (one out-of-line copy of the integer division: measured faster than a copy inlined
// at every call site, 4.2 against 5.6 ms for the part of a step at 262,144 columns
// outside the Richards solve, and 10.5 against 17.7 ms for the Richards solve)
static __device__ __noinline__ double cm_div_call(double x, double y) { return cm_div(x, y); }
__device__ __forceinline__ double jl_div(double x, double y) {
  const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
  const unsigned long long by = (unsigned long long)__double_as_longlong(y);
  // (by << 1) - 1 < 0xffdffffffffffffe: y is nonzero and finite
  if ((bx << 1) == 0 && (by << 1) - 1ull < 0xffdffffffffffffeull)
    return __longlong_as_double((long long)((bx ^ by) & 0x8000000000000000ull));
  return cm_div_call(x, y);
}
// other scalar types (the recording adjoint's): their own division
template <class A, class B>
__device__ __forceinline__ auto jl_div(A x, B y) {
  return x / y;
}
// |x| < t for a positive threshold t, on the integer pipes (false for NaN, as in IEEE).
__device__ __forceinline__ bool abs_lt(double x, double t) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffLL) < __double_as_longlong(t);
}
// Julia's Float64 x^4 (Base.Math.pow_body, compensated squaring).
__device__ __forceinline__ double jl_pow4(double x) {
  double x2 = __dmul_rn(x, x);
  double lo1 = __fma_rn(x, x, -x2);
  double x4 = __dmul_rn(x2, x2);
  double lo2 = __fma_rn(x2, x2, -x4);
  double xnlo = lo2 + (x2 * 2.0 * lo1);
  if (isfinite(x4) && isfinite(xnlo)) return x4 + xnlo;
  return x4;
}

// level-indexed access, jj 1-based like the Julia code
template <typename T>
__device__ __forceinline__ T& LV(T* p, int64_t c, int jj, int64_t ld) {
  return p[c + (int64_t)(jj - 1) * ld];
}
template <typename T>
__device__ __forceinline__ T LVc(const T* p, int64_t c, int jj, int64_t ld) {
  return __ldg(p + c + (int64_t)(jj - 1) * ld);
}

__device__ __forceinline__ bool is_wallroof(int64_t it) {
  return it == ICOL_SUNWALL || it == ICOL_SHADEWALL || it == ICOL_ROOF;
}

// Value of a scalar: the identity for double.  The step adjoint's recording scalar
// (adjoint_step.cu) overloads it.
__device__ __forceinline__ double VAL(double x) { return x; }

// ===========================================================================
// Banded pivoted LU for one column (band_diagonal.jl:87-170).
//
// The reference densifies the 5-band system into an n x n matrix and runs partial-
// pivot Gaussian elimination over all n columns.  Every entry outside the band is
// an exact zero, so each elimination it performs there is x - 0*y == x: the banded
// form below performs exactly the in-band operations, in the same order, and gives
// the same bits for every finite non-singular system.  With partial pivoting the
// upper factor widens to kl+ku, so each row keeps 2*kl+ku+1 entries:
// ab[r*W + d] holds A[r, r-kl+d].
// ===========================================================================
template <int KL, int KU, class S>
__device__ __forceinline__ void band_lu_solve(S* ab, S* x, int n) {
  constexpr int W = 2 * KL + KU + 1;
  // Partial-pivot elimination: step k picks the largest |A[i,k]| of rows k..k+KL,
  // swaps it into row k (columns k..k+KL+KU and the right-hand side), and subtracts
  // f = A[i,k]/A[k,k] times row k from each row below (the same steps as
  // band_lu_factor_solve below).  Step k touches rows k..k+KL over columns
  // k..k+KL+KU only; that window is kept in registers (w[i][c] = A[k+i, k+c]), so each
  // row comes in once from the assembled band and leaves once as its row of U, which
  // the back substitution reads.
  constexpr int R = KL + 1, C = KL + KU + 1;
#define AB(r, col) ab[(r) * W + ((col) - (r) + KL)]
  S w[R][C];
#pragma unroll
  for (int i = 0; i < R; i++)
#pragma unroll
    for (int c = 0; c < C; c++) w[i][c] = i < n ? AB(i, c) : S(0.0);
  for (int k = 0; k < n - 1; k++) {
    const int ni = min(n - 1, k + KL) - k;          // rows k+1..k+ni are in the system
    const int nc = min(n - 1, k + KL + KU) - k;     // columns k..k+nc are in the system
    int piv = 0;
    double maxv = fabs(VAL(w[0][0]));
#pragma unroll
    for (int i = 1; i < R; i++) {
      if (i <= ni) {
        const double v = fabs(VAL(w[i][0]));
        if (v > maxv) {
          maxv = v;
          piv = i;
        }
      }
    }
#pragma unroll
    for (int i = 1; i < R; i++) {
      if (i == piv) {
#pragma unroll
        for (int c = 0; c < C; c++) {
          if (c <= nc) {
            const S a = w[0][c];
            w[0][c] = w[i][c];
            w[i][c] = a;
          }
        }
        const S xk = x[k], xp = x[k + i];
        x[k] = xp;
        x[k + i] = xk;
      }
    }
    const S akk = w[0][0];
#pragma unroll
    for (int i = 1; i < R; i++) {
      if (i <= ni) {
        const S f = jl_div(w[i][0], akk);
#pragma unroll
        for (int c = 1; c < C; c++)
          if (c <= nc) w[i][c] = w[i][c] - f * w[0][c];
        x[k + i] = x[k + i] - f * x[k];
      }
    }
#pragma unroll
    for (int c = 0; c < C; c++)
      if (c <= nc) AB(k, k + c) = w[0][c];
    // slide down a row: the column the window gains comes from storage (no step has
    // written it yet), and row k+1+KL enters with its band
#pragma unroll
    for (int i = 0; i < R - 1; i++) {
#pragma unroll
      for (int c = 0; c < C - 1; c++) w[i][c] = w[i + 1][c + 1];
      w[i][C - 1] = k + 1 + i < n ? AB(k + 1 + i, k + C) : S(0.0);
    }
    const int r = k + 1 + KL;
#pragma unroll
    for (int c = 0; c < C; c++) w[R - 1][c] = r < n ? AB(r, k + 1 + c) : S(0.0);
  }
  if (n > 0) AB(n - 1, n - 1) = w[0][0];
  for (int i = n - 1; i >= 0; i--) {
    S s = x[i];
    const int jl = min(n - 1, i + KL + KU);
    for (int j = i + 1; j <= jl; j++) s = s - AB(i, j) * x[j];
    x[i] = jl_div(s, AB(i, i));
  }
#undef AB
}

// The same elimination keeping its factorisation (LAPACK gbtrf's product form): each
// multiplier f_ik stays in the slot of the entry it eliminated and piv[k] = p - k
// records the row exchange of step k.  x is bit-identical to band_lu_solve's.
template <int KL, int KU>
__device__ __forceinline__ void band_lu_factor_solve(double* ab, double* x, uint8_t* piv, int n) {
  // band_lu_solve's elimination and register window; the multiplier of row k+i leaves
  // with the window into A[k+i, k], the slot of the entry it eliminated
  constexpr int W = 2 * KL + KU + 1;
  constexpr int R = KL + 1, C = KL + KU + 1;
#define AB(r, col) ab[(r) * W + ((col) - (r) + KL)]
  double w[R][C];
#pragma unroll
  for (int i = 0; i < R; i++)
#pragma unroll
    for (int c = 0; c < C; c++) w[i][c] = i < n ? AB(i, c) : 0.0;
  for (int k = 0; k < n - 1; k++) {
    const int ni = min(n - 1, k + KL) - k;
    const int nc = min(n - 1, k + KL + KU) - k;
    int p = 0;
    double maxv = fabs(w[0][0]);
#pragma unroll
    for (int i = 1; i < R; i++) {
      if (i <= ni) {
        const double v = fabs(w[i][0]);
        if (v > maxv) {
          maxv = v;
          p = i;
        }
      }
    }
    piv[k] = (uint8_t)p;
#pragma unroll
    for (int i = 1; i < R; i++) {
      if (i == p) {
#pragma unroll
        for (int c = 0; c < C; c++) {
          if (c <= nc) {
            const double a = w[0][c];
            w[0][c] = w[i][c];
            w[i][c] = a;
          }
        }
        const double xk = x[k], xp = x[k + i];
        x[k] = xp;
        x[k + i] = xk;
      }
    }
    const double akk = w[0][0];
#pragma unroll
    for (int i = 1; i < R; i++) {
      if (i <= ni) {
        const double f = jl_div(w[i][0], akk);
#pragma unroll
        for (int c = 1; c < C; c++)
          if (c <= nc) w[i][c] = w[i][c] - f * w[0][c];
        x[k + i] = x[k + i] - f * x[k];
        AB(k + i, k) = f;
      }
    }
#pragma unroll
    for (int c = 0; c < C; c++)
      if (c <= nc) AB(k, k + c) = w[0][c];
#pragma unroll
    for (int i = 0; i < R - 1; i++) {
#pragma unroll
      for (int c = 0; c < C - 1; c++) w[i][c] = w[i + 1][c + 1];
      w[i][C - 1] = k + 1 + i < n ? AB(k + 1 + i, k + C) : 0.0;
    }
    const int r = k + 1 + KL;
#pragma unroll
    for (int c = 0; c < C; c++) w[R - 1][c] = r < n ? AB(r, k + 1 + c) : 0.0;
  }
  if (n > 0) {
    AB(n - 1, n - 1) = w[0][0];
    piv[n - 1] = 0;
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = x[i];
    const int jl = min(n - 1, i + KL + KU);
    for (int j = i + 1; j <= jl; j++) s = s - AB(i, j) * x[j];
    x[i] = jl_div(s, AB(i, i));
  }
#undef AB
}

// A^T w = b from the factors of band_lu_factor_solve (LAPACK gbtrs 'T' order):
// U^T y = b by forward substitution, then for k = n-2..0: y_k -= sum_i f_ik y_i and
// the row exchange of step k.  w holds b on entry.
template <int KL, int KU>
__device__ __forceinline__ void band_lu_transpose_solve(const double* ab, const uint8_t* piv, double* w, int n) {
  constexpr int W = 2 * KL + KU + 1;
#define AB(r, col) ab[(r) * W + ((col) - (r) + KL)]
  for (int i = 0; i < n; i++) {
    double s = w[i];
    for (int j = max(0, i - KL - KU); j < i; j++) s = s - AB(j, i) * w[j];
    w[i] = jl_div(s, AB(i, i));
  }
  for (int k = n - 2; k >= 0; k--) {
    double s = w[k];
    const int ilast = min(n - 1, k + KL);
    for (int i = k + 1; i <= ilast; i++) s = s - AB(i, k) * w[i];
    w[k] = s;
    const int p = k + (int)piv[k];
    if (p != k) {
      const double t = w[k];
      w[k] = w[p];
      w[p] = t;
    }
  }
#undef AB
}

// Where a column's active state lives.  The production kernels read and write the
// caller's fields in place (FieldState over clmgb_soiltemp_fields or
// clmgb_soilwater_fields; only the members a kernel uses are instantiated).  The
// step adjoint keeps the same quantities in per-thread storage with their tape
// indices.  Every column function below takes its state through such an accessor
// X, with X::S the scalar type of the active quantities, and the banded solve of
// soil_temperature! goes through X.band_solve.
template <class F>
struct FieldState {
  typedef double S;
  const F& f;
  int64_t c, ld;
  __device__ __forceinline__ FieldState(const F& ff, int64_t cc, int64_t l) : f(ff), c(cc), ld(l) {}
  __device__ __forceinline__ decltype(auto) T(int jj) const { return LV(f.t_soisno, c, jj, ld); }
  __device__ __forceinline__ decltype(auto) Liq(int jj) const { return LV(f.h2osoi_liq, c, jj, ld); }
  __device__ __forceinline__ decltype(auto) Ice(int jj) const { return LV(f.h2osoi_ice, c, jj, ld); }
  __device__ __forceinline__ decltype(auto) Fact(int jj) const { return LV(f.fact, c, jj, ld); }
  __device__ __forceinline__ decltype(auto) Icefrac(int j) const { return LV(f.icefrac, c, j, ld); }
  __device__ __forceinline__ decltype(auto) Tgrnd() const { return f.t_grnd[c]; }
  __device__ __forceinline__ decltype(auto) Th2osfc() const { return f.t_h2osfc[c]; }
  __device__ __forceinline__ decltype(auto) Qcharge() const { return f.qcharge[c]; }
  __device__ __forceinline__ double ForcLwrad() const { return f.forc_lwrad[c]; }
  __device__ __forceinline__ double Watsat(int j) const { return LVc(f.watsat, c, j, ld); }
  __device__ __forceinline__ double Bsw(int j) const { return LVc(f.bsw, c, j, ld); }
  __device__ __forceinline__ double Sucsat(int j) const { return LVc(f.sucsat, c, j, ld); }
  __device__ __forceinline__ double Hksat(int j) const { return LVc(f.hksat, c, j, ld); }
  // the banded solve of soil_temperature! (ab, x: the column's band rows and right-hand side)
  __device__ __forceinline__ void band_solve(double* ab, double* x, int n) const { band_lu_solve<2, 2>(ab, x, n); }
};

// ===========================================================================
// phase_change_h2osfc! (soil_temperature.jl:1757-1855), column c.
// ===========================================================================
template <class ST>
__device__ inline void phase_change_h2osfc_col(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c,
                                               double dtime, typename ST::S dhsdT, ST& X) {
  typedef typename ST::S S;
  const int joff = D.nlevsno;
  const int64_t snl = f.col_snl[c];
  f.xmf_h2osfc[c] = 0.0;
  f.qflx_h2osfc_to_ice[c] = 0.0;
  f.eflx_h2osfc_to_snow[c] = 0.0;
  const double fh = f.frac_h2osfc[c];
  if (fh > 0.0 && X.Th2osfc() <= TFRZ) {
    const S tinc = TFRZ - X.Th2osfc();
    X.Th2osfc() = TFRZ;
    const double ch = f.c_h2osfc[c];
    const S hm = fh * (dhsdT * tinc - tinc * ch / dtime);
    const S xm = hm * dtime / HFUS;
    const S temp1 = f.h2osfc[c] + xm;
    S h2osno_total = f.h2osno_no_layers[c];
    if (snl < 0)
      for (int j = (int)snl + 1; j <= 0; j++) h2osno_total += X.Ice(j + joff) + X.Liq(j + joff);
    const double fs = f.frac_sno_eff[c];
    const double z_avg = fs * f.snow_depth[c];
    S rho_avg = z_avg > 0.0 ? jl_min(800.0, h2osno_total / z_avg) : S(200.0);
    if (temp1 >= 0.0) {
      f.int_snow[c] -= VAL(xm);
      if (snl == 0) f.h2osno_no_layers[c] -= VAL(xm);
      else X.Ice(joff) -= xm;
      h2osno_total -= xm;
      f.h2osfc[c] += VAL(xm);
      f.xmf_h2osfc[c] = VAL(hm);
      f.qflx_h2osfc_to_ice[c] = -VAL(xm) / dtime;
      if (fs > 0.0 && snl < 0) f.snow_depth[c] = VAL(h2osno_total / (rho_avg * fs));
      else f.snow_depth[c] = VAL(h2osno_total) / DENICE;
      if (snl == 0) {
        X.T(joff) = X.Th2osfc();
        f.eflx_h2osfc_to_snow[c] = 0.0;
      } else {
        S c1;
        if (snl == -1) c1 = fs * (dtime / X.Fact(joff) - dhsdT * dtime);
        else c1 = fs / X.Fact(joff) * dtime;
        const S c2 = fh != 0.0 ? (-CPLIQ * xm - fh * dhsdT * dtime) : S(0.0);
        X.T(joff) = (c1 * X.T(joff) + c2 * X.Th2osfc()) / (c1 + c2);
        f.eflx_h2osfc_to_snow[c] = VAL((X.Th2osfc() - X.T(joff)) * c2 / dtime);
      }
    } else {
      const double h2osfc0 = f.h2osfc[c];
      rho_avg = (h2osno_total * rho_avg + h2osfc0 * DENICE) / (h2osno_total + h2osfc0);
      f.int_snow[c] += h2osfc0;
      if (snl == 0) f.h2osno_no_layers[c] += h2osfc0;
      else X.Ice(joff) += h2osfc0;
      h2osno_total += h2osfc0;
      f.qflx_h2osfc_to_ice[c] = h2osfc0 / dtime;
      X.Th2osfc() -= temp1 * HFUS / (dtime * dhsdT - ch);
      f.xmf_h2osfc[c] = VAL(hm - fh * temp1 * HFUS / dtime);
      if (snl == 0) {
        X.T(joff) = X.Th2osfc();
      } else {
        S c1;
        if (snl == -1) c1 = fs * (dtime / X.Fact(joff) - dhsdT * dtime);
        else c1 = fs / X.Fact(joff) * dtime;
        const S c2 = fh != 0.0 ? fh * (ch - dtime * dhsdT) : S(0.0);
        X.T(joff) = (c1 * X.T(joff) + c2 * X.Th2osfc()) / (c1 + c2);
        X.Th2osfc() = X.T(joff);
      }
      f.h2osfc[c] = 0.0;
      if (fs > 0.0 && snl < 0) f.snow_depth[c] = VAL(h2osno_total / (rho_avg * fs));
      else f.snow_depth[c] = VAL(h2osno_total) / DENICE;
    }
  }
}

__device__ inline void phase_change_h2osfc_col(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c,
                                               double dtime, double dhsdT) {
  FieldState<clmgb_soiltemp_fields> X(f, c, D.ldc);
  phase_change_h2osfc_col(D, f, c, dtime, dhsdT, X);
}

// ===========================================================================
// phase_change_beta! (soil_temperature.jl:1929-2230), hard Float64 path, column c.
// The reference's four level loops (the levels' starting state, the snow levels' and
// the soil levels' melt/freeze decisions, the phase change) run as one pass per
// level, and its per-call scratch rows (PcbTmp) become that level's registers.
// ===========================================================================
template <class ST>
__device__ inline void phase_change_beta_col(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c,
                                             double dtime, typename ST::S dhsdT, ST& X) {
  typedef typename ST::S S;
  const int64_t ld = D.ldc;
  const int nlevsno = D.nlevsno, nlevgrnd = D.nlevgrnd, nlevmax = D.nlevmax;
  const int joff = nlevsno;
  const int64_t snl = f.col_snl[c];
  const int64_t l = f.col_landunit[c] - 1;
  const int64_t it = f.col_itype[c];
  const int64_t lit = f.lun_itype[l];
  const bool wallroof = is_wallroof(it);
  double* EXI = f.excess_ice;
  const double fse = f.frac_sno_eff[c];
  const double fh = f.frac_h2osfc[c];
  const bool supercool_type = (lit == ISTSOIL || lit == ISTCROP || it == ICOL_ROAD_PERV);
  f.xmf[c] = 0.0;
  f.qflx_snomelt[c] = 0.0;
  f.qflx_snofrz[c] = 0.0;
  f.qflx_snow_drain[c] = 0.0;
  // No level reads another level's values in the reference's four loops, and the
  // column sums (xmf, qflx_snomelt, qflx_snofrz, snomelt_accum, and level 1's
  // overwrite of the first two) are formed in ascending level order either way, so one
  // pass per level gives the same bits.
  for (int j = -nlevsno + 1; j <= nlevmax; j++) {
    const int jj = j + joff;
    // ---- the level's starting state ----
    S tinc, hm, xm, wice0, wmass0, sc;
    tinc = 0.0;
    hm = 0.0;
    xm = 0.0;
    wice0 = 0.0;
    wmass0 = 0.0;
    sc = 0.0;
    double wexice0 = 0.0;
    if (j >= snl + 1) {
      LV(f.imelt, c, jj, ld) = 0;
      wice0 = X.Ice(jj);
      wexice0 = j >= 1 ? LV(EXI, c, j, ld) : 0.0;
      wmass0 = X.Ice(jj) + X.Liq(jj) + wexice0;
      if (j >= 1) LV(f.exice_subs, c, j, ld) = 0.0;
    }
    if (j <= 0) {
      LV(f.qflx_snomelt_lyr, c, jj, ld) = 0.0;
      LV(f.qflx_snofrz_lyr, c, jj, ld) = 0.0;
    }
    if (j < snl + 1) continue;
    const bool active = (!wallroof && j <= nlevgrnd) || (wallroof && j <= D.nlevurb);
    // ---- melt / freeze decision ----
    if (j <= 0) {
      if (X.Ice(jj) > 0.0 && X.T(jj) > TFRZ) {
        LV(f.imelt, c, jj, ld) = 1;
        tinc = TFRZ - X.T(jj);
        X.T(jj) = TFRZ;
      }
      if (X.Liq(jj) > 0.0 && X.T(jj) < TFRZ) {
        LV(f.imelt, c, jj, ld) = 2;
        tinc = TFRZ - X.T(jj);
        X.T(jj) = TFRZ;
      }
    } else if (active) {
      if (X.Ice(jj) > 0.0 && X.T(jj) > TFRZ) {
        LV(f.imelt, c, jj, ld) = 1; tinc = TFRZ - X.T(jj); X.T(jj) = TFRZ;
      }
      if (LV(EXI, c, j, ld) > 0.0 && X.T(jj) > TFRZ) {
        LV(f.imelt, c, jj, ld) = 1; tinc = TFRZ - X.T(jj); X.T(jj) = TFRZ;
      }
      if (supercool_type) {
        const S tt = X.T(jj);
        if (tt < TFRZ) {
          const S smp = HFUS * (TFRZ - tt) / (GRAV * tt) * 1000.0;
          S scv = X.Watsat(j) * cm_pow(smp / X.Sucsat(j), -1.0 / X.Bsw(j));
          scv *= LVc(f.dz, c, jj, ld) * 1000.0;
          sc = scv;
        }
      }
      if (X.Liq(jj) > sc && X.T(jj) < TFRZ) {
        LV(f.imelt, c, jj, ld) = 2; tinc = TFRZ - X.T(jj); X.T(jj) = TFRZ;
      }
      if (f.h2osno_no_layers[c] > 0.0 && j == 1) {
        if (X.T(jj) > TFRZ) {
          LV(f.imelt, c, jj, ld) = 1; tinc = TFRZ - X.T(jj); X.T(jj) = TFRZ;
        }
      }
    }
    if (!active) continue;
    // ---- phase change ----
    int64_t im = LV(f.imelt, c, jj, ld);
    const S fct = X.Fact(jj);
    if (im > 0) {
      if (j == snl + 1) {
        if (j > 0) hm = dhsdT * tinc - tinc / fct;
        else hm = fse * (dhsdT * tinc - tinc / fct);
        if (j == 1 && fh != 0.0) hm -= fh * dhsdT * tinc;
      } else if (j == 1) {
        hm = (1.0 - fse - fh) * dhsdT * tinc - tinc / fct;
      } else {
        if (j < 1) hm = -fse * tinc / fct;
        else hm = -tinc / fct;
      }
    }
    if (im == 1 && hm < 0.0) { hm = 0.0; im = 0; }
    if (im == 2 && hm > 0.0) { hm = 0.0; im = 0; }
    LV(f.imelt, c, jj, ld) = im;
    if (im > 0 && fabs(VAL(hm)) > 0.0) {
      xm = hm * dtime / HFUS;
      if (j == 1) {
        if (f.h2osno_no_layers[c] > 0.0 && xm > 0.0) {
          const double temp1 = f.h2osno_no_layers[c];
          const S h2n = jl_max(0.0, temp1 - xm);
          f.h2osno_no_layers[c] = VAL(h2n);
          const S propor = h2n / temp1;
          f.snow_depth[c] = VAL(propor * f.snow_depth[c]);
          const S heatr0 = hm - HFUS * (temp1 - h2n) / dtime;
          if (heatr0 > 0.0) { xm = heatr0 * dtime / HFUS; hm = heatr0; }
          else { xm = 0.0; hm = 0.0; }
          const S qsm = jl_max(0.0, temp1 - h2n) / dtime;
          f.qflx_snomelt[c] = VAL(qsm);
          f.xmf[c] = HFUS * VAL(qsm);
          f.qflx_snow_drain[c] = VAL(qsm);
        }
      }
      S heatr = 0.0;
      S ice = X.Ice(jj);
      if (xm > 0.0) {
        ice = jl_max(0.0, wice0 - xm);
        X.Ice(jj) = ice;
        heatr = hm - jl_div(HFUS * (wice0 - ice), dtime);
        const S xm2 = xm - ice;
        if (ice == 0.0) {
          if (wexice0 >= 0.0 && xm2 > 0.0 && j >= 2) {
            const S ex = jl_max(0.0, wexice0 - xm2);
            LV(EXI, c, j, ld) = VAL(ex);
            heatr = hm - jl_div(HFUS * (wexice0 - ex + wice0 - ice), dtime);
          }
        }
      } else if (xm < 0.0) {
        if (j <= 0) {
          ice = jl_min(wmass0, wice0 - xm);
        } else {
          if (wmass0 - wexice0 < sc) ice = 0.0;
          else ice = jl_min(wmass0 - wexice0 - sc, wice0 - xm);
        }
        X.Ice(jj) = ice;
        heatr = hm - jl_div(HFUS * (wice0 - ice), dtime);
      }
      const double ei_val = j >= 1 ? LV(EXI, c, j, ld) : 0.0;
      const S liq = jl_max(0.0, wmass0 - ice - ei_val);
      X.Liq(jj) = liq;
      if (fabs(VAL(heatr)) > 0.0) {
        S tt = X.T(jj);
        if (j == snl + 1) {
          if (j == 1) tt += fct * heatr / (1.0 - (1.0 - fh) * fct * dhsdT);
          else if (fse > 0.0) tt += (fct / fse) * heatr / (1.0 - fct * dhsdT);
        } else if (j == 1) {
          tt += fct * heatr / (1.0 - (1.0 - fse - fh) * fct * dhsdT);
        } else {
          if (j > 0) tt += fct * heatr;
          else if (fse > 0.0) tt += (fct / fse) * heatr;
        }
        if (j <= 0)
          if (VAL(liq) * VAL(ice) > 0.0) tt = TFRZ;
        X.T(jj) = tt;
      }
      if (j >= 1) {
        const double ex = LV(EXI, c, j, ld);
        f.xmf[c] += jl_div(HFUS * (VAL(wice0) - VAL(ice)), dtime) + jl_div(HFUS * (wexice0 - ex), dtime);
        LV(f.exice_subs, c, j, ld) = jl_max(0.0, jl_div(wexice0 - ex, DENICE));
      } else {
        f.xmf[c] += jl_div(HFUS * (VAL(wice0) - VAL(ice)), dtime);
      }
      if (im == 1 && j < 1) {
        const double q = jl_div(jl_max(0.0, VAL(wice0) - VAL(ice)), dtime);
        LV(f.qflx_snomelt_lyr, c, jj, ld) = q;
        f.qflx_snomelt[c] += q;
        f.snomelt_accum[c] += q * dtime * 1.0e-3;
      }
      if (im == 2 && j < 1) {
        const double q = jl_div(jl_max(0.0, VAL(ice) - VAL(wice0)), dtime);
        LV(f.qflx_snofrz_lyr, c, jj, ld) = q;
        f.qflx_snofrz[c] += q;
      }
    }
  }
  f.eflx_snomelt[c] = f.qflx_snomelt[c] * HFUS;
  if (f.lun_urbpoi[l]) f.eflx_snomelt_u[c] = f.eflx_snomelt[c];
  else if (lit == ISTSOIL || lit == ISTCROP) f.eflx_snomelt_r[c] = f.eflx_snomelt[c];
}

__device__ inline void phase_change_beta_col(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c,
                                             double dtime, double dhsdT) {
  FieldState<clmgb_soiltemp_fields> X(f, c, D.ldc);
  phase_change_beta_col(D, f, c, dtime, dhsdT, X);
}

// ===========================================================================
// soil_temperature! (soil_temperature.jl:358-593) for one non-urban column,
// all of its kernels fused in the reference's call order.
// ===========================================================================
template <class ST>
__device__ inline uint32_t soil_temperature_col(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c,
                                                double dtime, int snow_method, ST& X) {
  typedef typename ST::S S;
  const int64_t ld = D.ldc, ldp = D.ldp;
  const int nlevsno = D.nlevsno, nlevgrnd = D.nlevgrnd, nlevsoi = D.nlevsoi;
  const int nlevmax = D.nlevmax;
  const int joff = nlevsno;
  const int nlev = nlevsno + nlevmax;
  const int64_t snl = f.col_snl[c];
  if (snl > 0 || snl < -nlevsno) return CLMGB_COL_LEVEL_RANGE;
  const int64_t l = f.col_landunit[c] - 1;
  const int64_t it = f.col_itype[c];
  const int64_t lit = f.lun_itype[l];
  if (f.lun_urbpoi[l] || is_wallroof(it) || it == ICOL_ROAD_IMPERV || it == ICOL_ROAD_PERV)
    return CLMGB_COL_URBAN;
  const int jtop = (int)snl + 1;          // top active layer (Fortran numbering)
  const int jjtop = jtop + joff;          // its 1-based level index
  const bool is_special = (lit == ISTWET || lit == ISTICE);
  const int64_t nbedrock = f.col_nbedrock[c];
  const double fse = f.frac_sno_eff[c];
  const double fh = f.frac_h2osfc[c];
  const double* DZ = f.dz;
  const double* Z = f.z;
  const double* ZI = f.zi;
  const double* EXI = f.excess_ice;

  // per-column working rows (level index jj, 1-based; entries outside the active
  // range are never read)
  S tk[MAXL + 2], fn[MAXL + 2], fct[MAXL + 2], tt[MAXL + 2];
  double zz[MAXL + 2];

  // ---- soil_therm_prop!: layer conductivity thk (_soil_snow_tk_kernel! :647-716) ----
  // the logarithms of the two constant bases of tkwat^x and tkice^x, formed once
  double ln_tkwat_lo, ln_tkice_lo;
  const double ln_tkwat = cm_log_dd(TKWAT, &ln_tkwat_lo), ln_tkice = cm_log_dd(TKICE, &ln_tkice_lo);
  // thk kept in tk[] first, interface conductivity computed in place afterwards.
  for (int jj = jjtop; jj <= nlev; jj++) {
    tt[jj] = X.T(jj);
    zz[jj] = LVc(Z, c, jj, ld);
  }
  for (int jj = jjtop; jj <= nlevsno + nlevgrnd; jj++) {
    const int j = jj - nlevsno;
    S thkv = 0.0;
    if (j >= 1) {
      if (!is_special) {
        if (j > nbedrock) {
          thkv = THK_BEDROCK;             // bedrock overrides the soil value (:684-686)
        } else {
          const S liq = X.Liq(jj), ice = X.Ice(jj);
          const double exi = LV(EXI, c, j, ld);
          const double dzv = LVc(DZ, c, jj, ld);
          const S ws = X.Watsat(j);
          S satw = jl_div(jl_div(liq, DENH2O) + jl_div(ice, DENICE) + jl_div(exi, DENICE), dzv * ws);
          satw = jl_min(1.0, satw);
          if (satw > 1.0e-7) {
            S dke;
            if (tt[jj] >= TFRZ) dke = jl_max(0.0, cm_log10(satw) + 1.0);
            else dke = satw;
            const S a1 = jl_div(liq, DENH2O * dzv);
            const S fl_denom = a1 + jl_div(ice, DENICE * dzv) + jl_div(exi, DENICE * dzv);
            const S fl = jl_div(a1, fl_denom);
            const S dksat =
                LVc(f.tkmg, c, j, ld) * cm_pow_lx(TKWAT, ln_tkwat, ln_tkwat_lo, fl * ws) *
                cm_pow_lx(TKICE, ln_tkice, ln_tkice_lo, (1.0 - fl) * ws);
            thkv = dke * dksat + (1.0 - dke) * LVc(f.tkdry, c, j, ld);
          } else {
            thkv = LVc(f.tkdry, c, j, ld);
          }
        }
      } else if (lit == ISTICE) {
        thkv = tt[jj] < TFRZ ? TKICE : TKWAT;
      } else {  // ISTWET
        if (j > nlevsoi) thkv = THK_BEDROCK;
        else thkv = tt[jj] < TFRZ ? TKICE : TKWAT;
      }
    } else {
      // snow layer (snl+1 <= j <= 0) — Jordan1991 or Sturm1997
      const double denom = jl_max(fse, 1.0e-6) * jl_max(LVc(DZ, c, jj, ld), 1.0e-6);
      const S bwv = jl_div(X.Ice(jj) + X.Liq(jj), denom);
      LV(f.bw, c, jj, ld) = VAL(bwv);
      if (snow_method == CLMGB_SNOW_JORDAN1991) {
        thkv = TKAIR + (7.75e-5 * bwv + 1.105e-6 * (bwv * bwv)) * (TKICE - TKAIR);
      } else {
        if (bwv <= 156.0) thkv = 0.023 + 0.234 * (bwv / 1000.0);
        else thkv = 0.138 - 1.01 * (bwv / 1000.0) + 3.233 * ((bwv / 1000.0) * (bwv / 1000.0));
      }
    }
    LV(f.thk, c, jj, ld) = VAL(thkv);
    tk[jj] = thkv;
  }
  // _tk_h2osfc_kernel! (:762-776): uses the soil-1 layer conductivity
  S tk_h2osfc;
  {
    const double zh2osfc = 1.0e-3 * (0.5 * f.h2osfc[c]);
    const double z1 = zz[1 + joff];
    const S tk1 = tk[1 + joff];
    const S denom = TKWAT * z1 + tk1 * zh2osfc;
    if (denom > 0.0) tk_h2osfc = jl_div(TKWAT * tk1 * (z1 + zh2osfc), denom);
    else tk_h2osfc = tk1;
  }
  // interface conductivity (_soil_tk_interface_kernel! :599-629), ascending so
  // tk[jj+1] still holds the layer value when tk[jj] is formed
  for (int jj = jjtop; jj <= nlev; jj++) {
    const int j = jj - nlevsno;
    if (j <= nlevgrnd - 1) {
      const S tkj = tk[jj], tkj1 = tk[jj + 1];
      const double zj = zz[jj], zj1 = zz[jj + 1], zij1 = LVc(ZI, c, jj + 1, ld);
      tk[jj] = jl_div(tkj * tkj1 * (zj1 - zj), tkj * (zj1 - zij1) + tkj1 * (zij1 - zj));
    } else if (j == nlevgrnd) {
      tk[jj] = 0.0;
    }
  }

  // ---- heat capacity cv (_soil_cv, _unresolved_snow_cv, _snow_cv) -> fact, fn ----
  // (_heat_diff_kernel! :1271-1319): fact = dtime/cv, top layer with the CAPR factor
  for (int jj = jjtop; jj <= nlevsno + nlevgrnd; jj++) {
    const int j = jj - nlevsno;
    const double dzv = LVc(DZ, c, jj, ld);
    S cv;
    if (j >= 1) {
      if (!is_special) {
        cv = LVc(f.csol, c, j, ld) * (1.0 - X.Watsat(j)) * dzv + (X.Ice(jj) * CPICE + X.Liq(jj) * CPLIQ) +
             LV(EXI, c, j, ld) * CPICE;
      } else {
        cv = X.Ice(jj) * CPICE + X.Liq(jj) * CPLIQ;
      }
      if (j > nbedrock) cv = CSOL_BEDROCK * dzv;
      if (j == 1 && f.h2osno_no_layers[c] > 0.0) cv += CPICE * f.h2osno_no_layers[c];
    } else {
      if (fse > 0.0)
        cv = jl_max(THIN_SFCLAYER, jl_div(CPLIQ * X.Liq(jj) + CPICE * X.Ice(jj), fse));
      else
        cv = THIN_SFCLAYER;
    }
    S fc;
    if (j == jtop) {
      fc = jl_div(jl_div(dtime, cv) * dzv, 0.5 * (zz[jj] - LVc(ZI, c, jj, ld) + CAPR * (zz[jj + 1] - LVc(ZI, c, jj, ld))));
      fn[jj] = jl_div(tk[jj] * (tt[jj + 1] - tt[jj]), zz[jj + 1] - zz[jj]);
    } else if (j <= nlevgrnd - 1) {
      fc = jl_div(dtime, cv);
      fn[jj] = jl_div(tk[jj] * (tt[jj + 1] - tt[jj]), zz[jj + 1] - zz[jj]);
    } else {
      fc = jl_div(dtime, cv);
      fn[jj] = f.eflx_bot[c];
    }
    fct[jj] = fc;
    X.Fact(jj) = fc;
  }

  // ---- compute_ground_heat_flux_and_deriv! (:1200-1263) ----
  const double eg = f.emg[c];
  const S tg = X.Tgrnd();
  const S lwrad_emit = eg * SB * jl_pow4(tg);
  const S dlwrad_emit = 4.0 * eg * SB * (tg * tg * tg);
  const S lwrad_emit_snow = eg * SB * jl_pow4(tt[jjtop]);
  const S lwrad_emit_soil = eg * SB * jl_pow4(tt[1 + joff]);
  const S lwrad_emit_h2osfc = eg * SB * jl_pow4(X.Th2osfc());
  const double htvp = f.htvp[c];
  const S forc = X.ForcLwrad();
  const int64_t pi = f.col_patchi[c], pf = f.col_patchf[c];
  if (pi < 1 || pf > D.np || pf < pi - 1) return CLMGB_COL_PATCH_RANGE;
  S dhsdT = 0.0, hs_soil = 0.0, hs_h2osfc = 0.0, hs_top_snow = 0.0;
  double sabg_lyr_col[MAXSNO + 2];
  for (int k = 0; k <= nlevsno + 1; k++) sabg_lyr_col[k] = 0.0;
  for (int64_t p1 = pi; p1 <= pf; p1++) {
    const int64_t p = p1 - 1;
    if (f.patch_column[p] != c + 1 + D.c0) continue;
    S dh_p = 0.0, hsoil_p = 0.0, hh_p = 0.0;
    const bool act = f.mask_nolakep[p] != 0;
    const S base = f.dlrad[p] + (1.0 - (double)f.frac_veg_nosno[p]) * eg * forc;
    if (act && !f.lun_urbpoi[f.patch_landunit[p] - 1]) {
      const S gnet = f.sabg[p] + base - lwrad_emit - (f.eflx_sh_grnd[p] + f.qflx_evap_soi[p] * htvp);
      f.eflx_gnet[p] = VAL(gnet);
      f.sabg_chk[p] = fse * f.sabg_snow[p] + (1.0 - fse) * f.sabg_soil[p];
      const S dg = -f.cgrnd[p] - dlwrad_emit;
      f.dgnetdT[p] = VAL(dg);
      const double wt = f.patch_wtcol[p];
      const S gsoil = f.sabg_soil[p] + base - lwrad_emit_soil - (f.eflx_sh_soil[p] + f.qflx_ev_soil[p] * htvp);
      const S gh2o = f.sabg_soil[p] + base - lwrad_emit_h2osfc - (f.eflx_sh_h2osfc[p] + f.qflx_ev_h2osfc[p] * htvp);
      if (wt != 0.0) {
        dh_p = dg * wt;
        hsoil_p = gsoil * wt;
        hh_p = gh2o * wt;
      }
    }
    dhsdT += dh_p; hs_soil += hsoil_p; hs_h2osfc += hh_p;
    if (act) {   // SNICAR top-layer flux + per-layer solar (:1139-1167)
      const double wt = f.patch_wtcol[p];
      const double sab = LVc(f.sabg_lyr, p, jtop + joff, ldp);
      const S gsnow = sab + base - lwrad_emit_snow - (f.eflx_sh_snow[p] + f.qflx_ev_snow[p] * htvp);
      hs_top_snow += gsnow * wt;
      for (int j = jtop; j <= 1; j++) sabg_lyr_col[j + nlevsno] += LVc(f.sabg_lyr, p, j + joff, ldp) * wt;
    }
  }

  // ---- _h2osfc_thermprop_kernel! (:116-130) ----
  double ch, dz_h2osfc;
  if (f.h2osfc[c] > THIN_SFCLAYER && fh > THIN_SFCLAYER) {
    ch = jl_max(THIN_SFCLAYER, CPLIQ * f.h2osfc[c] / fh);
    dz_h2osfc = jl_max(THIN_SFCLAYER, 1.0e-3 * f.h2osfc[c] / fh);
  } else {
    ch = THIN_SFCLAYER;
    dz_h2osfc = THIN_SFCLAYER;
  }
  f.c_h2osfc[c] = ch;

  // ---- set_rhs_vec! + set_matrix! straight into band rows (row r = system row,
  //      r = 0 is the top active layer; the surface-water row sits between the
  //      snow layers and soil layer 1), ab[r][d] = A[r, r-2+d] ----
  constexpr int W = 7;
  S ab[MAXROWS * W];
  S x[MAXROWS];
  const int n = nlevgrnd - (int)snl + 1;
  const int rsw = -(int)snl;              // row of the surface-water equation
  const double omc = 1.0 - CNFAC;
  for (int k = 0; k < n * W; k++) ab[k] = 0.0;
  // snow rows: r = j - jtop  (j = jtop..0)
  for (int j = jtop; j <= 0; j++) {
    const int jj = j + joff;
    const int r = j - jtop;
    const S fc = fct[jj];
    const double dzp = zz[jj + 1] - zz[jj];
    if (j == jtop) {
      x[r] = tt[jj] + fc * (hs_top_snow - dhsdT * tt[jj] + CNFAC * fn[jj]);
      ab[r * W + 2] = 1.0 + jl_div(omc * fc * tk[jj], dzp) - fc * dhsdT;
    } else {
      x[r] = tt[jj] + CNFAC * fc * (fn[jj] - fn[jj - 1]);
      x[r] += fc * sabg_lyr_col[jj];
      const double dzm = zz[jj] - zz[jj - 1];
      ab[r * W + 1] = jl_div(-omc * fc * tk[jj - 1], dzm);
      ab[r * W + 2] = 1.0 + omc * fc * (jl_div(tk[jj], dzp) + jl_div(tk[jj - 1], dzm));
    }
    if (j != 0) ab[r * W + 3] = jl_div(-omc * fc * tk[jj], dzp);
    else ab[r * W + 4] = jl_div(-omc * fc * tk[jj], dzp);   // snow-soil coupling skips the h2osfc row
  }
  // surface-water row
  S fn_h2osfc;
  {
    const double dzm = 0.5 * dz_h2osfc + zz[1 + joff];
    const S th = X.Th2osfc();
    const S fnh = tk_h2osfc * (tt[1 + joff] - th) / dzm;
    fn_h2osfc = fnh;
    x[rsw] = th + (dtime / ch) * (hs_h2osfc - dhsdT * th + CNFAC * fnh);
    ab[rsw * W + 2] = 1.0 + omc * (dtime / ch) * tk_h2osfc / dzm - (dtime / ch) * dhsdT;
    ab[rsw * W + 3] = -omc * (dtime / ch) * tk_h2osfc / dzm;
  }
  // soil rows: r = rsw + j
  for (int j = 1; j <= nlevgrnd; j++) {
    const int jj = j + joff;
    const int r = rsw + j;
    const S fc = fct[jj];
    const S t0 = tt[jj];
    if (j == jtop) {   // snl == 0
      const double dzp = zz[jj + 1] - zz[jj];
      x[r] = t0 + fc * (hs_top_snow - dhsdT * t0 + CNFAC * fn[jj]);
      ab[r * W + 2] = 1.0 + jl_div(omc * fc * tk[jj], dzp) - fc * dhsdT;
      ab[r * W + 3] = jl_div(-omc * fc * tk[jj], dzp);
    } else if (j == 1) {
      const double dzm = zz[jj] - zz[jj - 1];
      const double dzp = zz[jj + 1] - zz[jj];
      x[r] = t0 + fc * ((1.0 - fse) * (hs_soil - dhsdT * t0) + CNFAC * (fn[jj] - fse * fn[jj - 1]));
      x[r] += fse * fc * sabg_lyr_col[j + nlevsno];
      ab[r * W + 3] = jl_div(-omc * fc * tk[jj], dzp);
      ab[r * W + 2] = 1.0 + omc * fc * (jl_div(tk[jj], dzp) + jl_div(fse * tk[jj - 1], dzm)) - (1.0 - fse) * fc * dhsdT;
      ab[r * W + 0] = jl_div(-fse * omc * fc * tk[jj - 1], dzm);
    } else if (j <= nlevgrnd - 1) {
      const double dzm = zz[jj] - zz[jj - 1];
      const double dzp = zz[jj + 1] - zz[jj];
      x[r] = t0 + CNFAC * fc * (fn[jj] - fn[jj - 1]);
      ab[r * W + 3] = jl_div(-omc * fc * tk[jj], dzp);
      ab[r * W + 2] = 1.0 + omc * fc * (jl_div(tk[jj], dzp) + jl_div(tk[jj - 1], dzm));
      ab[r * W + 1] = jl_div(-omc * fc * tk[jj - 1], dzm);
    } else {
      const double dzm = zz[jj] - zz[jj - 1];
      x[r] = t0 - CNFAC * fc * fn[jj - 1] + fc * fn[jj];
      ab[r * W + 2] = 1.0 + jl_div(omc * fc * tk[jj - 1], dzm);
      ab[r * W + 1] = jl_div(-omc * fc * tk[jj - 1], dzm);
    }
  }
  if (fh != 0.0) {   // surface-water corrections to soil layer 1 (:1480-1494, :1689-1707)
    const int jj = 1 + joff;
    const int r = rsw + 1;
    const S fc = fct[jj];
    x[r] -= fh * fc * ((hs_soil - dhsdT * tt[jj]) + CNFAC * fn_h2osfc);
    const double dzm = 0.5 * dz_h2osfc + zz[1 + joff];
    ab[r * W + 2] += fh * (omc * fc * tk_h2osfc / dzm + fc * dhsdT);
    ab[r * W + 1] = -fh * omc * fc * tk_h2osfc / dzm;
  }
  // the reference's densify drops band entries that fall outside the n x n system
  ab[0 * W + 0] = 0.0; ab[0 * W + 1] = 0.0;
  if (n > 1) ab[1 * W + 0] = 0.0;

  // ---- batched_band_solve! (band_diagonal.jl:87-170), banded form ----
  X.band_solve(ab, x, n);

  // ---- _tvector_extract_kernel! (:149-167) ----
  for (int j = jtop; j <= 0; j++) tt[j + joff] = x[j - jtop];
  for (int j = 1; j <= nlevgrnd; j++) tt[j + joff] = x[rsw + j];
  for (int jj = jjtop; jj <= nlev; jj++) X.T(jj) = tt[jj];
  if (fh == 0.0) X.Th2osfc() = tt[1 + joff];
  else X.Th2osfc() = x[rsw];

  // ---- _fn1_kernel! (:170-206) and _eflx_fgr_kernel! (:250-269) ----
  const bool issoilcrop = (lit == ISTSOIL || lit == ISTCROP);
  {
    f.eflx_fgr12[c] = 0.0;
    for (int jj = jjtop; jj <= nlev; jj++) {
      const int j = jj - nlevsno;
      double fn1v;
      if (j <= nlevgrnd - 1) fn1v = jl_div(VAL(tk[jj]) * (VAL(tt[jj + 1]) - VAL(tt[jj])), zz[jj + 1] - zz[jj]);
      else fn1v = 0.0;
      if (j == 1) f.eflx_fgr12[c] = -CNFAC * VAL(fn[jj]) - (1.0 - CNFAC) * fn1v;
      if (j >= 1 && j < nlevgrnd && issoilcrop) LV(f.eflx_fgr, c, j, ld) = -CNFAC * VAL(fn[jj]) - (1.0 - CNFAC) * fn1v;
      else if (j == nlevgrnd && issoilcrop) LV(f.eflx_fgr, c, j, ld) = 0.0;
    }
  }

  // ---- phase change (:552-561) ----
  phase_change_h2osfc_col(D, f, c, dtime, dhsdT, X);
  phase_change_beta_col(D, f, c, dtime, dhsdT, X);

  // ---- _tgrnd_kernel! (:224-247) ----
  {
    const S t1 = X.T(1 + joff), th = X.Th2osfc();
    S tgn;
    if (snl < 0) {
      const S ts = X.T(jjtop);
      if (fh != 0.0) tgn = fse * ts + (1.0 - fse - fh) * t1 + fh * th;
      else tgn = fse * ts + (1.0 - fse) * t1;
    } else {
      if (fh != 0.0) tgn = (1.0 - fh) * t1 + fh * th;
      else tgn = t1;
    }
    X.Tgrnd() = tgn;
  }
  uint32_t status = 0;
  for (int jj = jjtop; jj <= nlev; jj++)
    if (!isfinite(VAL(X.T(jj)))) status |= CLMGB_COL_NONFINITE;
  return status;
}

__device__ inline uint32_t soil_temperature_col(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c,
                                                double dtime, int snow_method) {
  FieldState<clmgb_soiltemp_fields> X(f, c, D.ldc);
  return soil_temperature_col(D, f, c, dtime, snow_method, X);
}

// ===========================================================================
// set_soil_water_fractions! kernel (soil_hydrology.jl:110-130), column c.
// ===========================================================================
template <class ST>
__device__ __forceinline__ void water_fractions_col(const Dims& D, const clmgb_soilwater_fields& f, int64_t c,
                                                    ST& X) {
  typedef typename ST::S S;
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  for (int j = 1; j <= D.nlevsoi; j++) {
    const double exi = LV(f.excess_ice, c, j, ld);
    const double dz_ext = LVc(f.dz, c, j + joff, ld) + jl_div(exi, DENICE);
    const S ws = X.Watsat(j);
    const S vol_ice = jl_min(ws, jl_div(X.Ice(j + joff) + exi, dz_ext * DENICE));
    LV(f.eff_porosity, c, j, ld) = jl_max(0.01, VAL(ws) - VAL(vol_ice));
    X.Icefrac(j) = jl_min(1.0, jl_div(vol_ice, ws));
  }
}

__device__ __forceinline__ void water_fractions_col(const Dims& D, const clmgb_soilwater_fields& f, int64_t c) {
  FieldState<clmgb_soilwater_fields> X(f, c, D.ldc);
  water_fractions_col(D, f, c, X);
}

// ===========================================================================
// _soilwm_moisture_form_kernel! (soil_water_movement.jl:1250-1489) as a per-column
// state machine: mf_begin loads a column, mf_attempt runs one substep attempt of
// the reference's `while true` loop, mf_end stores the results.  A thread can then
// work through several columns, one attempt at a time (see k_moisture_form_queue).
//
// Identical arithmetic to the reference, with three exact hoists:
//  * the ice impedance 10^(-e_ice*icefrac) depends only on icefrac, fixed during
//    the call, so it is formed once per column instead of once per attempt;
//  * a rejected attempt leaves h2osoi_liq unchanged, so the hydraulic properties,
//    fluxes and flux derivatives of the retry equal the previous attempt's bit for
//    bit; they are recomputed only after an accepted substep;
//  * dt_dz = dtsub/(1000*dz): when dtsub is halved or doubled the quotient scales
//    by exactly the same power of two, so it is rescaled through its exponent bits
//    instead of divided again; any other change of dtsub divides afresh.
// The accept/reject test and the error estimate only decide the substep schedule,
// so they are formed from the values of the active quantities.
// ===========================================================================
template <class S>
struct MfLaneT {
  static constexpr bool kRefreshInline = true;   // mf_attempt runs mf_refresh itself
  static constexpr bool kDzw = false;            // dzv holds dz (mf_dzw forms 1000*dz)
  int64_t c;
  int nlayers;
  int nsub;
  bool fresh;
  uint32_t status;
  double dtsub, dtdone, dt_cur;
  S qc;
  // the refresh's values the attempts read: the inflow of level 1, the bottom
  // level's conductivity and its derivative (the flux lower boundary's recharge)
  S qin1, hk_bot, dhkdw_bot;
  double dzv[MAXSOI + 1], dt_dz[MAXSOI + 1];
  S liq[MAXSOI + 1], imp[MAXSOI + 1];
  // outflow of each level and its derivatives; the inflow of level j > 1 and its
  // derivatives are the outflow ones of level j-1 (qin[j] = qout[j-1],
  // dqidw0[j] = dqodw1[j-1], dqidw1[j] = dqodw2[j-1], :1372-1376)
  S qout[MAXSOI + 1], dqodw1[MAXSOI + 1], dqodw2[MAXSOI + 1], fnet1[MAXSOI + 1];
  S gam[MAXSOI + 1], dwat[MAXSOI + 1];
};
typedef MfLaneT<double> MfLane;

// 1000*dz of level j of a lane: the product M_TO_MM*dz, or the lane's own copy of it
// (LT::kDzw), which has the same bits (DENH2O*dz of the column record)
template <class LT>
__device__ __forceinline__ double mf_dzw(const LT& L, int j) {
  if constexpr (LT::kDzw) return L.dzv[j];
  else return M_TO_MM * L.dzv[j];
}

// Substep log record (clmgb_substep_log): the liquid water of levels 1..nlevsoi at
// the start of an accepted substep, its dtsub, the time done before it.  After a
// column's cap records: its final liquid water, smp_l, hk_l (nlevsoi each),
// qcharge, attempts and status.
constexpr int SUB_REC = MAXSOI + 2;
constexpr int LOG_FIN = 3 * MAXSOI + 3;

// Ice impedance 10^(-e_ice*icefrac) of layer j (interface mean above the bottom
// layer), as formed at soil_water_movement.jl:1287-1293.
template <class ST>
__device__ __forceinline__ typename ST::S mf_impedance(double e_ice, int j, int nlayers, ST& X) {
  double ln10_lo;
  const double ln10 = cm_log_dd(10.0, &ln10_lo);
  if (j == nlayers) return cm_pow_lx(10.0, ln10, ln10_lo, -e_ice * X.Icefrac(j));
  return cm_pow_lx(10.0, ln10, ln10_lo, -e_ice * (0.5 * (X.Icefrac(j) + X.Icefrac(j + 1))));
}
__device__ __forceinline__ double mf_impedance(const Dims& D, const clmgb_soilwater_fields& f, double e_ice,
                                               int64_t c, int j, int nlayers) {
  FieldState<clmgb_soilwater_fields> X(f, c, D.ldc);
  return mf_impedance(e_ice, j, nlayers, X);
}

// returns false (and sets L.status) when the column cannot be solved.  imp_cache,
// when given, holds the impedances formed by k_impedance ([nlevsoi, ld_imp]).
// dt_init, when given, is a proposed size of the first substep per column (the
// warm start); it is clamped to [dtmin, dtime] and the solver's own error test
// accepts or halves it like any other substep.
template <class ST>
__device__ __forceinline__ bool mf_begin(MfLaneT<typename ST::S>& L, const Dims& D, const clmgb_soilwater_fields& f,
                                         const clmgb_swm_config& cfg, double dtime, int64_t c, ST& X,
                                         const double* imp_cache = nullptr, int64_t ld_imp = 0,
                                         const double* dt_init = nullptr) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  L.c = c;
  L.status = 0;
  const int64_t nl = f.col_nbedrock[c];
  if (nl < 1 || nl > D.nlevsoi) {
    L.status = CLMGB_COL_LEVEL_RANGE;
    return false;
  }
  const int nlayers = (int)nl;
  L.nlayers = nlayers;
  for (int j = 1; j <= nlayers; j++) {
    L.liq[j] = X.Liq(joff + j);
    L.dzv[j] = LVc(f.dz, c, joff + j, ld);
  }
  if (imp_cache) {
    for (int j = 1; j <= nlayers; j++) L.imp[j] = imp_cache[(int64_t)(j - 1) * ld_imp + c];
  } else {
    for (int j = 1; j <= nlayers; j++) L.imp[j] = mf_impedance(cfg.e_ice, j, nlayers, X);
  }
  L.nsub = 0;
  L.dtsub = dtime;
  if (dt_init) {
    const double d = dt_init[c];
    if (d == d) L.dtsub = jl_min(jl_max(d, cfg.dtmin), dtime);   // NaN keeps dtime
  }
  L.dtdone = 0.0;
  L.qc = 0.0;
  L.fresh = true;
  L.dt_cur = -1.0;
  return true;
}

// The hydraulic properties, fluxes and flux derivatives of an accepted substep's
// starting water (the `fresh` part of an attempt, soil_water_movement.jl:1280-1378).
// mf_attempt calls it at the first attempt after an accepted substep; the
// work-queue kernel may also call it on its own, before that attempt, when it
// batches this block across the lanes of a warp (same operations, same order).
template <class ST>
__device__ __forceinline__ void mf_refresh(MfLaneT<typename ST::S>& L, const Dims& D,
                                           const clmgb_soilwater_fields& f, const clmgb_swm_config& cfg, ST& X) {
  typedef typename ST::S S;
  const int64_t ld = D.ldc;
  const int64_t c = L.c;
  const int joff = D.nlevsno, joff_zi = D.nlevsno + 1, nlevsoi = D.nlevsoi;
  const int nlayers = L.nlayers;
  const int lower_bc = cfg.lower_boundary_condition;
  // Level by level: the saturation of level j+1, the hydraulic properties of level j
  // (Clapp-Hornberger inlined, :1280-1308), then the flux between levels j-1 and j
  // and its derivatives (:1310-1345), which need both levels' properties.  Every
  // value is formed by the reference's expression; only the loop order differs, so
  // no level's arrays are kept beyond the two the flux needs.
  auto saturation = [&](int j) -> S {
    const S vwc = jl_max(L.liq[j], 1.0e-6) / (L.dzv[j] * DENH2O);
    S s = vwc / X.Watsat(j);
    s = jl_min(s, 1.0);
    return jl_max(0.01, s);
  };
  S s_j = saturation(1);
  S hk_p = 0.0, dhkdw_p = 0.0, smp_p = 0.0, dsmpdw_p = 0.0;   // level j-1
  S hk_j = 0.0, dhkdw_j = 0.0, smp_j = 0.0, dsmpdw_j = 0.0;
  for (int j = 1; j <= nlayers; j++) {
    const S s_n = (j < nlayers) ? saturation(j + 1) : s_j;
    S s1 = (j == nlayers) ? s_j : 0.5 * (s_j + s_n);
    s1 = jl_min(s1, 1.0);
    s1 = jl_max(0.01, s1);
    const S b = X.Bsw(j);
    hk_j = L.imp[j] * X.Hksat(j) * cm_pow(s1, 2.0 * b + 3.0);
    dhkdw_j = (2.0 * b + 3.0) * hk_j / s1;
    const S sn = s_j;
    smp_j = -X.Sucsat(j) * cm_pow(sn, -b);
    const S dsmpds = -b * smp_j / sn;
    dsmpdw_j = dsmpds / X.Watsat(j);
    LV(f.smp_l, c, j, ld) = VAL(smp_j);
    LV(f.hk_l, c, j, ld) = VAL(hk_j);
    if (j >= 2) {
      const int k = j - 1;
      const S dhkds1 = 0.5 * dhkdw_p / X.Watsat(k);
      const S dhkds2 = 0.5 * dhkdw_p / X.Watsat(k + 1);
      const S num = smp_j - smp_p;
      const double den = M_TO_MM * (LVc(f.z, c, joff + k + 1, ld) - LVc(f.z, c, joff + k, ld));
      L.qout[k] = -hk_p * num / den + hk_p;
      L.dqodw1[k] = (hk_p * dsmpdw_p - dhkds1 * num) / den + dhkds1;
      L.dqodw2[k] = (-hk_p * dsmpdw_j - dhkds2 * num) / den + dhkds2;
    }
    hk_p = hk_j; dhkdw_p = dhkdw_j; smp_p = smp_j; dsmpdw_p = dsmpdw_j;
    s_j = s_n;
  }
  L.hk_bot = hk_j;
  L.dhkdw_bot = dhkdw_j;
  // ---- bottom level (:1347-1370) ----
  {
    const int j = nlayers;
    L.qout[j] = 0.0; L.dqodw1[j] = 0.0; L.dqodw2[j] = 0.0;
    if (lower_bc == CLMGB_BC_WATERTABLE) {
      int jwt = nlevsoi;
      for (int jj = 1; jj <= nlevsoi; jj++) {
        if (f.zwt[c] <= LVc(f.zi, c, joff_zi + jj, ld)) { jwt = jj - 1; break; }
      }
      if (j <= jwt) {
        const S dhkds1l = dhkdw_j / X.Watsat(j);
        const S num = -smp_j;
        const double den = M_TO_MM * (f.zwt[c] - LVc(f.z, c, joff + j, ld));
        L.qout[j] = -hk_j * num / den + hk_j;
        L.dqodw1[j] = (hk_j * dsmpdw_j - dhkds1l * num) / den + dhkds1l;
      }
    } else if (lower_bc == CLMGB_BC_FLUX) {
      L.qout[j] = hk_j;
      L.dqodw1[j] = dhkdw_j / X.Watsat(j);
    }
  }
  L.qin1 = f.qflx_infl[c];
  L.fnet1[1] = L.qin1 - L.qout[1] - LVc(f.qflx_rootsoi, c, 1, ld);
  for (int j = 2; j <= nlayers; j++) L.fnet1[j] = L.qout[j - 1] - L.qout[j] - LVc(f.qflx_rootsoi, c, j, ld);
  L.fresh = false;
}

// one attempt; returns true when the column's substep loop has finished.  LT is
// MfLaneT or a lane whose refresh is run elsewhere (LT::kRefreshInline false: the
// caller has refreshed it before the attempt).
template <class LT, class ST>
__device__ __forceinline__ bool mf_attempt(LT& L, const Dims& D, const clmgb_soilwater_fields& f,
                                           const clmgb_swm_config& cfg, double dtime, ST& X) {
  typedef typename ST::S S;
  const int64_t ld = D.ldc;
  const int64_t c = L.c;
  const int nlayers = L.nlayers;
  const int lower_bc = cfg.lower_boundary_condition;
  L.nsub += 1;
  if (L.nsub > D.attempt_cap) {
    L.status |= CLMGB_COL_SUBSTEP_CAP;
    return true;
  }
  const double dtsub = L.dtsub;
  // ---- dt_dz = dtsub / (1000*dz) ----
  if (dtsub != L.dt_cur) {
    const uint64_t a = (uint64_t)__double_as_longlong(dtsub), b = (uint64_t)__double_as_longlong(L.dt_cur);
    const uint64_t MANT = 0x000fffffffffffffULL;
    const int ea = (int)((a >> 52) & 0x7ff), eb = (int)((b >> 52) & 0x7ff);
    if (L.dt_cur > 0.0 && (a & MANT) == (b & MANT) && ea > 0 && eb > 0 && ea < 2047 && eb < 2047) {
      const long long shift = (long long)(ea - eb) << 52;
      for (int j = 1; j <= nlayers; j++) {
        const long long v = __double_as_longlong(L.dt_dz[j]);
        const int ev = (int)((v >> 52) & 0x7ff);
        if (ev + (ea - eb) > 0 && ev + (ea - eb) < 2047 && ev > 0)
          L.dt_dz[j] = __longlong_as_double(v + shift);
        else
          L.dt_dz[j] = jl_div(dtsub, mf_dzw(L, j));
      }
    } else {
      for (int j = 1; j <= nlayers; j++) L.dt_dz[j] = jl_div(dtsub, mf_dzw(L, j));
    }
    L.dt_cur = dtsub;
  }
  if constexpr (LT::kRefreshInline) {
    if (L.fresh) mf_refresh(L, D, f, cfg, X);
  }
  // ---- RHS / LHS (:1380-1397) fused into the Thomas forward sweep (:1421-1438) ----
  S bet, dwat_prev;
  {
    const S rmx = -L.fnet1[1] * L.dt_dz[1];
    const S dqidw1_1 = 0.0;                                   // no inflow derivative at level 1
    const S bmx = -1.0 - (-dqidw1_1 + L.dqodw1[1]) * L.dt_dz[1];
    bet = bmx;
    if (abs_lt(VAL(bet), 1.0e-30)) bet = 1.0e-30;
    dwat_prev = jl_div(rmx, bet);
    L.dwat[1] = dwat_prev;
  }
  S cmx_prev = -L.dqodw2[1] * L.dt_dz[1];
  for (int j = 2; j <= nlayers; j++) {
    const S amx = L.dqodw1[j - 1] * L.dt_dz[j];
    const S bmx = -1.0 - (-L.dqodw2[j - 1] + L.dqodw1[j]) * L.dt_dz[j];
    S cmx = 0.0;
    if (j != nlayers) cmx = -L.dqodw2[j] * L.dt_dz[j];
    const S rmx = -L.fnet1[j] * L.dt_dz[j];
    L.gam[j] = jl_div(cmx_prev, bet);
    bet = bmx - amx * L.gam[j];
    if (abs_lt(VAL(bet), 1.0e-30)) bet = copysign(1.0e-30, VAL(bet) == 0.0 ? 1.0 : VAL(bet));
    dwat_prev = jl_div(rmx - amx * dwat_prev, bet);
    L.dwat[j] = dwat_prev;
    cmx_prev = cmx;
  }
  {
    S dwat_next = dwat_prev;
    for (int j = nlayers - 1; j >= 1; j--) {
      dwat_next = L.dwat[j] - L.gam[j + 1] * dwat_next;
      L.dwat[j] = dwat_next;
    }
  }
  // ---- error estimate (:1440-1457) ----
  const bool expensive = (cfg.flux_calculation == 42);
  double errorMax = 0.0;
  for (int j = 1; j <= nlayers; j++) {
    double fnet0;
    if (expensive) {
      const double dqidw1_1 = 0.0;
      const double qin_test = j == 1 ? VAL(L.qin1) + dqidw1_1 * VAL(L.dwat[j])
                                     : VAL(L.qout[j - 1]) + VAL(L.dqodw1[j - 1]) * VAL(L.dwat[j - 1]) +
                                           VAL(L.dqodw2[j - 1]) * VAL(L.dwat[j]);
      const double qout_test = j == nlayers ? VAL(L.qout[j]) + VAL(L.dqodw1[j]) * VAL(L.dwat[j])
                                            : VAL(L.qout[j]) + VAL(L.dqodw1[j]) * VAL(L.dwat[j]) +
                                                  VAL(L.dqodw2[j]) * VAL(L.dwat[j + 1]);
      fnet0 = qin_test - qout_test - LVc(f.qflx_rootsoi, c, j, ld);
    } else {
      fnet0 = jl_div(VAL(L.dwat[j]), L.dt_dz[j]);
    }
    const double ev = fabs(VAL(L.fnet1[j]) - fnet0) * dtsub * 0.5;
    errorMax = jl_max(errorMax, ev);
  }
  // ---- reject (:1460-1463) ----
  if (errorMax > cfg.xTolerUpper && dtsub > cfg.dtmin) {
    L.dtsub = jl_max(dtsub / 2.0, cfg.dtmin);
    return false;
  }
  // ---- accept (:1466-1483) ----
  for (int j = 1; j <= nlayers; j++) L.liq[j] = L.liq[j] + L.dwat[j] * mf_dzw(L, j);
  L.fresh = true;
  S qcTemp;
  if (lower_bc == CLMGB_BC_FLUX) qcTemp = L.hk_bot + L.dhkdw_bot * L.dwat[nlayers];
  else if (lower_bc == CLMGB_BC_ZERO_FLUX) qcTemp = 0.0;
  else qcTemp = L.qout[nlayers] + L.dqodw1[nlayers] * L.dwat[nlayers];
  L.qc += qcTemp * (dtsub / dtime);
  L.dtdone += dtsub;
  if (fabs(dtime - L.dtdone) < cfg.verySmall) return true;
  double nd = dtsub;
  if (errorMax < cfg.xTolerLower) nd = dtsub * 2.0;
  L.dtsub = jl_min(nd, dtime - L.dtdone);
  return false;
}

template <class LT, class ST>
__device__ __forceinline__ uint32_t mf_end(LT& L, const Dims& D, const clmgb_soilwater_fields& f, ST& X) {
  const int64_t c = L.c;
  const int joff = D.nlevsno;
  uint32_t status = L.status;
  for (int j = 1; j <= L.nlayers; j++) {
    X.Liq(joff + j) = L.liq[j];
    if (!isfinite(VAL(L.liq[j]))) status |= CLMGB_COL_NONFINITE;
  }
  X.Qcharge() = L.qc;
  f.num_substeps[c] = (double)L.nsub;
  return status;
}

// production forms: the column's state in the caller's fields
__device__ __forceinline__ bool mf_begin(MfLane& L, const Dims& D, const clmgb_soilwater_fields& f,
                                         const clmgb_swm_config& cfg, double dtime, int64_t c,
                                         const double* imp_cache = nullptr, int64_t ld_imp = 0,
                                         const double* dt_init = nullptr) {
  FieldState<clmgb_soilwater_fields> X(f, c, D.ldc);
  return mf_begin(L, D, f, cfg, dtime, c, X, imp_cache, ld_imp, dt_init);
}
__device__ __forceinline__ bool mf_attempt(MfLane& L, const Dims& D, const clmgb_soilwater_fields& f,
                                           const clmgb_swm_config& cfg, double dtime) {
  FieldState<clmgb_soilwater_fields> X(f, L.c, D.ldc);
  return mf_attempt(L, D, f, cfg, dtime, X);
}
__device__ __forceinline__ uint32_t mf_end(MfLane& L, const Dims& D, const clmgb_soilwater_fields& f) {
  FieldState<clmgb_soilwater_fields> X(f, L.c, D.ldc);
  return mf_end(L, D, f, X);
}

// The whole substep loop for one column (one thread, one column).
template <class ST>
__device__ inline uint32_t moisture_form_col(const Dims& D, const clmgb_soilwater_fields& f,
                                             const clmgb_swm_config& cfg, double dtime, int64_t c, ST& X) {
  MfLaneT<typename ST::S> L;
  if (!mf_begin(L, D, f, cfg, dtime, c, X)) return L.status;
  while (!mf_attempt(L, D, f, cfg, dtime, X)) {
  }
  return mf_end(L, D, f, X);
}
__device__ inline uint32_t moisture_form_col(const Dims& D, const clmgb_soilwater_fields& f,
                                             const clmgb_swm_config& cfg, double dtime, int64_t c) {
  FieldState<clmgb_soilwater_fields> X(f, c, D.ldc);
  return moisture_form_col(D, f, cfg, dtime, c, X);
}

// ===========================================================================
// compute_qcharge! (soil_water_movement.jl:1153-1215) as soilwater_moisture_form! runs it
// after the solve under use_aquifer_layer(cfg) (:1575-1598; of those lower boundaries the
// moisture form accepts BC_WATERTABLE only).  The reference hands it freshly zeroed dwat,
// smp and imped rows, and vwc_liq = max(h2osoi_liq, 1e-6)/(dz*1000) of the solved water on
// levels 1..min(nbedrock, nlevsoi), zero below.  So the conductivity ka = 0*hksat*s1^(2b+3)
// is zero and the recharge written is a signed zero, for every column whose water table
// lies within the soil column (jwt < nlevsoi); the other columns keep the solve's qcharge.
// ===========================================================================
// jwt: the number of soil levels above the water table (:1177-1184)
__device__ __forceinline__ int watertable_level(const Dims& D, const clmgb_soilwater_fields& f, int64_t c) {
  int jwt = D.nlevsoi;
  for (int j = 1; j <= D.nlevsoi; j++) {
    if (f.zwt[c] <= LVc(f.zi, c, D.nlevsno + 1 + j, D.ldc)) {
      jwt = j - 1;
      break;
    }
  }
  return jwt;
}

// True when that pass replaces the solve's qcharge of column c.  The value it writes then
// depends on no state or parameter (ka is exactly zero), so the qcharge adjoint the
// step's reverse receives stops there.
__device__ __forceinline__ bool qcharge_replaced(const Dims& D, const clmgb_soilwater_fields& f,
                                                 const clmgb_swm_config& cfg, int64_t c) {
  return cfg.lower_boundary_condition == CLMGB_BC_WATERTABLE && watertable_level(D, f, c) < D.nlevsoi;
}

// The pass for column c (nbedrock in 1..nlevsoi); returns true when it wrote qcharge.
__device__ inline bool compute_qcharge_col(const Dims& D, const clmgb_soilwater_fields& f, double dtime,
                                           int64_t c) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  const int jwt = watertable_level(D, f, c);
  if (jwt >= D.nlevsoi) return false;
  const int nlayers = (int)f.col_nbedrock[c];
  const int jp = jwt + 1;
  const double zwt = f.zwt[c];
  const double wh_zwt = -LVc(f.sucsat, c, jp, ld) - zwt * M_TO_MM;
  const double vwc = jp <= nlayers ? jl_max(LV(f.h2osoi_liq, c, joff + jp, ld), 1.0e-6) /
                                         (LVc(f.dz, c, joff + jp, ld) * DENH2O)
                                   : 0.0;
  double s1 = jl_max(vwc / LVc(f.watsat, c, jp, ld), 0.01);
  s1 = jl_min(1.0, s1);
  const double imped = 0.0, smp = 0.0;   // the zeroed scratch rows the reference passes
  const double b = LVc(f.bsw, c, jp, ld);
  const double ka = imped * LVc(f.hksat, c, jp, ld) * cm_pow(s1, 2.0 * b + 3.0);
  const int jm = jwt > 1 ? jwt : 1;
  const double smp1 = jl_max(__ldg(f.smpmin + c), smp);
  const double wh = smp1 - LVc(f.z, c, joff + jm, ld) * M_TO_MM;
  double q;
  if (jwt == 0)
    q = -ka * (wh_zwt - wh) / ((zwt + 1.0e-3) * M_TO_MM);
  else
    q = -ka * (wh_zwt - wh) / ((zwt - LVc(f.z, c, joff + jwt, ld)) * M_TO_MM * 2.0);
  q = jl_max(-10.0 / dtime, q);
  q = jl_min(10.0 / dtime, q);
  f.qcharge[c] = q;
  return true;
}

}  // namespace clmgb
