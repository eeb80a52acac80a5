// clm_math.h — table-driven log/exp/pow/log10, and sin and acos, in binary64 for C and CUDA alike.
//
// Method: P. T. P. Tang's table-driven algorithms ("Table-driven implementation of
// the exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
// 1989, and "... the logarithm function", ACM TOMS 16(4), 1990), with Taylor
// polynomials of log1p and expm1 on the reduced argument.  The tables and split
// constants are generated by gen_math_tables.py (clm_math_tables.h).
//
// Every operation is an IEEE-754 binary64 add, multiply or fused multiply-add
// written out explicitly (CUDA: __dadd_rn/__dmul_rn/__fma_rn; C: +, *, fma() built
// with -ffp-contract=off), so a C build and a CUDA build return the same bits.  On
// GB300, whose FP64 pipe issues about 1.9 FMA/clk/SM, a pow() here costs about 40 FP64
// instructions; exponent and table-index handling use the integer pipes.
//
// pow and log10 go through a double-double logarithm (cm_log_dd: Tang's table with an
// extra-precision log(c) and an exactly formed reduced argument, the error-free sums
// written out) and an exponential of a double-double argument (cm_exp_dd, 256-entry
// table in two parts), so y*log(x) keeps about 2^-67 of absolute accuracy and the
// result is rounded once at the end: nearly always the correctly rounded value, as
// Julia's own Float64 ^ (base/math.jl, double-double log and exp) nearly always is.
// Integral y in [-4096, 24576] takes Julia's compensated power by squaring instead
// (Base.Math.pow_body(x::Float64, n::Integer)), as Julia's ^ does.
//
// Accuracy (tests/test_math.py checks these against 200-bit mpmath):
//   cm_log:           absolute error below 1 ulp of max(1, |result|)
//   cm_log10:         below 0.51 ulp of max(2^-10, |result|) (double-double log)
//   cm_exp:           relative error below 2 ulp
//   cm_pow(x, y):     relative error below 0.51 ulp off the integral-y path (below 1 ulp on it);
//                     the correctly rounded value in all but a few in 10^4 random cases
//   cm_sin:           error below 1 ulp of max(|result|, 2^-53 |x|) for |x| < 2^20 pi/2
//   cm_acos:          error below 1.5 ulp on [-1, 1]
//                     (Cody-Waite reduction; the 2^-53 |x| term covers x near multiples of pi)
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CM_FN static __device__ __forceinline__
#define CM_TABLE(name, n) static __device__ const double name[n]
#define CM_TABLE_U16(name, n) static __device__ const uint16_t name[n]
#define CM_LD(p) __ldg(&(p))
#define CM_FMA(a, b, c) __fma_rn((a), (b), (c))
#define CM_MUL(a, b) __dmul_rn((a), (b))
#define CM_ADD(a, b) __dadd_rn((a), (b))
#define CM_SUB(a, b) __dsub_rn((a), (b))
#define CM_SQRT(a) __dsqrt_rn(a)
#define CM_DIV(a, b) __ddiv_rn((a), (b))
#define CM_ISFINITE(x) isfinite(x)
#define CM_AS_U64(x) ((uint64_t)__double_as_longlong(x))
#define CM_AS_F64(u) __longlong_as_double((long long)(u))
#define CM_INF __longlong_as_double(0x7ff0000000000000LL)
#define CM_NAN __longlong_as_double(0x7ff8000000000000LL)
#else
#include <math.h>
#include <stdbool.h>
#include <string.h>
#define CM_FN static inline
#define CM_TABLE(name, n) static const double name[n]
#define CM_TABLE_U16(name, n) static const uint16_t name[n]
#define CM_LD(p) (p)
#define CM_FMA(a, b, c) fma((a), (b), (c))
#define CM_MUL(a, b) ((a) * (b))
#define CM_ADD(a, b) ((a) + (b))
#define CM_SUB(a, b) ((a) - (b))
#define CM_SQRT(a) sqrt(a)
#define CM_DIV(a, b) ((a) / (b))
#define CM_ISFINITE(x) isfinite(x)
static inline uint64_t cm_as_u64_(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double cm_as_f64_(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
#define CM_AS_U64(x) cm_as_u64_(x)
#define CM_AS_F64(u) cm_as_f64_(u)
#define CM_INF cm_as_f64_(0x7ff0000000000000ULL)
#define CM_NAN cm_as_f64_(0x7ff8000000000000ULL)
#endif

#include "clm_math_tables.h"

// ---- binary64 division on the integer pipes ----
// The correctly rounded quotient x / y formed with 64-bit integer arithmetic: on GB300
// an FP64 instruction occupies its sub-partition's FP64 unit for about 64 cycles (2
// lanes per clock per SM) while a 32-bit integer multiply-add takes about 2, so a
// division done in integers leaves the FP64 pipe, which bounds the column kernels, to
// the rest of the arithmetic.  Method: N. Moller and T. Granlund, "Improved division
// by invariant integers", IEEE Trans. Computers 60(2), 2011: the reciprocal
// v = floor((2^128 - 1) / d) - 2^64 of a normalised 64-bit divisor d (their
// reciprocal_word, seeded from CM_RECIP_V0) and the 2/1 division of a two-word
// numerator by d with v (div_2by1), which gives the exact quotient and remainder.
// With d = my * 2^11 and the numerator mx * 2^66 (mx, my the 53-bit significands) the
// quotient is floor(mx * 2^55 / my), 55 or 56 bits, and the remainder says whether
// anything was cut off: round to nearest even from there.  Zero, subnormal, infinite
// or NaN operands, and quotients below the normal range or above it, take the
// ordinary division (CM_DIV), so the result always equals it.
CM_FN uint64_t cm_umulhi_(uint64_t a, uint64_t b) {
#if defined(__CUDACC__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// floor((2^128 - 1) / d) - 2^64 for d >= 2^63
CM_FN uint64_t cm_recip_word_(uint64_t d) {
  const uint64_t d0 = d & 1;
  const uint64_t d9 = d >> 55;                               // 256..511
  const uint64_t d40 = (d >> 24) + 1;
  const uint64_t d63 = (d >> 1) + d0;                        // ceil(d / 2)
  const uint64_t v0 = CM_LD(CM_RECIP_V0[d9 - 256]);
  const uint64_t v1 = (v0 << 11) - ((v0 * v0 * d40) >> 40) - 1;
  const uint64_t v2 = (v1 << 13) + ((v1 * ((1ULL << 60) - v1 * d40)) >> 47);
  const uint64_t e = ((v2 >> 1) & (0 - d0)) - v2 * d63;    // 2^96 - v2 d63 + floor(v2/2) d0, mod 2^64
  const uint64_t v3 = (v2 << 31) + (cm_umulhi_(v2, e) >> 1);
  // v3 - floor((v3 + 2^64 + 1) d / 2^64)
  const uint64_t lo = v3 * d;
  const uint64_t lo2 = lo + d;
  const uint64_t hi = cm_umulhi_(v3, d) + (lo2 < lo) + d;
  return v3 - hi;
}

// floor((u1 2^64 + u0) / d) and its remainder, for u1 < d, d >= 2^63, v its reciprocal
CM_FN uint64_t cm_div2by1_(uint64_t u1, uint64_t u0, uint64_t d, uint64_t v, uint64_t* rem) {
  uint64_t q0 = v * u1;
  uint64_t q1 = cm_umulhi_(v, u1);
  q0 += u0;
  q1 += u1 + (q0 < u0);
  q1 += 1;
  uint64_t r = u0 - q1 * d;
  if (r > q0) {
    q1 -= 1;
    r += d;
  }
  if (r >= d) {
    q1 += 1;
    r -= d;
  }
  *rem = r;
  return q1;
}

CM_FN double cm_div(double x, double y) {
  const uint64_t bx = CM_AS_U64(x), by = CM_AS_U64(y);
  const uint64_t ex = (bx >> 52) & 0x7ff, ey = (by >> 52) & 0x7ff;
  if (ex - 1 >= 0x7fe || ey - 1 >= 0x7fe) return CM_DIV(x, y);   // zero, subnormal, Inf or NaN
  const uint64_t frac = 0x000fffffffffffffULL, hidden = 0x0010000000000000ULL;
  const uint64_t sign = (bx ^ by) & 0x8000000000000000ULL;
  const uint64_t mx = (bx & frac) | hidden, my = (by & frac) | hidden;
  int64_t e = (int64_t)ex - (int64_t)ey + 1023;
  uint64_t m = mx;                                          // y a power of two: x rescaled
  if (my != hidden) {
    const uint64_t d = my << 11;
    uint64_t r;
    const uint64_t q = cm_div2by1_(mx << 2, 0, d, cm_recip_word_(d), &r);   // floor(mx 2^55 / my)
    const int sh = (q >> 55) ? 3 : 2;                       // 56 bits: quotient >= 1
    if (sh == 2) e -= 1;
    m = q >> sh;
    const uint64_t cut = q & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    if (cut > half || (cut == half && (r != 0 || (m & 1)))) m += 1;
    if (m >> 53) {
      m >>= 1;
      e += 1;
    }
  }
  if (e < 1 || e > 0x7fe) return CM_DIV(x, y);             // subnormal or infinite quotient
  return CM_AS_F64(sign | ((uint64_t)e << 52) | (m & frac));
}

// Natural logarithm.
CM_FN double cm_log(double x) {
  uint64_t ix = CM_AS_U64(x);
  if (ix - 0x0010000000000000ULL >= 0x7ff0000000000000ULL - 0x0010000000000000ULL) {
    if (x != x) return x;                                   // NaN
    if ((ix << 1) == 0) return -CM_INF;                     // +-0
    if (ix >> 63) return CM_NAN;                            // negative
    if (ix == 0x7ff0000000000000ULL) return x;              // +Inf
    ix = CM_AS_U64(CM_MUL(x, 0x1p54)) - (54ULL << 52);      // subnormal: rescale
  }
  if (ix == 0x3ff0000000000000ULL) return 0.0;              // log(1) = 0 exactly
  // x = 2^k * z with z in [0.75, 1.5); i = table interval of z
  const uint64_t tmp = ix - 0x3fe8000000000000ULL;
  const int i = (int)((tmp >> 45) & 127);
  const int64_t k = ((int64_t)tmp) >> 52;
  const double z = CM_AS_F64(ix - (tmp & 0xfff0000000000000ULL));
  const double invc = CM_LD(CM_LOG_INVC[i]);
  const double logc = CM_LD(CM_LOG_LOGC[i]);
  const double r = CM_FMA(z, invc, -1.0);                   // |r| < 0.0039
  const double kd = (double)k;
  double q = CM_FMA(r, CM_LOG_C7, CM_LOG_C6);
  q = CM_FMA(r, q, CM_LOG_C5);
  q = CM_FMA(r, q, CM_LOG_C4);
  q = CM_FMA(r, q, CM_LOG_C3);
  q = CM_FMA(r, q, CM_LOG_C2);
  const double r2 = CM_MUL(r, r);
  const double w = CM_FMA(kd, CM_LN2_HI, logc);             // k*ln2_hi is exact
  const double lo = CM_FMA(kd, CM_LN2_LO, CM_MUL(r2, q));
  return CM_ADD(w, CM_ADD(r, lo));
}

// Exponential.
CM_FN double cm_exp(double x) {
  const uint64_t ix = CM_AS_U64(x);
  const uint32_t top = (uint32_t)(ix >> 52) & 0x7ffu;
  if (top - 0x3c9u >= 0x408u - 0x3c9u) {                   // |x| < 2^-54 or |x| >= 512 or NaN/Inf
    if (top < 0x3c9u) return CM_ADD(1.0, x);
    if (x != x) return x;
    if (x > 709.782712893383973096) return CM_INF;
    if (x < -745.1332191019412076235) return 0.0;
  }
  const double shift = 0x1.8p52;
  const double z = CM_MUL(CM_INVLN2N, x);
  double kd = CM_ADD(z, shift);
  const int64_t kk = (int64_t)(CM_AS_U64(kd) - 0x4338000000000000ULL);   // round(x*64/ln2)
  kd = CM_SUB(kd, shift);
  double r = CM_FMA(-kd, CM_LN2N_HI, x);                    // kd*hi exact (36-bit hi)
  r = CM_FMA(-kd, CM_LN2N_LO, r);                           // |r| <= ln2/128
  const int j = (int)(kk & 63);
  const int64_t n = kk >> 6;                                // floor(kk / 64)
  const double tj = CM_LD(CM_EXP_T[j]);
  double p = CM_FMA(r, CM_EXP_C6, CM_EXP_C5);
  p = CM_FMA(r, p, CM_EXP_C4);
  p = CM_FMA(r, p, CM_EXP_C3);
  p = CM_FMA(r, p, CM_EXP_C2);
  p = CM_FMA(CM_MUL(r, r), p, r);                           // expm1(r)
  const double res = CM_FMA(tj, p, tj);                     // 2^(j/64) * exp(r), in [0.99, 2.01)
  if (n >= -1020 && n <= 1020) return CM_AS_F64(CM_AS_U64(res) + ((uint64_t)n << 52));
  if (n > 0) return CM_MUL(CM_AS_F64(CM_AS_U64(res) + ((uint64_t)(n - 3) << 52)), 8.0);
  // result may be subnormal: scale to normal range first, round once at the end
  return CM_MUL(CM_AS_F64(CM_AS_U64(res) + ((uint64_t)(n + 1000) << 52)), 0x1p-1000);
}

// log(x) = hi + *lo (returned: hi) for a positive finite x, subnormals included:
// |hi + lo - log(x)| below about 2^-67 max(1, |log x|), and below 2^-67 |log x| near 1.
// The pair is not renormalised: |lo| < 2^-20 max(1, |hi|), which the callers (pow and
// log10, whose products with it are formed exactly or with a single rounding) allow.
// x = 2^k z, z in [0.75, 1.5); log(x) = k ln2 + log(1/invc) + log1p(r), r = z*invc - 1
// formed exactly by one fma (the table's invc has few fractional bits), |r| < 2^-7.
CM_FN double cm_log_dd(double x, double* lo_out) {
  uint64_t ix = CM_AS_U64(x);
  if (ix < 0x0010000000000000ULL) ix = CM_AS_U64(CM_MUL(x, 0x1p54)) - (54ULL << 52);   // subnormal
  const uint64_t tmp = ix - 0x3fe8000000000000ULL;
  const int i = (int)((tmp >> 45) & 127);
  const int64_t k = ((int64_t)tmp) >> 52;
  const double z = CM_AS_F64(ix - (tmp & 0xfff0000000000000ULL));
  const double invc = CM_LD(CM_LOGD_INVC[i]);
  const double lch = CM_LD(CM_LOGD_HI[i]);
  const double lcl = CM_LD(CM_LOGD_LO[i]);
  const double r = CM_FMA(z, invc, -1.0);                    // exact
  const double kd = (double)k;
  const double t1 = CM_FMA(kd, CM_LN2_HI, lch);              // exact: multiples of 2^-42 below 2^10
  // s + e = t1 + r exactly (Dekker's Fast2Sum: |t1| >= |r| or t1 == 0, checked by the
  // table generator for every interval)
  const double s = CM_ADD(t1, r);
  const double e = CM_SUB(r, CM_SUB(s, t1));
  // -r^2/2 = ar2 + e3 exactly
  const double ar = CM_MUL(-0.5, r);
  const double ar2 = CM_MUL(ar, r);
  const double e3 = CM_FMA(ar, r, -ar2);
  // hi + e2 = s + ar2 exactly (|s| >= |ar2|)
  const double hi = CM_ADD(s, ar2);
  const double e2 = CM_ADD(CM_SUB(s, hi), ar2);
  // r^3 (1/3 - r/4 + ... + r^6/9) = (r ar2) (-2/3 + r/2 - ...): the coefficients carry
  // the factor -2 (exact); truncation below 2^-70
  double p = CM_FMA(r, CM_LOGD_C9, CM_LOGD_C8);
  p = CM_FMA(r, p, CM_LOGD_C7);
  p = CM_FMA(r, p, CM_LOGD_C6);
  p = CM_FMA(r, p, CM_LOGD_C5);
  p = CM_FMA(r, p, CM_LOGD_C4);
  p = CM_FMA(r, p, CM_LOGD_C3);
  *lo_out = CM_ADD(CM_ADD(CM_FMA(kd, CM_LN2_LO, lcl), e), CM_FMA(CM_MUL(r, ar2), p, CM_ADD(e2, e3)));
  return hi;
}

// exp(x + xl) for |xl| <= ulp(x): the value before the final rounding is within about
// 2^-61 relative; x = k ln2/256 + r with k*hi exact, 2^(j/256) = t_hi + t_lo, expm1(r)
// by its Taylor series to r^5 on |r| <= ln2/512.
CM_FN double cm_exp_dd(double x, double xl) {
  const uint64_t ix = CM_AS_U64(x);
  const uint32_t top = (uint32_t)(ix >> 52) & 0x7ffu;
  if (top - 0x3c9u >= 0x408u - 0x3c9u) {                   // |x| < 2^-54 or |x| >= 512 or NaN/Inf
    if (top < 0x3c9u) return CM_ADD(1.0, x);
    if (x != x) return x;
    if (x > 709.782712893383973096) return CM_INF;
    if (x < -745.1332191019412076235) return 0.0;
  }
  const double shift = 0x1.8p52;
  double kd = CM_FMA(x, CM_EXPD_INVLN2N, shift);
  const int64_t kk = (int64_t)(CM_AS_U64(kd) - 0x4338000000000000ULL);   // round(x*256/ln2)
  kd = CM_SUB(kd, shift);
  double r = CM_FMA(-kd, CM_EXPD_LN2N_HI, x);               // exact
  r = CM_FMA(-kd, CM_EXPD_LN2N_LO, r);
  r = CM_ADD(r, xl);
  const int j = (int)(kk & 255);
  const int64_t n = kk >> 8;                                // floor(kk / 256)
  const double th = CM_LD(CM_EXPD_THI[j]);
  const double tl = CM_LD(CM_EXPD_TLO[j]);
  double q = CM_FMA(r, CM_EXPD_C5, CM_EXPD_C4);
  q = CM_FMA(r, q, CM_EXPD_C3);
  q = CM_FMA(r, q, CM_EXPD_C2);
  const double pm = CM_FMA(CM_MUL(r, r), q, r);             // expm1(r)
  const double res = CM_ADD(th, CM_FMA(th, pm, tl));        // 2^(j/256) exp(r), in [0.99, 2.01)
  if (n >= -1020 && n <= 1020) return CM_AS_F64(CM_AS_U64(res) + ((uint64_t)n << 52));
  if (n > 0) return CM_MUL(CM_AS_F64(CM_AS_U64(res) + ((uint64_t)(n - 3) << 52)), 8.0);
  return CM_MUL(CM_AS_F64(CM_AS_U64(res) + ((uint64_t)(n + 1000) << 52)), 0x1p-1000);
}

// Julia's x^n for an integer n (Base.Math.pow_body(x::Float64, n::Integer)): power by
// squaring with the products' rounding errors carried in a second word.
CM_FN double jl_pow_int(double x, int64_t n) {
  double y = 1.0, xnlo = 0.0, ynlo = 0.0;
  if (n == 3) return CM_MUL(CM_MUL(x, x), x);
  if (n < 0) {
    const double rx = CM_DIV(1.0, x);
    if (n == -2) return CM_MUL(rx, rx);
    if (CM_ISFINITE(x)) xnlo = CM_MUL(-CM_FMA(x, rx, -1.0), rx);
    x = rx;
    n = -n;
  }
  while (n > 1) {
    if (n & 1) {
      const double err = CM_FMA(y, xnlo, CM_MUL(x, ynlo));
      const double yh = CM_MUL(x, y);
      ynlo = CM_ADD(CM_FMA(x, y, -yh), err);
      y = yh;
    }
    const double err = CM_MUL(CM_MUL(x, 2.0), xnlo);
    const double xh = CM_MUL(x, x);
    xnlo = CM_ADD(CM_FMA(x, x, -xh), err);
    x = xh;
    n >>= 1;
  }
  const double err = CM_FMA(y, xnlo, CM_MUL(x, ynlo));
  if (CM_ISFINITE(x) && CM_ISFINITE(err)) return CM_FMA(x, y, err);
  return CM_MUL(x, y);
}

// Integral y in Julia's power-by-squaring range (Base.Math.use_power_by_squaring),
// -4096 <= y <= 24576, decided on the bit pattern (integer pipes only).
CM_FN bool cm_pow_by_squaring(uint64_t uy, int64_t* n) {
  if ((uy << 1) == 0) {                                     // y = +-0
    *n = 0;
    return true;
  }
  const int ex = (int)((uy >> 52) & 0x7ff) - 1023;          // |y| in [2^ex, 2^(ex+1))
  if (ex < 0 || ex > 14) return false;                      // |y| < 1 (not 0), or |y| >= 32768
  const int sh = 52 - ex;
  const uint64_t mant = (uy & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
  if (mant & ((1ULL << sh) - 1)) return false;              // a fraction
  const int64_t m = (int64_t)(mant >> sh);
  const int64_t v = (uy >> 63) ? -m : m;
  if (v < -4096 || v > 24576) return false;
  *n = v;
  return true;
}

// x^y with Julia Base's rules for Float64 (base/math.jl `^`): x == 1 -> 1; y NaN ->
// NaN; y integral in [-4096, 24576] -> compensated power by squaring (y == 0 -> 1);
// x == 0 -> 0 or Inf; x < 0 with non-integral y -> NaN (Julia raises a DomainError);
// otherwise exp(y log x) in double-double.  The tests of the common case look at bit
// patterns (integer pipes).
CM_FN double cm_pow(double x, double y) {
  const uint64_t ux = CM_AS_U64(x), uy = CM_AS_U64(y);
  if (ux == 0x3ff0000000000000ULL) return 1.0;
  if ((uy << 1) > 0xffe0000000000000ULL) return y;          // y NaN
  int64_t n;
  if (cm_pow_by_squaring(uy, &n)) return n == 0 ? 1.0 : jl_pow_int(x, n);
  bool neg = false;
  if (ux - 1 >= 0x7fefffffffffffffULL) {                    // not a positive finite nonzero x
    if ((ux << 1) == 0) return y > 0.0 ? 0.0 : CM_INF;     // x = +-0
    if ((ux << 1) > 0xffe0000000000000ULL) return x;        // x NaN
    const double ay = y < 0.0 ? -y : y;
    if (ux >> 63) {                                         // x < 0
      const bool yint = ay >= 0x1p53 || (double)(int64_t)y == y;
      if (!yint) return CM_NAN;
      neg = ay < 0x1p53 && ((int64_t)y & 1);
      x = -x;
    }
    if (x == CM_INF) {
      const double v = y > 0.0 ? CM_INF : 0.0;
      return neg ? -v : v;
    }
  }
  double lxl;
  const double lxh = cm_log_dd(x, &lxl);
  const double eh = CM_MUL(y, lxh);
  const double el = CM_FMA(y, lxl, CM_FMA(y, lxh, -eh));
  const double v = cm_exp_dd(eh, el);
  return neg ? -v : v;
}

// x^y for a positive finite x other than 1 whose logarithm lxh + lxl = cm_log_dd(x) the
// caller formed once: the value of cm_pow(x, y) for every y, without forming the
// logarithm again.
CM_FN double cm_pow_lx(double x, double lxh, double lxl, double y) {
  const uint64_t uy = CM_AS_U64(y);
  if ((uy << 1) > 0xffe0000000000000ULL) return y;
  int64_t n;
  if (cm_pow_by_squaring(uy, &n)) return n == 0 ? 1.0 : jl_pow_int(x, n);
  const double eh = CM_MUL(y, lxh);
  const double el = CM_FMA(y, lxl, CM_FMA(y, lxh, -eh));
  return cm_exp_dd(eh, el);
}

// Base-10 logarithm: the double-double log times 1/ln10 in two parts.
CM_FN double cm_log10(double x) {
  const uint64_t ix = CM_AS_U64(x);
  if (ix - 0x0010000000000000ULL >= 0x7ff0000000000000ULL - 0x0010000000000000ULL) {
    if (x != x) return x;                                   // NaN
    if ((ix << 1) == 0) return -CM_INF;                     // +-0
    if (ix >> 63) return CM_NAN;                            // negative
    if (ix == 0x7ff0000000000000ULL) return x;              // +Inf
  }
  if (ix == 0x3ff0000000000000ULL) return 0.0;
  double l;
  const double h = cm_log_dd(x, &l);
  const double v = CM_MUL(h, CM_INVLN10_HI);
  const double vl = CM_ADD(CM_FMA(h, CM_INVLN10_HI, -v), CM_FMA(h, CM_INVLN10_LO, CM_MUL(l, CM_INVLN10_HI)));
  return CM_ADD(v, vl);
}

// sin and cos of a reduced argument r + lo, |r| <= pi/4, |lo| <= ulp(r) (Taylor
// polynomials in r^2; lo enters to first order: sin' = cos ~ 1 - r^2/2, cos' = -sin ~ -r).
CM_FN double cm_sin_poly(double r, double lo) {
  const double z = CM_MUL(r, r);
  double p = CM_FMA(z, CM_SIN_S8, CM_SIN_S7);
  p = CM_FMA(z, p, CM_SIN_S6);
  p = CM_FMA(z, p, CM_SIN_S5);
  p = CM_FMA(z, p, CM_SIN_S4);
  p = CM_FMA(z, p, CM_SIN_S3);
  p = CM_FMA(z, p, CM_SIN_S2);
  p = CM_FMA(z, p, CM_SIN_S1);
  const double lo1 = CM_FMA(CM_MUL(-0.5, z), lo, lo);       // lo (1 - r^2/2)
  return CM_ADD(r, CM_FMA(CM_MUL(r, z), p, lo1));            // r + (r^3 p + lo1)
}
CM_FN double cm_cos_poly(double r, double lo) {
  const double z = CM_MUL(r, r);
  double q = CM_FMA(z, CM_COS_C8, CM_COS_C7);
  q = CM_FMA(z, q, CM_COS_C6);
  q = CM_FMA(z, q, CM_COS_C5);
  q = CM_FMA(z, q, CM_COS_C4);
  q = CM_FMA(z, q, CM_COS_C3);
  q = CM_FMA(z, q, CM_COS_C2);
  // 1 - z/2 + z^2 q - r lo, with the rounding error of w = 1 - z/2 carried into the tail
  const double hz = CM_MUL(0.5, z);
  const double w = CM_SUB(1.0, hz);
  const double c = CM_FMA(-r, lo, CM_SUB(CM_SUB(1.0, w), hz));
  return CM_ADD(w, CM_FMA(CM_MUL(z, z), q, c));
}

// Sine for |x| < 2^20 * pi/2 (NaN beyond, and for NaN or infinite x): the reduced
// argument x - k pi/2 = r + lo with pi/2 in three parts (k*hi and k*mid exact, the
// subtraction of k*mid error-free by Knuth's two-sum), then sin or cos by k mod 4.
CM_FN double cm_sin(double x) {
  const double ax = x < 0.0 ? -x : x;
  if (!(ax < 1647099.0)) return CM_NAN;                     // 2^20 * pi/2, NaN, Inf
  if (ax < 0x1p-27) return x;                               // sin(x) = x in binary64
  if (ax <= CM_PIO4) return cm_sin_poly(x, 0.0);
  const double shift = 0x1.8p52;
  double kd = CM_FMA(x, CM_INVPIO2, shift);
  const int64_t k = (int64_t)(CM_AS_U64(kd) - 0x4338000000000000ULL);   // round(x*2/pi)
  kd = CM_SUB(kd, shift);
  const double a = CM_FMA(-kd, CM_PIO2_HI, x);              // exact
  const double b = CM_MUL(-kd, CM_PIO2_MID);                // exact
  const double r0 = CM_ADD(a, b);
  const double bv = CM_SUB(r0, a);
  const double err = CM_ADD(CM_SUB(a, CM_SUB(r0, bv)), CM_SUB(b, bv));   // a + b - r0
  const double lo0 = CM_FMA(-kd, CM_PIO2_LO, err);
  const double r = CM_ADD(r0, lo0);
  const double lo = CM_SUB(lo0, CM_SUB(r, r0));
  const int q = (int)(k & 3);
  const double v = (q & 1) ? cm_cos_poly(r, lo) : cm_sin_poly(r, lo);
  return (q & 2) ? -v : v;
}

// asin(t) for |t| <= 1/2: t + t^3 P(t^2) (Taylor series, 27 terms).
CM_FN double cm_asin_small(double t) {
  const double z = CM_MUL(t, t);
  double p = CM_ASIN_A27;
  p = CM_FMA(z, p, CM_ASIN_A26);
  p = CM_FMA(z, p, CM_ASIN_A25);
  p = CM_FMA(z, p, CM_ASIN_A24);
  p = CM_FMA(z, p, CM_ASIN_A23);
  p = CM_FMA(z, p, CM_ASIN_A22);
  p = CM_FMA(z, p, CM_ASIN_A21);
  p = CM_FMA(z, p, CM_ASIN_A20);
  p = CM_FMA(z, p, CM_ASIN_A19);
  p = CM_FMA(z, p, CM_ASIN_A18);
  p = CM_FMA(z, p, CM_ASIN_A17);
  p = CM_FMA(z, p, CM_ASIN_A16);
  p = CM_FMA(z, p, CM_ASIN_A15);
  p = CM_FMA(z, p, CM_ASIN_A14);
  p = CM_FMA(z, p, CM_ASIN_A13);
  p = CM_FMA(z, p, CM_ASIN_A12);
  p = CM_FMA(z, p, CM_ASIN_A11);
  p = CM_FMA(z, p, CM_ASIN_A10);
  p = CM_FMA(z, p, CM_ASIN_A9);
  p = CM_FMA(z, p, CM_ASIN_A8);
  p = CM_FMA(z, p, CM_ASIN_A7);
  p = CM_FMA(z, p, CM_ASIN_A6);
  p = CM_FMA(z, p, CM_ASIN_A5);
  p = CM_FMA(z, p, CM_ASIN_A4);
  p = CM_FMA(z, p, CM_ASIN_A3);
  p = CM_FMA(z, p, CM_ASIN_A2);
  p = CM_FMA(z, p, CM_ASIN_A1);
  return CM_FMA(CM_MUL(t, z), p, t);
}

// Arc cosine for |x| <= 1 (NaN outside): pi/2 - asin(x) on |x| <= 1/2, else through
// asin(sqrt((1 -+ x)/2)), whose argument is formed exactly ((1 -+ x) by Sterbenz, the
// halving) and rounded once by the square root.
CM_FN double cm_acos(double x) {
  if (!(x >= -1.0 && x <= 1.0)) return CM_NAN;
  if (x <= 0.5 && x >= -0.5) return CM_ADD(CM_PIO2_H, CM_SUB(CM_PIO2_L, cm_asin_small(x)));
  if (x > 0.5) return CM_MUL(2.0, cm_asin_small(CM_SQRT(CM_MUL(0.5, CM_SUB(1.0, x)))));
  const double a = CM_MUL(2.0, cm_asin_small(CM_SQRT(CM_MUL(0.5, CM_ADD(1.0, x)))));
  return CM_ADD(CM_PI_HI, CM_SUB(CM_PI_LO, a));
}
