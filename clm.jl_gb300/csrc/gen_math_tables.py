"""Generates clm_math_tables.h: the lookup tables of clm_math.h (log/exp).

Run from this directory:  python gen_math_tables.py > clm_math_tables.h
Needs mpmath (bundled with sympy).  Values are computed at 200-bit precision and
rounded once to binary64, written as C99 hex-float literals so C and CUDA compile
exactly the same bits.

log table (Tang's table-driven logarithm): the reduced argument z = x*2^-k lies in
[0.75, 1.5) and is split into 128 subintervals by the top 7 bits of (bits(x) -
bits(0.75)): 64 intervals of width 1/256 on [0.75, 1) and 64 of width 1/128 on
[1, 1.5).  For the centre c_i of interval i the table stores invc_i = RN(1/c_i) and
logc_i = RN(-log(invc_i)), so log(z) = logc_i + log1p(z*invc_i - 1) with
|z*invc_i - 1| < 0.004.

exp table (Tang's table-driven exponential, N = 64): T_j = RN(2^(j/64)), j = 0..63.
Also the split constants ln2/N = hi + lo with hi holding 36 significant bits (k*hi
exact for |k| < 2^17) and ln2 = hi + lo with 42-bit hi (k*hi exact for |k| < 2^11).

sin: Cody and Waite's reduction by pi/2 in three parts (pi/2 = hi + mid + lo, hi and
mid with 33 significant bits, so k*hi and k*mid are exact for |k| < 2^20), then the
Taylor polynomials of sin (to r^17) and cos (to r^16) on |r| <= pi/4, whose
truncation errors are below 2^-60 relative.  DEG2RAD is RN(RN(pi) / 180), the binary64
quotient that pi/180.0 gives.

acos: asin's Taylor series on [0, 1/2] (27 terms), with acos(x) = pi/2 - asin(x) for
|x| <= 1/2 and acos(x) = 2 asin(sqrt((1-x)/2)), pi - 2 asin(sqrt((1+x)/2)) beyond;
pi and pi/2 in two parts.

Double-double log for pow and log10 (Tang's method with an extra-precision table):
the same 128 intervals as the log table.  invc_i is the binary64 nearest 1/c_i among
numbers with few fractional bits, chosen so that r = z*invc_i - 1 is exactly
representable for every z of the interval (a single fma forms it with no rounding);
the generator checks this at both ends of every interval (r is monotonic in z).  The
two intervals next to 1 use invc = 1, so r = z - 1 and log near 1 keeps its relative
accuracy.  -log(invc_i) = logc_hi + logc_lo with logc_hi a multiple of 2^-42 (so
k*ln2_hi + logc_hi is exact for |k| < 2^11), and |logc_hi| >= |r| on its interval
(checked), so adding r to it is error-free by Fast2Sum.  |r| < 2^-7 everywhere; log1p(r) is its
Taylor series to r^9 (truncation below 2^-70), its r^3 tail evaluated on r * (-r^2/2)
with the coefficients times -2.

exp of a double-double argument (N = 256): 2^(j/256) = t_hi + t_lo (t_hi = RN, t_lo =
RN of the rest), ln2/256 = hi + lo with 33-bit hi (k*hi exact for |k| < 2^20), and
expm1 on |r| <= ln2/512 by its Taylor series to r^5 (truncation below 2^-66).
"""
from fractions import Fraction
import mpmath as mp

mp.mp.prec = 200


def hexd(v):
    return float(v).hex()


def round_bits(v, bits):
    """Round mpf v to `bits` significant bits (returned as a Python float)."""
    m, e = mp.frexp(v)
    scale = mp.mpf(2) ** bits
    return float(mp.nint(m * scale) / scale * mp.mpf(2) ** e)


def main():
    lines = ["// clm_math_tables.h — generated by gen_math_tables.py; do not edit.", "#pragma once", ""]
    invc, logc = [], []
    for i in range(128):
        if i < 64:
            lo = mp.mpf(0.75) + mp.mpf(i) / 256
            w = mp.mpf(1) / 256
        else:
            lo = mp.mpf(1) + mp.mpf(i - 64) / 128
            w = mp.mpf(1) / 128
        c = lo + w / 2
        ic = float(1 / c)
        invc.append(ic)
        logc.append(float(-mp.log(mp.mpf(ic))))
    lines.append("CM_TABLE(CM_LOG_INVC, 128) = {")
    lines += ["  %s," % hexd(v) for v in invc]
    lines.append("};")
    lines.append("CM_TABLE(CM_LOG_LOGC, 128) = {")
    lines += ["  %s," % hexd(v) for v in logc]
    lines.append("};")
    lines.append("CM_TABLE(CM_EXP_T, 64) = {")
    lines += ["  %s," % hexd(mp.mpf(2) ** (mp.mpf(j) / 64)) for j in range(64)]
    lines.append("};")
    ln2 = mp.log(2)
    ln2n = ln2 / 64
    hi_n = round_bits(ln2n, 36)
    lo_n = float(ln2n - mp.mpf(hi_n))
    hi = round_bits(ln2, 42)
    lo = float(ln2 - mp.mpf(hi))
    consts = {
        "CM_LN2N_HI": hi_n, "CM_LN2N_LO": lo_n, "CM_INVLN2N": float(64 / ln2),
        "CM_LN2_HI": hi, "CM_LN2_LO": lo, "CM_INVLN10": float(1 / mp.log(10)),
    }
    lines.append("")
    for k, v in consts.items():
        lines.append("#define %s (%s)" % (k, hexd(v)))
    # log1p(r) = r - r^2/2 + ... : coefficients 1/n, n = 2..7 (signs applied in code)
    for n in range(2, 8):
        lines.append("#define CM_LOG_C%d (%s)" % (n, hexd(mp.mpf((-1) ** (n + 1)) / n)))
    for n in range(2, 7):
        lines.append("#define CM_EXP_C%d (%s)" % (n, hexd(1 / mp.factorial(n))))
    pio2 = mp.pi / 2
    p_hi = round_bits(pio2, 33)
    p_mid = round_bits(pio2 - mp.mpf(p_hi), 33)
    p_lo = float(pio2 - mp.mpf(p_hi) - mp.mpf(p_mid))
    for k, v in (("CM_PIO2_HI", p_hi), ("CM_PIO2_MID", p_mid), ("CM_PIO2_LO", p_lo),
                 ("CM_INVPIO2", float(2 / mp.pi)), ("CM_PIO4", float(mp.pi / 4)),
                 ("CM_DEG2RAD", float(mp.mpf(float(mp.pi)) / 180))):
        lines.append("#define %s (%s)" % (k, hexd(v)))
    for k in range(1, 9):        # sin: (-1)^k / (2k+1)!
        lines.append("#define CM_SIN_S%d (%s)" % (k, hexd(mp.mpf((-1) ** k) / mp.factorial(2 * k + 1))))
    for k in range(2, 9):        # cos: (-1)^k / (2k)!
        lines.append("#define CM_COS_C%d (%s)" % (k, hexd(mp.mpf((-1) ** k) / mp.factorial(2 * k))))
    # asin(t) = t + t^3 sum_k A_k t^(2k-2), A_k = (2k)! / (4^k (k!)^2 (2k+1)), k = 1..27:
    # on |t| <= 1/2 the first omitted term is below 2^-58 relative
    for k in range(1, 28):
        a = mp.factorial(2 * k) / (mp.mpf(4) ** k * mp.factorial(k) ** 2 * (2 * k + 1))
        lines.append("#define CM_ASIN_A%d (%s)" % (k, hexd(a)))
    lines += logd_tables()
    lines += expd_tables()
    pi_hi = float(mp.pi)
    lines.append("#define CM_PI_HI (%s)" % hexd(pi_hi))
    lines.append("#define CM_PI_LO (%s)" % hexd(mp.pi - mp.mpf(pi_hi)))
    p2 = float(mp.pi / 2)
    lines.append("#define CM_PIO2_H (%s)" % hexd(p2))
    lines.append("#define CM_PIO2_L (%s)" % hexd(mp.pi / 2 - mp.mpf(p2)))
    # seed of the integer reciprocal (Moller and Granlund 2011, reciprocal_word):
    # floor((2^19 - 3*2^8) / d9) for the top 9 bits d9 = 256..511 of a normalised divisor
    lines.append("CM_TABLE_U16(CM_RECIP_V0, 256) = {")
    for i in range(0, 256, 8):
        lines.append("  " + " ".join("%d," % ((2 ** 19 - 3 * 2 ** 8) // (256 + k)) for k in range(i, i + 8)))
    lines.append("};")
    print("\n".join(lines))


def _interval(i):
    """The z range [lo, hi) of log interval i and the ulp of its z values."""
    if i < 64:
        lo = Fraction(3, 4) + Fraction(i, 256)
        return lo, lo + Fraction(1, 256), Fraction(1, 2 ** 53)
    lo = Fraction(1) + Fraction(i - 64, 128)
    return lo, lo + Fraction(1, 128), Fraction(1, 2 ** 52)


def _r_exact_all(zlo, zlast, u, invc):
    """True when z*invc - 1 is a binary64 number for every binary64 z in [zlo, zlast]
    (spacing u).  z*invc - 1 is a multiple of u/den(invc) (den a power of two) and its
    magnitude is largest at an end of the interval, so it suffices that the largest
    magnitude is below 2^53 such multiples."""
    step = u / invc.denominator
    rmax = max(abs(zlo * invc - 1), abs(zlast * invc - 1))
    return rmax / step < 2 ** 53


def logd_tables():
    out = []
    invc_l, hi_l, lo_l = [], [], []
    rmax = Fraction(0)
    for i in range(128):
        zlo, zhi, u = _interval(i)
        zlast = zhi - u
        if i in (63, 64):
            invc = Fraction(1)
        else:
            c = (zlo + zhi) / 2
            invc = None
            for fb in range(40, 4, -1):          # fractional bits of invc, most first
                cand = Fraction(round(Fraction(2 ** fb) / c), 2 ** fb)
                if _r_exact_all(zlo, zlast, u, cand):
                    invc = cand
                    break
            assert invc is not None, i
        rm = max(abs(zlo * invc - 1), abs(zlast * invc - 1))
        rmax = max(rmax, rm)
        iv = float(invc)
        assert Fraction(iv) == invc
        lg = -mp.log(mp.mpf(iv))
        hi = float(mp.nint(lg * mp.mpf(2) ** 42) / mp.mpf(2) ** 42)
        lo = float(lg - mp.mpf(hi))
        invc_l.append(iv)
        hi_l.append(hi)
        lo_l.append(lo)
        # k*ln2_hi + logc_hi + r is summed error-free by Fast2Sum, which needs
        # |logc_hi| >= |r| whenever logc_hi != 0 (for k != 0, |k ln2_hi + logc_hi| > 0.28)
        assert hi == 0.0 or abs(hi) >= float(rm), (i, hi, float(rm))
    assert rmax < Fraction(1, 128), float(rmax)
    for name, vals in (("CM_LOGD_INVC", invc_l), ("CM_LOGD_HI", hi_l), ("CM_LOGD_LO", lo_l)):
        out.append("CM_TABLE(%s, 128) = {" % name)
        out += ["  %s," % hexd(v) for v in vals]
        out.append("};")
    out.append("// max |r| over the intervals: %.6g" % float(rmax))
    # log1p(r) = r - r^2/2 + r^3 sum_{n>=3} (-1)^(n+1) r^(n-3) / n, the sum evaluated on
    # (r * (-r^2/2)) with each coefficient times -2
    for n in range(3, 10):
        out.append("#define CM_LOGD_C%d (%s)" % (n, hexd(-2 * mp.mpf((-1) ** (n + 1)) / n)))
    ln10 = mp.log(10)
    ih = float(1 / ln10)
    out.append("#define CM_INVLN10_HI (%s)" % hexd(ih))
    out.append("#define CM_INVLN10_LO (%s)" % hexd(1 / ln10 - mp.mpf(ih)))
    return out


def expd_tables():
    out = []
    th, tl = [], []
    for j in range(256):
        v = mp.mpf(2) ** (mp.mpf(j) / 256)
        h = float(v)
        th.append(h)
        tl.append(float(v - mp.mpf(h)))
    for name, vals in (("CM_EXPD_THI", th), ("CM_EXPD_TLO", tl)):
        out.append("CM_TABLE(%s, 256) = {" % name)
        out += ["  %s," % hexd(v) for v in vals]
        out.append("};")
    ln2n = mp.log(2) / 256
    hi = round_bits(ln2n, 33)
    out.append("#define CM_EXPD_LN2N_HI (%s)" % hexd(hi))
    out.append("#define CM_EXPD_LN2N_LO (%s)" % hexd(ln2n - mp.mpf(hi)))
    out.append("#define CM_EXPD_INVLN2N (%s)" % hexd(256 / mp.log(2)))
    for n in range(2, 6):
        out.append("#define CM_EXPD_C%d (%s)" % (n, hexd(1 / mp.factorial(n))))
    return out


if __name__ == "__main__":
    main()
