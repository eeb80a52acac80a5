"""Accuracy of the shared table-driven log/exp/pow/log10 (clm_math.h) against
200-bit mpmath, over the argument ranges of the column solve and beyond.

pow and log10 go through a double-double logarithm and are rounded once at the end:
their results must stay within 0.51 ulp and be the correctly rounded value in all but
a few in 10^4 cases, as Julia's own Float64 ^ (base/math.jl) nearly always is.  For
integral exponents in [-4096, 24576] Julia's ^ takes compensated power by squaring
(Base.Math.pow_body(x, n::Integer)); a step-by-step restatement of it here pins that
path bit for bit."""
import ctypes as C
import math

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
from oracle import oracle as orc  # noqa: E402

mp.mp.prec = 200


def _fn(name, nargs):
    f = getattr(orc.lib(), name)
    f.argtypes = [C.c_double] * nargs
    f.restype = C.c_double
    return f


def ulp(x):
    return math.ulp(abs(x)) if x != 0 else 5e-324


def test_log_and_log10_accuracy():
    rng = np.random.default_rng(1)
    xs = np.concatenate([10 ** rng.uniform(-300, 300, 3000), rng.uniform(0.5, 2.0, 3000),
                         1 + rng.uniform(-1e-6, 1e-6, 500), 10 ** rng.uniform(-7, 0, 2000),
                         [5e-324, 1e-310, 2.2250738585072014e-308, 1.0, 2.0, 0.75, 1.5, 1.7976931348623157e308]])
    flog, flog10 = _fn("orc_cm_log", 1), _fn("orc_cm_log10", 1)
    worst = worst10 = 0.0
    for x in xs:
        x = float(x)
        ref = mp.log(mp.mpf(x))
        got = flog(x)
        worst = max(worst, float(abs(mp.mpf(got) - ref)) / ulp(max(1.0, abs(float(ref)))))
        ref10 = mp.log10(mp.mpf(x))
        got10 = flog10(x)
        worst10 = max(worst10, float(abs(mp.mpf(got10) - ref10)) / ulp(max(1.0, abs(float(ref10)))))
    assert worst < 2.0, worst
    assert worst10 < 0.51, worst10
    # log10 relative to its own result, near 1 included
    worst_rel = 0.0
    for x in xs:
        x = float(x)
        ref10 = mp.log10(mp.mpf(x))
        if ref10 == 0:
            continue
        worst_rel = max(worst_rel, float(abs(mp.mpf(flog10(x)) - ref10)) / ulp(float(ref10)))
    assert worst_rel < 0.51, worst_rel
    assert flog10(1000.0) == 3.0 and flog10(1e-5) == -5.0
    assert flog(1.0) == 0.0 and flog10(1.0) == 0.0
    assert flog(0.0) == -math.inf and math.isnan(flog(-1.0)) and flog(math.inf) == math.inf


def test_exp_accuracy():
    rng = np.random.default_rng(2)
    xs = np.concatenate([rng.uniform(-745, 709.7, 4000), rng.uniform(-1, 1, 2000), [0.0, 1e-300, -1e-300,
                                                                                    709.78, -708.4, -744.0]])
    fexp = _fn("orc_cm_exp", 1)
    worst = 0.0
    for x in xs:
        x = float(x)
        ref = mp.exp(mp.mpf(x))
        got = fexp(x)
        if float(ref) < 2.2250738585072014e-308:      # subnormal results: absolute
            assert abs(mp.mpf(got) - ref) <= 5e-324
            continue
        worst = max(worst, float(abs(mp.mpf(got) - ref) / ref) / (2.0 ** -52))
    assert worst < 2.0, worst
    assert fexp(710.0) == math.inf and fexp(-746.0) == 0.0 and fexp(0.0) == 1.0


@pytest.mark.parametrize("xr,yr", [((0.01, 1.0), (5.0, 45.0)),      # s^(2b+3)
                                   ((0.01, 1.0), (-20.0, -2.0)),    # s^(-b)
                                   ((0.57, 0.57), (0.0, 0.95)),     # TKWAT^(fl*watsat)
                                   ((2.29, 2.29), (0.0, 0.95)),     # TKICE^((1-fl)*watsat)
                                   ((10.0, 10.0), (-6.0, 0.0)),     # ice impedance
                                   ((1.0, 1e7), (-0.5, -0.04)),     # supercool (smp/sucsat)^(-1/b)
                                   ((1e-3, 1e3), (-60.0, 60.0))])
def test_pow_accuracy(xr, yr):
    rng = np.random.default_rng(int(xr[0] * 100 + yr[0] * 7) & 0xffff)
    fpow = _fn("orc_cm_pow", 2)
    xs = rng.uniform(*xr, 1500) if xr[0] != xr[1] else np.full(1500, xr[0])
    ys = rng.uniform(*yr, 1500)
    misrounded = 0
    for x, y in zip(xs, ys):
        x, y = float(x), float(y)
        ref = mp.power(mp.mpf(x), mp.mpf(y))
        got = fpow(x, y)
        cr = float(ref)
        if float(y).is_integer():
            continue                       # the power-by-squaring path, pinned below
        err_ulp = float(abs(mp.mpf(got) - ref)) / ulp(cr)
        assert err_ulp < 0.51, (x, y, err_ulp)
        misrounded += got != cr
    assert misrounded <= 3, misrounded     # 1500 cases: nearly always correctly rounded


def _fma(a, b, c):
    return float(mp.mpf(a) * mp.mpf(b) + mp.mpf(c))


def julia_pow_int(x, n):
    """Base.Math.pow_body(x::Float64, n::Integer), step by step in binary64."""
    y, xnlo, ynlo = 1.0, 0.0, 0.0
    if n == 3:
        return x * x * x
    if n < 0:
        rx = 1.0 / x
        if n == -2:
            return rx * rx
        if math.isfinite(x):
            xnlo = -_fma(x, rx, -1.0) * rx
        x, n = rx, -n
    while n > 1:
        if n & 1:
            err = _fma(y, xnlo, x * ynlo)
            yh = x * y
            ynlo = _fma(x, y, -yh) + err
            y = yh
        err = x * 2.0 * xnlo
        xh = x * x
        xnlo = _fma(x, x, -xh) + err
        x = xh
        n >>= 1
    err = _fma(y, xnlo, x * ynlo)
    if math.isfinite(x) and math.isfinite(err):
        return _fma(x, y, err)
    return x * y


def test_pow_integral_exponents_follow_julia_power_by_squaring():
    fpow = _fn("orc_cm_pow", 2)
    rng = np.random.default_rng(9)
    xs = np.concatenate([[10.0, 0.57, 2.29, 0.1, 3.0, 1.0000001, 0.999999], rng.uniform(0.01, 50.0, 60)])
    for x in xs:
        for n in list(range(-13, 14)) + [-4096, 100, 24576]:
            x, n = float(x), int(n)
            if n == 0:
                assert fpow(x, 0.0) == 1.0
                continue
            want = julia_pow_int(x, n)
            got = fpow(x, float(n))
            assert got == want or (math.isnan(got) and math.isnan(want)), (x, n, got, want)
    # beyond the range the general path runs (no power by squaring)
    assert abs(fpow(1.0001, 30000.0) / float(mp.power(mp.mpf(1.0001), 30000)) - 1) < 2e-16


def test_pow_special_values():
    """Julia's rules for Float64 ^ (base/math.jl); Julia raises a DomainError for a
    negative base with a non-integral exponent, which is NaN here."""
    fpow = _fn("orc_cm_pow", 2)
    assert fpow(2.0, 0.0) == 1.0 and fpow(1.0, 1e300) == 1.0 and fpow(math.nan, 0.0) == 1.0
    assert fpow(1.0, math.nan) == 1.0 and math.isnan(fpow(2.0, math.nan))
    assert fpow(0.0, 2.0) == 0.0 and fpow(0.0, -1.0) == math.inf and fpow(0.0, 0.5) == 0.0
    assert fpow(0.0, -0.5) == math.inf and fpow(-0.0, -1.0) == -math.inf
    assert math.isnan(fpow(-2.0, 0.5)) and fpow(-2.0, 3.0) == -8.0 and fpow(-2.0, 1e20) == math.inf
    assert fpow(-2.0, 30001.0) == -math.inf and fpow(-0.5, 30001.0) == -0.0
    assert fpow(math.inf, 2.0) == math.inf and fpow(math.inf, -2.0) == 0.0
    assert fpow(math.inf, 0.5) == math.inf and fpow(-math.inf, 3.0) == -math.inf
    assert fpow(2.0, 2000.0) == math.inf and fpow(2.0, -1200.0) == 0.0 and fpow(2.0, -1074.0) == 5e-324


def test_sin_accuracy():
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-math.pi, math.pi, 4000), rng.uniform(-1e5, 1e5, 2000),
                         rng.uniform(0.0, 90.0, 2000) * float.fromhex("0x1.1df46a2529d39p-6"),
                         10 ** rng.uniform(-12, 0, 500),
                         [0.0, -0.0, 1e-300, math.pi / 4, math.pi / 2, math.pi, 3 * math.pi / 4, 1.6e6]])
    fsin = _fn("orc_cm_sin", 1)
    worst = 0.0
    for x in xs:
        x = float(x)
        ref = mp.sin(mp.mpf(x))
        got = fsin(x)
        scale = max(abs(float(ref)), 2.0 ** -53 * abs(x), 5e-324)
        worst = max(worst, float(abs(mp.mpf(got) - ref)) / ulp(scale))
    assert worst < 1.0, worst
    assert fsin(0.0) == 0.0 and math.copysign(1.0, fsin(-0.0)) == -1.0
    assert math.isnan(fsin(math.inf)) and math.isnan(fsin(math.nan)) and math.isnan(fsin(2e6))


def test_acos_accuracy():
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(-1, 1, 6000), 1 - 10 ** rng.uniform(-16, 0, 1000),
                         -1 + 10 ** rng.uniform(-16, 0, 1000), [1.0, -1.0, 0.5, -0.5, 0.0, -0.0]])
    facos = _fn("orc_cm_acos", 1)
    worst = 0.0
    for x in xs:
        x = float(x)
        ref = mp.acos(mp.mpf(x))
        got = facos(x)
        if ref == 0:
            assert got == 0.0
            continue
        worst = max(worst, float(abs(mp.mpf(got) - ref) / ref) / (2.0 ** -52))
    assert worst < 1.5, worst
    assert facos(1.0) == 0.0 and math.isnan(facos(1.0000000000000002)) and math.isnan(facos(math.nan))


def test_integer_division_is_the_ieee_quotient():
    """cm_div (64-bit integer reciprocal and 2/1 division, Moller and Granlund 2011) is
    the binary64 quotient x / y bit for bit: random bit patterns (every exponent,
    subnormals, zeros, infinities, NaN), operands with close exponents, divisors and
    numerators with short significands, products of random significands (quotients
    next to a representable value), and powers of two."""
    f = orc.lib().orc_cm_div_n
    f.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = None
    rng = np.random.default_rng(71)
    n = 2_000_000
    a = rng.integers(0, 2 ** 64, n, dtype=np.uint64)
    b = rng.integers(0, 2 ** 64, n, dtype=np.uint64)
    frac = np.uint64(0x000FFFFFFFFFFFFF)
    sgn = np.uint64(0x8000000000000000)
    close = rng.integers(1000, 1048, (2, n), dtype=np.uint64) << np.uint64(52)
    k = n // 5
    a[k:2 * k] = (a[k:2 * k] & (frac | sgn)) | close[0, k:2 * k]
    b[k:2 * k] = (b[k:2 * k] & (frac | sgn)) | close[1, k:2 * k]
    b[2 * k:3 * k] &= ~np.uint64(0x000FFFFFFFFFFF00)            # short divisor significands
    x = a.view(np.float64)
    y = b.view(np.float64)
    q = (rng.integers(0, 2 ** 52, n, dtype=np.uint64) | np.uint64(1023 << 52)).view(np.float64)
    with np.errstate(all="ignore"):
        x[3 * k:4 * k] = q[3 * k:4 * k] * y[3 * k:4 * k]           # quotients next to q
    y[4 * k:4 * k + 1000] = 2.0 ** rng.integers(-1000, 1000, 1000)   # powers of two
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.0, -3.0, 1e300,
                        1.7976931348623157e308, np.inf, -np.inf, np.nan])
    sx, sy = np.meshgrid(special, special, indexing="ij")
    x = np.concatenate([x, sx.ravel()])
    y = np.concatenate([y, sy.ravel()])
    out = np.empty_like(x)
    f(len(x), x.ctypes.data, y.ctypes.data, out.ctypes.data)
    with np.errstate(all="ignore"):
        want = x / y
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(out), nan)
    assert np.array_equal(out[~nan].view(np.uint64), want[~nan].view(np.uint64))
