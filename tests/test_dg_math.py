"""dg_log / dg_ipow (dengo_gb300/csrc/dg_math.h) compiled for the host.

The device build runs the same IEEE operations, so what holds here holds on
the GPU: dg_log is correctly rounded on a sample checked against 200-bit
arithmetic, it differs from glibc's log only where glibc itself is not
correctly rounded, and dg_ipow<2>(x) == x*x == glibc pow(x, 2)."""
import ctypes as C
import math
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include "dg_math.h"
extern "C" double h_dg_log(double x) { return dg_log(x); }
extern "C" double h_pow2(double x) { return dg_ipow<2>(x); }
extern "C" double h_pow3(double x) { return dg_ipow<3>(x); }
extern "C" double h_pow4(double x) { return dg_ipow<4>(x); }
extern "C" double h_glibc_log(double x) { return log(x); }
/* dg_div(a, b, 1/b) and dg_quot(a, b) against a / b on random bit patterns: a and b with
 * uniformly random sign, exponent field and mantissa (every class of value),
 * on pairs whose exponents straddle the guarded range's edges, and on signed
 * zero numerators over every class of b (zero, subnormal, normal, inf,
 * NaN).  Returns the number of results whose bits differ (NaNs compare
 * equal). */
extern "C" long long h_div_mismatch(long long n, unsigned long long seed) {
    long long bad = 0;
    for (long long i = 0; i < n; i++) {
        seed ^= seed << 13; seed ^= seed >> 7; seed ^= seed << 17;
        unsigned long long ba = seed;
        seed ^= seed << 13; seed ^= seed >> 7; seed ^= seed << 17;
        unsigned long long bb = seed;
        if (i & 1) {   /* exponents near the guard's bounds (150, 1900, +-800) */
            static const int ea[] = {149, 150, 151, 1899, 1900, 1901, 1023, 1100, 300};
            static const int eb[] = {150, 1900, 1023, 949, 950, 951, 1851, 1852, 151};
            const int ka = (int)((seed >> 3) % 9), kb = (int)((seed >> 9) % 9);
            ba = (ba & 0x800fffffffffffffull) | ((unsigned long long)ea[ka] << 52);
            bb = (bb & 0x800fffffffffffffull) | ((unsigned long long)eb[kb] << 52);
        } else if ((i & 3) == 2) {   /* +-0 over b of every class */
            static const int eb[] = {0, 0, 1, 150, 1023, 2046, 2047, 2047};
            const int kb = (int)((seed >> 5) % 8);
            ba &= 0x8000000000000000ull;
            bb = (bb & 0x800fffffffffffffull) | ((unsigned long long)eb[kb] << 52);
            if (kb == 0) bb &= 0x8000000000000000ull;            /* b = +-0 */
            if (kb == 6) bb &= 0x8000000000000000ull | (0x7ffull << 52);   /* b = +-inf */
        }
        double a, b;
        memcpy(&a, &ba, 8);
        memcpy(&b, &bb, 8);
        const double q = dg_div(a, b, 1.0 / b), r = a / b, q2 = dg_quot(a, b);
        uint64_t bq, br, bq2;
        memcpy(&bq, &q, 8);
        memcpy(&br, &r, 8);
        memcpy(&bq2, &q2, 8);
        bad += !(bq == br || (q != q && r != r));
        bad += !(bq2 == br || (q2 != q2 && r != r));
    }
    return bad;
}
extern "C" double h_glibc_pow(double x, double y) { return pow(x, y); }
extern "C" long long h_log_mismatch(long long n, unsigned long long seed) {
    long long bad = 0;
    for (long long i = 0; i < n; i++) {
        seed ^= seed << 13; seed ^= seed >> 7; seed ^= seed << 17;
        double u = (double)(seed >> 11) * 0x1p-53;
        double x = exp(u * 20.723265836946414);   /* [1, 1e9] */
        bad += dg_log(x) != log(x);
    }
    return bad;
}
'''


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("dgmath")
    src = d / "m.cpp"
    src.write_text(SRC)
    so = d / "m.so"
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                           "-I", os.path.join(ROOT, "dengo_gb300", "csrc"), str(src),
                           "-o", str(so)])
    L = C.CDLL(str(so))
    for f in ("h_dg_log", "h_pow2", "h_pow3", "h_pow4", "h_glibc_log"):
        getattr(L, f).restype = C.c_double
        getattr(L, f).argtypes = [C.c_double]
    L.h_glibc_pow.restype = C.c_double
    L.h_glibc_pow.argtypes = [C.c_double, C.c_double]
    L.h_log_mismatch.restype = C.c_longlong
    L.h_log_mismatch.argtypes = [C.c_longlong, C.c_ulonglong]
    L.h_div_mismatch.restype = C.c_longlong
    L.h_div_mismatch.argtypes = [C.c_longlong, C.c_ulonglong]
    return L


def test_log_correctly_rounded(lib):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(1)
    xs = np.exp(rng.uniform(0, np.log(1e9), 20000))
    xs = np.concatenate([xs, [1.0, 2.0, 10.0, 1e9, 0.5, 3.0e-5, 1e300, 5e-300]])
    for x in xs:
        assert lib.h_dg_log(float(x)) == float(mpmath.log(mpmath.mpf(float(x)))), x


def test_log_special_values(lib):
    assert lib.h_dg_log(1.0) == 0.0
    assert math.isnan(lib.h_dg_log(float("nan")))
    assert lib.h_dg_log(0.0) == -math.inf
    assert lib.h_dg_log(math.inf) == math.inf


def test_log_agrees_with_glibc_except_its_misroundings(lib):
    bad = lib.h_log_mismatch(2_000_000, 88172645463325252)
    assert bad / 2_000_000 < 2e-4


def test_shared_reciprocal_division_is_exact(lib):
    """dg_div(a, b, 1/b) -- one correctly rounded reciprocal shared by all
    quotients with divisor b, then Markstein's FMA correction inside a
    guarded exponent range, a true division outside it -- equals a / b bit
    for bit (Markstein, IA-64 and Elementary Functions, 2000: the corrected
    quotient is correctly rounded when neither step under- or overflows)."""
    assert lib.h_div_mismatch(20_000_000, 0x9E3779B97F4A7C15) == 0


def test_integer_powers(lib):
    # The reference is built with gcc, which folds pow(x, 2) with a literal 2
    # into x*x at compile time; dg_ipow<2> is that product.  Cubes go to
    # glibc's pow at run time, which is not always correctly rounded.
    rng = np.random.default_rng(2)
    xs = np.ldexp(rng.uniform(1, 2, 5000), rng.integers(-200, 200, 5000))
    misround3 = 0
    for x in xs:
        x = float(x)
        assert lib.h_pow2(x) == x * x
        misround3 += lib.h_pow3(x) != lib.h_glibc_pow(x, 3.0)
        exact3 = Fraction(x) ** 3
        assert abs(Fraction(lib.h_pow3(x)) - exact3) <= Fraction(math.ulp(lib.h_pow3(x))) / 2
        exact4 = Fraction(x) ** 4
        assert abs(Fraction(lib.h_pow4(x)) - exact4) <= Fraction(math.ulp(lib.h_pow4(x))) / 2
    assert misround3 / len(xs) < 5e-3


CMP_SRC = r'''
#include "dg_math.h"
extern "C" int h_cmp(double a, double b) {
    int r = 0;
    r |= (dg_isnan(a) == (a != a)) << 0;
    r |= (dg_nonzero(a) == (a != 0.0)) << 1;
    r |= (dg_lt0(a) == (a < 0.0)) << 2;
    r |= (dg_abs_gt(a, b) == (fabs(a) > fabs(b))) << 3;
    r |= (dg_abs_gt_val(a, b) == (fabs(a) > b)) << 4;
    r |= (b > 0 ? (dg_lt_pos(a, b) == (a < b)) : 1) << 5;
    r |= (dg_finite(a) == (bool)isfinite(a)) << 6;
    return r;
}
'''


def test_integer_comparisons_match_ieee(tmp_path):
    """The bit-pattern comparisons used on the device agree with the C
    operators on every class of value (zeros of both signs, subnormals,
    normals, infinities, NaNs)."""
    src = tmp_path / "c.cpp"
    src.write_text(CMP_SRC)
    so = tmp_path / "c.so"
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                           "-I", os.path.join(ROOT, "dengo_gb300", "csrc"), str(src),
                           "-o", str(so)])
    L = C.CDLL(str(so))
    L.h_cmp.restype = C.c_int
    L.h_cmp.argtypes = [C.c_double, C.c_double]
    special = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1e-25, -1e-25, 1.0, -1.0,
               1.5, 1e308, -1e308, math.inf, -math.inf, math.nan, -math.nan]
    rng = np.random.default_rng(5)
    rand = list(np.ldexp(rng.uniform(-2, 2, 300), rng.integers(-1074, 1024, 300)))
    vals = special + [float(v) for v in rand]
    for a in vals:
        for b in special + [float(v) for v in rand[:40]]:
            assert L.h_cmp(a, b) == 0x7F, (a, b, bin(L.h_cmp(a, b)))
