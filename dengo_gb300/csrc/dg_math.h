/*
 * Elementary functions whose results are reproducible across host and
 * device.  The solver's decisions (Newton convergence, substep acceptance)
 * compare quantities near thresholds, so the device must compute what the
 * reference's host build computes.  Plain IEEE operations (+ - * / sqrt)
 * already agree when the device build does not contract a*b+c into an FMA
 * (nvcc --fmad=false) and the host build uses -ffp-contract=off; these two
 * functions cover the rest of the solver's arithmetic:
 *
 *   dg_log(x)      natural log with an error below 2^-68 relative before the
 *                  final rounding, so it returns the correctly rounded value
 *                  except when log(x) lies within ~2^-16 ulp of a rounding
 *                  midpoint.  glibc's log is correctly rounded on all but a
 *                  few in 10^5 inputs, so the two agree on all but about that
 *                  many.
 *   dg_ipow<n>(x)  x^n for integer n >= 2, the exact power rounded once
 *                  (compensated products).  x^2 is the single product x*x,
 *                  which is what glibc's pow(x, 2) returns for every finite x.
 *
 * Method of dg_log (table-driven reduction, after P. T. P. Tang, "Table-driven
 * implementation of the logarithm function in IEEE floating-point
 * arithmetic", ACM TOMS 16(4), 1990, carried in double-double):
 *   x = 2^e * m, m in [1,2);  j = nearest of 128ths to m - 1;
 *   inv_j ~ 1/(1 + j/128) (a table constant);  m * inv_j - 1 = r_hi + r_lo
 *   exactly (one product error term via fma, Sterbenz for the subtraction);
 *   log x = e ln2 + (-log inv_j) + log1p(r_hi) + r_lo (1 - r_hi),
 *   with ln2 and -log inv_j stored as double-double and log1p(r) - r by its
 *   Taylor series to r^8 (|r| <= 2^-8).  High parts are added with
 *   error-free sums; the low parts are summed once at the end.
 * Both functions use only +, -, *, fma and bit manipulation, so host and
 * device builds return identical bits.
 */
#ifndef DG_MATH_H
#define DG_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "dg_logtab.h"

#ifdef __CUDACC__
#define DG_HD __host__ __device__ __forceinline__
#else
#define DG_HD static inline
#endif

#ifdef __CUDACC__
__device__ const double dg_logtab_dev[129][3] = DG_LOGTAB_DATA;
#endif
static const double dg_logtab_host[129][3] = DG_LOGTAB_DATA;

DG_HD uint64_t dg_bits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

DG_HD double dg_from_bits(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

DG_HD double dg_fma(double a, double b, double c)
{
#ifdef __CUDA_ARCH__
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}

/* s + err == a + b exactly (Knuth's TwoSum). */
DG_HD void dg_two_sum(double a, double b, double *s, double *err)
{
    double sum = a + b;
    double bb = sum - a;
    *err = (a - (sum - bb)) + (b - bb);
    *s = sum;
}

DG_HD double dg_log(double x)
{
    if (!(x >= 2.2250738585072014e-308 && x <= 1.7976931348623157e308))
        return log(x); /* NaN, <= 0, subnormal, inf: never on the solver path */
    const uint64_t b = dg_bits(x);
    const int e = (int)(b >> 52) - 1023;
    const uint64_t mb = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
    const double m = dg_from_bits(mb);
    const int j = ((int)((mb >> 44) & 0xFF) + 1) >> 1;
#ifdef __CUDA_ARCH__
    const double inv = __ldg(&dg_logtab_dev[j][0]);
    const double thi = __ldg(&dg_logtab_dev[j][1]);
    const double tlo = __ldg(&dg_logtab_dev[j][2]);
#else
    const double inv = dg_logtab_host[j][0];
    const double thi = dg_logtab_host[j][1];
    const double tlo = dg_logtab_host[j][2];
#endif
    const double p = m * inv;
    const double rlo = dg_fma(m, inv, -p);
    const double r = p - 1.0;
    /* log1p(r) - r = r^2 * (-1/2 + r/3 - r^2/4 + ... - r^6/8) */
    double q = dg_fma(r, -0.125, 1.0 / 7.0);
    q = dg_fma(r, q, -1.0 / 6.0);
    q = dg_fma(r, q, 0.2);
    q = dg_fma(r, q, -0.25);
    q = dg_fma(r, q, 1.0 / 3.0);
    q = dg_fma(r, q, -0.5);
    const double poly = (r * r) * q;
    const double corr = dg_fma(-rlo, r, rlo);
    const double ed = (double)e;
    double s1, t1, s2, t2;
    dg_two_sum(ed * DG_LN2_HI, thi, &s1, &t1);
    dg_two_sum(s1, r, &s2, &t2);
    const double low = ((ed * DG_LN2_LO + tlo) + (corr + poly)) + (t1 + t2);
    return s2 + low;
}

/* Binary exponent field of x (0 for zero/subnormal, 0x7FF for inf/NaN). */
DG_HD int dg_expo(double x) { return (int)((dg_bits(x) >> 52) & 0x7FF); }

DG_HD bool dg_finite(double x) { return dg_expo(x) != 0x7FF; }

/* IEEE comparisons evaluated on the bit patterns, with the results of the C
 * operators in every case (NaN, infinities, signed zeros).  On GB300 a
 * floating-point compare occupies the scarce FP64 pipe; these run on the
 * integer pipes.  Shifting the bits left by one drops the sign and orders
 * magnitudes as unsigned integers; NaN is any magnitude above infinity's. */
#define DG_INF2 0xFFE0000000000000ull

DG_HD bool dg_isnan(double x) { return (dg_bits(x) << 1) > DG_INF2; }

/* x != 0.0 */
DG_HD bool dg_nonzero(double x) { return (dg_bits(x) << 1) != 0; }

/* x < 0.0 */
DG_HD bool dg_lt0(double x)
{
    const uint64_t b = dg_bits(x), m = b << 1;
    return (b >> 63) && m != 0 && m <= DG_INF2;
}

/* fabs(a) > fabs(b) */
DG_HD bool dg_abs_gt(double a, double b)
{
    const uint64_t x = dg_bits(a) << 1, y = dg_bits(b) << 1;
    return x <= DG_INF2 && y <= DG_INF2 && x > y;
}

/* fabs(s) > t */
DG_HD bool dg_abs_gt_val(double s, double t)
{
    const uint64_t x = dg_bits(s) << 1, tb = dg_bits(t), y = tb << 1;
    if (x > DG_INF2 || y > DG_INF2) return false;
    if (tb >> 63) return y != 0 || x != 0;   /* t <= -0: true unless s and t are zeros */
    return x > y;
}

/* y < c for c > 0 */
DG_HD bool dg_lt_pos(double y, double c)
{
    const uint64_t b = dg_bits(y);
    if ((b << 1) > DG_INF2) return false;
    if (b >> 63) return true;
    return b < dg_bits(c);
}

/* Divisor in the range where dg_div's fast path applies. */
DG_HD bool dg_div_ok(double b)
{
    const int e = dg_expo(b);
    return e >= 150 && e <= 1900;
}

/* a / b, correctly rounded, given rb = 1.0 / b (correctly rounded).
 * Markstein's quotient theorem (P. Markstein, "Computation of elementary
 * functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
 * 1990): with q = RN(a rb) and the exact remainder r = a - b q from one
 * fma, RN(q + r rb) = RN(a/b), provided no intermediate leaves the normal
 * range.  The exponent guard keeps |a|, |b| in [2^-873, 2^877] and their
 * ratio within 2^800, which keeps q and r normal; every other operand
 * (zero, subnormal, huge, inf, NaN) takes the plain division -- except a
 * zero numerator over a nonzero finite b, whose quotient is the zero with
 * the sign sign(a) xor sign(b) (IEEE 754), formed from the bits: structural
 * zeros of the Jacobian reach this on every elimination step, and a plain
 * division costs about nine FP64 operations.  One reciprocal then serves
 * all quotients by the same divisor at 3 FP64 operations each. */
DG_HD double dg_div(double a, double b, double rb)
{
    const int ea = dg_expo(a), eb = dg_expo(b), d = ea - eb;
    if (ea >= 150 && ea <= 1900 && eb >= 150 && eb <= 1900 && d >= -800 && d <= 800) {
        const double q = a * rb;
        const double r = dg_fma(-b, q, a);
        return dg_fma(r, rb, q);
    }
    const uint64_t ba = dg_bits(a), bb = dg_bits(b);
    if ((ba << 1) == 0 && (bb << 1) != 0 && eb != 0x7FF)
        return dg_from_bits((ba ^ bb) & 0x8000000000000000ull);
    return a / b;
}

/* a / b, correctly rounded, with dg_div's zero-numerator case taken from
 * the bits: for a quotient whose divisor has no reciprocal at hand. */
DG_HD double dg_quot(double a, double b)
{
    const uint64_t ba = dg_bits(a), bb = dg_bits(b);
    if ((ba << 1) == 0 && (bb << 1) != 0 && dg_expo(b) != 0x7FF)
        return dg_from_bits((ba ^ bb) & 0x8000000000000000ull);
    return a / b;
}

/* x^n, n >= 2: the exact power rounded once (up to ~2^-100 relative error
 * before that rounding). */
/* x^n in FP32 for the mixed path's Jacobian: plain products (one
 * rounding each; the Jacobian only steers Newton's iteration). */
template <int n>
DG_HD float dg_ipow(float x)
{
    float p = x;
#pragma unroll
    for (int k = 1; k < n; k++) p = p * x;
    return p;
}

template <int n>
DG_HD double dg_ipow(double x)
{
    if (n == 2) return x * x;
    double h = x * x;
    double l = dg_fma(x, x, -h);
#pragma unroll
    for (int k = 2; k < n; k++) {
        const double ph = h * x;
        const double pl = dg_fma(h, x, -ph);
        l = dg_fma(l, x, pl);
        h = ph;
    }
    return h + l;
}

#endif
