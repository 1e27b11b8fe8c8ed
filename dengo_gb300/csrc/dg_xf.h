/*
 * Extended-range FP32 ("XF"): a float mantissa with a separate int exponent,
 * value = m * 2^e, 1 <= |m| < 2 (or m = 0; inf/NaN carry e = 0).
 *
 * The mixed-precision solve builds its Newton matrix in this arithmetic:
 * every product, quotient and sum rounds to FP32's 24-bit significand, as
 * FP32 arithmetic does, but the exponent never underflows or overflows.
 * Plain FP32 cannot hold this network's Jacobian: rate and cooling tables
 * reach 1e-57 and whole tables lie below FP32's normal range (1.2e-38), and
 * after the scaling by dt * scale_v / scale_q such entries can dominate a
 * row.  Measured on the host build of the engine, the Newton iteration with
 * a plain-FP32 Jacobian converged 28 of 64 converged config-1 cells; with
 * the FP64 Jacobian rounded to 24 bits but its exponent kept, all 64 with
 * the FP64 path's sweep counts.
 *
 * Every operation runs on the FP32 and integer pipes (the exponent
 * bookkeeping is integer arithmetic on the float's bit pattern), so the
 * Jacobian costs no FP64 instruction; conversions from and to FP64 are bit
 * manipulations as well.  Values below FP64's normal range convert to zero.
 */
#ifndef DG_XF_H
#define DG_XF_H

#include "dg_math.h"

namespace dg {

DG_HD unsigned int xf_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned int b;
    memcpy(&b, &f, sizeof b);
    return b;
#endif
}

DG_HD float xf_from_bits(unsigned int b)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
#endif
}

struct XF {
    float m;
    int e;
};

/* Normalises m * 2^e so that 1 <= |m| < 2 (m is a normal float, zero, inf
 * or NaN; FP32 subnormals cannot arise from normalised operands). */
DG_HD XF xf_norm(float m, int e)
{
    const unsigned int b = xf_bits(m);
    const int f = (int)((b >> 23) & 0xffu);
    if (f == 0) return XF{xf_from_bits(b & 0x80000000u), 0};
    if (f == 0xff) return XF{m, 0};
    return XF{xf_from_bits((b & 0x807fffffu) | 0x3f800000u), e + f - 127};
}

DG_HD bool xf_finite(XF a) { return ((xf_bits(a.m) >> 23) & 0xffu) != 0xffu; }
DG_HD bool xf_zero(XF a) { return (xf_bits(a.m) & 0x7fffffffu) == 0u; }

/* 2^k as a float, -126 <= k <= 127 */
DG_HD float xf_pow2(int k) { return xf_from_bits((unsigned int)(127 + k) << 23); }

/* double -> XF: the significand rounded to 24 bits (to nearest, ties to
 * even); FP64 subnormals become zero, inf and NaN stay. */
DG_HD XF xf(double d)
{
    const unsigned long long b = dg_bits(d);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    int E = (int)((b >> 52) & 0x7ff);
    if (E == 0) return XF{xf_from_bits(sign), 0};
    if (E == 0x7ff) {
        const unsigned long long man = b & 0xfffffffffffffull;
        return XF{xf_from_bits(sign | (man ? 0x7fc00000u : 0x7f800000u)), 0};
    }
    const unsigned long long man = b & 0xfffffffffffffull;
    unsigned int top = (unsigned int)(man >> 29);
    const unsigned int rem = (unsigned int)(man & 0x1fffffffu);
    if (rem > 0x10000000u || (rem == 0x10000000u && (top & 1u))) top++;
    if (top == 0x800000u) {
        top = 0;
        E++;
    }
    return XF{xf_from_bits(sign | 0x3f800000u | top), E - 1023};
}

DG_HD XF xf(float f) { return xf_norm(f, 0); }
DG_HD XF xf(int i) { return xf_norm((float)i, 0); }

/* XF -> double, exact inside FP64's normal range (zero below it,
 * infinity above). */
DG_HD double xf_to_double(XF a)
{
    const unsigned int b = xf_bits(a.m);
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    const unsigned int f = (b >> 23) & 0xffu;
    if (f == 0) return dg_from_bits(sign);
    if (f == 0xff) return (double)a.m;
    const long long E = (long long)a.e + 1023;
    if (E <= 0) return dg_from_bits(sign);
    if (E >= 0x7ff) return dg_from_bits(sign | 0x7ff0000000000000ull);
    return dg_from_bits(sign | ((unsigned long long)E << 52) |
                        ((unsigned long long)(b & 0x7fffffu) << 29));
}

DG_HD XF operator-(XF a) { return XF{-a.m, a.e}; }
DG_HD XF operator*(XF a, XF b) { return xf_norm(a.m * b.m, a.e + b.e); }
DG_HD XF operator/(XF a, XF b) { return xf_norm(a.m / b.m, a.e - b.e); }

DG_HD XF operator+(XF a, XF b)
{
    if (!xf_finite(a) || !xf_finite(b)) return XF{a.m + b.m, 0};
    if (xf_zero(a)) return b;
    if (xf_zero(b)) return a;
    const int d = a.e - b.e;
    if (d >= 0) return d > 40 ? a : xf_norm(a.m + b.m * xf_pow2(-d), a.e);
    return d < -40 ? b : xf_norm(b.m + a.m * xf_pow2(d), b.e);
}

DG_HD XF operator-(XF a, XF b) { return a + (-b); }

/* mixed operands: float and int literals of the generated expressions */
DG_HD XF operator+(XF a, float b) { return a + xf(b); }
DG_HD XF operator+(float a, XF b) { return xf(a) + b; }
DG_HD XF operator-(XF a, float b) { return a - xf(b); }
DG_HD XF operator-(float a, XF b) { return xf(a) - b; }
DG_HD XF operator*(XF a, float b) { return a * xf(b); }
DG_HD XF operator*(float a, XF b) { return xf(a) * b; }
DG_HD XF operator/(XF a, float b) { return a / xf(b); }
DG_HD XF operator/(float a, XF b) { return xf(a) / b; }
DG_HD XF operator+(XF a, int b) { return a + xf(b); }
DG_HD XF operator+(int a, XF b) { return xf(a) + b; }
DG_HD XF operator-(XF a, int b) { return a - xf(b); }
DG_HD XF operator-(int a, XF b) { return xf(a) - b; }
DG_HD XF operator*(XF a, int b) { return a * xf(b); }
DG_HD XF operator*(int a, XF b) { return xf(a) * b; }
DG_HD XF operator/(XF a, int b) { return a / xf(b); }
DG_HD XF operator/(int a, XF b) { return xf(a) / b; }

template <int n>
DG_HD XF dg_ipow(XF x)
{
    XF p = x;
#pragma unroll
    for (int k = 1; k < n; k++) p = p * x;
    return p;
}

}  // namespace dg
#endif
