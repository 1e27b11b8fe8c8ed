/*
 * Mixed-precision linear solve of one cell's Newton system (the precision =
 * DENGO_MIXED path).
 *
 * The reference solves the scaled system (I - dt J) s = g with FP64 Gaussian
 * elimination (BE_chem_solve.C:330-382).  Here the elimination runs in FP32 and
 * FP64 iterative refinement recovers the FP64 solution:
 *
 *   1. power-of-two row scales 2^s_i and column scales 2^t_j, from the
 *      exponent fields only (integer operations): every entry of the scaled
 *      matrix R A C lies below 1 and each row and column maximum in [2^-1, 1);
 *   2. R A C rounded to FP32 by integer operations (round to nearest even;
 *      entries below FP32's normal range become zeros);
 *   3. FP32 LU with partial pivoting, the pivots kept for repeated solves;
 *   4. x0 = C (LU)^-1 R g, the right-hand side normalised by a power of two;
 *   5. refinement: r = g - A x in FP64 (fused multiply-adds over the
 *      structural nonzeros), d = C (LU)^-1 R r, x = x + d, repeated (at most
 *      4 times) until the correction is below 2^-40 of max |x| or stops
 *      halving (the FP64 residual's own accuracy is reached).
 *
 * operator() runs it all on one lane; the split engine calls prepare /
 * residual_row / refine itself to spread the residual rows over its warps.
 *
 * The scale factors are powers of two and the FP32 <-> FP64 conversions are
 * exact integer re-encodings, so no step except the residual and the update
 * uses the FP64 pipe.  The FP64 matrix is left intact; when it or g holds
 * inf/NaN, or the FP32 solve yields a non-finite value, mixed_solve returns
 * false and the caller runs the FP64 elimination instead (which then
 * reproduces the reference's NaN propagation).
 *
 * A refinement that ends without meeting the 2^-40 criterion (its
 * correction stopped halving, or MAX_REFINE steps were taken) also hands the
 * system to the FP64 elimination, so no solve is kept less accurate than the
 * FP64 path's.  In the solver's own Newton systems that happens in well under
 * 0.1 % of solves.  Built with DG_MIXED_STRICT=0 such a solution is kept
 * instead and Newton's convergence test judges the sweep.
 */
#ifndef DG_MIXED_CUH
#define DG_MIXED_CUH

#ifndef DG_MIXED_STRICT
#define DG_MIXED_STRICT 1
#endif

#include "dg_math.h"
#include "dg_slots.cuh"

namespace dg {

/* (float)(v * 2^e), round to nearest even, by integer operations.  Requires
 * |v * 2^e| < 2^128 and v finite; results below FP32's normal range and FP64
 * subnormal inputs give a signed zero. */
__device__ __forceinline__ float dg_f32_scaled(double v, int e)
{
    const unsigned long long b = dg_bits(v);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int be = (int)((b >> 52) & 0x7ff);
    const int fe = be - 1023 + 127 + e;
    if (be == 0 || fe <= 0) return __uint_as_float(sign);
    const unsigned long long man = b & 0xfffffffffffffull;
    unsigned int m = (unsigned int)(man >> 29);
    const unsigned int rem = (unsigned int)(man & 0x1fffffffu);
    if (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) m++;
    /* a mantissa carry runs into the exponent field, as it should */
    return __uint_as_float(sign | (((unsigned int)fe << 23) + m));
}

/* (double)f * 2^e by integer operations (exact inside FP64's normal range;
 * below it a signed zero, above it a signed infinity).  f must be finite. */
__device__ __forceinline__ double dg_f64_scaled(float f, int e)
{
    const unsigned int b = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    int fe = (int)((b >> 23) & 0xff);
    unsigned int m = b & 0x7fffffu;
    if (fe == 0) {
        if (m == 0) return dg_from_bits(sign);
        const int sh = __clz(m) - 8; /* bring the leading one to bit 23 */
        m = (m << sh) & 0x7fffffu;
        fe = 1 - sh;
    }
    const int de = fe - 127 + 1023 + e;
    if (de <= 0) return dg_from_bits(sign);
    if (de >= 0x7ff) return dg_from_bits(sign | 0x7ff0000000000000ull);
    return dg_from_bits(sign | ((unsigned long long)de << 52) | ((unsigned long long)m << 29));
}

__device__ __forceinline__ bool dg_f32_finite(float f) { return ((__float_as_uint(f) >> 23) & 0xff) != 0xff; }

template <class Net, int BLOCK>
struct MixedSolve {
    static constexpr int N = Net::N;
    static constexpr int NONE = -100000;
    static constexpr int MAX_REFINE = 4;
    Slots<BLOCK> J;   /* FP64 scaled I - dt J, column-major, left intact */
    SlotsF<BLOCK> JF; /* FP32 factors */

    /* FP32 partial-pivot LU of R A C; the reciprocal pivots replace the
     * diagonal. */
    __device__ __forceinline__ void factor(int (&piv)[N]) const
    {
#pragma unroll
        for (int k = 0; k < N - 1; k++) {
            int p = k;
            float best = fabsf(JF[k * N + k]);
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                const float a = fabsf(JF[k * N + i]);
                if (a > best) {
                    best = a;
                    p = i;
                }
            }
            piv[k] = p;
            if (p != k) {
#pragma unroll
                for (int j = k; j < N; j++) {
                    const float t = JF[j * N + k];
                    JF[j * N + k] = JF[j * N + p];
                    JF[j * N + p] = t;
                }
            }
            const float rp = 1.0f / JF[k * N + k];
            JF[k * N + k] = rp;
            float m[N], row[N];
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                m[i] = JF[k * N + i] * rp;
                JF[k * N + i] = m[i];
            }
#pragma unroll
            for (int j = k + 1; j < N; j++) row[j] = JF[j * N + k];
#pragma unroll
            for (int i = k + 1; i < N; i++) {
#pragma unroll
                for (int j = k + 1; j < N; j++) JF[j * N + i] = fmaf(-m[i], row[j], JF[j * N + i]);
            }
        }
        piv[N - 1] = N - 1;
        JF[(N - 1) * N + (N - 1)] = 1.0f / JF[(N - 1) * N + (N - 1)];
    }

    __device__ __forceinline__ void solve32(const int (&piv)[N], float (&v)[N]) const
    {
#pragma unroll
        for (int k = 0; k < N - 1; k++) {
            const int p = piv[k];
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                if (i == p) {
                    const float t = v[k];
                    v[k] = v[i];
                    v[i] = t;
                }
            }
            const float vk = v[k];
#pragma unroll
            for (int i = k + 1; i < N; i++) v[i] = fmaf(-JF[k * N + i], vk, v[i]);
        }
#pragma unroll
        for (int i = N - 1; i >= 0; i--) {
            float vi = v[i];
#pragma unroll
            for (int j = i + 1; j < N; j++) vi = fmaf(-JF[j * N + i], v[j], vi);
            v[i] = vi * JF[i * N + i];
        }
    }

    /* d = C (LU)^-1 R r for an FP64 right-hand side r; returns false on a
     * non-finite FP32 result.  *emax receives the largest exponent in d. */
    __device__ __forceinline__ bool apply(const int (&piv)[N], const int (&s)[N], const int (&t)[N],
                                          const double (&r)[N], double (&d)[N], int &emax) const
    {
        int W = NONE;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const int e = dg_expo(r[i]);
            if (e != 0 && e + s[i] > W) W = e + s[i];
        }
        emax = 0;
        if (W == NONE) {
#pragma unroll
            for (int i = 0; i < N; i++) d[i] = 0.0;
            return true;
        }
        float v[N];
#pragma unroll
        for (int i = 0; i < N; i++) v[i] = dg_f32_scaled(r[i], s[i] + 1022 - W);
        solve32(piv, v);
        bool fin = true;
#pragma unroll
        for (int j = 0; j < N; j++) {
            fin = fin && dg_f32_finite(v[j]);
            d[j] = dg_f64_scaled(v[j], t[j] + W - 1022);
            const int e = dg_expo(d[j]);
            emax = e > emax ? e : emax;
        }
        return fin;
    }

    /* Equilibration, FP32 rounding and factorisation of A, and the first
     * solve x = C (LU)^-1 R g.  false: A or g holds inf/NaN or the FP32 solve
     * broke down (A and g untouched; the caller falls back to FP64). */
    __device__ __forceinline__ bool prepare(const double (&g)[N], int (&s)[N], int (&t)[N],
                                            int (&piv)[N], double (&x)[N]) const
    {
        bool fin = true;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const int eg = dg_expo(g[i]);
            fin = fin && eg != 0x7ff;
            int m = 0;
#pragma unroll
            for (int j = 0; j < N; j++) {
                const int e = dg_expo(J[j * N + i]);
                fin = fin && e != 0x7ff;
                m = e > m ? e : m;
            }
            s[i] = m ? 1022 - m : 0;
        }
        if (!fin) return false;
#pragma unroll
        for (int j = 0; j < N; j++) {
            int m = NONE;
#pragma unroll
            for (int i = 0; i < N; i++) {
                if (!Net::jnz(i, j)) continue;
                const int e = dg_expo(J[j * N + i]);
                if (e != 0 && e + s[i] > m) m = e + s[i];
            }
            t[j] = m == NONE ? 0 : 1022 - m;
        }
#pragma unroll
        for (int j = 0; j < N; j++) {
#pragma unroll
            for (int i = 0; i < N; i++)
                JF[j * N + i] = Net::jnz(i, j) ? dg_f32_scaled(J[j * N + i], s[i] + t[j]) : 0.0f;
        }
        factor(piv);
        int ed;
        return apply(piv, s, t, g, x, ed);
    }

    /* Residual of row i, g_i - sum_j A_ij x_j, in FP64 over the structural
     * nonzeros (i must be a compile-time constant after unrolling). */
    template <class XS>
    __device__ __forceinline__ double residual_row(int i, double gi, const XS &x) const
    {
        double acc = gi;
#pragma unroll
        for (int j = 0; j < N; j++)
            if (Net::jnz(i, j)) acc = __fma_rn(-J[j * N + i], x[j], acc);
        return acc;
    }

    /* One refinement step from the residual r: x += C (LU)^-1 R r.  Returns
     * false on a non-finite value; *more is cleared when the correction is
     * below 2^-40 of max|x| or did not halve (exponent eprev, updated). */
    __device__ __forceinline__ bool refine(const int (&piv)[N], const int (&s)[N], const int (&t)[N],
                                           const double (&r)[N], double (&x)[N], int &eprev,
                                           bool &more) const
    {
        double d[N];
        int ed;
        bool fin = apply(piv, s, t, r, d, ed);
        int ex = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            x[j] = x[j] + d[j];
            const int e = dg_expo(x[j]);
            ex = e > ex ? e : ex;
            fin = fin && e != 0x7ff;
        }
        more = !(ed <= ex - 40 || ed >= eprev);
        eprev = ed;
        return fin;
    }

    /* Whether a refinement that stopped with last-correction exponent ed met
     * the 2^-40 criterion (a zero correction meets it). */
    __device__ __forceinline__ static bool refined(const double (&x)[N], int ed)
    {
        int ex = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            const int e = dg_expo(x[j]);
            ex = e > ex ? e : ex;
        }
        return ed == 0 || ed <= ex - 40;
    }

    /* x = A^-1 g; false: A or g holds inf/NaN, the FP32 solve broke down
     * or (unless DG_MIXED_STRICT=0) the refinement stopped short of 2^-40;
     * x undefined, A and g untouched. */
    __device__ __forceinline__ bool operator()(const double (&g)[N], double (&x)[N]) const
    {
        int s[N], t[N], piv[N];
        if (!prepare(g, s, t, piv, x)) return false;
        int eprev = 0x7ff;
#pragma unroll 1
        for (int it = 0; it < MAX_REFINE; it++) {
            double r[N];
#pragma unroll
            for (int i = 0; i < N; i++) r[i] = residual_row(i, g[i], x);
            bool more;
            if (!refine(piv, s, t, r, x, eprev, more)) return false;
            if (!more) return !DG_MIXED_STRICT || refined(x, eprev);
        }
        return !DG_MIXED_STRICT;
    }
};

}  // namespace dg
#endif
