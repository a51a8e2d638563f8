/*
 * fdgpu_bound.cuh — single-precision lower bounds of stencil values, used to skip FP64
 * evaluations that cannot lower a running minimum.
 *
 * Most 2-D (fdsph2d) trials that pass the causality-floor test still lose to the running minimum
 * by far more than single-precision rounding: on the 201x201x81 benchmark station, 29 of 30 million
 * lose by more than 1e-4 relative, and only about 50 thousand win.  The FP64 pipe of this GPU is
 * narrow, so each skipped evaluation saves about 70 FP64 operations.
 *
 * The bound is rigorous, not a heuristic.  Every quantity of the stencil is computed in FP32, in the
 * same order as the FP64 evaluation, together with an upper bound e on its distance from the
 * double-precision value the FP64 path computes:
 *
 *     |v32 - v64| <= e.
 *
 * Each operation z = x op y propagates the input bounds exactly as the mathematics allows (for
 * example |xy - x'y'| <= |x| ey + (|y| + ey) ex).  It adds U|z32| for the rounding of both the FP32
 * and the FP64 result; U = 2^-22 covers 2^-24 + 2^-53 with room.  The bounds themselves are
 * computed with upward rounding (__fmaf_ru, __fmul_ru, ...), so they never shrink by rounding.
 * Table doubles enter through truncation toward zero to FP32, on the integer pipe (relative error
 * below 2^-23).  A NaN or an infinity anywhere makes the final comparison fail, so the caller
 * evaluates the trial in FP64.
 *
 * The kernel translation unit is compiled with --fmad=false, so the FP32 value operations are
 * rounded one by one, as the bound assumes.
 */
#ifndef FDGPU_BOUND_CUH
#define FDGPU_BOUND_CUH

#include "fdgpu_trials.cuh"

namespace fdk {

#define FB_U 2.384185791015625e-07f      /* 2^-22 */
#define FB_INFL 1.00000095367431640625f  /* 1 + 2^-20: absorbs the FP64 rounding of propagated error */

/* value and a bound of its distance from the FP64 path's value */
struct EB {
    float v, e;
};

/* a positive normal double truncated to float on the integer pipe (NaN outside float's normal
 * range, which makes every later comparison fail) */
__device__ __forceinline__ float d2f_trunc(double x)
{
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (b <= 0 || e < 1 || e > 254) return __int_as_float(0x7fc00000);
    return __int_as_float((e << 23) | (int)((b >> 29) & 0x7fffff));
}

__device__ __forceinline__ float eb_tail(float v, float prop)
{
    return __fmaf_ru(FB_U, fabsf(v), __fmul_ru(prop, FB_INFL));
}

__device__ __forceinline__ EB eb_exact(float v) { return {v, 0.f}; }

/* a tabulated double */
__device__ __forceinline__ EB eb_tab(double x)
{
    const float f = d2f_trunc(x);
    return {f, __fmul_ru(FB_U, fabsf(f))};
}

__device__ __forceinline__ EB eb_add(EB a, EB b)
{
    const float v = a.v + b.v;
    return {v, eb_tail(v, __fadd_ru(a.e, b.e))};
}

__device__ __forceinline__ EB eb_sub(EB a, EB b)
{
    const float v = a.v - b.v;
    return {v, eb_tail(v, __fadd_ru(a.e, b.e))};
}

__device__ __forceinline__ EB eb_mul(EB a, EB b)
{
    const float v = a.v * b.v;
    const float p = __fmaf_ru(fabsf(a.v), b.e, __fmul_ru(__fadd_ru(fabsf(b.v), b.e), a.e));
    return {v, eb_tail(v, p)};
}

__device__ __forceinline__ EB eb_sq(EB a)
{
    const float v = a.v * a.v;
    return {v, eb_tail(v, __fmul_ru(a.e, __fmaf_ru(2.f, fabsf(a.v), a.e)))};
}

/* x / d for a tabulated divisor d, as x times its tabulated reciprocal: the FP64 path rounds
 * the exact quotient x/d once, and the truncated reciprocal is within 2^-22 of 1/d, so this is
 * eb_mul by a tabulated value */
__device__ __forceinline__ EB eb_div_tab(EB a, double inv) { return eb_mul(a, eb_tab(inv)); }

/* times a power of two: exact in both precisions */
__device__ __forceinline__ EB eb_scale(EB a, float p2) { return {a.v * p2, a.e * fabsf(p2)}; }

/* sqrt: |sqrt(x) - sqrt(x')| <= min(e / sqrt(x), sqrt(e)) for x > 0, and <= sqrt(x + e) when x <= 0
 * (a negative FP64 argument makes the stencil reject, which no lower bound contradicts) */
__device__ __forceinline__ EB eb_sqrt(EB a)
{
    if (!(a.v > 0.f)) {
        const float hi = __fadd_ru(a.v, a.e);
        return {0.f, hi > 0.f ? __fsqrt_ru(hi) : 0.f};
    }
    const float v = __fsqrt_rn(a.v);
    /* rsqrtf is within 2 ulp of 1/sqrt(x) and __fsqrt_rn within half an ulp: the factors cover both */
    const float p = fminf(__fmul_ru(a.e, __fmul_ru(rsqrtf(a.v), 1.00000095367431640625f)),
                          __fmul_ru(__fsqrt_rn(a.e), 1.0000002384185791015625f));
    return {v, eb_tail(v, p)};
}

/* Lower bound of the value fdsph2d returns for trial d (the stencil of eval_2d, same order of
 * operations), given its causality floor fl or any float below it.  The roots of a x^2 + b x + c
 * (a > 0) satisfy x2 <= x1 in FP64 as well, every operation there being monotone, and the value is
 * x2 when x2 >= floor, else x1 when x1 >= floor, else the rejection value 1e11.  So when x2 is
 * certainly below fl the value is at least min(x1, 1e11); otherwise it is at least x2.  A floor
 * below the true one (the stale pair left out) only weakens the first test. */
__device__ __forceinline__ float lower_2d(const TrialDesc &d, const float *t18, const float *s18, const fd_geo_dev &g,
                                          int z, int y, float fl)
{
    double iv[4];   /* reciprocals of d01 d02 d13 d23 */
#pragma unroll
    for (int j = 0; j < 4; j++) {
        double dj;
        dist_rt(g, d.dcls[j], z + d.ddz[j], y + d.ddy[j], dj, iv[j]);
    }
    double a64, i2a;
    apair_rt(g, d.apair, z, y, a64, i2a);
    const EB a = eb_tab(a64);
    const EB t1 = eb_exact(t18[d.slot[1]]), t2 = eb_exact(t18[d.slot[2]]), t3 = eb_exact(t18[d.slot[3]]);
    const EB sum = eb_add(eb_add(eb_add(eb_exact(s18[NB_POINT]), eb_exact(s18[d.slot[1]])), eb_exact(s18[d.slot[2]])),
                          eb_exact(s18[d.slot[3]]));
    const EB slo = eb_scale(sum, 0.25f);
    const EB p = eb_sub(eb_div_tab(eb_sub(t1, t3), iv[2]), eb_div_tab(t2, iv[1]));
    const EB q = eb_sub(eb_div_tab(eb_sub(t2, t3), iv[3]), eb_div_tab(t1, iv[0]));
    const EB b = eb_scale(eb_add(eb_div_tab(p, iv[1]), eb_div_tab(q, iv[0])), 2.f);
    const EB c = eb_sub(eb_add(eb_sq(p), eb_sq(q)), eb_mul(sum, slo));
    const EB rad = eb_sub(eb_sq(b), eb_mul(eb_scale(a, 4.f), c));
    if (__fadd_ru(rad.v, rad.e) < 0.f) return 1.e10f;   /* the FP64 discriminant is negative: 1e11 */
    const EB sq = eb_sqrt(rad);
    const EB nb = eb_scale(b, -1.f);
    const EB x2 = eb_div_tab(eb_sub(nb, sq), i2a);   /* i2a = 1/(2a) */
    if (__fadd_ru(x2.v, x2.e) < fl) {
        const EB x1 = eb_div_tab(eb_add(nb, sq), i2a);
        return fminf(__fsub_rd(x1.v, x1.e), 1.e10f);
    }
    return __fsub_rd(x2.v, x2.e);
}

/* trial value v (>= the returned bound lo) cannot lower a running minimum that is at most g */
__device__ __forceinline__ bool bound_prunes(float lo, double g)
{
    return lo >= 0.f && !lt(1.e11, g) && !lt(f2d(lo), g);
}

}  // namespace fdk

#endif
