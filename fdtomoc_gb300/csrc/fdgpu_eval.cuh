/*
 * fdgpu_eval.cuh — evaluation of one face point on the GPU, bit-identical to the reference.
 *
 * The reference's face-point body (TOP: src/sphfd.c:1034-1761, the other faces mirrored) runs 22
 * trial stencils in a fixed order and keeps the minimum.  The sequence comes from fd_face_table.h.
 * The arithmetic keeps the reference's FP64 operation order exactly; what changes is how each
 * operation is obtained:
 *
 *   - geometry-only subexpressions (products of radius, sin(colatitude), angular steps, the
 *     fdsph3d coefficients, the quadratics' 'a') come from tables built with the reference's own
 *     formula, so they are the same doubles the reference computes;
 *   - x / d for a geometric divisor d is RN(x/d) computed from the tabulated RN(1/d) with two
 *     fused-multiply-add corrections (Markstein's theorem; 5 FP64 ops instead of ~17 for a
 *     generic division on this part);
 *   - float->double conversions and power-of-two scalings are done on the integer pipe;
 *   - a stencil whose causality floor (the largest time it reads, which its accepted root can
 *     never be below) is already >= the running minimum is not evaluated: it cannot lower the
 *     minimum, and its only side effect, the stale (t0,t4) state, is still applied.
 *
 * The kernel translation unit is compiled with --fmad=false: no multiply-add is contracted except
 * the explicit __fma_rn corrections of the division, whose results are exact by construction.
 */
#ifndef FDGPU_EVAL_CUH
#define FDGPU_EVAL_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "fd_face_table.h"
#include "fdgpu_check.cuh"
#include "fdgpu_layout.h"

namespace fdk {

/* ---------------------------------------------------------------------------------------------- */
/* exact helpers                                                                                   */

/* float -> double on the integer pipe (normal numbers and zeros; anything else converts normally) */
__device__ __forceinline__ double f2d(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    if (e - 1u < 254u) {
        const unsigned long long d = ((unsigned long long)(b & 0x80000000u) << 32)
                                     | ((unsigned long long)(e + 896u) << 52)
                                     | ((unsigned long long)(b & 0x7fffffu) << 29);
        return __longlong_as_double((long long)d);
    }
    if ((b << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)(b & 0x80000000u) << 32));
    return (double)f;
}

/* Comparisons of finite doubles on the integer pipe (an FP64 compare occupies this GPU's FP64 unit
 * like any FP64 instruction, 64 cycles per warp).  Each gives exactly the double comparison's result,
 * signed zeros included, for the operands it states; none is used where an operand may be NaN. */

/* a < b for finite a and b of any sign */
__device__ __forceinline__ bool flt(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    if ((ia | ib) >= 0) return ia < ib;                       /* both non-negative */
    if ((ia & ib) < 0) return ia > ib;                        /* both negative: the larger magnitude */
    if (ia < 0) return (ia << 1) != 0 || (ib << 1) != 0;      /* a negative: below b unless both zero */
    return false;                                             /* b negative, a not */
}

/* !(x >= 0.) for any x: negative and not -0, or NaN */
__device__ __forceinline__ bool not_ge0(double x)
{
    const long long ix = __double_as_longlong(x);
    return (ix < 0 && (ix << 1) != 0) || (ix & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

/* x * 2^k, exact: exponent arithmetic on the integer pipe when x and the result are normal;
 * zeros and subnormals take the floating-point multiply (never reached with physical inputs) */
template <int K>
__device__ __forceinline__ double scale2k(double x)
{
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e != 0 && e + K >= 1 && e + K <= 2046) return __longlong_as_double(b + ((long long)K << 52));
    constexpr double p2 = K >= 0 ? (double)(1ll << (K >= 0 ? K : 0)) : 1.0 / (double)(1ll << (K < 0 ? -K : 0));
    return x * p2;
}

/* RN(x / d) given inv = RN(1/d): q = RN(x*inv) then two exact-residual corrections.  Zero x keeps
 * its sign, as a true division would. */
__device__ __forceinline__ double div_rn(double x, double d, double inv)
{
    if ((__double_as_longlong(x) << 1) == 0) return __dmul_rn(x, inv);
    double q = __dmul_rn(x, inv);
    double e = __fma_rn(-d, q, x);
    q = __fma_rn(e, inv, q);
    e = __fma_rn(-d, q, x);
    return __fma_rn(e, inv, q);
}

/* ---------------------------------------------------------------------------------------------- */
/* compile-time face geometry                                                                      */

template <int F>
struct FaceT {
    static constexpr int AU = fd_face_frame[F].axis_u;
    static constexpr int AV = fd_face_frame[F].axis_v;
    static constexpr int AN = fd_face_frame[F].axis_n;
    static constexpr int IN = fd_face_frame[F].inner;
    static constexpr int HW = fd_face_frame[F].headw;
    /* offset of node (du,dv,w) along grid axis a (0 x, 1 y, 2 z) */
    __host__ __device__ static constexpr int off(int a, fdn_node n) { return a == AU ? n.du : a == AV ? n.dv : n.w * IN; }
};

/* What a face point needs from its surroundings: times and slownesses of the 3x3 block on the face
 * layer (w=0) and on the inner layer (w=1), and the indices that locate it. */
struct PointCtx {
    int u, v;                  /* face coordinates */
    int z, y;                  /* grid z and y of the point */
    int nu, nv;                /* grid extent along u and v */
    int ulo, uhi, vlo, vhi;    /* current face rectangle */
    long long pT;              /* index of the point in T */
    float t[2][3][3];
    float s[2][3][3];
};

__device__ __forceinline__ const double *node_row(const fd_geo_dev &g, int z, int y)
{
    if (!FD_OK(z, g.nz, 1) || !FD_OK(y, g.ny, 2)) { z = 0; y = 0; }
    return g.node + ((long long)z * g.ny + y) * FD_N_N;
}

/* canonical distance products of the new-edge / 2-D / new-face stencils */
enum { CH_H = 0, CH_RDQ = 1, CH_RSDF = 2 };
__host__ __device__ constexpr int chain_class(fdn_chain c)
{
    return c.n == 1 ? CH_H : c.n == 2 ? CH_RDQ : CH_RSDF;
}

#define FD_T(p, n) ((p).t[(n).w][(n).dv + 1][(n).du + 1])

/* roots of a x^2 + b x + c = 0 (rad = b*b - 4ac already formed), with the reference's
 * causality test against floor tmx; tie rule of fdsph3d (x1 preferred only if strictly smaller). */
__device__ __forceinline__ double roots_3d(double b, double rad, double twoa, double i2a, double tmx)
{
    if (not_ge0(rad)) return 1.e11;
    const double sq = __dsqrt_rn(rad);
    const double x1 = div_rn(-b + sq, twoa, i2a);
    const double x2 = div_rn(-b - sq, twoa, i2a);
    const bool bad1 = flt(x1, tmx), bad2 = flt(x2, tmx);
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return flt(x1, x2) ? x1 : x2;
}

/* same, with the tie rule of fdsphne / fdsph2d (x2 preferred only if strictly smaller) */
__device__ __forceinline__ double roots_2(double b, double rad, double twoa, double i2a, double tmx)
{
    if (not_ge0(rad)) return 1.e11;
    const double sq = __dsqrt_rn(rad);
    const double x1 = div_rn(-b + sq, twoa, i2a);
    const double x2 = div_rn(-b - sq, twoa, i2a);
    const bool bad1 = flt(x1, tmx), bad2 = flt(x2, tmx);
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return flt(x2, x1) ? x2 : x1;
}

}  // namespace fdk

#endif
