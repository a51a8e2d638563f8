/*
 * fdgpu_eval.cuh — evaluation of one face point on the GPU, bit-identical to the reference.
 *
 * The reference's face-point body (TOP: src/sphfd.c:1034-1761, the other faces mirrored) runs 22
 * trial stencils in a fixed order and keeps the minimum.  Here the sequence comes from
 * fd_face_table.h and is expanded at compile time per face (template recursion over the trial
 * index), so every node offset, guard and geometry lookup is a constant.  The arithmetic keeps the
 * reference's FP64 operation order exactly; what changes is how each operation is obtained:
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

/* per-point evaluation state: the reference's guess / fhead / t[0],t[4] */
struct EvalState {
    double guess;
    double fhead;
    float t0, t4;              /* the stale stencil slots 0 and 4 */
    int writers;               /* 3-D / new-edge / new-face calls made so far */
    bool gate;                 /* first-contact block gate */
    bool have_inherit;         /* t0,t4 hold a valid inherited state */
    bool defer;                /* needs the state left by an earlier point: stop */
    int n3d, nne, n2d, nnf, n1d;
};

__device__ __forceinline__ const double *node_row(const fd_geo_dev &g, int z, int y)
{
    return g.node + ((long long)z * g.ny + y) * FD_N_N;
}

/* canonical distance products of the new-edge / 2-D / new-face stencils */
enum { CH_H = 0, CH_RDQ = 1, CH_RSDF = 2 };
__host__ __device__ constexpr int chain_class(fdn_chain c)
{
    return c.n == 1 ? CH_H : c.n == 2 ? CH_RDQ : CH_RSDF;
}

template <int F, int K, int J>
struct Dist {
    static constexpr fdn_chain c = fd_face_trials[F][K].d[J];
    static constexpr int cls = chain_class(c);
    static_assert(cls != CH_H || (c.n == 1 && c.f[0].kind == FDN_H), "distance chain shape");
    static_assert(cls != CH_RDQ || (c.f[0].kind == FDN_R && c.f[1].kind == FDN_DQ), "distance chain shape");
    static_assert(cls != CH_RSDF || (c.n == 3 && c.f[0].kind == FDN_R && c.f[1].kind == FDN_S && c.f[2].kind == FDN_DF),
                  "distance chain shape");
    static constexpr int dz = FaceT<F>::off(2, c.f[0].at);
    static constexpr int dy = cls == CH_RSDF ? FaceT<F>::off(1, c.f[1].at) : 0;
    __device__ __forceinline__ static void get(const fd_geo_dev &g, const PointCtx &p, double &d, double &inv)
    {
        if constexpr (cls == CH_H) {
            d = g.h;
            inv = g.inv_h;
        } else if constexpr (cls == CH_RDQ) {
            const double *zr = g.zrow + (long long)(p.z + dz) * FD_Z_N;
            d = zr[FD_Z_RDQ];
            inv = zr[FD_Z_INV_RDQ];
        } else {
            const double *nr = node_row(g, p.z + dz, p.y + dy);
            d = nr[FD_N_RSDF];
            inv = nr[FD_N_INV_RSDF];
        }
    }
};

/* the quadratic's 'a' for a pair of distances taken at the point itself */
template <int CA, int CB>
__device__ __forceinline__ void pair_a(const fd_geo_dev &g, const PointCtx &p, double &a, double &i2a)
{
    static_assert(CA != CB, "distance pair");
    constexpr int lo = CA < CB ? CA : CB, hi = CA < CB ? CB : CA;
    const double *nr = node_row(g, p.z, p.y);
    if constexpr (lo == CH_H && hi == CH_RSDF) { a = nr[FD_N_A_SH]; i2a = nr[FD_N_I2A_SH]; }
    else if constexpr (lo == CH_H && hi == CH_RDQ) { a = nr[FD_N_A_QH]; i2a = nr[FD_N_I2A_QH]; }
    else { a = nr[FD_N_A_SQ]; i2a = nr[FD_N_I2A_SQ]; }
}

template <int F, int K, int J>
__device__ __forceinline__ static constexpr bool dist_at_point()
{
    return Dist<F, K, J>::dz == 0 && Dist<F, K, J>::dy == 0;
}

#define FD_T(p, n) ((p).t[(n).w][(n).dv + 1][(n).du + 1])
#define FD_S(p, n) ((p).s[(n).w][(n).dv + 1][(n).du + 1])

/* roots of a x^2 + b x + c = 0 (rad = b*b - 4ac already formed), with the reference's
 * causality test against floor tmx; tie rule of fdsph3d (x1 preferred only if strictly smaller). */
__device__ __forceinline__ double roots_3d(double b, double rad, double twoa, double i2a, double tmx)
{
    if (!(rad >= 0.)) return 1.e11;
    const double sq = __dsqrt_rn(rad);
    const double x1 = div_rn(-b + sq, twoa, i2a);
    const double x2 = div_rn(-b - sq, twoa, i2a);
    const bool bad1 = x1 < tmx, bad2 = x2 < tmx;
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return (x1 < x2) ? x1 : x2;
}

/* same, with the tie rule of fdsphne / fdsph2d (x2 preferred only if strictly smaller) */
__device__ __forceinline__ double roots_2(double b, double rad, double twoa, double i2a, double tmx)
{
    if (!(rad >= 0.)) return 1.e11;
    const double sq = __dsqrt_rn(rad);
    const double x1 = div_rn(-b + sq, twoa, i2a);
    const double x2 = div_rn(-b - sq, twoa, i2a);
    const bool bad1 = x1 < tmx, bad2 = x2 < tmx;
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return (x2 < x1) ? x2 : x1;
}

/* a trial whose accepted value can be no lower than tmx cannot improve guess */
__device__ __forceinline__ bool cannot_improve(float tmx, const EvalState &st)
{
    return f2d(tmx) >= st.guess && st.guess <= 1.e11;
}

/* ---------------------------------------------------------------------------------------------- */
/* guards                                                                                          */

template <int F, int K>
__device__ __forceinline__ bool guard(const PointCtx &p, EvalState &st)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    if constexpr (tr.big_guess) {
        /* the first-contact test is made once on entry to its block of trials */
        if constexpr (K == 0 || fd_face_trials[F][K - 1].kind != tr.kind) st.gate = st.guess > 1.0e9;
        if (!st.gate) return false;
    }
    if constexpr ((tr.need & FDN_NEED_UM) != 0) if (!(p.u > 0)) return false;
    if constexpr ((tr.need & FDN_NEED_UP) != 0) if (!(p.u < p.nu - 1)) return false;
    if constexpr ((tr.need & FDN_NEED_VM) != 0) if (!(p.v > 0)) return false;
    if constexpr ((tr.need & FDN_NEED_VP) != 0) if (!(p.v < p.nv - 1)) return false;
    if constexpr ((tr.inside & FDN_IN_ULO) != 0) if (!(p.u > p.ulo)) return false;
    if constexpr ((tr.inside & FDN_IN_UHI) != 0) if (!(p.u < p.uhi)) return false;
    if constexpr ((tr.inside & FDN_IN_VLO) != 0) if (!(p.v > p.vlo)) return false;
    if constexpr ((tr.inside & FDN_IN_VHI) != 0) if (!(p.v < p.vhi)) return false;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (c < tr.nchk) {
            const float tv = p.t[0][tr.chk[c].dv + 1][tr.chk[c].du + 1];
            const bool ok = ((tr.chk_nonzero >> c) & 1) ? (tv != 0.0f) : (tv < 1.e9f);
            if (!ok) return false;
        }
    }
    return true;
}

/* ---------------------------------------------------------------------------------------------- */
/* trials                                                                                          */

/* fdsph3d (src/sphfd.c:5906-6013) for corner trial K of face F */
template <int F, int K>
__device__ __forceinline__ void trial_3d(const fd_geo_dev &g, const PointCtx &p, EvalState &st)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    using FT = FaceT<F>;
    constexpr fdn_node P7 = {0, 0, 0};
    /* cell corner offsets (compile time) */
    constexpr int zmin = [] {
        int m = FT::off(2, P7);
        for (int i = 0; i < 7; i++) m = FT::off(2, tr.t[i]) < m ? FT::off(2, tr.t[i]) : m;
        return m;
    }();
    constexpr int ymin = [] {
        int m = FT::off(1, P7);
        for (int i = 0; i < 7; i++) m = FT::off(1, tr.t[i]) < m ? FT::off(1, tr.t[i]) : m;
        return m;
    }();
    float tf[7];
#pragma unroll
    for (int i = 0; i < 7; i++) tf[i] = FD_T(p, tr.t[i]);
    st.t0 = tf[0];
    st.t4 = tf[4];
    st.writers++;
    float tmx = tf[0];
#pragma unroll
    for (int i = 1; i < 7; i++) tmx = fmaxf(tmx, tf[i]);
    if (cannot_improve(tmx, st)) return;
    st.n3d++;
    const double *C = g.cell + ((long long)(p.z + zmin) * (g.ny - 1) + (p.y + ymin)) * FD_C_N;
    constexpr int r7 = FT::off(2, P7) - zmin, q7 = FT::off(1, P7) - ymin;
    double t[7];
#pragma unroll
    for (int i = 0; i < 7; i++) t[i] = f2d(tf[i]);
    /* slo = 0.125 * sum(s[0..7]) in slot order; 16*slo*slo = (2*sum)*slo */
    double sum = f2d(FD_S(p, tr.t[0]));
#pragma unroll
    for (int i = 1; i < 7; i++) sum = sum + f2d(FD_S(p, tr.t[i]));
    sum = sum + f2d(p.s[0][1][1]);
    const double slo = scale2k<-3>(sum);
    const double sl16 = scale2k<1>(sum) * slo;
    const double a = C[FD_C_DIAG(r7, q7)];
    const double i2a = C[FD_C_I2A(r7, q7)];
    /* b (already doubled through the table) */
    double b = 0.0;
#pragma unroll
    for (int i = 0; i < 7; i++) {
        const int ri = FT::off(2, tr.t[i]) - zmin, qi = FT::off(1, tr.t[i]) - ymin;
        const int sx = FT::off(0, tr.t[i]) == FT::off(0, P7);
        const double term = t[i] * C[FD_C_PROW(r7, q7, ri, qi, sx)];
        if (i == 0) b = term; else b = b + term;
    }
    double c = 0.0;
#pragma unroll
    for (int i = 0; i < 7; i++) {
        const int ri = FT::off(2, tr.t[i]) - zmin, qi = FT::off(1, tr.t[i]) - ymin;
        const double term = (t[i] * t[i]) * C[FD_C_DIAG(ri, qi)];
        if (i == 0) c = term; else c = c + term;
    }
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const int ri = FT::off(2, tr.t[i]) - zmin, qi = FT::off(1, tr.t[i]) - ymin;
        double c2 = 0.0;
#pragma unroll
        for (int j = i + 1; j < 7; j++) {
            const int rj = FT::off(2, tr.t[j]) - zmin, qj = FT::off(1, tr.t[j]) - ymin;
            const int sx = FT::off(0, tr.t[i]) == FT::off(0, tr.t[j]);
            const double term = t[j] * C[FD_C_PAIR(ri, qi, rj, qj, sx)];
            if (j == i + 1) c2 = term; else c2 = c2 + term;
        }
        c = c + c2 * t[i];
    }
    c = c - sl16;
    const double rad = b * b - scale2k<2>(a) * c;
    const double x = roots_3d(b, rad, scale2k<1>(a), i2a, f2d(tmx));
    if (x < st.guess) st.guess = x;
}

/* fdsphne (src/sphfd.c:6016-6074) */
template <int F, int K>
__device__ __forceinline__ void trial_ne(const fd_geo_dev &g, const PointCtx &p, EvalState &st)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    float tf[5];
#pragma unroll
    for (int i = 0; i < 5; i++) tf[i] = FD_T(p, tr.t[i]);
    st.t0 = tf[0];
    st.t4 = tf[4];
    st.writers++;
    const float tmx = fmaxf(fmaxf(fmaxf(tf[0], tf[1]), fmaxf(tf[2], tf[3])), tf[4]);
    if (cannot_improve(tmx, st)) return;
    st.nne++;
    double d01, i01, d12, i12, d14, i14, d25, i25, d45, i45;
    Dist<F, K, 0>::get(g, p, d01, i01);
    Dist<F, K, 1>::get(g, p, d12, i12);
    Dist<F, K, 2>::get(g, p, d14, i14);
    Dist<F, K, 3>::get(g, p, d25, i25);
    Dist<F, K, 4>::get(g, p, d45, i45);
    static_assert(dist_at_point<F, K, 3>() && dist_at_point<F, K, 4>(), "new-edge 'a' pair at the point");
    double a, i2a;
    pair_a<Dist<F, K, 3>::cls, Dist<F, K, 4>::cls>(g, p, a, i2a);
    const double t0 = f2d(tf[0]), t1 = f2d(tf[1]), t2 = f2d(tf[2]), t3 = f2d(tf[3]), t4 = f2d(tf[4]);
    const double sum = ((f2d(FD_S(p, tr.t[1])) + f2d(FD_S(p, tr.t[2]))) + f2d(FD_S(p, tr.t[4]))) + f2d(p.s[0][1][1]);
    const double slo = scale2k<-2>(sum);
    const double dt1 = div_rn(t4 - t1, d14, i14) - div_rn(t2, d25, i25);
    const double dt2 = div_rn(t2 - t1, d12, i12) - div_rn(t4, d45, i45);
    const double dt3 = div_rn(t0 - t3, d01, i01);
    const double b = scale2k<1>(div_rn(dt1, d25, i25) + div_rn(dt2, d45, i45));
    const double c = ((dt1 * dt1 + dt2 * dt2) + dt3 * dt3) - sum * slo;
    const double rad = b * b - scale2k<2>(a) * c;
    const double x = roots_2(b, rad, scale2k<1>(a), i2a, f2d(tmx));
    if (x < st.guess) st.guess = x;
}

/* fdsph2d (src/sphfd.c:6077-6143): reads the stale t0, t4 */
template <int F, int K>
__device__ __forceinline__ void trial_2d(const fd_geo_dev &g, const PointCtx &p, EvalState &st)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    const float tf1 = FD_T(p, tr.t[1]), tf2 = FD_T(p, tr.t[2]), tf3 = FD_T(p, tr.t[3]);
    const float tmx = fmaxf(fmaxf(fmaxf(tf1, tf2), fmaxf(tf3, st.t0)), st.t4);
    if (cannot_improve(tmx, st)) return;
    st.n2d++;
    double d01, i01, d02, i02, d13, i13, d23, i23;
    Dist<F, K, 0>::get(g, p, d01, i01);
    Dist<F, K, 1>::get(g, p, d02, i02);
    Dist<F, K, 2>::get(g, p, d13, i13);
    Dist<F, K, 3>::get(g, p, d23, i23);
    static_assert(dist_at_point<F, K, 0>() && dist_at_point<F, K, 1>(), "2-D 'a' pair at the point");
    double a, i2a;
    pair_a<Dist<F, K, 0>::cls, Dist<F, K, 1>::cls>(g, p, a, i2a);
    const double t1 = f2d(tf1), t2 = f2d(tf2), t3 = f2d(tf3);
    const float sp = p.s[0][1][1];
    const double sum = ((f2d(sp) + f2d(FD_S(p, tr.t[1]))) + f2d(FD_S(p, tr.t[2]))) + f2d(FD_S(p, tr.t[3]));
    const double slo = scale2k<-2>(sum);
    const double t1t3t2 = div_rn(t1 - t3, d13, i13) - div_rn(t2, d02, i02);
    const double t2t3t1 = div_rn(t2 - t3, d23, i23) - div_rn(t1, d01, i01);
    const double b = scale2k<1>(div_rn(t1t3t2, d02, i02) + div_rn(t2t3t1, d01, i01));
    const double c = (t1t3t2 * t1t3t2 + t2t3t1 * t2t3t1) - sum * slo;
    const double rad = b * b - scale2k<2>(a) * c;
    const double x = roots_2(b, rad, scale2k<1>(a), i2a, f2d(tmx));
    if constexpr (tr.head) {
        if (x < st.guess) {
            st.fhead = (st.guess - x) / (d01 * f2d(sp));
            st.guess = x;
        }
    } else {
        if (x < st.guess) st.guess = x;
    }
}

/* fdsphnf (src/sphfd.c:6146-6184) */
template <int F, int K>
__device__ __forceinline__ void trial_nf(const fd_geo_dev &g, const PointCtx &p, EvalState &st)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    float tf[5];
#pragma unroll
    for (int i = 0; i < 5; i++) tf[i] = FD_T(p, tr.t[i]);
    st.t0 = tf[0];
    st.t4 = tf[4];
    st.writers++;
    const float tchk = fmaxf(fmaxf(tf[0], tf[1]), fmaxf(tf[3], tf[4]));
    if (cannot_improve(fmaxf(tchk, tf[2]), st)) return;
    st.nnf++;
    double d02, i02, d12, i12, d25, i25;
    Dist<F, K, 0>::get(g, p, d02, i02);
    Dist<F, K, 1>::get(g, p, d12, i12);
    Dist<F, K, 2>::get(g, p, d25, i25);
    const double slo = scale2k<-1>(f2d(p.s[0][1][1]) + f2d(FD_S(p, tr.t[2])));
    const double t4t0 = div_rn(f2d(tf[4]) - f2d(tf[0]), d02, i02);
    const double t1t3 = div_rn(f2d(tf[1]) - f2d(tf[3]), d12, i12);
    double x = slo * slo - scale2k<-2>(t4t0 * t4t0 + t1t3 * t1t3);
    if (!(x >= 0.)) {
        x = 1.e11;
    } else {
        x = f2d(tf[2]) + d25 * __dsqrt_rn(x);
        if (x < f2d(tchk)) x = 1.e11;
    }
    if (x < st.guess) st.guess = x;
}

/* geometric factor of a 1-D product chain */
template <int F>
__device__ __forceinline__ double factor(const fd_geo_dev &g, const PointCtx &p, fdn_factor fa)
{
    using FT = FaceT<F>;
    switch (fa.kind) {
    case FDN_H: return g.h;
    case FDN_DQ: return g.dq;
    case FDN_DF: return g.df;
    case FDN_R: return g.zrow[(long long)(p.z + FT::off(2, fa.at)) * FD_Z_N + FD_Z_R];
    default: return g.ysin[p.y + FT::off(1, fa.at)];
    }
}

/* straight-edge trial: tc(nbr) + .5*(s_point + s_nbr) * f1 * f2 * f3 (e.g. src/sphfd.c:1727-1755) */
template <int F, int K>
__device__ __forceinline__ void trial_1d(const fd_geo_dev &g, const PointCtx &p, EvalState &st)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    const float tn = FD_T(p, tr.t[0]);
    /* the product is positive, so the trial is never below the neighbour's time */
    if (f2d(tn) >= st.guess) return;
    st.n1d++;
    const float sp = p.s[0][1][1];
    const float ssum = sp + FD_S(p, tr.t[0]);
    double x = scale2k<-1>(f2d(ssum));
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (k < tr.d[0].n) x = x * factor<F>(g, p, tr.d[0].f[k]);
    const double tr_ = f2d(tn) + x;
    if constexpr (tr.head) {
        if (tr_ < st.guess) {
            /* denominator chain, left to right, ending in the point's slowness */
            double den = factor<F>(g, p, tr.hd.f[0]);
#pragma unroll
            for (int k = 1; k < 4; k++)
                if (k < tr.hd.n) den = (tr.hd.f[k].kind == FDN_SLOW) ? den * f2d(sp) : den * factor<F>(g, p, tr.hd.f[k]);
            st.fhead = (st.guess - tr_) / den;
            st.guess = tr_;
        }
    } else {
        if (tr_ < st.guess) st.guess = tr_;
    }
}

template <int F, int K>
__device__ __forceinline__ void run_trials(const fd_geo_dev &g, const PointCtx &p, EvalState &st)
{
    if constexpr (K < FDN_NTRIAL) {
        constexpr fdn_trial tr = fd_face_trials[F][K];
        if (guard<F, K>(p, st)) {
            if constexpr (tr.kind == FDN_3D) trial_3d<F, K>(g, p, st);
            else if constexpr (tr.kind == FDN_NE) trial_ne<F, K>(g, p, st);
            else if constexpr (tr.kind == FDN_2D) {
                if (st.writers == 0 && !st.have_inherit) { st.defer = true; return; }
                trial_2d<F, K>(g, p, st);
            }
            else if constexpr (tr.kind == FDN_NF) trial_nf<F, K>(g, p, st);
            else trial_1d<F, K>(g, p, st);
        }
        run_trials<F, K + 1>(g, p, st);
    }
}

}  // namespace fdk

#endif
