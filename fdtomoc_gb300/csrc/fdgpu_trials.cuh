/*
 * fdgpu_trials.cuh — trial descriptors and the generic per-kind stencil evaluators.
 *
 * A round of the face walk evaluates many (point, trial) pairs at once.  To keep every lane of a
 * warp busy the evaluators are generic in the trial: what differs between the 22 trials of a face
 * (which neighbours fill which slots, which table entries hold the coefficients, which distances
 * the stencil takes) is read from a small descriptor, derived at compile time from
 * fd_face_table.h.  The arithmetic is the reference's, operation for operation (see
 * fdgpu_eval.cuh for how each operation is obtained exactly).
 *
 * Neighbourhood indexing: a point's context holds the 3x3 blocks of times and slownesses on the
 * face layer (w=0) and the inner layer (w=1); node (du,dv,w) sits at w*9 + (dv+1)*3 + (du+1), the
 * point itself at 4.
 */
#ifndef FDGPU_TRIALS_CUH
#define FDGPU_TRIALS_CUH

#include "fdgpu_eval.cuh"

namespace fdk {

enum { NB_POINT = 4, NB_N = 18 };
enum { AP_SH = 0, AP_QH = 1, AP_SQ = 2 };
enum { FK_H = 0, FK_DQ = 1, FK_DF = 2, FK_R = 3, FK_S = 4, FK_SLOW = 5 };

/* trial index ranges, identical on every face (checked below) */
enum { TK_3D0 = 0, TK_NE0 = 4, TK_2D0 = 8, TK_NF = 16, TK_1D0 = 17 };

struct TrialDesc {
    unsigned char kind, head;
    unsigned char slot[7];       /* neighbourhood index of t slots (2-D: slots 1..3; 1-D: slot 0) */
    /* fdsph3d */
    unsigned char prow[7], diag[7], pair[21], a_idx, i2a_idx;
    signed char zmin, ymin;
    /* distances of ne / 2-D / nf, in the stencil's argument order */
    unsigned char dcls[5];
    signed char ddz[5], ddy[5];
    unsigned char apair;
    /* 1-D: value chain after 0.5*(s_point + s_nbr), and the head-wave denominator chain */
    unsigned char vn, vk[3];
    signed char vdz[3], vdy[3];
    unsigned char hn, hk[4];
    signed char hdz[4], hdy[4];
};

constexpr int nb_index(fdn_node n) { return n.w * 9 + (n.dv + 1) * 3 + (n.du + 1); }

template <int F>
constexpr int geo_dz(fdn_node n) { return FaceT<F>::off(2, n); }
template <int F>
constexpr int geo_dy(fdn_node n) { return FaceT<F>::off(1, n); }

template <int F>
constexpr int apair_of(fdn_chain a, fdn_chain b)
{
    const int ca = chain_class(a), cb = chain_class(b);
    const int lo = ca < cb ? ca : cb, hi = ca < cb ? cb : ca;
    return (lo == CH_H && hi == CH_RSDF) ? AP_SH : (lo == CH_H && hi == CH_RDQ) ? AP_QH : AP_SQ;
}

template <int F>
constexpr TrialDesc make_desc(int K)
{
    using FT = FaceT<F>;
    const fdn_trial tr = fd_face_trials[F][K];
    TrialDesc d{};
    d.kind = tr.kind;
    d.head = tr.head;
    for (int i = 0; i < 7; i++) d.slot[i] = (unsigned char)nb_index(tr.t[i]);
    if (tr.kind == FDN_3D) {
        const fdn_node P7 = {0, 0, 0};
        int zmin = FT::off(2, P7), ymin = FT::off(1, P7);
        for (int i = 0; i < 7; i++) {
            zmin = FT::off(2, tr.t[i]) < zmin ? FT::off(2, tr.t[i]) : zmin;
            ymin = FT::off(1, tr.t[i]) < ymin ? FT::off(1, tr.t[i]) : ymin;
        }
        d.zmin = (signed char)zmin;
        d.ymin = (signed char)ymin;
        const int r7 = FT::off(2, P7) - zmin, q7 = FT::off(1, P7) - ymin;
        d.a_idx = FD_C_DIAG(r7, q7);
        d.i2a_idx = FD_C_I2A(r7, q7);
        int k = 0;
        for (int i = 0; i < 7; i++) {
            const int ri = FT::off(2, tr.t[i]) - zmin, qi = FT::off(1, tr.t[i]) - ymin;
            d.prow[i] = FD_C_PROW(r7, q7, ri, qi, FT::off(0, tr.t[i]) == FT::off(0, P7) ? 1 : 0);
            d.diag[i] = FD_C_DIAG(ri, qi);
            for (int j = i + 1; j < 7; j++) {
                const int rj = FT::off(2, tr.t[j]) - zmin, qj = FT::off(1, tr.t[j]) - ymin;
                d.pair[k++] = FD_C_PAIR(ri, qi, rj, qj, FT::off(0, tr.t[i]) == FT::off(0, tr.t[j]) ? 1 : 0);
            }
        }
    }
    if (tr.kind == FDN_NE || tr.kind == FDN_2D || tr.kind == FDN_NF) {
        const int nd = tr.kind == FDN_NE ? 5 : tr.kind == FDN_2D ? 4 : 3;
        for (int j = 0; j < nd; j++) {
            const fdn_chain c = tr.d[j];
            const int cls = chain_class(c);
            d.dcls[j] = (unsigned char)cls;
            d.ddz[j] = (signed char)(cls == CH_H ? 0 : FT::off(2, c.f[0].at));
            d.ddy[j] = (signed char)(cls == CH_RSDF ? FT::off(1, c.f[1].at) : 0);
        }
        if (tr.kind == FDN_NE) d.apair = (unsigned char)apair_of<F>(tr.d[3], tr.d[4]);
        if (tr.kind == FDN_2D) d.apair = (unsigned char)apair_of<F>(tr.d[0], tr.d[1]);
    }
    if (tr.kind == FDN_1D) {
        d.vn = tr.d[0].n;
        for (int j = 0; j < tr.d[0].n; j++) {
            d.vk[j] = tr.d[0].f[j].kind;
            d.vdz[j] = (signed char)FT::off(2, tr.d[0].f[j].at);
            d.vdy[j] = (signed char)FT::off(1, tr.d[0].f[j].at);
        }
        d.hn = tr.hd.n;
        for (int j = 0; j < tr.hd.n; j++) {
            d.hk[j] = tr.hd.f[j].kind;
            d.hdz[j] = (signed char)FT::off(2, tr.hd.f[j].at);
            d.hdy[j] = (signed char)FT::off(1, tr.hd.f[j].at);
        }
    }
    return d;
}

template <int F, int... K>
struct DescRow {
    static constexpr TrialDesc row[sizeof...(K)] = {make_desc<F>(K)...};
};

/* the kind layout is the same on all faces */
constexpr bool kinds_uniform()
{
    for (int f = 0; f < FDN_NFACE; f++)
        for (int k = 0; k < FDN_NTRIAL; k++) {
            const int want = k < TK_NE0 ? FDN_3D : k < TK_2D0 ? FDN_NE : k < TK_NF ? FDN_2D : k < TK_1D0 ? FDN_NF : FDN_1D;
            if (fd_face_trials[f][k].kind != want) return false;
        }
    return true;
}
static_assert(kinds_uniform(), "every face runs 4 corner, 4 new-edge, 8 2-D, 1 new-face, 5 1-D trials in that order");

/* ---------------------------------------------------------------------------------------------- */
/* geometry accessors at run time                                                                  */

__device__ __forceinline__ void dist_rt(const fd_geo_dev &g, int cls, int z, int y, double &d, double &inv)
{
    if (cls == CH_H) {
        d = g.h;
        inv = g.inv_h;
    } else if (cls == CH_RDQ) {
        if (!FD_OK(z, g.nz, 3)) z = 0;
        const double *zr = g.zrow + (long long)z * FD_Z_N;
        d = zr[FD_Z_RDQ];
        inv = zr[FD_Z_INV_RDQ];
    } else {
        const double *nr = node_row(g, z, y);
        d = nr[FD_N_RSDF];
        inv = nr[FD_N_INV_RSDF];
    }
}

__device__ __forceinline__ void apair_rt(const fd_geo_dev &g, int ap, int z, int y, double &a, double &i2a)
{
    const double *nr = node_row(g, z, y);
    const int o = ap == AP_SH ? FD_N_A_SH : ap == AP_QH ? FD_N_A_QH : FD_N_A_SQ;
    a = nr[o];
    i2a = nr[o + 1];
}

__device__ __forceinline__ double factor_rt(const fd_geo_dev &g, int kind, int z, int y, float slow)
{
    switch (kind) {
    case FK_H: return g.h;
    case FK_DQ: return g.dq;
    case FK_DF: return g.df;
    case FK_R: return g.zrow[(long long)(FD_OK(z, g.nz, 4) ? z : 0) * FD_Z_N + FD_Z_R];
    case FK_S: return g.ysin[FD_OK(y, g.ny, 5) ? y : 0];
    default: return f2d(slow);
    }
}

/* ---------------------------------------------------------------------------------------------- */
/* generic evaluators: t, s = the point's 18-node context                                         */

/* fdsph3d (src/sphfd.c:5906-6013): the accepted value or 1e11 */
__device__ __forceinline__ double eval_3d(const TrialDesc &d, const float *t18, const float *s18,
                                          const fd_geo_dev &g, int z, int y)
{
    float tf[7];
#pragma unroll
    for (int i = 0; i < 7; i++) tf[i] = t18[d.slot[i]];
    float tmx = tf[0];
#pragma unroll
    for (int i = 1; i < 7; i++) tmx = fmaxf(tmx, tf[i]);
    double t[7];
#pragma unroll
    for (int i = 0; i < 7; i++) t[i] = f2d(tf[i]);
    double sum = f2d(s18[d.slot[0]]);
#pragma unroll
    for (int i = 1; i < 7; i++) sum = sum + f2d(s18[d.slot[i]]);
    sum = sum + f2d(s18[NB_POINT]);
    const double slo = scale2k<-3>(sum);
    const double sl16 = scale2k<1>(sum) * slo;
    int zc = z + d.zmin, yc = y + d.ymin;
    if (!FD_OK(zc, g.nz - 1, 6) || !FD_OK(yc, g.ny - 1, 7)) { zc = 0; yc = 0; }
    const double *C = g.cell + ((long long)zc * (g.ny - 1) + yc) * FD_C_N;
    const double a = C[d.a_idx], i2a = C[d.i2a_idx];
    double b = t[0] * C[d.prow[0]];
#pragma unroll
    for (int i = 1; i < 7; i++) b = b + t[i] * C[d.prow[i]];
    double c = (t[0] * t[0]) * C[d.diag[0]];
#pragma unroll
    for (int i = 1; i < 7; i++) c = c + (t[i] * t[i]) * C[d.diag[i]];
    int k = 0;
#pragma unroll
    for (int i = 0; i < 6; i++) {
        double c2 = t[i + 1] * C[d.pair[k++]];
#pragma unroll
        for (int j = i + 2; j < 7; j++) c2 = c2 + t[j] * C[d.pair[k++]];
        c = c + c2 * t[i];
    }
    c = c - sl16;
    const double rad = b * b - scale2k<2>(a) * c;
    return roots_3d(b, rad, scale2k<1>(a), i2a, f2d(tmx));
}

/* fdsphne (src/sphfd.c:6016-6074) */
__device__ __forceinline__ double eval_ne(const TrialDesc &d, const float *t18, const float *s18,
                                          const fd_geo_dev &g, int z, int y)
{
    float tf[5];
#pragma unroll
    for (int i = 0; i < 5; i++) tf[i] = t18[d.slot[i]];
    const float tmx = fmaxf(fmaxf(fmaxf(tf[0], tf[1]), fmaxf(tf[2], tf[3])), tf[4]);
    double dd[5], iv[5];
#pragma unroll
    for (int j = 0; j < 5; j++) dist_rt(g, d.dcls[j], z + d.ddz[j], y + d.ddy[j], dd[j], iv[j]);
    double a, i2a;
    apair_rt(g, d.apair, z, y, a, i2a);
    const double t0 = f2d(tf[0]), t1 = f2d(tf[1]), t2 = f2d(tf[2]), t3 = f2d(tf[3]), t4 = f2d(tf[4]);
    const double sum = ((f2d(s18[d.slot[1]]) + f2d(s18[d.slot[2]])) + f2d(s18[d.slot[4]])) + f2d(s18[NB_POINT]);
    const double slo = scale2k<-2>(sum);
    /* d[] = d01 d12 d14 d25 d45 */
    const double dt1 = div_rn(t4 - t1, dd[2], iv[2]) - div_rn(t2, dd[3], iv[3]);
    const double dt2 = div_rn(t2 - t1, dd[1], iv[1]) - div_rn(t4, dd[4], iv[4]);
    const double dt3 = div_rn(t0 - t3, dd[0], iv[0]);
    const double b = scale2k<1>(div_rn(dt1, dd[3], iv[3]) + div_rn(dt2, dd[4], iv[4]));
    const double c = ((dt1 * dt1 + dt2 * dt2) + dt3 * dt3) - sum * slo;
    const double rad = b * b - scale2k<2>(a) * c;
    return roots_2(b, rad, scale2k<1>(a), i2a, f2d(tmx));
}

/* fdsph2d (src/sphfd.c:6077-6143) without its stale-slot test: returns both roots (x1 NaN when
 * the discriminant is negative); the caller applies the causality floor including t0,t4. */
__device__ __forceinline__ void eval_2d(const TrialDesc &d, const float *t18, const float *s18,
                                        const fd_geo_dev &g, int z, int y, double &x1, double &x2)
{
    const float tf1 = t18[d.slot[1]], tf2 = t18[d.slot[2]], tf3 = t18[d.slot[3]];
    double dd[4], iv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) dist_rt(g, d.dcls[j], z + d.ddz[j], y + d.ddy[j], dd[j], iv[j]);
    double a, i2a;
    apair_rt(g, d.apair, z, y, a, i2a);
    const double t1 = f2d(tf1), t2 = f2d(tf2), t3 = f2d(tf3);
    const double sum = ((f2d(s18[NB_POINT]) + f2d(s18[d.slot[1]])) + f2d(s18[d.slot[2]])) + f2d(s18[d.slot[3]]);
    const double slo = scale2k<-2>(sum);
    /* d[] = d01 d02 d13 d23 */
    const double t1t3t2 = div_rn(t1 - t3, dd[2], iv[2]) - div_rn(t2, dd[1], iv[1]);
    const double t2t3t1 = div_rn(t2 - t3, dd[3], iv[3]) - div_rn(t1, dd[0], iv[0]);
    const double b = scale2k<1>(div_rn(t1t3t2, dd[1], iv[1]) + div_rn(t2t3t1, dd[0], iv[0]));
    const double c = (t1t3t2 * t1t3t2 + t2t3t1 * t2t3t1) - sum * slo;
    const double rad = b * b - scale2k<2>(a) * c;
    if (not_ge0(rad)) {
        x1 = __longlong_as_double(0x7ff8000000000000ll);
        x2 = x1;
        return;
    }
    const double sq = __dsqrt_rn(rad);
    const double twoa = scale2k<1>(a);
    x1 = div_rn(-b + sq, twoa, i2a);
    x2 = div_rn(-b - sq, twoa, i2a);
}

/* fdsphnf (src/sphfd.c:6146-6184) */
__device__ __forceinline__ double eval_nf(const TrialDesc &d, const float *t18, const float *s18,
                                          const fd_geo_dev &g, int z, int y)
{
    float tf[5];
#pragma unroll
    for (int i = 0; i < 5; i++) tf[i] = t18[d.slot[i]];
    const float tchk = fmaxf(fmaxf(tf[0], tf[1]), fmaxf(tf[3], tf[4]));
    double dd[3], iv[3];
#pragma unroll
    for (int j = 0; j < 3; j++) dist_rt(g, d.dcls[j], z + d.ddz[j], y + d.ddy[j], dd[j], iv[j]);
    const double slo = scale2k<-1>(f2d(s18[NB_POINT]) + f2d(s18[d.slot[2]]));
    const double t4t0 = div_rn(f2d(tf[4]) - f2d(tf[0]), dd[0], iv[0]);
    const double t1t3 = div_rn(f2d(tf[1]) - f2d(tf[3]), dd[1], iv[1]);
    double x = slo * slo - scale2k<-2>(t4t0 * t4t0 + t1t3 * t1t3);
    if (not_ge0(x)) return 1.e11;
    x = f2d(tf[2]) + dd[2] * __dsqrt_rn(x);
    return flt(x, f2d(tchk)) ? 1.e11 : x;
}

/* straight edge: t_nbr + 0.5*(s_point + s_nbr) * f1 * f2 * f3 (e.g. src/sphfd.c:1727-1755) */
__device__ __forceinline__ double eval_1d(const TrialDesc &d, const float *t18, const float *s18,
                                          const fd_geo_dev &g, int z, int y)
{
    const float ssum = s18[NB_POINT] + s18[d.slot[0]];
    double x = scale2k<-1>(f2d(ssum));
    for (int j = 0; j < d.vn; j++) x = x * factor_rt(g, d.vk[j], z + d.vdz[j], y + d.vdy[j], 0.f);
    return f2d(t18[d.slot[0]]) + x;
}

/* head-wave denominator of a head trial: d01*s_point (2-D) or the 1-D chain ending in s_point */
__device__ __forceinline__ double head_den(const TrialDesc &d, const float *s18, const fd_geo_dev &g, int z, int y)
{
    const float sp = s18[NB_POINT];
    if (d.kind == FDN_2D) {
        double d01, i01;
        dist_rt(g, d.dcls[0], z + d.ddz[0], y + d.ddy[0], d01, i01);
        return d01 * f2d(sp);
    }
    double den = factor_rt(g, d.hk[0], z + d.hdz[0], y + d.hdy[0], sp);
    for (int j = 1; j < d.hn; j++) den = den * factor_rt(g, d.hk[j], z + d.hdz[j], y + d.hdy[j], sp);
    return den;
}

/* a < b, exactly as the double comparison, on the integer pipe when both are non-negative */
__device__ __forceinline__ bool lt(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    if ((ia | ib) >= 0) return ia < ib;
    return a < b;
}

}  // namespace fdk

#endif
