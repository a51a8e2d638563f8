/*
 * fdgpu_kernels.cu — GB300 kernels of the sphfd travel-time solver.
 *
 *   fd_geo_build    builds the geometry tables of one grid geometry (shared by its stations);
 *   fd_solve        one CTA per station: source box, then the expanding-box sweeps of
 *                   src/sphfd.c:1008-5678 with each face walked in dependency order.
 *
 * Face walk.  The reference updates a face's points one at a time in ascending order of the time
 * of their inner-layer neighbour (ties in fill order, src/sphfd.c:1024-1033 and glibc's stable
 * qsort); a point reads its eight in-face neighbours, seeing the new value of those already
 * updated and the old value of the others.  So the face is a DAG: an edge runs from each point to
 * every in-face neighbour with a larger key (time bits, fill index).  Walking it in Kahn rounds —
 * every point whose earlier neighbours are all done is evaluated in parallel, then releases its
 * later neighbours — reproduces the sequential order exactly.  No sort is needed.
 *
 * The one sequential coupling that is not a neighbour relation is the stale (t0,t4) pair of
 * fdsph2d (src/sphfd.c:6116-6121): a point whose first 2-D trial comes before any 3-D / new-edge
 * call of its own reads the pair left by the previous point in sort order.  Such a point is put
 * aside; when no other point is ready, the one with the smallest key has every smaller-key point
 * done, and its pair is the record of the largest-key earlier point that made a writer call (or
 * the face's entry pair).  This is rare (hundreds of points per million).
 *
 * There are no spin-waits: CTAs synchronise only with __syncthreads, and every loop is bounded.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fdgpu_eval.cuh"
#include "fdgpu_trials.cuh"
#include "fdgpu_layout.h"

#define FD_BLOCK 512

/* optional per-phase cycle counters (thread 0, between barriers) for profiling builds */
#ifdef FDGPU_PHASE_TIMERS
#define FD_TIC(v) long long v = clock64()
#define FD_TOC(k, v) do { if (threadIdx.x == 0) sh.cyc[k] += clock64() - (v); } while (0)
#else
#define FD_TIC(v) do { } while (0)
#define FD_TOC(k, v) do { } while (0)
#endif
#define FD_HEADTEST 1.e-3

namespace fdk {

/* ---------------------------------------------------------------------------------------------- */
/* geometry tables                                                                                 */

__global__ void fd_geo_build(int nx, int ny, int nz, double h, double dq, double df, double z0r,
                             const double *ysin, double *zrow, double *node, double *cell)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const double hsq = h * h, dqsq = dq * dq, dfsq = df * df;
    const double is_h = 1.0 / (h * h);
    for (long long z = tid; z < nz; z += stride) {
        const double r = z0r - h * (double)z;  /* rc(z), src/sphfd.c:154 */
        zrow[z * FD_Z_N + FD_Z_R] = r;
        zrow[z * FD_Z_N + FD_Z_RDQ] = r * dq;
        zrow[z * FD_Z_N + FD_Z_INV_RDQ] = 1.0 / (r * dq);
    }
    for (long long k = tid; k < (long long)nz * ny; k += stride) {
        const int z = (int)(k / ny), y = (int)(k % ny);
        const double r = z0r - h * (double)z, s = ysin[y];
        const double rsdf = (r * s) * df, rdq = r * dq;
        double *o = node + k * FD_N_N;
        o[FD_N_RSDF] = rsdf;
        o[FD_N_INV_RSDF] = 1.0 / rsdf;
        o[FD_N_RDFS] = (r * df) * s;
        const double is_s = 1.0 / (rsdf * rsdf), is_q = 1.0 / (rdq * rdq);
        const double a_sh = is_s + is_h, a_qh = is_q + is_h, a_sq = is_s + is_q;
        o[FD_N_A_SH] = a_sh;
        o[FD_N_I2A_SH] = 1.0 / (2.0 * a_sh);
        o[FD_N_A_QH] = a_qh;
        o[FD_N_I2A_QH] = 1.0 / (2.0 * a_qh);
        o[FD_N_A_SQ] = a_sq;
        o[FD_N_I2A_SQ] = 1.0 / (2.0 * a_sq);
    }
    /* fdsph3d coefficients (src/sphfd.c:5937-5972) for every cell */
    for (long long k = tid; k < (long long)(nz - 1) * (ny - 1); k += stride) {
        const int zc = (int)(k / (ny - 1)), yc = (int)(k % (ny - 1));
        const double rr[2] = {z0r - h * (double)zc, z0r - h * (double)(zc + 1)};
        const double sq[2] = {ysin[yc], ysin[yc + 1]};
        double *o = cell + k * FD_C_N;
        for (int ri = 0; ri < 2; ri++)
            for (int qi = 0; qi < 2; qi++) {
                const double dfs = df * sq[qi];
                const double a = 1.0 / hsq + (1.0 / dqsq + 1. / (dfs * dfs)) / (rr[ri] * rr[ri]);
                o[FD_C_DIAG(ri, qi)] = a;
                o[FD_C_I2A(ri, qi)] = 1.0 / (2.0 * a);
            }
        for (int r7 = 0; r7 < 2; r7++)
            for (int q7 = 0; q7 < 2; q7++)
                for (int ri = 0; ri < 2; ri++)
                    for (int qi = 0; qi < 2; qi++)
                        for (int sx = 0; sx < 2; sx++) {
                            const double gg = (r7 == ri) ? 1.0 : -1.0, nn = (q7 == qi) ? 1.0 : -1.0, mm = sx ? 1.0 : -1.0;
                            const double df2s7 = df * (df * sq[q7]);
                            const double kk = gg / hsq + (nn / dqsq + mm / (df2s7 * sq[qi])) / (rr[r7] * rr[ri]);
                            o[FD_C_PROW(r7, q7, ri, qi, sx)] = 2.0 * kk;
                        }
        for (int ri = 0; ri < 2; ri++)
            for (int qi = 0; qi < 2; qi++)
                for (int rj = 0; rj < 2; rj++)
                    for (int qj = 0; qj < 2; qj++)
                        for (int sx = 0; sx < 2; sx++) {
                            const double gg = (ri == rj) ? 1.0 : -1.0, nn = (qi == qj) ? 1.0 : -1.0, mm = sx ? 1.0 : -1.0;
                            const double df2si = dfsq * sq[qi];
                            const double kk = gg / hsq + (nn / dqsq + mm / (df2si * sq[qj])) / (rr[ri] * rr[rj]);
                            o[FD_C_PAIR(ri, qi, rj, qj, sx)] = 2.0 * kk;
                        }
    }
}

/* ---------------------------------------------------------------------------------------------- */
/* per-CTA state                                                                                   */

struct Shared {
    int wall[6], dflag[6];
    int radius, rad0, reverse, headpref;
    int headw[8];
    float carry_t0, carry_t4;
    int cnt[2];
    int ndef;
    unsigned long long exitkey;
    /* current face */
    int face, layer, ulo, uhi, vlo, vhi, nuf, n, n_pad;
    long long su, sv, sn, ssu, ssv, ssn;
    int nu, nv;
    int status;
    unsigned long long red[FD_BLOCK / 32];
    unsigned long long bcast;
    /* statistics */
    long long faces, node_updates, rounds, deferred;
    unsigned long long st[5];
    int sweeps;
    int restart_wall[8];
    long long cyc[6];
    /* plane-pipelined sweep: number of planes, layer of plane 0, queue tail, done flag */
    int pipelined, np, player0, qtail;
    long long psweeps;
};

/* face frame for a face number known only at run time */
__device__ __forceinline__ fdn_frame frame_of(int f)
{
    switch (f) {
    case 0: return fd_face_frame[0];
    case 1: return fd_face_frame[1];
    case 2: return fd_face_frame[2];
    case 3: return fd_face_frame[3];
    case 4: return fd_face_frame[4];
    default: return fd_face_frame[5];
    }
}

/* order-preserving 32-bit image of a float time (ties of -0 and +0 kept equal) */
__device__ __forceinline__ unsigned okey32(float f)
{
    unsigned b = __float_as_uint(f);
    if (b == 0x80000000u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ unsigned long long block_min_u64(unsigned long long x, Shared &sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_down_sync(0xffffffffu, x, o);
        x = y < x ? y : x;
    }
    if ((threadIdx.x & 31) == 0) sh.red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = sh.red[0];
        for (int w = 1; w < FD_BLOCK / 32; w++) m = sh.red[w] < m ? sh.red[w] : m;
        sh.bcast = m;
    }
    __syncthreads();
    return sh.bcast;
}

__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long x, Shared &sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_down_sync(0xffffffffu, x, o);
        x = y > x ? y : x;
    }
    if ((threadIdx.x & 31) == 0) sh.red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = sh.red[0];
        for (int w = 1; w < FD_BLOCK / 32; w++) m = sh.red[w] > m ? sh.red[w] : m;
        sh.bcast = m;
    }
    __syncthreads();
    return sh.bcast;
}

struct Counters {
    unsigned long long n[5];
};

/* ---------------------------------------------------------------------------------------------- */
/* trial-major rounds                                                                              */

#define FD_CHUNK 128   /* points per evaluation chunk */
#define FD_TPP 4       /* threads per point in phase A */

#define FD_DESC_ROW(F)                                                                              \
    make_desc<F>(0), make_desc<F>(1), make_desc<F>(2), make_desc<F>(3), make_desc<F>(4), make_desc<F>(5), \
    make_desc<F>(6), make_desc<F>(7), make_desc<F>(8), make_desc<F>(9), make_desc<F>(10), make_desc<F>(11), \
    make_desc<F>(12), make_desc<F>(13), make_desc<F>(14), make_desc<F>(15), make_desc<F>(16), make_desc<F>(17), \
    make_desc<F>(18), make_desc<F>(19), make_desc<F>(20), make_desc<F>(21)
__constant__ TrialDesc c_desc[FDN_NFACE * FDN_NTRIAL] = {FD_DESC_ROW(0), FD_DESC_ROW(1), FD_DESC_ROW(2),
                                                         FD_DESC_ROW(3), FD_DESC_ROW(4), FD_DESC_ROW(5)};

/* item list regions by kind: 3-D, new-edge, 2-D, new-face, 1-D */
__device__ __forceinline__ int item_off(int kind)
{
    return (kind == 0 ? 0 : kind == 1 ? 4 : kind == 2 ? 8 : kind == 3 ? 16 : 17) * FD_CHUNK;
}

__device__ __forceinline__ int kind_of(int K)
{
    return K < TK_NE0 ? 0 : K < TK_2D0 ? 1 : K < TK_NF ? 2 : K < TK_1D0 ? 3 : 4;
}

struct Smem {
    TrialDesc desc[FDN_NTRIAL];
    float t[FD_CHUNK][NB_N];
    float s[FD_CHUNK][NB_N];
    int idx[FD_CHUNK];               /* fill index of the chunk's point */
    int lay[FD_CHUNK];               /* its face layer */
    int pl[FD_CHUNK];                /* its plane in a pipelined sweep (-1 otherwise) */
    int z[FD_CHUNK], y[FD_CHUNK];
    unsigned guardm[FD_CHUNK];       /* trials whose guards pass (first-contact gates excluded) */
    unsigned evalm[FD_CHUNK];        /* trials whose value was computed in the parallel phases */
    double res[FD_CHUNK][FDN_NTRIAL];
    double x2[FD_CHUNK][8];
    unsigned short items[22 * FD_CHUNK];
    int cnt[5];
};

/* dependency state of the current face: one in-degree byte per point (0xFF once done) and one
 * byte marking which of its 8 neighbours come earlier in sort order; in shared memory after Smem
 * when the face fits, else in the station's global scratch */
__device__ __forceinline__ unsigned char *dag_indeg(const fd_station_dev &sd, Smem &sm, bool in_smem)
{
    return in_smem ? reinterpret_cast<unsigned char *>(&sm + 1) : sd.scr.dag;
}

__device__ __forceinline__ void nb_off(int k, int &du, int &dv)
{
    /* k = 0..7 over the 3x3 block without its centre, row by row */
    const int c = k < 4 ? k : k + 1;
    du = c % 3 - 1;
    dv = c / 3 - 1;
}

/* bits of the neighbours of fill index i that lie inside the face rectangle */
__device__ __forceinline__ unsigned inrect_mask(int iu, int iv, int nuf, int nvf)
{
    unsigned m = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int du, dv;
        nb_off(k, du, dv);
        const int ju = iu + du, jv = iv + dv;
        if (ju >= 0 && ju < nuf && jv >= 0 && jv < nvf) m |= 1u << k;
    }
    return m;
}

/* guards without the first-contact gates; t18 = the point's 18-node context */
template <int F, int K>
__device__ __forceinline__ bool guard_static(const float *t18, int u, int v, int nu, int nv, int ulo, int uhi,
                                             int vlo, int vhi)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    if constexpr ((tr.need & FDN_NEED_UM) != 0) if (!(u > 0)) return false;
    if constexpr ((tr.need & FDN_NEED_UP) != 0) if (!(u < nu - 1)) return false;
    if constexpr ((tr.need & FDN_NEED_VM) != 0) if (!(v > 0)) return false;
    if constexpr ((tr.need & FDN_NEED_VP) != 0) if (!(v < nv - 1)) return false;
    if constexpr ((tr.inside & FDN_IN_ULO) != 0) if (!(u > ulo)) return false;
    if constexpr ((tr.inside & FDN_IN_UHI) != 0) if (!(u < uhi)) return false;
    if constexpr ((tr.inside & FDN_IN_VLO) != 0) if (!(v > vlo)) return false;
    if constexpr ((tr.inside & FDN_IN_VHI) != 0) if (!(v < vhi)) return false;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (c < tr.nchk) {
            const float tv = t18[nb_index(tr.chk[c])];
            const bool ok = ((tr.chk_nonzero >> c) & 1) ? (tv != 0.0f) : (tv < 1.e9f);
            if (!ok) return false;
        }
    }
    return true;
}

/* causality floor of trial K: the largest time among the slots its accepted value cannot be below
 * (2-D: its three own slots; the stale pair is added in the scan) */
template <int F, int K>
__device__ __forceinline__ float floor_of(const float *t18)
{
    constexpr fdn_trial tr = fd_face_trials[F][K];
    constexpr int n = tr.kind == FDN_3D ? 7 : (tr.kind == FDN_NE || tr.kind == FDN_NF) ? 5 : tr.kind == FDN_2D ? 4 : 1;
    constexpr int i0 = tr.kind == FDN_2D ? 1 : 0;
    float m = t18[nb_index(tr.t[i0])];
#pragma unroll
    for (int i = i0 + 1; i < n; i++) m = fmaxf(m, t18[nb_index(tr.t[i])]);
    return m;
}

/* a trial with floor fl cannot lower a running minimum that is at most g (any earlier value of
 * the running minimum is such a bound): its accepted value is >= fl, and its rejection value
 * 1e11 is not below g */
__device__ __forceinline__ bool prunable(float fl, double g) { return f2d(fl) >= g && g <= 1.e11; }

struct Rect {
    int u, v, nu, nv, ulo, uhi, vlo, vhi;
};

/* phase A2: thread q of a point handles trials K = q, q+4, ...: guards, pruning, items.  Corner
 * and edge trials are queued now; new-edge trials only when no corner trial can run (the
 * first-contact gate is then decided by the initial value); 2-D trials after the corners. */
template <int F, int K>
__device__ __forceinline__ void a2_trials(Smem &sm, int slot, const Rect &r, double g0, bool any3d, unsigned &gm,
                                          unsigned &em)
{
    if constexpr (K < FDN_NTRIAL) {
        constexpr fdn_trial tr = fd_face_trials[F][K];
        const float *t18 = sm.t[slot];
        if (guard_static<F, K>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)) {
            gm |= 1u << K;
            if constexpr (tr.kind == FDN_3D) {
                if (!prunable(floor_of<F, K>(t18), g0)) em |= 1u << K;
            } else if constexpr (tr.kind == FDN_1D) {
                if (!(f2d(floor_of<F, K>(t18)) >= g0)) em |= 1u << K;
            } else if constexpr (tr.kind == FDN_NE) {
                if (!any3d && g0 > 1.0e9 && !prunable(floor_of<F, K>(t18), g0)) em |= 1u << K;
            }
        }
        a2_trials<F, K + FD_TPP>(sm, slot, r, g0, any3d, gm, em);
    }
}

template <int F>
__device__ __forceinline__ bool any_corner(const float *t18, const Rect &r)
{
    return guard_static<F, 0>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)
           || guard_static<F, 1>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)
           || guard_static<F, 2>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)
           || guard_static<F, 3>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi);
}

__device__ __forceinline__ Rect rect_of(const Shared &sh, int i)
{
    Rect r;
    r.u = sh.ulo + i % sh.nuf;
    r.v = sh.vlo + i / sh.nuf;
    r.nu = sh.nu; r.nv = sh.nv;
    r.ulo = sh.ulo; r.uhi = sh.uhi; r.vlo = sh.vlo; r.vhi = sh.vhi;
    return r;
}

template <int F>
__device__ void phase_a2(Smem &sm, const Shared &sh, int slot, int q)
{
    const int i = sm.idx[slot];
    const Rect r = rect_of(sh, i);
    const float *t18 = sm.t[slot];
    const double g0 = f2d(t18[NB_POINT]);
    const bool any3d = any_corner<F>(t18, r);
    unsigned gm = 0, em = 0;
    switch (q) {
    case 0: a2_trials<F, 0>(sm, slot, r, g0, any3d, gm, em); break;
    case 1: a2_trials<F, 1>(sm, slot, r, g0, any3d, gm, em); break;
    case 2: a2_trials<F, 2>(sm, slot, r, g0, any3d, gm, em); break;
    default: a2_trials<F, 3>(sm, slot, r, g0, any3d, gm, em); break;
    }
    if (gm) atomicOr(&sm.guardm[slot], gm);
    if (em) atomicOr(&sm.evalm[slot], em);
    unsigned m = em;
    while (m) {
        const int K = __ffs(m) - 1;
        m &= m - 1;
        const int kind = kind_of(K);
        sm.items[item_off(kind) + atomicAdd(&sm.cnt[kind], 1)] = (unsigned short)((slot << 5) | K);
    }
}

/* phase G: replay the corner and new-edge trials (all writers of the stencil state come before
 * the 2-D block) to get the running minimum entering the 2-D block — an upper bound for every
 * 2-D trial's turn — and the stale (t0,t4) those trials test against; queue the 2-D trials that
 * can still lower the minimum.  Thread q takes 2-D trials 8+q and 12+q. */
__device__ void phase_g(Smem &sm, int slot, int q, float it0, float it4)
{
    const float *t18 = sm.t[slot];
    const unsigned gm = sm.guardm[slot], em = sm.evalm[slot];
    double g1 = f2d(t18[NB_POINT]);
    float s0 = it0, s4 = it4;
    for (int K = 0; K < TK_NE0; K++) {
        if (!((gm >> K) & 1u)) continue;
        s0 = t18[sm.desc[K].slot[0]];
        s4 = t18[sm.desc[K].slot[4]];
        if ((em >> K) & 1u) {
            const double v = sm.res[slot][K];
            if (lt(v, g1)) g1 = v;
        }
    }
    const bool gate = lt(1.0e9, g1);
    for (int K = TK_NE0; K < TK_2D0; K++) {
        if (!gate || !((gm >> K) & 1u)) continue;
        s0 = t18[sm.desc[K].slot[0]];
        s4 = t18[sm.desc[K].slot[4]];
        if ((em >> K) & 1u) {
            const double v = sm.res[slot][K];
            if (lt(v, g1)) g1 = v;
        }
    }
    unsigned add = 0;
    for (int K = TK_2D0 + q; K < TK_NF; K += FD_TPP) {
        if (!((gm >> K) & 1u)) continue;
        const TrialDesc &d = sm.desc[K];
        const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], s0)), s4);
        if (prunable(fl, g1)) continue;
        add |= 1u << K;
        sm.items[item_off(2) + atomicAdd(&sm.cnt[2], 1)] = (unsigned short)((slot << 5) | K);
    }
    if (add) atomicOr(&sm.evalm[slot], add);
}

/* evaluate queued items of kinds [k0, k1] with all threads */
__device__ void run_items(const fd_station_dev &sd, Smem &sm, int k0, int k1, Counters &cn)
{
    int start[6];
    start[0] = 0;
    for (int k = 0; k < 5; k++) start[k + 1] = start[k] + ((k >= k0 && k <= k1) ? sm.cnt[k] : 0);
    const int total = start[5];
    for (int j = threadIdx.x; j < total; j += blockDim.x) {
        int kind = 0;
        while (j >= start[kind + 1]) kind++;
        const unsigned it = sm.items[item_off(kind) + (j - start[kind])];
        const int slot = (int)(it >> 5), K = (int)(it & 31);
        const TrialDesc &d = sm.desc[K];
        const int z = sm.z[slot], y = sm.y[slot];
        const float *t18 = sm.t[slot], *s18 = sm.s[slot];
        switch (kind) {
        case 0: sm.res[slot][K] = eval_3d(d, t18, s18, sd.g, z, y); break;
        case 1: sm.res[slot][K] = eval_ne(d, t18, s18, sd.g, z, y); break;
        case 2: {
            double x1, x2;
            eval_2d(d, t18, s18, sd.g, z, y, x1, x2);
            sm.res[slot][K] = x1;
            sm.x2[slot][K - TK_2D0] = x2;
            break;
        }
        case 3: sm.res[slot][K] = eval_nf(d, t18, s18, sd.g, z, y); break;
        default: sm.res[slot][K] = eval_1d(d, t18, s18, sd.g, z, y); break;
        }
        cn.n[kind]++;
    }
}

/* ---------------------------------------------------------------------------------------------- */
/* plane-pipelined sweeps                                                                          */
/*                                                                                                 */
/* After a restart the box is one whole model wall and a sweep is a run of full planes, each one's */
/* inner layer being the previous plane (src/sphfd.c:5623-5674).  A point of plane p+1 needs only  */
/* the 3x3 block below it in plane p and its earlier neighbours in its own plane; so the planes    */
/* are walked as one dependency graph instead of one after the other.  Every node has one counter  */
/* word: inner-layer nodes pending in bits 0-7, in-plane neighbours pending in bits 8-15.  When a   */
/* node's inner block is complete, the keys of its in-plane neighbours (their inner-layer times)   */
/* are final, so it learns which neighbours come later and drops them from its count; earlier      */
/* neighbours drop themselves when they finish.  The word reaching zero queues the node.  The run */
/* is taken only when no point can need an earlier point's stencil state (see fd_solve).          */

__device__ __forceinline__ unsigned long long node_key(float tin, int i)
{
    return ((unsigned long long)okey32(tin) << 32) | (unsigned)i;
}

/* earlier-neighbour byte of fill index i, keys from the inner-layer field at `inner_layer` */
__device__ unsigned earlier_mask(const fd_station_dev &sd, const Shared &sh, int i, int inner_layer)
{
    const fdn_frame fr = frame_of(sh.face);
    const int nvf = sh.n / sh.nuf, iu = i % sh.nuf, iv = i / sh.nuf;
    auto tin = [&](int ju, int jv) {
        int xyz[3];
        xyz[fr.axis_u] = sh.ulo + ju;
        xyz[fr.axis_v] = sh.vlo + jv;
        xyz[fr.axis_n] = inner_layer;
        return sd.T[((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0]];
    };
    const unsigned long long ki = node_key(tin(iu, iv), i);
    unsigned em = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int du, dv;
        nb_off(k, du, dv);
        const int ju = iu + du, jv = iv + dv;
        if (ju < 0 || ju >= sh.nuf || jv < 0 || jv >= nvf) continue;
        if (node_key(tin(ju, jv), jv * sh.nuf + ju) < ki) em |= 1u << k;
    }
    return em;
}

/* node (plane pp, fill index i) is final: record (last plane), release its later in-plane
 * neighbours and the plane pp+1 nodes whose inner block contains it */
__device__ void pipelined_release(const fd_station_dev &sd, Shared &sh, int slot, int i, int pp, bool writer,
                                  float st0, float st4, const float *t18)
{
    const int nplane = sh.n, nvf = sh.n / sh.nuf, iu = i % sh.nuf, iv = i / sh.nuf;
    const fdn_frame fr = frame_of(sh.face);
    if (pp == sh.np - 1) {
        if (writer) {
            sd.scr.rec[i] = make_float2(st0, st4);
            atomicMax(&sh.exitkey, node_key(t18[13], i));
        } else {
            sd.scr.rec[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        }
    }
    const long long base = (long long)pp * nplane;
    unsigned later = inrect_mask(iu, iv, sh.nuf, nvf) & ~(unsigned)sd.scr.pemask[base + i];
    while (later) {
        const int k = __ffs(later) - 1;
        later &= later - 1;
        int du, dv;
        nb_off(k, du, dv);
        const int j = (iv + dv) * sh.nuf + iu + du;
        const unsigned old = atomicSub(&sd.scr.pcount[base + j], 1u << 8);
        if (old == (1u << 8)) sd.scr.pqueue[atomicAdd(&sh.qtail, 1)] = (int)(base + j);
    }
    if (pp + 1 < sh.np) {
        const long long nb = base + nplane;
        const int layer = sh.player0 - pp * fr.inner;   /* this plane = the next plane's inner layer */
        for (int dv = -1; dv <= 1; dv++)
            for (int du = -1; du <= 1; du++) {
                const int ju = iu + du, jv = iv + dv;
                if (ju < 0 || ju >= sh.nuf || jv < 0 || jv >= nvf) continue;
                const int j = jv * sh.nuf + ju;
                const unsigned old = atomicSub(&sd.scr.pcount[nb + j], 1u);
                if ((old & 0xFFu) != 1u) continue;
                /* inner block of node j complete: its in-plane order is now known */
                const unsigned em = earlier_mask(sd, sh, j, layer);
                sd.scr.pemask[nb + j] = (unsigned char)em;
                const unsigned lat = (unsigned)__popc(inrect_mask(ju, jv, sh.nuf, nvf) & ~em);
                const unsigned w = old - 1u;
                const unsigned prev = lat ? atomicSub(&sd.scr.pcount[nb + j], lat << 8) : w;
                if (prev - (lat << 8) == 0u) sd.scr.pqueue[atomicAdd(&sh.qtail, 1)] = (int)(nb + j);
            }
    }
}

/* Phase C for one point: the reference's sequential minimum over the 22 trials, from the values
 * computed in the parallel phases (new-edge and new-face values that were not precomputed are
 * evaluated here — they are needed only at first contact), then the commit
 * (src/sphfd.c:1756-1760), the point's stencil-state record and the release of its later
 * neighbours into list `out`.  Returns false if the point must wait for an inherited state. */
__device__ bool phase_c(const fd_station_dev &sd, Shared &sh, Smem &sm, int slot, bool have_inherit, float it0,
                        float it4, int out, unsigned char *dag, Counters &cn)
{
    const int i = sm.idx[slot];
    const float *t18 = sm.t[slot], *s18 = sm.s[slot];
    const unsigned gm = sm.guardm[slot], em = sm.evalm[slot];
    const double told = f2d(t18[NB_POINT]);
    /* a 2-D trial before any corner / new-edge call would read the previous point's t0,t4 */
    if (!have_inherit && (gm & 0xFu) == 0 && !((gm & 0xF0u) && told > 1.0e9) && (gm & 0xFF00u)) {
        if (sh.pipelined) sh.status = 6;   /* excluded by the pipelining precondition */
        return false;
    }
    const int z = sm.z[slot], y = sm.y[slot];
    double guess = told;
    float st0 = it0, st4 = it4;
    int writers = 0;
    bool gate = false;
    int lastK = -1;
    double last_gb = 0.0, last_v = 0.0;
#pragma unroll 1
    for (int K = 0; K < FDN_NTRIAL; K++) {
        /* the first-contact tests are made on entry to their blocks (src/sphfd.c:1375, :1698) */
        if (K == TK_NE0 || K == TK_NF) gate = lt(1.0e9, guess);
        if (!((gm >> K) & 1u)) continue;
        const TrialDesc &d = sm.desc[K];
        const bool ev = (em >> K) & 1u;
        double v;
        if (K < TK_2D0 || K == TK_NF) {
            /* corner, new-edge, new-face: writers of the stencil state */
            if (K >= TK_NE0 && !gate) continue;
            st0 = t18[d.slot[0]];
            st4 = t18[d.slot[4]];
            writers++;
            if (ev) {
                v = sm.res[slot][K];
            } else if (K >= TK_NE0) {
                /* new-edge / new-face value not precomputed: evaluate unless it cannot improve */
                float fl = t18[d.slot[0]];
                for (int k = 1; k < 5; k++) fl = fmaxf(fl, t18[d.slot[k]]);
                if (prunable(fl, guess)) continue;
                v = (K == TK_NF) ? eval_nf(d, t18, s18, sd.g, z, y) : eval_ne(d, t18, s18, sd.g, z, y);
                cn.n[K == TK_NF ? 3 : 1]++;
            } else {
                continue;
            }
        } else if (K < TK_NF) {
            /* 2-D: the causality floor includes the stale t0,t4 */
            if (!ev) continue;
            const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], st0)), st4);
            const double x1 = sm.res[slot][K], x2 = sm.x2[slot][K - TK_2D0];
            if (x1 != x1) {
                v = 1.e11;
            } else {
                const double f = f2d(fl);
                const bool bad1 = lt(x1, f), bad2 = lt(x2, f);
                v = bad1 ? (bad2 ? 1.e11 : x2) : (bad2 ? x1 : (lt(x2, x1) ? x2 : x1));
            }
        } else {
            if (!ev) continue;
            v = sm.res[slot][K];
        }
        if (lt(v, guess)) {
            if (d.head) { lastK = K; last_gb = guess; last_v = v; }
            guess = v;
        }
    }
    if (lt(guess, told)) {
        const fdn_frame fr = frame_of(sh.face);
        int xyz[3];
        xyz[fr.axis_u] = sh.ulo + i % sh.nuf;
        xyz[fr.axis_v] = sh.vlo + i / sh.nuf;
        xyz[fr.axis_n] = sm.lay[slot];
        const long long pT = ((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0];
        sd.T[pT] = __double2float_rn(guess);
        if (lastK >= 0) {
            /* only the last head trial that lowered the minimum sets the measure that is tested */
            const double fhead = (last_gb - last_v) / head_den(sm.desc[lastK], s18, sd.g, z, y);
            if (fhead > FD_HEADTEST) atomicAdd(&sh.headw[fr.headw], 1);
        }
    }
    if (sh.pipelined) {
        pipelined_release(sd, sh, slot, i, sm.pl[slot], writers != 0, st0, st4, t18);
        return true;
    }
    if (writers) {
        sd.scr.rec[i] = make_float2(st0, st4);
        atomicMax(&sh.exitkey, sd.scr.key[i]);
    } else {
        sd.scr.rec[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    }
    /* done; release the later in-face neighbours */
    const int nvf = sh.n / sh.nuf, iu = i % sh.nuf, iv = i / sh.nuf;
    unsigned char *emask = dag + sh.n_pad;
    unsigned later = inrect_mask(iu, iv, sh.nuf, nvf) & ~(unsigned)emask[i];
    atomicOr(reinterpret_cast<unsigned *>(dag) + (i >> 2), 0xFFu << ((i & 3) * 8));
    while (later) {
        const int k = __ffs(later) - 1;
        later &= later - 1;
        int du, dv;
        nb_off(k, du, dv);
        const int j = (iv + dv) * sh.nuf + iu + du;
        const unsigned sh8 = (j & 3) * 8;
        const unsigned old = atomicSub(reinterpret_cast<unsigned *>(dag) + (j >> 2), 1u << sh8);
        if (((old >> sh8) & 0xFFu) == 1u) sd.scr.wl[out][atomicAdd(&sh.cnt[out], 1)] = j;
    }
    return true;
}

__device__ __forceinline__ void phase_a2_dispatch(Smem &sm, const Shared &sh, int slot, int q)
{
    switch (sh.face) {
    case 0: phase_a2<0>(sm, sh, slot, q); break;
    case 1: phase_a2<1>(sm, sh, slot, q); break;
    case 2: phase_a2<2>(sm, sh, slot, q); break;
    case 3: phase_a2<3>(sm, sh, slot, q); break;
    case 4: phase_a2<4>(sm, sh, slot, q); break;
    default: phase_a2<5>(sm, sh, slot, q); break;
    }
}

/* Evaluate points list[0..m) (m <= FD_CHUNK).  All threads call this. */
__device__ void run_chunk(const fd_station_dev &sd, Shared &sh, Smem &sm, const int *list, int m, bool have_inherit,
                          float it0, float it4, int out, unsigned char *dag, Counters &cn)
{
    const int tid = threadIdx.x;
    if (tid < 5) sm.cnt[tid] = 0;
    FD_TIC(ta);
    /* A1: the 18-node context of each point, FD_TPP threads per point */
    const fdn_frame fr = frame_of(sh.face);
    for (int r = tid; r < m * FD_TPP; r += blockDim.x) {
        const int slot = r / FD_TPP, q = r % FD_TPP;
        /* list entries: fill indices, or plane*n + fill index in a pipelined sweep */
        const int e = list[slot];
        const int pp = sh.pipelined ? e / sh.n : -1;
        const int i = sh.pipelined ? e - pp * sh.n : e;
        const int layer = sh.pipelined ? sh.player0 - pp * fr.inner : sh.layer;
        const int u = sh.ulo + i % sh.nuf, v = sh.vlo + i / sh.nuf;
        int xyz[3];
        xyz[fr.axis_u] = u;
        xyz[fr.axis_v] = v;
        xyz[fr.axis_n] = layer;
        const long long pT = ((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0];
        const long long pS = (long long)xyz[2] * sd.s_sz + (long long)xyz[1] * sd.s_sy + xyz[0];
        if (q == 0) {
            sm.idx[slot] = i;
            sm.lay[slot] = layer;
            sm.pl[slot] = pp;
            sm.z[slot] = xyz[2];
            sm.y[slot] = xyz[1];
            sm.guardm[slot] = 0;
            sm.evalm[slot] = 0;
        }
        for (int nb = q; nb < NB_N; nb += FD_TPP) {
            const int w = nb / 9, dv = (nb / 3) % 3 - 1, du = nb % 3 - 1;
            const int uu = u + du, vv = v + dv;
            float tv = 0.f, svv = 0.f;
            if (uu >= 0 && uu < sh.nu && vv >= 0 && vv < sh.nv) {
                const long long off_n = (long long)(w * fr.inner);
                tv = sd.T[pT + du * sh.su + dv * sh.sv + off_n * sh.sn];
                svv = __ldg(&sd.S[pS + du * sh.ssu + dv * sh.ssv + off_n * sh.ssn]);
            }
            sm.t[slot][nb] = tv;
            sm.s[slot][nb] = svv;
        }
    }
    __syncthreads();
    /* A2: guards, pruning, corner / edge / first-contact items */
    for (int r = tid; r < m * FD_TPP; r += blockDim.x) phase_a2_dispatch(sm, sh, r / FD_TPP, r % FD_TPP);
    __syncthreads();
    FD_TOC(1, ta);
    FD_TIC(tb);
    run_items(sd, sm, 0, 4, cn);   /* corner, new-edge, 1-D (2-D not queued yet, new-face never) */
    __syncthreads();
    if (tid < 5) sm.cnt[tid] = 0;
    __syncthreads();
    for (int r = tid; r < m * FD_TPP; r += blockDim.x) phase_g(sm, r / FD_TPP, r % FD_TPP, it0, it4);
    __syncthreads();
    run_items(sd, sm, 2, 2, cn);
    __syncthreads();
    FD_TOC(2, tb);
    FD_TIC(tc);
    if (tid < m) {
        if (!phase_c(sd, sh, sm, tid, have_inherit, it0, it4, out, dag, cn))
            sd.scr.deferred[atomicAdd(&sh.ndef, 1)] = list[tid];
    }
    __syncthreads();
    FD_TOC(3, tc);
}

/* Walk the current face (parameters in sh) in dependency order. */
__device__ void face_walk(const fd_station_dev &sd, Shared &sh, Smem &sm, bool dag_in_smem, Counters &cn)
{
    const int n = sh.n, nuf = sh.nuf, nvf = n / nuf;
    const int tid = threadIdx.x;
    const float *T = sd.T;
    const fdn_frame fr = frame_of(sh.face);
    unsigned char *dag = dag_indeg(sd, sm, dag_in_smem);
    unsigned char *emask = dag + sh.n_pad;
    FD_TIC(t0);
    /* trial descriptors of this face */
    for (int k = tid; k < FDN_NTRIAL; k += blockDim.x) sm.desc[k] = c_desc[sh.face * FDN_NTRIAL + k];
    /* keys: time of the inner-layer neighbour, then fill index */
    for (int i = tid; i < n; i += blockDim.x) {
        int xyz[3];
        xyz[fr.axis_u] = sh.ulo + i % nuf;
        xyz[fr.axis_v] = sh.vlo + i / nuf;
        xyz[fr.axis_n] = sh.layer + fr.inner;
        const float tin = T[((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0]];
        sd.scr.key[i] = ((unsigned long long)okey32(tin) << 32) | (unsigned)i;
    }
    if (tid == 0) { sh.cnt[0] = 0; sh.cnt[1] = 0; sh.ndef = 0; sh.exitkey = 0ull; }
    __syncthreads();
    /* earlier-neighbour masks and in-degrees */
    for (int i = tid; i < n; i += blockDim.x) {
        const unsigned long long ki = sd.scr.key[i];
        const int iu = i % nuf, iv = i / nuf;
        unsigned em = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int du, dv;
            nb_off(k, du, dv);
            const int ju = iu + du, jv = iv + dv;
            if (ju < 0 || ju >= nuf || jv < 0 || jv >= nvf) continue;
            if (sd.scr.key[jv * nuf + ju] < ki) em |= 1u << k;
        }
        emask[i] = (unsigned char)em;
        dag[i] = (unsigned char)__popc(em);
        if (em == 0) sd.scr.wl[0][atomicAdd(&sh.cnt[0], 1)] = i;
    }
    __syncthreads();
    FD_TOC(0, t0);
    int cur = 0;
    long long rounds = 0;
    const long long max_rounds = 2ll * n + 8;
    for (;;) {
        FD_TIC(tr);
        __syncthreads();
        const int ncur = sh.cnt[cur];
        const int ndef = sh.ndef;
        if (++rounds > max_rounds) {
            if (tid == 0) sh.status = 3;
            break;
        }
        if (ncur == 0) {
            if (ndef == 0) break;
            /* the deferred point with the smallest key: every point below it is done */
            unsigned long long lm = ~0ull;
            for (int j = tid; j < ndef; j += blockDim.x) {
                const unsigned long long k = sd.scr.key[sd.scr.deferred[j]];
                lm = k < lm ? k : lm;
            }
            const unsigned long long dmin = block_min_u64(lm, sh);
            /* the last writer before it in sort order */
            unsigned long long lw = 0ull;
            for (int i = tid; i < n; i += blockDim.x) {
                const unsigned long long k = sd.scr.key[i];
                if (k < dmin && dag[i] == 0xFFu && !isnan(sd.scr.rec[i].x)) lw = k > lw ? k : lw;
            }
            const unsigned long long wkey = block_max_u64(lw, sh);
            const int d = (int)(dmin & 0xffffffffu);
            float t0 = sh.carry_t0, t4 = sh.carry_t4;
            if (wkey) {
                const float2 r = sd.scr.rec[(int)(wkey & 0xffffffffu)];
                t0 = r.x;
                t4 = r.y;
            }
            if (tid == 0) {
                for (int j = 0; j < ndef; j++)
                    if (sd.scr.deferred[j] == d) { sd.scr.deferred[j] = sd.scr.deferred[ndef - 1]; break; }
                sh.ndef = ndef - 1;
                sh.deferred++;
            }
            __syncthreads();
            const int one[1] = {d};
            run_chunk(sd, sh, sm, one, 1, true, t0, t4, cur, dag, cn);
            FD_TOC(5, tr);
            continue;
        }
        if (tid == 0) { sh.cnt[cur ^ 1] = 0; sh.rounds++; }
        __syncthreads();
        FD_TOC(4, tr);
        for (int c0 = 0; c0 < ncur; c0 += FD_CHUNK) {
            const int m = ncur - c0 < FD_CHUNK ? ncur - c0 : FD_CHUNK;
            run_chunk(sd, sh, sm, sd.scr.wl[cur] + c0, m, false, 0.f, 0.f, cur ^ 1, dag, cn);
        }
        cur ^= 1;
    }
    __syncthreads();
    if (tid == 0) {
        if (sh.exitkey) {
            const float2 r = sd.scr.rec[(int)(sh.exitkey & 0xffffffffu)];
            sh.carry_t0 = r.x;
            sh.carry_t4 = r.y;
        }
        sh.faces++;
        sh.node_updates += n;
    }
}

/* face parameters of face `face` for the current walls (thread 0) */
__device__ void setup_face(const fd_station_dev &sd, Shared &sh, int face)
{
    const int nx = sd.g.nx, ny = sd.g.ny, nz = sd.g.nz;
    const long long nxy = (long long)nx * ny;
    /* walls: 0 z1, 1 z2, 2 x2, 3 x1, 4 y1, 5 y2 */
    const int x1 = sh.wall[3], x2 = sh.wall[2], y1 = sh.wall[4], y2 = sh.wall[5];
    const int z1 = sh.wall[0], z2 = sh.wall[1];
    sh.face = face;
    sh.layer = sh.wall[face];
    if (face < 2) {
        sh.ulo = x1 + 1; sh.uhi = x2 - 1; sh.vlo = y1 + 1; sh.vhi = y2 - 1;
        sh.nu = nx; sh.nv = ny;
        sh.su = 1; sh.sv = nx; sh.sn = nxy;
        sh.ssu = 1; sh.ssv = sd.s_sy; sh.ssn = sd.s_sz;
    } else if (face < 4) {
        sh.ulo = y1 + 1; sh.uhi = y2 - 1; sh.vlo = z1 + 1; sh.vhi = z2 - 1;
        sh.nu = ny; sh.nv = nz;
        sh.su = nx; sh.sv = nxy; sh.sn = 1;
        sh.ssu = sd.s_sy; sh.ssv = sd.s_sz; sh.ssn = 1;
    } else {
        sh.ulo = x1 + 1; sh.uhi = x2 - 1; sh.vlo = z1 + 1; sh.vhi = z2 - 1;
        sh.nu = nx; sh.nv = nz;
        sh.su = 1; sh.sv = nxy; sh.sn = nx;
        sh.ssu = 1; sh.ssv = sd.s_sz; sh.ssn = sd.s_sy;
    }
    sh.nuf = sh.uhi - sh.ulo + 1;
    const int nvf = sh.vhi - sh.vlo + 1;
    sh.n = (sh.nuf > 0 && nvf > 0) ? sh.nuf * nvf : 0;
    sh.n_pad = (sh.n + 15) & ~15;
}

/* One sweep of face F as a plane-pipelined dependency graph.  Leaves walls, flags and radius as
 * the radius loop of src/sphfd.c:1018-5566 would. */
__device__ void pipelined_sweep(const fd_station_dev &sd, Shared &sh, Smem &sm, Counters &cn, int F)
{
    const int tid = threadIdx.x;
    const fdn_frame fr = frame_of(F);
    if (tid == 0) {
        setup_face(sd, sh, F);
        /* the planes the radius loop would visit: up to grow[F] per radius step, until the wall
         * reaches the model side or the radius reaches maxrad */
        const int nmax = F < 2 ? sd.g.nz : F < 4 ? sd.g.nx : sd.g.ny;
        int w = sh.wall[F], flag = sh.dflag[F], radius = sh.radius, rad0 = sh.rad0, np = 0;
        while (rad0 && flag) {
            for (int ig = 1; ig <= sd.grow[F]; ig++) {
                if (!flag) continue;
                np++;
                if (fr.inner > 0 ? (w == 0) : (w == nmax - 1)) flag = 0;
                w -= fr.inner;
            }
            radius++;
            if (radius == sd.maxrad) rad0 = 0;
        }
        sh.np = np;
        sh.player0 = sh.wall[F];
        sh.wall[F] = w;
        sh.dflag[F] = flag;
        sh.radius = radius;
        sh.rad0 = rad0;
        sh.qtail = 0;
        sh.exitkey = 0ull;
        sh.pipelined = 1;
    }
    for (int k = tid; k < FDN_NTRIAL; k += blockDim.x) sm.desc[k] = c_desc[F * FDN_NTRIAL + k];
    __syncthreads();
    const int np = sh.np, nplane = sh.n, nuf = sh.nuf, nvf = nplane > 0 ? nplane / nuf : 0;
    const long long total = (long long)np * nplane;
    if (total > 0) {
        /* counters: plane 0 reads the static wall layer, so its in-plane order is known now */
        const int wall_layer = sh.player0 + fr.inner;
        for (long long id = tid; id < total; id += blockDim.x) {
            const int pp = (int)(id / nplane), i = (int)(id - (long long)pp * nplane);
            const unsigned inr = inrect_mask(i % nuf, i / nuf, nuf, nvf);
            const unsigned c2 = (unsigned)__popc(inr);
            unsigned wd = (pp > 0 ? 1u + c2 : 0u) | (c2 << 8);
            if (pp == 0) {
                const unsigned em = earlier_mask(sd, sh, i, wall_layer);
                sd.scr.pemask[id] = (unsigned char)em;
                wd -= (unsigned)__popc(inr & ~em) << 8;
            }
            sd.scr.pcount[id] = wd;
            if (wd == 0u) sd.scr.pqueue[atomicAdd(&sh.qtail, 1)] = (int)id;
        }
        long long head = 0, steps = 0;
        for (;;) {
            __syncthreads();
            const long long tail = sh.qtail;
            if (head >= total || sh.status) break;
            const long long avail = tail - head;
            if (avail <= 0 || ++steps > total + 8) {
                if (tid == 0) sh.status = 5;   /* cannot happen: every node is queued exactly once */
                break;
            }
            const int m = avail < FD_CHUNK ? (int)avail : FD_CHUNK;
            run_chunk(sd, sh, sm, sd.scr.pqueue + head, m, false, 0.f, 0.f, 0, sd.scr.dag, cn);
            head += m;
        }
        __syncthreads();
        if (tid == 0) sh.rounds += steps;
    }
    if (tid == 0) {
        if (sh.exitkey) {
            const float2 r = sd.scr.rec[(int)(sh.exitkey & 0xffffffffu)];
            sh.carry_t0 = r.x;
            sh.carry_t4 = r.y;
        }
        sh.faces += np;
        sh.node_updates += total;
        sh.psweeps++;
        sh.pipelined = 0;
    }
    __syncthreads();
}

/* ---------------------------------------------------------------------------------------------- */
/* source box (src/sphfd.c:724-825)                                                                */

__device__ void init_field(const fd_station_dev &sd)
{
    const long long nxyz = (long long)sd.g.nx * sd.g.ny * sd.g.nz;
    const float u = 1.0e10f;
    /* T may start anywhere a float can: scalar head up to a 16-byte boundary, float4 body, scalar tail */
    const long long head = (long long)(((16u - ((unsigned)(uintptr_t)sd.T & 15u)) & 15u) / 4u);
    const long long h = head < nxyz ? head : nxyz;
    for (long long i = threadIdx.x; i < h; i += blockDim.x) sd.T[i] = u;
    float4 *T4 = reinterpret_cast<float4 *>(sd.T + h);
    const long long nv4 = (nxyz - h) / 4;
    for (long long i = threadIdx.x; i < nv4; i += blockDim.x) T4[i] = make_float4(u, u, u, u);
    for (long long i = h + nv4 * 4 + threadIdx.x; i < nxyz; i += blockDim.x) sd.T[i] = u;
    __syncthreads();
    const int nc = sd.ncube, w = 2 * nc + 1;
    const long long nx = sd.g.nx, nxy = (long long)sd.g.nx * sd.g.ny;
    const float s000 = sd.S[(long long)sd.zs * sd.s_sz + (long long)sd.ys * sd.s_sy + sd.xs];
    for (int k = threadIdx.x; k < w * w * w; k += blockDim.x) {
        const int zz = sd.zs - nc + k / (w * w), yy = sd.ys - nc + (k / w) % w, xx = sd.xs - nc + k % w;
        if (zz < 0 || zz >= sd.g.nz || yy < 0 || yy >= sd.g.ny || xx < 0 || xx >= sd.g.nx) continue;
        const int jy = yy - (sd.ys - nc), jx = xx - (sd.xs - nc);
        const double cq = sd.box_trig[2 * jy], sq = sd.box_trig[2 * jy + 1];
        const double cf = sd.box_trig[2 * w + 2 * jx], sf = sd.box_trig[2 * w + 2 * jx + 1];
        const double rz1 = sd.g.zrow[(long long)zz * FD_Z_N + FD_Z_R];
        const double x2p = rz1 * cq;
        const double y2p = rz1 * sq * cf;
        const double z2p = rz1 * sq * sf;
        const double dx = sd.src_xyz[0] - x2p, dy = sd.src_xyz[1] - y2p, dz = sd.src_xyz[2] - z2p;
        const double dist = __dsqrt_rn(dx * dx + dy * dy + dz * dz);
        sd.T[(long long)zz * nxy + (long long)yy * nx + xx] = __double2float_rn((double)s000 * dist);
    }
    __syncthreads();
}

/* ---------------------------------------------------------------------------------------------- */
/* the sweep loop (src/sphfd.c:1008-5678)                                                          */

__global__ void __launch_bounds__(FD_BLOCK, 1) fd_solve(const fd_station_dev *stations, int nst, int dag_smem_bytes)
{
    __shared__ Shared sh;
    extern __shared__ __align__(16) unsigned char fd_dyn_smem[];
    Smem &sm = *reinterpret_cast<Smem *>(fd_dyn_smem);
    if ((int)blockIdx.x >= nst) return;
    const fd_station_dev &sd = stations[blockIdx.x];
    const int tid = threadIdx.x;
    unsigned long long t_start = 0;
    if (tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    /* the dependency bytes of the station's largest face go to shared memory when they fit */
    const bool dag_in_smem = 2ll * sd.max_face_pad <= dag_smem_bytes;
    if (sd.init_mode == 0) init_field(sd);
    if (tid == 0) {
        for (int f = 0; f < 6; f++) { sh.wall[f] = sd.wall[f]; sh.dflag[f] = sd.dflag[f]; }
        sh.radius = sd.radius;
        sh.rad0 = 1;
        sh.reverse = sd.reverse;
        sh.headpref = sd.headpref;
        sh.carry_t0 = sd.carry_t0;
        sh.carry_t4 = sd.carry_t4;
        sh.status = 0;
        sh.faces = sh.node_updates = sh.rounds = sh.deferred = 0;
        for (int k = 0; k < 5; k++) sh.st[k] = 0;
        sh.sweeps = 0;
        for (int k = 0; k < 8; k++) sh.restart_wall[k] = 0;
        for (int k = 0; k < 6; k++) sh.cyc[k] = 0;
        sh.pipelined = 0;
        sh.psweeps = 0;
    }
    __syncthreads();
    Counters cn;
    for (int k = 0; k < 5; k++) cn.n[k] = 0;
    const int nx = sd.g.nx, ny = sd.g.ny, nz = sd.g.nz;
    const long long nxy = (long long)nx * ny;
    int guard_sweeps = 0;
    while (sh.reverse > -1 && sh.status == 0) {
        if (tid == 0) for (int k = 0; k < 8; k++) sh.headw[k] = 0;
        __syncthreads();
        /* A sweep with one active face (every sweep after a restart) walks full planes.  It runs as
         * one plane-pipelined graph when no point can need an earlier point's stencil state: every
         * time below 1e9 makes every corner guard that is inside the grid pass (so each point calls
         * a corner stencil before its 2-D trials), except the EAST corner whose guard tests the node
         * above for being non-zero (src/sphfd.c:2544), which fails only next to a zero time. */
        int act = -1, nact = 0;
        for (int f = 0; f < 6; f++)
            if (sh.dflag[f]) { act = f; nact++; }
        bool piped = false;
        if (nact == 1 && sh.rad0 && sd.scr.pcount) {
            int bad = 0;
            const long long nxyz = nxy * nz;
            for (long long i = tid; i < nxyz; i += blockDim.x) {
                const float t = sd.T[i];
                if (!(t < 1.e9f)) bad = 1;
                else if (act == 2 && t == 0.0f && (i / nx) % ny == 0 && i / nxy == 1) bad = 1;
            }
            piped = !__syncthreads_or(bad);
        }
        if (piped) pipelined_sweep(sd, sh, sm, cn, act);
        while (!piped && sh.rad0
               && (sh.dflag[0] || sh.dflag[1] || sh.dflag[2] || sh.dflag[3] || sh.dflag[4] || sh.dflag[5])
               && sh.status == 0) {
            for (int face = 0; face < 6; face++) {
                for (int ig = 1; ig <= sd.grow[face]; ig++) {
                    if (!sh.dflag[face]) continue;
                    if (tid == 0) setup_face(sd, sh, face);
                    __syncthreads();
                    if (sh.n > 0) face_walk(sd, sh, sm, dag_in_smem, cn);
                    __syncthreads();
                    if (tid == 0) {
                        /* move the wall outward (e.g. src/sphfd.c:1762-1764) */
                        const int inner = frame_of(face).inner;
                        const int nmax = face < 2 ? nz : face < 4 ? nx : ny;
                        const bool limit = inner > 0 ? (sh.wall[face] == 0) : (sh.wall[face] == nmax - 1);
                        if (limit) sh.dflag[face] = 0;
                        sh.wall[face] -= inner;
                    }
                    __syncthreads();
                }
            }
            if (tid == 0) {
                sh.radius++;
                if (sh.radius == sd.maxrad) sh.rad0 = 0;
            }
            __syncthreads();
        }
        if (tid == 0) {
            sh.sweeps++;
            /* restart test (src/sphfd.c:5570-5676) */
            const int *hw = sh.headw;
            if (!hw[1] && !hw[2] && !hw[3] && !hw[4] && !hw[5] && !hw[6]) {
                sh.reverse = 0;
            } else {
                int head = 0, srcwall = 0;
                for (int w = 1; w <= 6; w++)
                    if (hw[w] > 0 && hw[w] > head) { head = hw[w]; srcwall = w; }
                if (sh.headpref > 0 && hw[sh.headpref] > 0) srcwall = sh.headpref;
                for (int f = 0; f < 6; f++) sh.dflag[f] = 1;
                sh.rad0 = 1;
                sh.radius = 1;
                /* face order walls: 0 z1, 1 z2, 2 x2, 3 x1, 4 y1, 5 y2 */
                if (srcwall == 1) sh.wall[2] = 1; else { sh.wall[2] = nx; sh.dflag[2] = 0; }
                if (srcwall == 2) sh.wall[3] = nx - 2; else { sh.wall[3] = -1; sh.dflag[3] = 0; }
                if (srcwall == 3) sh.wall[5] = 1; else { sh.wall[5] = ny; sh.dflag[5] = 0; }
                if (srcwall == 4) sh.wall[4] = ny - 2; else { sh.wall[4] = -1; sh.dflag[4] = 0; }
                if (srcwall == 5) sh.wall[1] = 1; else { sh.wall[1] = nz; sh.dflag[1] = 0; }
                if (srcwall == 6) sh.wall[0] = nz - 2; else { sh.wall[0] = -1; sh.dflag[0] = 0; }
                if (sh.reverse > 0) sh.restart_wall[srcwall]++;
            }
            sh.reverse--;
        }
        __syncthreads();
        if (++guard_sweeps > 1000000) { if (tid == 0) sh.status = 4; break; }
    }
    /* statistics */
    for (int k = 0; k < 5; k++) atomicAdd(&sh.st[k], cn.n[k]);
    __syncthreads();
    if (tid == 0 && sd.stats) {
        fd_station_stats *o = sd.stats;
        o->status = sh.status;
        o->sweeps = sh.sweeps;
        o->node_updates = sh.node_updates;
        o->faces = sh.faces;
        o->rounds = sh.rounds;
        o->deferred = sh.deferred;
        for (int k = 0; k < 5; k++) o->stencils[k] = (int64_t)sh.st[k];
        for (int k = 0; k < 8; k++) o->restart_wall[k] = sh.restart_wall[k];
        for (int k = 0; k < 6; k++) o->phase_cycles[k] = sh.cyc[k];
        unsigned long long t_end;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
        o->t_start_ns = (int64_t)t_start;
        o->t_end_ns = (int64_t)t_end;
    }
}

}  // namespace fdk

/* launch wrappers used by the host runtime */
extern "C" cudaError_t fdk_launch_geo_build(int nx, int ny, int nz, double h, double dq, double df, double z0r,
                                            const double *ysin, double *zrow, double *node, double *cell,
                                            cudaStream_t stream)
{
    fdk::fd_geo_build<<<152, 256, 0, stream>>>(nx, ny, nz, h, dq, df, z0r, ysin, zrow, node, cell);
    return cudaGetLastError();
}

extern "C" cudaError_t fdk_launch_solve(const fd_station_dev *stations, int nst, long long max_face_pad,
                                        cudaStream_t stream)
{
    if (nst <= 0) return cudaSuccess;
    /* dynamic shared memory: the evaluation chunk, plus the face's dependency bytes if they fit */
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const long long base = (long long)sizeof(fdk::Smem);
    const long long want = base + 2 * max_face_pad;
    const long long bytes = want <= optin - 1024 ? want : base;
    const cudaError_t e = cudaFuncSetAttribute(fdk::fd_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    fdk::fd_solve<<<nst, FD_BLOCK, (size_t)bytes, stream>>>(stations, nst, (int)(bytes - base));
    return cudaGetLastError();
}

/* slowness = 1/velocity, float division as the reference does it (src/sphfd.c:689-690) */
__global__ void fd_v2s(const float *v, float *s, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s[i] = 1.0f / v[i];
}

extern "C" cudaError_t fdk_launch_v2s(const float *v, float *s, long long n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    fd_v2s<<<(int)blocks, 256, 0, stream>>>(v, s, n);
    return cudaGetLastError();
}

/* FP64 pipe rate probe: 8 independent fused multiply-add chains per thread, all SMs */
__global__ void fd_fp64_probe(double *out, int iters)
{
    double a0 = threadIdx.x * 1e-9 + 1.0, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
    double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
    const double m = 1.0000001, c = 1e-12;
    for (int i = 0; i < iters; i++) {
        a0 = __fma_rn(a0, m, c); a1 = __fma_rn(a1, m, c); a2 = __fma_rn(a2, m, c); a3 = __fma_rn(a3, m, c);
        a4 = __fma_rn(a4, m, c); a5 = __fma_rn(a5, m, c); a6 = __fma_rn(a6, m, c); a7 = __fma_rn(a7, m, c);
    }
    out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

extern "C" cudaError_t fdk_probe_fp64(double *scratch, int blocks, int threads, int iters, float *ms, cudaStream_t s)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fd_fp64_probe<<<blocks, threads, 0, s>>>(scratch, iters);
    cudaEventRecord(e0, s);
    fd_fp64_probe<<<blocks, threads, 0, s>>>(scratch, iters);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return e == cudaSuccess ? cudaGetLastError() : e;
}
