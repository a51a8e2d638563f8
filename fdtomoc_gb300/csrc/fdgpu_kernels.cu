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
 * every in-face neighbour with a larger key (time bits, fill index).  Walking it in dependency order —
 * every point whose earlier neighbours are all done may be evaluated, then releases its later
 * neighbours — reproduces the sequential order exactly.  No sort is needed.
 *
 * The one sequential coupling that is not a neighbour relation is the stale (t0,t4) pair of
 * fdsph2d (src/sphfd.c:6116-6121): a point whose first 2-D trial comes before any 3-D / new-edge
 * call of its own reads the pair left by the previous point in sort order.  Such a point is put
 * aside; when no other point is ready, the one with the smallest key has every smaller-key point
 * done, and its pair is the record of the largest-key earlier point that made a writer call (or
 * the face's entry pair).  This is rare (hundreds of points per million).
 *
 * Within a walk the warps of the CTA are independent workers that meet only at shared-memory
 * counters (see "warp workers" below); every wait among them is bounded and ends in an error
 * status, never in a hang.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fdgpu_eval.cuh"
#include "fdgpu_trials.cuh"
#include "fdgpu_bound.cuh"
#include "fdgpu_layout.h"

#define FD_WARPS 12                 /* independent workers per station */
#define FD_BLOCK (FD_WARPS * 32)

/* optional per-phase cycle counters (thread 0, between barriers) for profiling builds */
#ifdef FDGPU_PHASE_TIMERS
#define FD_TIC(v) long long v = clock64()
#define FD_TOC(k, v) \
    do { if ((threadIdx.x & 31) == 0) atomicAdd(reinterpret_cast<unsigned long long *>(&sh.cyc[k]), (unsigned long long)(clock64() - (v))); } while (0)
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
    /* current walk: ready queue, queue of points waiting for an inherited stencil state, idle
     * workers, finished nodes */
    int qhead, qtail, qcap, rqhead, rqtail, rqcap, idle, ndone;
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
    /* plane-pipelined sweep: on/off, number of planes, layer of plane 0 */
    int pipelined, np, player0;
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
/* warp workers                                                                                    */
/*                                                                                                 */
/* A walk — one face, or one plane-pipelined sweep — is a dependency graph whose ready nodes sit   */
/* in a queue.  Every warp of the CTA is an independent worker: it claims up to 32 ready nodes,     */
/* evaluates them (one lane per node for the per-node steps, the stencil trials of all its nodes   */
/* spread over the 32 lanes), commits them and queues the nodes they complete.  Warps meet only at */
/* shared-memory counters, so the FP64 work of some warps hides the memory and control latency of  */
/* the others, and a node starts as soon as its own inputs are final instead of at the next round. */
/*                                                                                                 */
/* Queue: positions are taken with an atomic on the tail and written after; every entry starts as */
/* -1, so a worker that claimed a position not yet written waits for it (briefly: the writer is    */
/* between two instructions).  Stores of a node's time and of its queue entries are ordered by     */
/* __threadfence_block before the counters that publish them.                                     */
/*                                                                                                 */
/* Quiescence: a worker with nothing to claim counts itself idle.  When every worker is idle and   */
/* the queue is empty and stays so (tail read before and after the idle count), no node is in      */
/* flight and none can become ready; if points were put aside for an inherited stencil state, one  */
/* worker (elected with a lock, the test repeated under it) resolves the first of them.  Every     */
/* wait is bounded: a worker idle for FD_WAIT_CYCLES without progress sets the station's status    */
/* and all workers leave the walk.                                                                  */

#define NB_PAD 19                    /* context row stride: the 32 rows fall on distinct banks */
#define FD_WAIT_CYCLES (4ll << 30)   /* about 2 s at the maximum SM clock */
#ifndef FD_FACE_WARPS
#define FD_FACE_WARPS FD_WARPS       /* workers that take part in a face walk */
#endif
#define FD_QSPIN (1 << 22)           /* polls of an unwritten queue entry before giving up */

#define FD_DESC_ROW(F)                                                                              \
    make_desc<F>(0), make_desc<F>(1), make_desc<F>(2), make_desc<F>(3), make_desc<F>(4), make_desc<F>(5), \
    make_desc<F>(6), make_desc<F>(7), make_desc<F>(8), make_desc<F>(9), make_desc<F>(10), make_desc<F>(11), \
    make_desc<F>(12), make_desc<F>(13), make_desc<F>(14), make_desc<F>(15), make_desc<F>(16), make_desc<F>(17), \
    make_desc<F>(18), make_desc<F>(19), make_desc<F>(20), make_desc<F>(21)
__constant__ TrialDesc c_desc[FDN_NFACE * FDN_NTRIAL] = {FD_DESC_ROW(0), FD_DESC_ROW(1), FD_DESC_ROW(2),
                                                         FD_DESC_ROW(3), FD_DESC_ROW(4), FD_DESC_ROW(5)};

__device__ __forceinline__ int kind_of(int K)
{
    return K < TK_NE0 ? 0 : K < TK_2D0 ? 1 : K < TK_NF ? 2 : K < TK_1D0 ? 3 : 4;
}

/* shared by the CTA: the current face's trial descriptors */
struct CtaSmem {
    TrialDesc desc[FDN_NTRIAL];
};
constexpr int kCtaSmemBytes = (int)((sizeof(CtaSmem) + 15) & ~(size_t)15);

/* one warp's chunk of up to 32 nodes; slot = lane of the node */
struct WarpSmem {
    double res[32][FDN_NTRIAL];            /* trial values (2-D: after the causality selection) */
    float t[32][NB_PAD];                   /* 18-node time context */
    float s[32][NB_PAD];                   /* 18-node slowness context */
    float s0[32], s4[32];                  /* stencil state entering the 2-D block */
    int z[32], y[32];                      /* grid z and y of the node */
    unsigned short items[FDN_NTRIAL * 32]; /* (slot << 5 | trial) to evaluate, trial-major */
};
static_assert(sizeof(WarpSmem) % 16 == 0, "keeps the dependency bytes after the warp areas aligned");
constexpr int kSmemBase = kCtaSmemBytes + FD_WARPS * (int)sizeof(WarpSmem);

template <class T>
__device__ __forceinline__ T vload(const T &x) { return *const_cast<const volatile T *>(&x); }

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
 * (2-D: its three own slots; the stale pair is added later) */
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
__device__ __forceinline__ bool any_corner(const float *t18, const Rect &r)
{
    return guard_static<F, 0>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)
           || guard_static<F, 1>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)
           || guard_static<F, 2>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi)
           || guard_static<F, 3>(t18, r.u, r.v, r.nu, r.nv, r.ulo, r.uhi, r.vlo, r.vhi);
}

/* Guards, pruning and the trials to evaluate before the 2-D block: gm = trials whose guards pass
 * (first-contact gates excluded), em = corner and 1-D trials that can lower the minimum, and
 * new-edge trials when no corner can run (their gate is then decided by the initial value). */
template <int F, int K>
__device__ __forceinline__ void guard_trials(const float *t18, const Rect &r, double g0, bool any3d, unsigned &gm,
                                             unsigned &em)
{
    if constexpr (K < FDN_NTRIAL) {
        constexpr fdn_trial tr = fd_face_trials[F][K];
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
        guard_trials<F, K + 1>(t18, r, g0, any3d, gm, em);
    }
}

template <int F>
__device__ __forceinline__ void guards_face(const float *t18, const Rect &r, unsigned &gm, unsigned &em)
{
    const double g0 = f2d(t18[NB_POINT]);
    const bool any3d = any_corner<F>(t18, r);
    gm = 0;
    em = 0;
    guard_trials<F, 0>(t18, r, g0, any3d, gm, em);
}

__device__ __forceinline__ void guards(int face, const float *t18, const Rect &r, unsigned &gm, unsigned &em)
{
    switch (face) {
    case 0: guards_face<0>(t18, r, gm, em); break;
    case 1: guards_face<1>(t18, r, gm, em); break;
    case 2: guards_face<2>(t18, r, gm, em); break;
    case 3: guards_face<3>(t18, r, gm, em); break;
    case 4: guards_face<4>(t18, r, gm, em); break;
    default: guards_face<5>(t18, r, gm, em); break;
    }
}

/* append the items (lane, K) for K in [k0, k1) whose bit is set in the lane's em, trial-major */
__device__ __forceinline__ int push_items(unsigned short *items, int n, unsigned em, int k0, int k1, int lane)
{
    const unsigned below = (1u << lane) - 1u;
    for (int K = k0; K < k1; K++) {
        const bool on = (em >> K) & 1u;
        const unsigned b = __ballot_sync(0xffffffffu, on);
        if (on) items[n + __popc(b & below)] = (unsigned short)((lane << 5) | K);
        n += __popc(b);
    }
    return n;
}

/* evaluate items[0..n) with the warp's lanes; a 2-D value is stored after the causality selection
 * against its floor, which includes the stencil state entering the 2-D block (src/sphfd.c:6116-6121) */
__device__ void eval_items(const fd_station_dev &sd, const CtaSmem &cs, WarpSmem &ws, int n, int lane, Counters &cn)
{
    for (int j = lane; j < n; j += 32) {
        const unsigned it = ws.items[j];
        const int slot = (int)(it >> 5), K = (int)(it & 31);
        const TrialDesc &d = cs.desc[K];
        const int z = ws.z[slot], y = ws.y[slot];
        const float *t18 = ws.t[slot], *s18 = ws.s[slot];
        const int kind = kind_of(K);
        double v;
        switch (kind) {
        case 0: v = eval_3d(d, t18, s18, sd.g, z, y); break;
        case 1: v = eval_ne(d, t18, s18, sd.g, z, y); break;
        case 2: {
            double x1, x2;
            eval_2d(d, t18, s18, sd.g, z, y, x1, x2);
            if (x1 != x1) {
                v = 1.e11;
            } else {
                const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], ws.s0[slot])),
                                       ws.s4[slot]);
                const double f = f2d(fl);
                const bool bad1 = lt(x1, f), bad2 = lt(x2, f);
                v = bad1 ? (bad2 ? 1.e11 : x2) : (bad2 ? x1 : (lt(x2, x1) ? x2 : x1));
            }
            break;
        }
        case 3: v = eval_nf(d, t18, s18, sd.g, z, y); break;
        default: v = eval_1d(d, t18, s18, sd.g, z, y); break;
        }
        ws.res[slot][K] = v;
        cn.n[kind]++;
    }
}

/* Replay of the corner and new-edge trials (every writer of the stencil state comes before the
 * 2-D block): the running minimum entering the 2-D block — an upper bound for every 2-D trial's
 * turn — and the stale (t0,t4) those trials test against.  Returns the 2-D trials that can still
 * lower the minimum. */
__device__ unsigned stale_pair(const CtaSmem &cs, WarpSmem &ws, int slot, unsigned gm, unsigned em, float it0,
                               float it4)
{
    const float *t18 = ws.t[slot];
    double g1 = f2d(t18[NB_POINT]);
    float s0 = it0, s4 = it4;
    for (int K = 0; K < TK_NE0; K++) {
        if (!((gm >> K) & 1u)) continue;
        s0 = t18[cs.desc[K].slot[0]];
        s4 = t18[cs.desc[K].slot[4]];
        if ((em >> K) & 1u) {
            const double v = ws.res[slot][K];
            if (lt(v, g1)) g1 = v;
        }
    }
    const bool gate = lt(1.0e9, g1);
    for (int K = TK_NE0; K < TK_2D0; K++) {
        if (!gate || !((gm >> K) & 1u)) continue;
        s0 = t18[cs.desc[K].slot[0]];
        s4 = t18[cs.desc[K].slot[4]];
        if ((em >> K) & 1u) {
            const double v = ws.res[slot][K];
            if (lt(v, g1)) g1 = v;
        }
    }
    ws.s0[slot] = s0;
    ws.s4[slot] = s4;
    ws.res[slot][TK_NF] = g1;   /* for filter_2d: the new-face value is never precomputed */
    unsigned add = 0;
    for (int K = TK_2D0; K < TK_NF; K++) {
        if (!((gm >> K) & 1u)) continue;
        const TrialDesc &d = cs.desc[K];
        const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], s0)), s4);
        if (!prunable(fl, g1)) add |= 1u << K;
    }
    return add;
}

/* Drop the queued 2-D items whose single-precision lower bound shows they cannot lower the
 * running minimum entering the 2-D block (kept in res[slot][TK_NF]); their value is recorded as the
 * rejection value, which leaves the minimum and the head-wave test as the true value would.
 * Compacts items[0..n) in place and returns the number left. */
__device__ int filter_2d(const fd_station_dev &sd, const CtaSmem &cs, WarpSmem &ws, int n, int lane)
{
    int out = 0;
    for (int j0 = 0; j0 < n; j0 += 32) {
        const int j = j0 + lane;
        unsigned it = 0;
        bool keep = false;
        if (j < n) {
            it = ws.items[j];
            const int slot = (int)(it >> 5), K = (int)(it & 31);
            const TrialDesc &d = cs.desc[K];
            const float *t18 = ws.t[slot];
            const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], ws.s0[slot])),
                                   ws.s4[slot]);
            const float lo = lower_2d(d, t18, ws.s[slot], sd.g, ws.z[slot], ws.y[slot], fl);
            if (bound_prunes(lo, ws.res[slot][TK_NF]))
                ws.res[slot][K] = 1.e11;
            else
                keep = true;
        }
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        if (keep) ws.items[out + __popc(b & ((1u << lane) - 1u))] = (unsigned short)it;
        out += __popc(b);
    }
    return out;
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
        return vload(sd.T[((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0]]);
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

/* append e to a queue with tail counter `tail`; a position past the capacity (a node queued more
 * often than the walk allows) is refused */
__device__ __forceinline__ void enqueue_to(int *queue, int &tail, int cap, Shared &sh, int e)
{
    const int pos = atomicAdd(&tail, 1);
    if (pos < cap)
        queue[pos] = e;
    else
        atomicCAS(&sh.status, 0, 10);
}

__device__ __forceinline__ void enqueue(int *queue, Shared &sh, int e) { enqueue_to(queue, sh.qtail, sh.qcap, sh, e); }

/* node (plane pp, fill index i) is final: record (last plane), release its later in-plane
 * neighbours and the plane pp+1 nodes whose inner block contains it */
__device__ void pipelined_release(const fd_station_dev &sd, Shared &sh, int i, int pp, bool writer, float st0,
                                  float st4, float tin)
{
    const int nplane = sh.n, nvf = sh.n / sh.nuf, iu = i % sh.nuf, iv = i / sh.nuf;
    const fdn_frame fr = frame_of(sh.face);
    if (pp == sh.np - 1) {
        if (writer) {
            sd.scr.rec[i] = make_float2(st0, st4);
            atomicMax(&sh.exitkey, node_key(tin, i));
        } else {
            sd.scr.rec[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        }
    }
    __threadfence_block();
    const long long base = (long long)pp * nplane;
    unsigned later = inrect_mask(iu, iv, sh.nuf, nvf) & ~(unsigned)sd.scr.pemask[base + i];
    while (later) {
        const int k = __ffs(later) - 1;
        later &= later - 1;
        int du, dv;
        nb_off(k, du, dv);
        const int j = (iv + dv) * sh.nuf + iu + du;
        const unsigned old = atomicSub(&sd.scr.pcount[base + j], 1u << 8);
        if (old == (1u << 8)) enqueue(sd.scr.pqueue, sh, (int)(base + j));
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
                __threadfence_block();
                const unsigned lat = (unsigned)__popc(inrect_mask(ju, jv, sh.nuf, nvf) & ~em);
                const unsigned w = old - 1u;
                const unsigned prev = lat ? atomicSub(&sd.scr.pcount[nb + j], lat << 8) : w;
                if (prev - (lat << 8) == 0u) enqueue(sd.scr.pqueue, sh, (int)(nb + j));
            }
    }
}

/* face walk: node i is final; mark it done and release its later in-face neighbours */
__device__ void face_release(const fd_station_dev &sd, Shared &sh, unsigned char *dag, int i, bool writer,
                             float st0, float st4)
{
    if (writer) {
        sd.scr.rec[i] = make_float2(st0, st4);
        atomicMax(&sh.exitkey, sd.scr.key[i]);
    } else {
        sd.scr.rec[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    }
    __threadfence_block();
    /* done; a point waiting for the stencil state left before it resumes its search */
    const int waiter = atomicExch(&sd.scr.pst[i], -2);
    if (waiter >= 0) enqueue_to(sd.scr.rq, sh.rqtail, sh.rqcap, sh, waiter);
    const int nvf = sh.n / sh.nuf, iu = i % sh.nuf, iv = i / sh.nuf;
    const unsigned char *emask = dag + sh.n_pad;
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
        if (((old >> sh8) & 0xFFu) == 1u) enqueue(sd.scr.queue, sh, j);
    }
}

/* The reference's sequential minimum over the 22 trials of one node, from the values computed
 * by the warp (new-edge and new-face values that were not precomputed are evaluated here — they
 * are needed only at first contact), then the commit (src/sphfd.c:1756-1760), the node's
 * stencil-state record and the release of the nodes that wait on it.
 *
 * `permissive`: the node makes no writer call before its 2-D trials, so those test against a
 * stencil state left by an earlier point; their values were computed with no stale floor.  A
 * stale floor can only turn a 2-D value into the rejection value, so if no 2-D value lowered
 * the running minimum the result is the one the true state gives and the node commits; else it
 * returns false without committing. */
__device__ bool commit_node(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int slot, int i,
                            int pp, long long pT, unsigned gm, unsigned em, float it0, float it4, bool permissive,
                            unsigned char *dag, Counters &cn)
{
    const float *t18 = ws.t[slot], *s18 = ws.s[slot];
    const double told = f2d(t18[NB_POINT]);
    const int z = ws.z[slot], y = ws.y[slot];
    double guess = told;
    float st0 = it0, st4 = it4;
    int writers = 0;
    bool gate = false, win2d = false;
    int lastK = -1;
    double last_gb = 0.0, last_v = 0.0;
#pragma unroll 1
    for (int K = 0; K < FDN_NTRIAL; K++) {
        /* the first-contact tests are made on entry to their blocks (src/sphfd.c:1375, :1698) */
        if (K == TK_NE0 || K == TK_NF) gate = lt(1.0e9, guess);
        if (!((gm >> K) & 1u)) continue;
        const TrialDesc &d = cs.desc[K];
        const bool ev = (em >> K) & 1u;
        double v;
        if (K < TK_2D0 || K == TK_NF) {
            /* corner, new-edge, new-face: writers of the stencil state */
            if (K >= TK_NE0 && !gate) continue;
            st0 = t18[d.slot[0]];
            st4 = t18[d.slot[4]];
            writers++;
            if (ev) {
                v = ws.res[slot][K];
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
        } else {
            if (!ev) continue;
            v = ws.res[slot][K];
            if (K < TK_NF && lt(v, guess)) win2d = true;
        }
        if (lt(v, guess)) {
            if (d.head) { lastK = K; last_gb = guess; last_v = v; }
            guess = v;
        }
    }
    if (permissive && win2d) return false;
    if (lt(guess, told)) {
        sd.T[pT] = __double2float_rn(guess);
        if (lastK >= 0) {
            /* only the last head trial that lowered the minimum sets the measure that is tested */
            const double fhead = (last_gb - last_v) / head_den(cs.desc[lastK], s18, sd.g, z, y);
            if (fhead > FD_HEADTEST) atomicAdd(&sh.headw[frame_of(sh.face).headw], 1);
        }
    }
    if (sh.pipelined)
        pipelined_release(sd, sh, i, pp, writers != 0, st0, st4, t18[13]);
    else
        face_release(sd, sh, dag, i, writers != 0, st0, st4);
    return true;
}

/* Evaluate and commit one chunk: lane l holds queue entry e (-1 for none).  A node given with
 * have_inherit uses (it0, it4) as the stencil state entering it.  All 32 lanes call. */
__device__ void warp_chunk(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int e,
                           bool have_inherit, float it0, float it4, unsigned char *dag, Counters &cn)
{
    const int lane = threadIdx.x & 31;
    const bool valid = e >= 0;
    const fdn_frame fr = frame_of(sh.face);
    int i = 0, pp = -1;
    long long pT = 0;
    unsigned gm = 0, em = 0;
    bool permissive = false;
    FD_TIC(ta);
    if (valid) {
        /* entries: fill indices, or plane * n + fill index in a pipelined sweep */
        int layer = sh.layer;
        if (sh.pipelined) {
            pp = e / sh.n;
            i = e - pp * sh.n;
            layer = sh.player0 - pp * fr.inner;
        } else {
            i = e;
        }
        const int u = sh.ulo + i % sh.nuf, v = sh.vlo + i / sh.nuf;
        int xyz[3];
        xyz[fr.axis_u] = u;
        xyz[fr.axis_v] = v;
        xyz[fr.axis_n] = layer;
        pT = ((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0];
        const long long pS = (long long)xyz[2] * sd.s_sz + (long long)xyz[1] * sd.s_sy + xyz[0];
        ws.z[lane] = xyz[2];
        ws.y[lane] = xyz[1];
        float *tr = ws.t[lane], *sr = ws.s[lane];
        const long long inner_t = (long long)fr.inner * sh.sn, inner_s = (long long)fr.inner * sh.ssn;
#pragma unroll
        for (int nb = 0; nb < NB_N; nb++) {
            const int w = nb / 9, dv = (nb / 3) % 3 - 1, du = nb % 3 - 1;
            const int uu = u + du, vv = v + dv;
            float tv = 0.f, svv = 0.f;
            if (uu >= 0 && uu < sh.nu && vv >= 0 && vv < sh.nv) {
                tv = sd.T[pT + du * sh.su + dv * sh.sv + (w ? inner_t : 0ll)];
                svv = __ldg(&sd.S[pS + du * sh.ssu + dv * sh.ssv + (w ? inner_s : 0ll)]);
            }
            tr[nb] = tv;
            sr[nb] = svv;
        }
        guards(sh.face, tr, rect_of(sh, i), gm, em);
        /* a 2-D trial before any corner / new-edge call reads the state an earlier point left */
        const double told = f2d(tr[NB_POINT]);
        permissive = !have_inherit && (gm & 0xFu) == 0 && !((gm & 0xF0u) && told > 1.0e9) && (gm & 0xFF00u);
    }
    __syncwarp();
    int n1 = push_items(ws.items, 0, em, TK_3D0, TK_2D0, lane);
    n1 = push_items(ws.items, n1, em, TK_1D0, FDN_NTRIAL, lane);
    __syncwarp();
    FD_TOC(1, ta);
    FD_TIC(tb);
    eval_items(sd, cs, ws, n1, lane, cn);
    __syncwarp();
    const float lo = __int_as_float(0xff800000);   /* -inf: no stale floor */
    const float p0 = permissive ? lo : it0, p4 = permissive ? lo : it4;
    if (valid) em |= stale_pair(cs, ws, lane, gm, em, p0, p4);
    __syncwarp();
    int n2 = push_items(ws.items, 0, em, TK_2D0, TK_NF, lane);
    __syncwarp();
    n2 = filter_2d(sd, cs, ws, n2, lane);
    __syncwarp();
    eval_items(sd, cs, ws, n2, lane, cn);
    __syncwarp();
    FD_TOC(2, tb);
    FD_TIC(tc);
    bool fin = false;
    if (valid) {
        fin = commit_node(sd, sh, cs, ws, lane, i, pp, pT, gm, em, p0, p4, permissive, dag, cn);
        if (!fin) {
            if (sh.pipelined) {
                atomicCAS(&sh.status, 0, 6);   /* excluded by the pipelining precondition */
            } else {
                atomicAdd(reinterpret_cast<unsigned long long *>(&sh.deferred), 1ull);
                enqueue_to(sd.scr.rq, sh.rqtail, sh.rqcap, sh, e);
            }
        }
    }
    const unsigned done = __ballot_sync(0xffffffffu, fin);
    if (lane == 0 && done) {
        __threadfence_block();
        atomicAdd(&sh.ndone, __popc(done));
    }
    __syncwarp();
    FD_TOC(3, tc);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long x)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
        x = y > x ? y : x;
    }
    return x;
}

/* the face point that precedes point c in sort order (largest key below c's), -1 if none */
__device__ int predecessor(const fd_station_dev &sd, int n, int c, int lane)
{
    const unsigned long long kc = sd.scr.key[c];
    unsigned long long best = 0ull;   /* every key is above 0: times are not negative */
    int j = lane;
    for (; j + 96 < n; j += 128) {
        const unsigned long long k0 = sd.scr.key[j], k1 = sd.scr.key[j + 32];
        const unsigned long long k2 = sd.scr.key[j + 64], k3 = sd.scr.key[j + 96];
        if (k0 < kc && k0 > best) best = k0;
        if (k1 < kc && k1 > best) best = k1;
        if (k2 < kc && k2 > best) best = k2;
        if (k3 < kc && k3 > best) best = k3;
    }
    for (; j < n; j += 32) {
        const unsigned long long k = sd.scr.key[j];
        if (k < kc && k > best) best = k;
    }
    best = warp_max_u64(best);
    return best ? (int)(best & 0xffffffffu) : -1;
}

/* Point w needs the stencil state left by the last point before it in sort order that made a
 * writer call.  Walk back through the sort order: a done writer gives its record; a done
 * non-writer passes the search to its predecessor; a point not yet done takes w as its waiter and
 * queues it again when it finishes (a point has at most one waiter: waiters lie between it and the
 * next pending point).  Before the face's first point the state is the one the face started with.
 * Keys fall along the walk, so waits cannot form a cycle.  One warp; evaluates w when found. */
__device__ void resume_waiter(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int w,
                              unsigned char *dag, Counters &cn)
{
    const int lane = threadIdx.x & 31;
    int c = w;
    for (int guard = 0; guard <= 2 * sh.n + 2; guard++) {
        const int p = predecessor(sd, sh.n, c, lane);
        int verdict = 0;   /* 0 continue from p, 1 found (t0,t4), 2 waiting, 3 retry p */
        float t0 = sh.carry_t0, t4 = sh.carry_t4;
        if (lane == 0) {
            if (p < 0) {
                verdict = 1;
            } else {
                int st = vload(sd.scr.pst[p]);
                if (st != -2) {
                    const int old = atomicCAS(&sd.scr.pst[p], -1, w);
                    if (old == -1) verdict = 2;
                    else if (old == -2) verdict = 3;
                    else { atomicCAS(&sh.status, 0, 11); verdict = 2; }   /* a second waiter */
                    st = old;
                }
                if (verdict == 0 || verdict == 3) {
                    __threadfence_block();
                    const float r0 = vload(sd.scr.rec[p].x), r4 = vload(sd.scr.rec[p].y);
                    if (!isnan(r0)) { verdict = 1; t0 = r0; t4 = r4; }
                    else verdict = 0;
                }
            }
        }
        verdict = __shfl_sync(0xffffffffu, verdict, 0);
        if (verdict == 2) return;
        if (verdict == 1) {
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            t4 = __shfl_sync(0xffffffffu, t4, 0);
            warp_chunk(sd, sh, cs, ws, lane == 0 ? w : -1, true, t0, t4, dag, cn);
            return;
        }
        c = p;
    }
    if (lane == 0) atomicCAS(&sh.status, 0, 12);
}

/* nothing queued, every worker idle, and both queues unchanged across the idle count (lane 0) */
__device__ __forceinline__ bool quiescent(Shared &sh)
{
    const int t0 = vload(sh.qtail), h0 = vload(sh.qhead), r0 = vload(sh.rqtail), g0 = vload(sh.rqhead);
    if (h0 != t0 || r0 != g0) return false;
    __threadfence_block();
    if (vload(sh.idle) != FD_WARPS) return false;
    __threadfence_block();
    return vload(sh.qtail) == t0 && vload(sh.qhead) == t0 && vload(sh.rqtail) == r0 && vload(sh.rqhead) == r0;
}

/* claim one entry of a queue (lane 0): spins briefly for an entry whose writer is between its two
 * instructions; -1 and a status on failure */
__device__ __forceinline__ int read_entry(const int *queue, int pos, Shared &sh)
{
    const volatile int *q = queue + pos;
    int e = *q;
    for (int spin = 0; e < 0 && spin < FD_QSPIN; spin++) {
        __nanosleep(32);
        e = *q;
    }
    if (e < 0) atomicCAS(&sh.status, 0, 9);   /* a claimed entry never written */
    return e;
}

/* the worker loop of one walk over `total` nodes; all warps call it between two CTA barriers */
__device__ void run_walk(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int *queue,
                         int total, unsigned char *dag, Counters &cn)
{
    const int lane = threadIdx.x & 31;
    bool idle = false;
    long long since = clock64();
    long long chunks = 0;
    for (;;) {
        int act = 0, h = 0, m = 0;   /* act: 0 wait, 1 chunk, 2 resume a waiter, 3 leave */
        if (lane == 0) {
            if (vload(sh.status) != 0 || vload(sh.ndone) >= total) {
                act = 3;
            } else {
                const int rh = vload(sh.rqhead), rt0 = vload(sh.rqtail), rt = rt0 < sh.rqcap ? rt0 : sh.rqcap;
                const int head = vload(sh.qhead), qt = vload(sh.qtail), tail = qt < sh.qcap ? qt : sh.qcap;
                if (rh < rt) {
                    if (idle) { atomicSub(&sh.idle, 1); idle = false; }
                    if (atomicCAS(&sh.rqhead, rh, rh + 1) == rh) { act = 2; h = read_entry(sd.scr.rq, rh, sh); }
                } else if (head < tail && (sh.pipelined || (int)(threadIdx.x >> 5) < FD_FACE_WARPS)) {
                    if (idle) { atomicSub(&sh.idle, 1); idle = false; }
                    const int want = tail - head < 32 ? tail - head : 32;
                    if (atomicCAS(&sh.qhead, head, head + want) == head) { act = 1; h = head; m = want; }
                } else {
                    if (!idle) { __threadfence_block(); atomicAdd(&sh.idle, 1); idle = true; }
                    /* all idle with nothing queued and nodes left: nothing can release them */
                    if (quiescent(sh) && vload(sh.ndone) < total) {
                        atomicCAS(&sh.status, 0, 3);
                        act = 3;
                    }
                }
                if (act == 1 || act == 2) {
                    since = clock64();
                } else if (act == 0 && clock64() - since > FD_WAIT_CYCLES) {
                    atomicCAS(&sh.status, 0, 8);   /* no work for this worker for too long */
                    act = 3;
                }
            }
        }
        act = __shfl_sync(0xffffffffu, act, 0);
        if (act == 3) break;
        h = __shfl_sync(0xffffffffu, h, 0);
        if (act == 1) {
            m = __shfl_sync(0xffffffffu, m, 0);
            int e = -1;
            if (lane < m) {
                const volatile int *q = queue + h + lane;
                e = *q;
                for (int spin = 0; e < 0 && spin < FD_QSPIN; spin++) {
                    __nanosleep(32);
                    e = *q;
                }
                if (e < 0) atomicCAS(&sh.status, 0, 9);   /* a claimed entry never written */
            }
            __threadfence_block();
            warp_chunk(sd, sh, cs, ws, e, false, 0.f, 0.f, dag, cn);
            chunks++;
            continue;
        }
        if (act == 2) {
            __threadfence_block();
            if (h >= 0) resume_waiter(sd, sh, cs, ws, h, dag, cn);
            continue;
        }
        __nanosleep(64);
    }
    if (lane == 0 && chunks) atomicAdd(reinterpret_cast<unsigned long long *>(&sh.rounds), (unsigned long long)chunks);
}

/* Walk the current face (parameters in sh) in dependency order. */
__device__ void face_walk(const fd_station_dev &sd, Shared &sh, CtaSmem &cs, WarpSmem &ws, unsigned char *dag,
                          Counters &cn)
{
    const int n = sh.n, nuf = sh.nuf, nvf = n / nuf;
    const int tid = threadIdx.x;
    const float *T = sd.T;
    const fdn_frame fr = frame_of(sh.face);
    unsigned char *emask = dag + sh.n_pad;
    int *queue = sd.scr.queue;
    FD_TIC(t0);
    /* trial descriptors of this face */
    for (int k = tid; k < FDN_NTRIAL; k += blockDim.x) cs.desc[k] = c_desc[sh.face * FDN_NTRIAL + k];
    /* keys: time of the inner-layer neighbour, then fill index */
    for (int i = tid; i < n; i += blockDim.x) {
        int xyz[3];
        xyz[fr.axis_u] = sh.ulo + i % nuf;
        xyz[fr.axis_v] = sh.vlo + i / nuf;
        xyz[fr.axis_n] = sh.layer + fr.inner;
        const float tin = T[((long long)xyz[2] * sd.g.ny + xyz[1]) * sd.g.nx + xyz[0]];
        sd.scr.key[i] = ((unsigned long long)okey32(tin) << 32) | (unsigned)i;
        sd.scr.pst[i] = -1;
        queue[i] = -1;
        sd.scr.rq[2 * i] = -1;
        sd.scr.rq[2 * i + 1] = -1;
    }
    if (tid == 0) {
        sh.qhead = sh.qtail = sh.rqhead = sh.rqtail = sh.idle = sh.ndone = 0;
        sh.qcap = n;
        sh.rqcap = 2 * n;
        sh.exitkey = 0ull;
    }
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
        if (em == 0) enqueue(queue, sh, i);
    }
    __syncthreads();
    FD_TOC(0, t0);
    FD_TIC(tw);
    run_walk(sd, sh, cs, ws, queue, n, dag, cn);
    __syncthreads();
    FD_TOC(4, tw);
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
__device__ void pipelined_sweep(const fd_station_dev &sd, Shared &sh, CtaSmem &cs, WarpSmem &ws, Counters &cn, int F)
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
        sh.qhead = sh.qtail = sh.rqhead = sh.rqtail = sh.idle = sh.ndone = 0;
        sh.qcap = (int)((long long)np * sh.n);
        sh.rqcap = 0;
        sh.exitkey = 0ull;
        sh.pipelined = 1;
    }
    for (int k = tid; k < FDN_NTRIAL; k += blockDim.x) cs.desc[k] = c_desc[F * FDN_NTRIAL + k];
    __syncthreads();
    const int np = sh.np, nplane = sh.n, nuf = sh.nuf, nvf = nplane > 0 ? nplane / nuf : 0;
    const long long total = (long long)np * nplane;
    if (total > 0) {
        for (long long id = tid; id < total; id += blockDim.x) sd.scr.pqueue[id] = -1;
        __syncthreads();
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
            if (wd == 0u) enqueue(sd.scr.pqueue, sh, (int)id);
        }
        __syncthreads();
        run_walk(sd, sh, cs, ws, sd.scr.pqueue, (int)total, nullptr, cn);
        __syncthreads();
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
    CtaSmem &cs = *reinterpret_cast<CtaSmem *>(fd_dyn_smem);
    WarpSmem &ws = reinterpret_cast<WarpSmem *>(fd_dyn_smem + kCtaSmemBytes)[threadIdx.x >> 5];
    if ((int)blockIdx.x >= nst) return;
    const fd_station_dev &sd = stations[blockIdx.x];
    const int tid = threadIdx.x;
    unsigned long long t_start = 0;
    if (tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    /* the dependency bytes of the station's largest face go to shared memory when they fit */
    unsigned char *dag = 2ll * sd.max_face_pad <= dag_smem_bytes ? fd_dyn_smem + kSmemBase : sd.scr.dag;
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
        FD_TIC(tsweep);
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
        if (piped) pipelined_sweep(sd, sh, cs, ws, cn, act);
        while (!piped && sh.rad0
               && (sh.dflag[0] || sh.dflag[1] || sh.dflag[2] || sh.dflag[3] || sh.dflag[4] || sh.dflag[5])
               && sh.status == 0) {
            for (int face = 0; face < 6; face++) {
                for (int ig = 1; ig <= sd.grow[face]; ig++) {
                    if (!sh.dflag[face]) continue;
                    if (tid == 0) setup_face(sd, sh, face);
                    __syncthreads();
                    if (sh.n > 0) face_walk(sd, sh, cs, ws, dag, cn);
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
            if (sh.sweeps == 0) FD_TOC(5, tsweep);   /* profiling builds: the first sweep's cycles */
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
        o->pipelined_sweeps = (int32_t)sh.psweeps;
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
    const long long base = (long long)fdk::kSmemBase;
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
