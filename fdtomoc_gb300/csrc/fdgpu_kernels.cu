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
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fdgpu_eval.cuh"
#include "fdgpu_trials.cuh"
#include "fdgpu_bound.cuh"
#include "fdgpu_layout.h"

#define FD_WARPS 12                 /* independent workers per station */
/* Largest cluster of CTAs one station may use.  Multi-CTA solving (the walk state shared through
 * distributed shared memory) passed the bit-exactness tests but hung or faulted intermittently on
 * this GPU; until the cause is found every station runs on one CTA. */
#ifndef FD_MAX_CLUSTER
#define FD_MAX_CLUSTER 1
#endif
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

/* state of the current walk that all CTAs of a station's cluster share; it lives in the shared
 * memory of the cluster's first CTA and the others reach it through distributed shared memory */
struct WalkShared {
    /* ready queues (one per face in a sweep graph; a face walk uses queue 0), the queue of points
     * resuming a search for an inherited stencil state, idle workers, finished nodes, parked points
     * and wait pairs */
    int nq;
    int qhead[6], qtail[6], qcap[6], qbase[6];
    int rqhead, rqtail, rqcap, idle, ndone, npark, nwait;
    int status;
    int headw[8];
    unsigned long long exitkey;
    long long rounds, deferred;
    unsigned long long st[5];
    int bar_count;            /* cluster barrier: arrivals so far */
};

struct Shared {
    WalkShared wl;
    WalkShared *w;           /* the cluster's shared walk state (wl of rank 0) */
    int cs, rank;            /* CTAs per station, this CTA's rank */
    int stat;                /* the station's status as this CTA read it at its last barrier */
    int wall[6], dflag[6];
    int radius, rad0, reverse, headpref;
    float carry_t0, carry_t4;
    /* current face of a face walk */
    int face, layer, ulo, uhi, vlo, vhi, nuf, n, n_pad;
    long long su, sv, sn, ssu, ssv, ssn;
    int nu, nv;
    /* current sweep graph: on/off, face instances, points; per face, the 27-bit masks of the
     * neighbour offsets a node of that face reads, and of those in its inner plane */
    int graph, gok, ninst, single, nodefer;
    unsigned gfaces;
    long long gM;
    unsigned ctxm[6], innm[6];
    void *gsm;
    unsigned long long red[FD_BLOCK / 32];
    unsigned long long bcast;
    /* statistics */
    long long faces, node_updates;
    int sweeps;
    int restart_wall[8];
    long long cyc[6];
    long long gsweeps;
};

/* ordering of a worker's global and shared stores before the counters that publish them, at the
 * scope of the CTAs that share the walk */
__device__ __forceinline__ void wfence(const Shared &sh)
{
    if (sh.cs > 1)
        asm volatile("fence.acq_rel.cluster;" ::: "memory");
    else
        __threadfence_block();
}

#ifndef FD_BAR_SPINS
#define FD_BAR_SPINS (1ll << 26)   /* polls (about 64 ns apart) before a cluster barrier gives up */
#endif

/* Barrier of all threads of the station's CTAs: the CTA's threads meet, its thread 0 meets the other
 * CTAs' at an arrival counter in the first CTA's shared memory that only grows (barrier k is passed
 * once it reaches (k+1) * CTAs, so no arrival can be lost to a reset).  The wait is bounded: a CTA
 * that waits too long records which barrier (site) gave up in the station's status and goes on, so
 * a fault in the schedule ends in an error, never in a hang.  Thread 0 then takes the station's
 * status for the whole CTA (sh.stat), so every branch that depends on it is taken by all threads. */
__device__ __forceinline__ void csync(Shared &sh, int site)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        if (sh.cs > 1) {
            asm volatile("fence.acq_rel.cluster;" ::: "memory");
            const int my = atomicAdd(&sh.w->bar_count, 1);
            const int target = (my / sh.cs + 1) * sh.cs;
            long long spins = 0;
            while (*const_cast<volatile int *>(&sh.w->bar_count) < target) {
                __nanosleep(64);
                if (++spins > FD_BAR_SPINS) {
                    atomicCAS(&sh.w->status, 0, 100 + site);
                    break;
                }
            }
            asm volatile("fence.acq_rel.cluster;" ::: "memory");
        }
        sh.stat = *const_cast<volatile int *>(&sh.w->status);
    }
    __syncthreads();
}

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

/* stencil evaluations by kind (3-D, new-edge, 2-D, new-face, 1-D): the warp's counts in its
 * shared area, passed by value (a pointer), so that no per-thread memory is involved */
struct Counters {
    unsigned long long *n;
};

__device__ __forceinline__ void count_eval(Counters cn, int kind) { atomicAdd(&cn.n[kind], 1ull); }

/* coordinate of node (x,y,z) along a grid axis, and a node placed from face coordinates: selects on
 * registers (arrays indexed by a run-time axis would live in per-thread local memory, whose L1 lines
 * this kernel's large shared-memory carve-out leaves little room for) */
__device__ __forceinline__ int coord(int axis, int x, int y, int z) { return axis == 0 ? x : axis == 1 ? y : z; }

__device__ __forceinline__ void place(const fdn_frame &fr, int u, int v, int n, int &x, int &y, int &z)
{
    x = fr.axis_u == 0 ? u : fr.axis_v == 0 ? v : n;
    y = fr.axis_u == 1 ? u : fr.axis_v == 1 ? v : n;
    z = fr.axis_u == 2 ? u : fr.axis_v == 2 ? v : n;
}

/* ---------------------------------------------------------------------------------------------- */
/* warp workers                                                                                    */
/*                                                                                                 */
/* A walk — one face, or a whole sweep as one graph — is a dependency graph whose ready nodes sit   */
/* in queues.  Every warp of the CTA is an independent worker: it claims up to 32 ready nodes of    */
/* one face direction, evaluates them (one lane per node for the per-node steps, the stencil       */
/* trials of all its nodes spread over the 32 lanes), commits them and queues the nodes they       */
/* complete.  Warps meet only at shared-memory counters, so the FP64 work of some warps hides the  */
/* memory and control latency of the others, and a node starts as soon as its own inputs are      */
/* final.                                                                                          */
/*                                                                                                 */
/* Queues: positions are taken with an atomic on the tail and written after; every entry starts as */
/* -1, so a worker that claimed a position not yet written waits for it (briefly: the writer is    */
/* between two instructions).  Stores of a node's time and of its queue entries are ordered by     */
/* __threadfence_block before the counters that publish them.  Every wait is bounded: a worker     */
/* idle for FD_WAIT_CYCLES without progress sets the station's status and all workers leave the   */
/* walk; all idle with nothing queued and nodes left is reported the same way.                    */

#define NB_PAD 19                    /* context row stride: the 32 rows fall on distinct banks */
#define FD_WAIT_CYCLES (4ll << 30)   /* about 2 s at the maximum SM clock */
#ifndef FD_WALK_CYCLES
#define FD_WALK_CYCLES (1ll << 37)   /* about 66 s: no walk of a real grid comes near it */
#endif
#define FD_QSPIN (1 << 22)           /* polls of an unwritten queue entry before giving up */
#define FD_KEYED 0x80000000u         /* counter word: the node's sort key is final */

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

/* shared by the CTA: the trial descriptors of all six faces */
struct CtaSmem {
    TrialDesc desc[FDN_NFACE][FDN_NTRIAL];
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
    unsigned long long cnt[6];             /* stencil evaluations by kind (5 used) */
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
__device__ __forceinline__ bool prunable(float fl, double g) { return !lt(f2d(fl), g) && !lt(1.e11, g); }

struct Rect {
    int u, v, nu, nv, ulo, uhi, vlo, vhi;
};

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
                if (lt(f2d(floor_of<F, K>(t18)), g0)) em |= 1u << K;
            } else if constexpr (tr.kind == FDN_NE) {
                if (!any3d && lt(1.0e9, g0) && !prunable(floor_of<F, K>(t18), g0)) em |= 1u << K;
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
__device__ void eval_items(const fd_station_dev &sd, const TrialDesc *dsc, WarpSmem &ws, int n, int lane, Counters cn)
{
    for (int j = lane; j < n; j += 32) {
        const unsigned it = ws.items[j];
        const int slot = (int)(it >> 5), K = (int)(it & 31);
        const TrialDesc &d = dsc[K];
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
            if ((__double_as_longlong(x1) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) {   /* NaN: no root */
                v = 1.e11;
            } else {
                const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], ws.s0[slot])),
                                       ws.s4[slot]);
                const double f = f2d(fl);
                const bool bad1 = flt(x1, f), bad2 = flt(x2, f);
                v = bad1 ? (bad2 ? 1.e11 : x2) : (bad2 ? x1 : (flt(x2, x1) ? x2 : x1));
            }
            break;
        }
        case 3: v = eval_nf(d, t18, s18, sd.g, z, y); break;
        default: v = eval_1d(d, t18, s18, sd.g, z, y); break;
        }
        ws.res[slot][K] = v;
        count_eval(cn, kind);
    }
}

/* Replay of the corner and new-edge trials (every writer of the stencil state comes before the
 * 2-D block): the running minimum entering the 2-D block — an upper bound for every 2-D trial's
 * turn — and the stale (t0,t4) those trials test against.  Returns the 2-D trials that can still
 * lower the minimum. */
__device__ unsigned stale_pair(const TrialDesc *dsc, WarpSmem &ws, int slot, unsigned gm, unsigned em, float it0,
                               float it4)
{
    const float *t18 = ws.t[slot];
    double g1 = f2d(t18[NB_POINT]);
    float s0 = it0, s4 = it4;
    for (int K = 0; K < TK_NE0; K++) {
        if (!((gm >> K) & 1u)) continue;
        s0 = t18[dsc[K].slot[0]];
        s4 = t18[dsc[K].slot[4]];
        if ((em >> K) & 1u) {
            const double v = ws.res[slot][K];
            if (lt(v, g1)) g1 = v;
        }
    }
    const bool gate = lt(1.0e9, g1);
    for (int K = TK_NE0; K < TK_2D0; K++) {
        if (!gate || !((gm >> K) & 1u)) continue;
        s0 = t18[dsc[K].slot[0]];
        s4 = t18[dsc[K].slot[4]];
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
        const TrialDesc &d = dsc[K];
        const float fl = fmaxf(fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), fmaxf(t18[d.slot[3]], s0)), s4);
        if (!prunable(fl, g1)) add |= 1u << K;
    }
    return add;
}

/* Drop the queued 2-D items whose single-precision lower bound shows they cannot lower the
 * running minimum entering the 2-D block (kept in res[slot][TK_NF]); their value is recorded as the
 * rejection value, which leaves the minimum and the head-wave test as the true value would.
 * Compacts items[0..n) in place and returns the number left. */
__device__ int filter_2d(const fd_station_dev &sd, const TrialDesc *dsc, WarpSmem &ws, int n, int lane)
{
    int out = 0;
    for (int j0 = 0; j0 < n; j0 += 32) {
        const int j = j0 + lane;
        unsigned it = 0;
        bool keep = false;
        if (j < n) {
            it = ws.items[j];
            const int slot = (int)(it >> 5), K = (int)(it & 31);
            const TrialDesc &d = dsc[K];
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
/* node addressing                                                                                 */

__device__ __forceinline__ unsigned long long node_key(float tin, int i)
{
    return ((unsigned long long)okey32(tin) << 32) | (unsigned)i;
}

/* grid extent and node strides of the time field and of the slowness model along an axis */
__device__ __forceinline__ int axis_len(const fd_station_dev &sd, int a) { return a == 0 ? sd.g.nx : a == 1 ? sd.g.ny : sd.g.nz; }
__device__ __forceinline__ long long t_stride(const fd_station_dev &sd, int a)
{
    return a == 0 ? 1ll : a == 1 ? (long long)sd.g.nx : (long long)sd.g.nx * sd.g.ny;
}
__device__ __forceinline__ long long s_stride(const fd_station_dev &sd, int a) { return a == 0 ? 1ll : a == 1 ? sd.s_sy : sd.s_sz; }

/* where a node sits: grid index, coordinates, face rectangle, fill index */
struct Where {
    long long p;
    int x, y, z;
    int i;       /* fill index in its face (instance) */
    int inst;    /* face instance of a sweep graph, -1 in a face walk */
    Rect r;
};

/* append e to a queue with tail counter `tail`; a position past the capacity (a node queued more
 * often than the walk allows) is refused */
__device__ __forceinline__ void enqueue_to(int *queue, int &tail, int cap, Shared &sh, int e)
{
    const int pos = atomicAdd(&tail, 1);
    if (pos < cap)
        *const_cast<volatile int *>(&queue[pos]) = e;   /* a strong store: readers synchronise on it */
    else
        atomicCAS(&sh.w->status, 0, 10);
}

/* ---------------------------------------------------------------------------------------------- */
/* face walks (one face at a time; used when the sweep-graph arrays are not available)             */

/* face walk: node i is final; mark it done and release its later in-face neighbours */
__device__ void face_release(const fd_station_dev &sd, Shared &sh, unsigned char *dag, int i, bool writer,
                             float st0, float st4)
{
    if (writer) {
        sd.scr.rec[i] = make_float2(st0, st4);
        atomicMax(&sh.w->exitkey, sd.scr.key[i]);
    } else {
        sd.scr.rec[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    }
    wfence(sh);
    /* done; a point waiting for the stencil state left before it resumes its search */
    const int waiter = atomicExch(&sd.scr.pst[i], -2);
    if (waiter >= 0) enqueue_to(sd.scr.rq, sh.w->rqtail, sh.w->rqcap, sh, waiter);
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
        if (((old >> sh8) & 0xFFu) == 1u) enqueue_to(sd.scr.queue, sh.w->qtail[0], sh.w->qcap[0], sh, j);
    }
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long x)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
        x = y > x ? y : x;
    }
    return x;
}

/* ---------------------------------------------------------------------------------------------- */
/* sweep graphs                                                                                    */
/*                                                                                                 */
/* A whole sweep runs as one dependency graph.  Which face instance (a face at one wall position)  */
/* computes which node depends only on the walls, not on times, so the sweep's schedule of face    */
/* instances is simulated first; a node's owner then follows from two small shared-memory tables  */
/* (the instance of each face at each layer, and each instance's rectangle).  A node reads its     */
/* own-plane 3x3 block and the 3x3 block of its inner layer.  For each pair of nodes where one     */
/* reads the other and their owners differ, the earlier-owned one must finish first: the reader    */
/* needs its new value, or it must read the other's old one.  Within one face instance the order   */
/* is the sort order of the inner-layer times, known once a node's inner block is final (its inner */
/* block holds the inner nodes of all its in-face neighbours).  Every node keeps one counter word: */
/* inner block pending (bits 0-7), same-instance neighbours pending (8-15), other-instance nodes    */
/* pending (16-23), a point waits on it (bit 29), done (bit 30), key final (bit 31).  After a      */
/* restart (one face) this is a plane pipeline; in the forward sweep it lets all six faces and     */
/* successive wall positions advance together.                                                     */
/*                                                                                                 */
/* Inherited stencil state: a point whose 2-D trials need the state an earlier point left, and    */
/* whose result depends on it, waits for the last point before it (in the reference's order) that  */
/* made a writer call: the predecessor by key in its own instance once all keys there are final,   */
/* else the last writer of the nearest earlier instance once that instance is complete.  Waits    */
/* are registered on a point (a wait pair and the counter's wait bit) or on an instance event (all */
/* keys final, all points done; a parked-point entry).                                            */

#define FD_LMAX 1024                 /* largest grid extent a sweep graph handles */
#ifndef FD_GRAPH_FORWARD
#define FD_GRAPH_FORWARD 1           /* the first sweep as a graph too */
#endif
#define FD_IMAX 3088                 /* face instances: at most nx + ny + nz + 8 */
#define FD_WAITB 0x20000000u
#define FD_DONEB 0x40000000u

struct GRect {
    short face, layer, ulo, uhi, vlo, vhi, nuf, pad;
};

/* in the dynamic shared memory after the warp areas (the face walks' dependency bytes otherwise) */
struct GraphSmem {
    short lay2inst[FDN_NFACE][FD_LMAX];   /* instance of face f at layer l, -1 if none */
    GRect rect[FD_IMAX];
};

/* the warp areas and the sweep-graph tables fit one CTA's 227 KB, with 2 KB left for the static
 * shared memory of fd_solve */
static_assert(kSmemBase + sizeof(GraphSmem) + 2048 <= 227 * 1024, "shared memory of one CTA");

__device__ __forceinline__ GraphSmem &gsmem(const Shared &sh) { return *reinterpret_cast<GraphSmem *>(sh.gsm); }

/* Neighbour offsets (dx,dy,dz) are numbered k = (dz+1)*9 + (dy+1)*3 + (dx+1), 13 being the node
 * itself; the opposite offset is 26 - k.  An owner word holds (face << 24) | instance, -1 for a
 * node no instance of the sweep computes. */
__device__ __forceinline__ int own_inst(int w) { return w & 0xFFFFFF; }
__device__ __forceinline__ int own_face(int w) { return w >> 24; }

/* masks of the offsets a node of face f reads (own plane and inner plane) and of its inner plane */
__device__ void relation_masks(int f, unsigned &ctx, unsigned &inn)
{
    const fdn_frame fr = frame_of(f);
    ctx = 0;
    inn = 0;
    for (int k = 0; k < 27; k++) {
        if (k == 13) continue;
        const int on = coord(fr.axis_n, k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1);
        if (on == 0 || on == fr.inner) ctx |= 1u << k;
        if (on == fr.inner) inn |= 1u << k;
    }
}

__device__ __forceinline__ int rect_n(const GRect &r) { return r.nuf * (r.vhi - r.vlo + 1); }

/* owner word of node (x,y,z), which must lie in the grid */
__device__ __forceinline__ int owner_of(const GraphSmem &gs, unsigned faces, int x, int y, int z)
{
#pragma unroll
    for (int f = 0; f < 6; f++) {
        if (!((faces >> f) & 1u)) continue;
        const fdn_frame fr = frame_of(f);
        const int I = gs.lay2inst[f][coord(fr.axis_n, x, y, z)];
        if (I < 0) continue;
        const GRect &r = gs.rect[I];
        const int u = coord(fr.axis_u, x, y, z), v = coord(fr.axis_v, x, y, z);
        if (u >= r.ulo && u <= r.uhi && v >= r.vlo && v <= r.vhi) return (f << 24) | I;
    }
    return -1;
}

/* owner word of node (x,y,z) when face F is the likely owner: F's instance at the node's layer is
 * looked at first (one table entry and one rectangle), the full search only if it is not F's.  Each
 * node belongs to at most one instance of a sweep, so the answer is owner_of's. */
__device__ __forceinline__ int owner_near(const GraphSmem &gs, unsigned faces, int F, int x, int y, int z)
{
    const fdn_frame fr = frame_of(F);
    if ((faces >> F) & 1u) {
        const int I = gs.lay2inst[F][coord(fr.axis_n, x, y, z)];
        if (I >= 0) {
            const GRect &r = gs.rect[I];
            const int u = coord(fr.axis_u, x, y, z), v = coord(fr.axis_v, x, y, z);
            if (u >= r.ulo && u <= r.uhi && v >= r.vlo && v <= r.vhi) return (F << 24) | I;
        }
    }
    return owner_of(gs, faces, x, y, z);
}

/* node index of point j of instance r */
__device__ __forceinline__ long long inst_node(const fd_station_dev &sd, const GRect &r, int j)
{
    const fdn_frame fr = frame_of(r.face);
    int x, y, z;
    place(fr, r.ulo + j % r.nuf, r.vlo + j / r.nuf, r.layer, x, y, z);
    return ((long long)z * sd.g.ny + y) * sd.g.nx + x;
}

/* sort key of point j of instance r: time of its inner-layer node, then fill index */
__device__ __forceinline__ unsigned long long inst_key(const fd_station_dev &sd, const GRect &r, int j)
{
    const fdn_frame fr = frame_of(r.face);
    const long long p = inst_node(sd, r, j) + fr.inner * t_stride(sd, fr.axis_n);
    return node_key(vload(sd.T[p]), j);
}

/* fill index of node (x,y,z) in instance r */
__device__ __forceinline__ int inst_fill(const GRect &r, int x, int y, int z)
{
    const fdn_frame fr = frame_of(r.face);
    return (coord(fr.axis_v, x, y, z) - r.vlo) * r.nuf + (coord(fr.axis_u, x, y, z) - r.ulo);
}

/* points parked on instance I's event `kind` (1: all keys final, 2: all done) go to the resume queue */
__device__ void fire_event(const fd_station_dev &sd, Shared &sh, int I, int kind)
{
    wfence(sh);
    if (!(vload(sd.scr.ginst[I].evwait) & kind)) return;
    const int st = (kind << 24) | I;
    const int np = min(vload(sh.w->npark), FD_GPARK_CAP);
    for (int k = 0; k < np; k++) {
        if (vload(sd.scr.gpark[k].y) == st && atomicCAS(&sd.scr.gpark[k].y, st, -2) == st) {
            wfence(sh);
            enqueue_to(sd.scr.grq, sh.w->rqtail, sh.w->rqcap, sh, vload(sd.scr.gpark[k].x));
        }
    }
}

/* Key event of node j of instance I (its inner block is final): its earlier same-instance
 * neighbours, recorded, and the later ones dropped from its counter.  Returns the counter word
 * after the update. */
__device__ unsigned key_event(const fd_station_dev &sd, Shared &sh, int I, int j, long long q)
{
    const GRect &r = gsmem(sh).rect[I];
    const fdn_frame fr = frame_of(r.face);
    const int n = rect_n(r), nvf = r.vhi - r.vlo + 1, iv = j / r.nuf, iu = j - iv * r.nuf;
    const long long su = t_stride(sd, fr.axis_u), sv = t_stride(sd, fr.axis_v);
    const long long qin = q + fr.inner * t_stride(sd, fr.axis_n);   /* q's inner-layer node */
    const unsigned inr = inrect_mask(iu, iv, r.nuf, nvf);
    /* the inner-layer times of q and of its in-rectangle neighbours, all loads issued together */
    float tn[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int du, dv;
        nb_off(k, du, dv);
        const long long qk = qin + du * su + dv * sv;
        tn[k] = (((inr >> k) & 1u) && FD_OK(qk, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 12)) ? vload(sd.T[qk]) : 0.f;
    }
    const unsigned long long kj = node_key(vload(sd.T[qin]), j);
    unsigned em = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int du, dv;
        nb_off(k, du, dv);
        if (((inr >> k) & 1u) && node_key(tn[k], j + du + dv * r.nuf) < kj) em |= 1u << k;
    }
    if (!FD_OK(q, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 13) || !FD_OK(qin, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 29)
        || !FD_OK(I, sd.scr.ginst_cap, 14))
        return 0u;
    sd.scr.gemask[q] = (unsigned char)em;
    wfence(sh);
    const unsigned lat = (unsigned)__popc(inr & ~em);
    const unsigned add = FD_KEYED - (lat << 8);
    const unsigned nw = atomicAdd(&sd.scr.gcnt[q], add) + add;
    if (!sh.nodefer && atomicAdd(&sd.scr.ginst[I].nkeyed, 1) == n - 1) fire_event(sd, sh, I, 1);
    return nw;
}

__device__ __forceinline__ bool ready_word(unsigned w) { return (w & ~FD_WAITB) == FD_KEYED; }

__device__ __forceinline__ void graph_ready(const fd_station_dev &sd, Shared &sh, int face, long long q)
{
    enqueue_to(sd.scr.gqueue + sh.w->qbase[face], sh.w->qtail[face], sh.w->qcap[face], sh, (int)q);
}

/* drop one inner-block (inner) or other-instance dependency of node q (instance oq, face fq) */
__device__ __forceinline__ void graph_dec(const fd_station_dev &sd, Shared &sh, long long q, int oq, int fq,
                                          int qx, int qy, int qz, bool inner)
{
    const unsigned dec = inner ? 1u : (1u << 16);
    if (!FD_OK(q, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 19)) return;
    const unsigned nw = atomicSub(&sd.scr.gcnt[q], dec) - dec;
    if (inner && (nw & 0xFFu) == 0u) {
        /* q's inner block is complete: its key and in-face order are now known */
        if (ready_word(key_event(sd, sh, oq, inst_fill(gsmem(sh).rect[oq], qx, qy, qz), q))) graph_ready(sd, sh, fq, q);
    } else if (ready_word(nw)) {
        graph_ready(sd, sh, fq, q);
    }
}

/* node p (instance I, face F, fill index i) is final: record, release what waits on it */
__device__ void graph_release(const fd_station_dev &sd, Shared &sh, int F, long long p, int x, int y, int z, int I,
                              int i, bool writer, float st0, float st4, float tin)
{
    const GraphSmem &gs = gsmem(sh);
    if (!FD_OK(p, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 15) || !FD_OK(I, sd.scr.ginst_cap, 16)) return;
    const GRect &r = gs.rect[I];
    fd_ginst &gi = sd.scr.ginst[I];
    /* records: of every point when a point may need an earlier one's; else only the last instance's,
     * for the state the sweep leaves */
    if (!sh.nodefer || I == sh.ninst - 1) {
        if (writer) {
            sd.scr.grec[p] = make_float2(st0, st4);
            atomicMax(&gi.exitkey, node_key(tin, i));
        } else {
            sd.scr.grec[p] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        }
    }
    wfence(sh);
    /* done; a point waiting for the stencil state left before it resumes its search */
    if (!sh.nodefer && (atomicOr(&sd.scr.gcnt[p], FD_DONEB) & FD_WAITB)) {
        wfence(sh);
        const int nw = min(vload(sh.w->nwait), FD_GWAIT_CAP);
        for (int k = 0; k < nw; k++)
            if (vload(sd.scr.gwait[k].x) == (int)p && atomicCAS(&sd.scr.gwait[k].x, (int)p, -1) == (int)p)
                enqueue_to(sd.scr.grq, sh.w->rqtail, sh.w->rqcap, sh, vload(sd.scr.gwait[k].y));
    }
    const int nx = sd.g.nx, ny = sd.g.ny;
    const fdn_frame fr = frame_of(F);
    if (sh.single) {
        /* one face: the next instance's nodes whose inner block holds p */
        if (I + 1 < sh.ninst && gs.rect[I + 1].layer == r.layer - fr.inner) {
            const GRect &rn = gs.rect[I + 1];
            const int u0 = coord(fr.axis_u, x, y, z), v0 = coord(fr.axis_v, x, y, z);
            for (int dv = -1; dv <= 1; dv++)
                for (int du = -1; du <= 1; du++) {
                    const int u = u0 + du, v = v0 + dv;
                    if (u < rn.ulo || u > rn.uhi || v < rn.vlo || v > rn.vhi) continue;
                    int qx, qy, qz;
                    place(fr, u, v, rn.layer, qx, qy, qz);
                    const long long q = ((long long)qz * ny + qy) * nx + qx;
                    graph_dec(sd, sh, q, I + 1, F, qx, qy, qz, true);
                }
        }
    } else {
        /* nodes of later instances that read p, or that p read */
        const unsigned myctx = sh.ctxm[F];
        for (int k = 0; k < 27; k++) {
            if (k == 13) continue;
            const int qx = x + k % 3 - 1, qy = y + (k / 3) % 3 - 1, qz = z + k / 9 - 1;
            if (qx < 0 || qx >= nx || qy < 0 || qy >= ny || qz < 0 || qz >= sd.g.nz) continue;
            const int w = owner_near(gs, sh.gfaces, F, qx, qy, qz);
            if (w < 0 || own_inst(w) <= I) continue;
            const int fq = own_face(w);
            if (!((myctx >> k) & 1u) && !((sh.ctxm[fq] >> (26 - k)) & 1u)) continue;
            const long long q = ((long long)qz * ny + qy) * nx + qx;
            graph_dec(sd, sh, q, own_inst(w), fq, qx, qy, qz, (sh.innm[fq] >> (26 - k)) & 1u);
        }
    }
    /* later neighbours in the same instance */
    const int nvf = r.vhi - r.vlo + 1, iu = i % r.nuf, iv = i / r.nuf;
    const unsigned char gem = sh.cs > 1 ? __ldcg(&sd.scr.gemask[p]) : sd.scr.gemask[p];
    unsigned later = inrect_mask(iu, iv, r.nuf, nvf) & ~(unsigned)gem;
    while (later) {
        const int k = __ffs(later) - 1;
        later &= later - 1;
        int du, dv;
        nb_off(k, du, dv);
        const long long q = p + du * t_stride(sd, fr.axis_u) + dv * t_stride(sd, fr.axis_v);
        if (!FD_OK(q, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 17)) continue;
        const unsigned nw = atomicSub(&sd.scr.gcnt[q], 1u << 8) - (1u << 8);
        if (ready_word(nw)) graph_ready(sd, sh, F, q);
    }
}

/* point w waits for an event of instance I (kind 1: all keys final, 2: all points done) (lane 0) */
__device__ void wait_event(const fd_station_dev &sd, Shared &sh, int w, int I, int kind)
{
    const int k = atomicAdd(&sh.w->npark, 1);
    if (k >= FD_GPARK_CAP) {
        atomicCAS(&sh.w->status, 0, 15);
        return;
    }
    const int st = (kind << 24) | I;
    sd.scr.gpark[k].x = w;
    wfence(sh);
    atomicExch(&sd.scr.gpark[k].y, st);
    atomicOr(&sd.scr.ginst[I].evwait, kind);
    wfence(sh);
    const int n = rect_n(gsmem(sh).rect[I]);
    const bool now = kind == 1 ? vload(sd.scr.ginst[I].nkeyed) >= n : vload(sd.scr.ginst[I].ndone) >= n;
    if (now && atomicCAS(&sd.scr.gpark[k].y, st, -2) == st) enqueue_to(sd.scr.grq, sh.w->rqtail, sh.w->rqcap, sh, w);
}

/* point w waits for point p to be done (lane 0).  Returns false if p is already done (no wait). */
__device__ bool wait_point(const fd_station_dev &sd, Shared &sh, int w, long long p)
{
    const int k = atomicAdd(&sh.w->nwait, 1);
    if (k >= FD_GWAIT_CAP) {
        atomicCAS(&sh.w->status, 0, 15);
        return true;
    }
    sd.scr.gwait[k].y = w;
    wfence(sh);
    atomicExch(&sd.scr.gwait[k].x, (int)p);
    wfence(sh);
    if (!(atomicOr(&sd.scr.gcnt[p], FD_WAITB) & FD_DONEB)) return true;
    /* p finished meanwhile: take the pair back unless p's release already took it (and queued w) */
    return atomicCAS(&sd.scr.gwait[k].x, (int)p, -1) != (int)p;
}

/* ---------------------------------------------------------------------------------------------- */
/* evaluation of one chunk                                                                         */

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
__device__ bool commit_node(const fd_station_dev &sd, Shared &sh, const TrialDesc *dsc, WarpSmem &ws, int slot,
                            int F, const Where &wh, unsigned gm, unsigned em, float it0, float it4, bool permissive,
                            unsigned char *dag, Counters cn)
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
        const TrialDesc &d = dsc[K];
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
                count_eval(cn, K == TK_NF ? 3 : 1);
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
    if (lt(guess, told) && FD_OK(wh.p, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 11)) {
        sd.T[wh.p] = __double2float_rn(guess);
        if (lastK >= 0) {
            /* only the last head trial that lowered the minimum sets the measure that is tested */
            const double fhead = (last_gb - last_v) / head_den(dsc[lastK], s18, sd.g, z, y);
            if (fhead > FD_HEADTEST) atomicAdd(&sh.w->headw[frame_of(F).headw], 1);
        }
    }
    if (sh.graph)
        graph_release(sd, sh, F, wh.p, wh.x, wh.y, wh.z, wh.inst, wh.i, writers != 0, st0, st4, t18[13]);
    else
        face_release(sd, sh, dag, wh.i, writers != 0, st0, st4);
    return true;
}

/* where the node of queue entry e lies: a fill index in a face walk, a grid index in a graph;
 * ok false for a graph node no instance owns */
__device__ __forceinline__ Where locate(const fd_station_dev &sd, const Shared &sh, int F, int e, bool &ok)
{
    const fdn_frame fr = frame_of(F);
    Where wh;
    ok = true;
    if (sh.graph) {
        wh.p = e;
        const int nx = sd.g.nx, ny = sd.g.ny, exy = e / nx;
        wh.x = e - exy * nx;
        wh.z = exy / ny;
        wh.y = exy - wh.z * ny;
        const int w = owner_near(gsmem(sh), sh.gfaces, F, wh.x, wh.y, wh.z);
        if (w < 0) {
            ok = false;
            return wh;
        }
        wh.inst = own_inst(w);
        const GRect &gr = gsmem(sh).rect[wh.inst];
        wh.r.u = coord(fr.axis_u, wh.x, wh.y, wh.z);
        wh.r.v = coord(fr.axis_v, wh.x, wh.y, wh.z);
        wh.r.ulo = gr.ulo; wh.r.uhi = gr.uhi; wh.r.vlo = gr.vlo; wh.r.vhi = gr.vhi;
        wh.i = inst_fill(gr, wh.x, wh.y, wh.z);
    } else {
        wh.i = e;
        wh.inst = -1;
        wh.r.u = sh.ulo + e % sh.nuf;
        wh.r.v = sh.vlo + e / sh.nuf;
        wh.r.ulo = sh.ulo; wh.r.uhi = sh.uhi; wh.r.vlo = sh.vlo; wh.r.vhi = sh.vhi;
        place(fr, wh.r.u, wh.r.v, sh.layer, wh.x, wh.y, wh.z);
        wh.p = ((long long)wh.z * sd.g.ny + wh.y) * sd.g.nx + wh.x;
    }
    wh.r.nu = axis_len(sd, fr.axis_u);
    wh.r.nv = axis_len(sd, fr.axis_v);
    return wh;
}

/* Evaluate and commit one chunk of face F: lane l holds queue entry e (-1 for none).  A node given
 * with have_inherit uses (it0, it4) as the stencil state entering it.  All 32 lanes call. */
__device__ void warp_chunk(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int F, int e,
                           bool have_inherit, float it0, float it4, unsigned char *dag, Counters cn)
{
    const int lane = threadIdx.x & 31;
    const fdn_frame fr = frame_of(F);
    const TrialDesc *dsc = cs.desc[F];
    Where wh;
    unsigned gm = 0, em = 0;
    bool permissive = false;
    FD_TIC(ta);
    if (e >= 0) {
        bool ok;
        wh = locate(sd, sh, F, e, ok);
        if (!ok) {
            atomicCAS(&sh.w->status, 0, 14);   /* a queued node no face instance owns */
            e = -1;
        }
    }
    const bool valid = e >= 0;
    if (valid) {
        const long long pS = (long long)wh.z * sd.s_sz + (long long)wh.y * sd.s_sy + wh.x;
        ws.z[lane] = wh.z;
        ws.y[lane] = wh.y;
        float *tr = ws.t[lane], *sr = ws.s[lane];
        const long long su = t_stride(sd, fr.axis_u), sv = t_stride(sd, fr.axis_v);
        const long long ssu = s_stride(sd, fr.axis_u), ssv = s_stride(sd, fr.axis_v);
        const long long inner_t = fr.inner * t_stride(sd, fr.axis_n), inner_s = fr.inner * s_stride(sd, fr.axis_n);
#pragma unroll
        for (int nb = 0; nb < NB_N; nb++) {
            const int w = nb / 9, dv = (nb / 3) % 3 - 1, du = nb % 3 - 1;
            const int uu = wh.r.u + du, vv = wh.r.v + dv;
            float tv = 0.f, svv = 0.f;
            if (uu >= 0 && uu < wh.r.nu && vv >= 0 && vv < wh.r.nv) {
                /* with several CTAs, through L2: another SM may have written it since this SM last
                 * read it; one CTA's own stores keep its L1 current */
                const long long it = wh.p + du * su + dv * sv + (w ? inner_t : 0ll);
                if (FD_OK(it, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 27)) {
                    const float *pt = &sd.T[it];
                    tv = sh.cs > 1 ? __ldcg(pt) : *pt;
                    svv = __ldg(&sd.S[pS + du * ssu + dv * ssv + (w ? inner_s : 0ll)]);
                }
            }
            tr[nb] = tv;
            sr[nb] = svv;
        }
        guards(F, tr, wh.r, gm, em);
        /* a 2-D trial before any corner / new-edge call reads the state an earlier point left */
        const double told = f2d(tr[NB_POINT]);
        permissive = !have_inherit && (gm & 0xFu) == 0 && !((gm & 0xF0u) && lt(1.0e9, told)) && (gm & 0xFF00u);
    }
    __syncwarp();
    int n1 = push_items(ws.items, 0, em, TK_3D0, TK_2D0, lane);
    n1 = push_items(ws.items, n1, em, TK_1D0, FDN_NTRIAL, lane);
    __syncwarp();
    FD_TOC(1, ta);
    FD_TIC(tb);
    eval_items(sd, dsc, ws, n1, lane, cn);
    __syncwarp();
    const float lo = __int_as_float(0xff800000);   /* -inf: no stale floor */
    const float p0 = permissive ? lo : it0, p4 = permissive ? lo : it4;
    if (valid) em |= stale_pair(dsc, ws, lane, gm, em, p0, p4);
    __syncwarp();
    int n2 = push_items(ws.items, 0, em, TK_2D0, TK_NF, lane);
    __syncwarp();
    n2 = filter_2d(sd, dsc, ws, n2, lane);
    __syncwarp();
    eval_items(sd, dsc, ws, n2, lane, cn);
    __syncwarp();
    FD_TOC(2, tb);
    FD_TIC(tc);
    bool fin = false;
    if (valid) {
        fin = commit_node(sd, sh, dsc, ws, lane, F, wh, gm, em, p0, p4, permissive, dag, cn);
        if (!fin) {
            atomicAdd(reinterpret_cast<unsigned long long *>(&sh.w->deferred), 1ull);
            if (sh.nodefer)
                atomicCAS(&sh.w->status, 0, 6);   /* excluded by the sweep's precondition */
            else
                enqueue_to(sh.graph ? sd.scr.grq : sd.scr.rq, sh.w->rqtail, sh.w->rqcap, sh, e);
        }
    }
    if (sh.graph && !sh.nodefer) {
        /* points done per face instance, one atomic per instance in the chunk; the instance
         * complete wakes points waiting for its last writer */
        const int key = fin ? wh.inst : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (fin && lane == __ffs(peers) - 1) {
            const int c = __popc(peers);
            const int old = atomicAdd(&sd.scr.ginst[key].ndone, c);
            if (old + c == rect_n(gsmem(sh).rect[key])) fire_event(sd, sh, key, 2);
        }
    }
    const unsigned done = __ballot_sync(0xffffffffu, fin);
    if (lane == 0 && done) {
        wfence(sh);
        atomicAdd(&sh.w->ndone, __popc(done));
    }
    __syncwarp();
    FD_TOC(3, tc);
}

/* ---------------------------------------------------------------------------------------------- */
/* inherited stencil state                                                                         */

/* face walk: the point that precedes point c in sort order (largest key below c's), -1 if none */
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

/* Face walk: point w needs the stencil state left by the last point before it in sort order that
 * made a writer call.  Walk back through the sort order: a done writer gives its record; a done
 * non-writer passes the search to its predecessor; a point not yet done takes w as its waiter and
 * queues it again when it finishes (a point has at most one waiter: waiters lie between it and the
 * next pending point).  Before the face's first point the state is the one the face started with.
 * Keys fall along the walk, so waits cannot form a cycle.  One warp; evaluates w when found. */
__device__ void resume_waiter(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int w,
                              unsigned char *dag, Counters cn)
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
                if (vload(sd.scr.pst[p]) != -2) {
                    const int old = atomicCAS(&sd.scr.pst[p], -1, w);
                    if (old == -1) verdict = 2;
                    else if (old == -2) verdict = 3;
                    else { atomicCAS(&sh.w->status, 0, 11); verdict = 2; }   /* a second waiter */
                }
                if (verdict == 0 || verdict == 3) {
                    wfence(sh);
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
            warp_chunk(sd, sh, cs, ws, sh.face, lane == 0 ? w : -1, true, t0, t4, dag, cn);
            return;
        }
        c = p;
    }
    if (lane == 0) atomicCAS(&sh.w->status, 0, 12);
}

/* Sweep graph: the same search for point w (a grid index), by the reference's order of face
 * instances and, within one, of keys.  Registers w on an instance event or a point when the
 * answer is not yet known.  One warp; evaluates w when found. */
__device__ void resume_graph(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int w,
                             Counters cn)
{
    const int lane = threadIdx.x & 31;
    const GraphSmem &gs = gsmem(sh);
    const int nx = sd.g.nx, ny = sd.g.ny;
    if (!FD_OK(w, (long long)sd.g.nx * sd.g.ny * sd.g.nz, 20)) return;
    const int wxy = w / nx;
    const int wx = w - wxy * nx, wy = wxy % ny, wz = wxy / ny;
    const int ow = owner_of(gs, sh.gfaces, wx, wy, wz);
    if (ow < 0) {
        if (lane == 0) atomicCAS(&sh.w->status, 0, 14);
        return;
    }
    const int I = own_inst(ow);
    const GRect &r = gs.rect[I];
    const int n = rect_n(r);
    if (vload(sd.scr.ginst[I].nkeyed) < n) {   /* keys below w's not all known yet */
        if (lane == 0) wait_event(sd, sh, w, I, 1);
        return;
    }
    unsigned long long kc = inst_key(sd, r, inst_fill(r, wx, wy, wz));
    for (int guard = 0; guard <= 2 * n + 2; guard++) {
        /* predecessor in the instance */
        unsigned long long best = 0ull;
        for (int j = lane; j < n; j += 32) {
            const unsigned long long k = inst_key(sd, r, j);
            if (k < kc && k > best) best = k;
        }
        best = warp_max_u64(best);
        int verdict = 0;   /* 0 continue below best, 1 found, 2 waiting */
        float t0 = sh.carry_t0, t4 = sh.carry_t4;
        if (lane == 0) {
            if (best) {
                const long long p = inst_node(sd, r, (int)(best & 0xffffffffu));
                if (!FD_OK((long long)(best & 0xffffffffu), n, 21)) {
                    verdict = 2;
                } else if (!(vload(sd.scr.gcnt[p]) & FD_DONEB) && wait_point(sd, sh, w, p)) {
                    verdict = 2;
                } else {
                    wfence(sh);
                    const float r0 = vload(sd.scr.grec[p].x), r4 = vload(sd.scr.grec[p].y);
                    if (!isnan(r0)) { verdict = 1; t0 = r0; t4 = r4; }
                }
            } else {
                /* no earlier point in the instance: the last writer of an earlier instance */
                verdict = 1;
                for (int J = I - 1; J >= 0; J--) {
                    const GRect &rj = gs.rect[J];
                    if (vload(sd.scr.ginst[J].ndone) < rect_n(rj)) { wait_event(sd, sh, w, J, 2); verdict = 2; break; }
                    wfence(sh);
                    const unsigned long long ek = vload(sd.scr.ginst[J].exitkey);
                    if (ek) {
                        const long long p = inst_node(sd, rj, (int)(ek & 0xffffffffu));
                        if (!FD_OK((long long)(ek & 0xffffffffu), rect_n(rj), 22)) break;
                        t0 = vload(sd.scr.grec[p].x);
                        t4 = vload(sd.scr.grec[p].y);
                        break;
                    }
                }
            }
        }
        verdict = __shfl_sync(0xffffffffu, verdict, 0);
        if (verdict == 2) return;
        if (verdict == 1) {
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            t4 = __shfl_sync(0xffffffffu, t4, 0);
            warp_chunk(sd, sh, cs, ws, r.face, lane == 0 ? w : -1, true, t0, t4, nullptr, cn);
            return;
        }
        kc = best;
    }
    if (lane == 0) atomicCAS(&sh.w->status, 0, 12);
}

/* ---------------------------------------------------------------------------------------------- */
/* the worker loop                                                                                 */

/* nothing queued, every worker idle, and all queues unchanged across the idle count (lane 0) */
__device__ __forceinline__ bool quiescent(Shared &sh)
{
    int t0[6], r0 = vload(sh.w->rqtail);
    for (int k = 0; k < sh.w->nq; k++) {
        t0[k] = vload(sh.w->qtail[k]);
        if (vload(sh.w->qhead[k]) != t0[k]) return false;
    }
    if (vload(sh.w->rqhead) != r0) return false;
    wfence(sh);
    if (vload(sh.w->idle) != sh.cs * FD_WARPS) return false;
    wfence(sh);
    for (int k = 0; k < sh.w->nq; k++)
        if (vload(sh.w->qtail[k]) != t0[k] || vload(sh.w->qhead[k]) != t0[k]) return false;
    return vload(sh.w->rqtail) == r0 && vload(sh.w->rqhead) == r0;
}

/* read a claimed queue entry: spins briefly for an entry whose writer is between its two
 * instructions; -1 and a status on failure */
__device__ __forceinline__ int read_entry(const int *queue, int pos, Shared &sh)
{
    const volatile int *q = queue + pos;
    int e = *q;
    for (int spin = 0; e < 0 && spin < FD_QSPIN; spin++) {
        __nanosleep(32);
        e = *q;
    }
    if (e < 0) atomicCAS(&sh.w->status, 0, 9);   /* a claimed entry never written */
    return e;
}

/* the worker loop of one walk over `total` nodes; all warps call it between two CTA barriers */
__device__ void run_walk(const fd_station_dev &sd, Shared &sh, const CtaSmem &cs, WarpSmem &ws, int total,
                         unsigned char *dag, Counters cn)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    int *queue = sh.graph ? sd.scr.gqueue : sd.scr.queue;
    int *rq = sh.graph ? sd.scr.grq : sd.scr.rq;
    bool idle = false;
    long long since = clock64();
    const long long started = since;
    const long long wait_lim = sd.wait_cycles > 0 ? sd.wait_cycles : FD_WAIT_CYCLES;
    const long long walk_lim = sd.walk_cycles > 0 ? sd.walk_cycles : FD_WALK_CYCLES;
    long long chunks = 0;
    unsigned idle_polls = 0;
    for (;;) {
        int act = 0, h = 0, m = 0, qf = 0;   /* act: 0 wait, 1 chunk, 2 resume a waiter, 3 leave */
        if (lane == 0) {
            if (vload(sh.w->status) != 0 || vload(sh.w->ndone) >= total) {
                act = 3;
            } else {
                const int rh = vload(sh.w->rqhead), rt0 = vload(sh.w->rqtail), rt = rt0 < sh.w->rqcap ? rt0 : sh.w->rqcap;
                if (rh < rt) {
                    if (idle) { atomicSub(&sh.w->idle, 1); idle = false; }
                    if (atomicCAS(&sh.w->rqhead, rh, rh + 1) == rh) { act = 2; h = read_entry(rq, rh, sh); }
                } else {
                    /* the fullest queue, starting the scan at a warp-dependent face */
                    int best = -1, bavail = 0, bhead = 0;
                    for (int k0 = 0; k0 < sh.w->nq; k0++) {
                        const int k = (k0 + warp) % sh.w->nq;
                        const int hd = vload(sh.w->qhead[k]), qt = vload(sh.w->qtail[k]);
                        const int tl = qt < sh.w->qcap[k] ? qt : sh.w->qcap[k];
                        if (tl - hd > bavail) { bavail = tl - hd; best = k; bhead = hd; }
                    }
                    if (best >= 0) {
                        if (idle) { atomicSub(&sh.w->idle, 1); idle = false; }
                        const int want = bavail < 32 ? bavail : 32;
                        if (atomicCAS(&sh.w->qhead[best], bhead, bhead + want) == bhead) {
                            act = 1; h = sh.w->qbase[best] + bhead; m = want; qf = best;
                        }
                    } else {
                        if (!idle) { wfence(sh); atomicAdd(&sh.w->idle, 1); idle = true; idle_polls = 0; }
                        /* all idle with nothing queued and nodes left: nothing can release them.  The
                         * check (two fences and a scan of every queue) runs on every 64th idle poll
                         * only: idle warps are most of the CTA in a forward sweep, and their polls
                         * share the SM's shared-memory pipe with the working warps */
                        if ((++idle_polls & 63u) == 0u && quiescent(sh) && vload(sh.w->ndone) < total) {
                            atomicCAS(&sh.w->status, 0, 3);
                            act = 3;
                        }
                    }
                }
                if (act == 1 || act == 2) {
                    since = clock64();
                } else if (act == 0 && clock64() - since > wait_lim) {
                    atomicCAS(&sh.w->status, 0, 8);   /* no work for this worker for too long */
                    act = 3;
                }
                if (act != 3 && clock64() - started > walk_lim) {
                    atomicCAS(&sh.w->status, 0, 17);   /* the walk as a whole ran far too long */
                    act = 3;
                }
            }
        }
        act = __shfl_sync(0xffffffffu, act, 0);
        if (act == 3) break;
        h = __shfl_sync(0xffffffffu, h, 0);
        if (act == 1) {
            m = __shfl_sync(0xffffffffu, m, 0);
            qf = __shfl_sync(0xffffffffu, qf, 0);
            int e = -1;
            if (lane < m) {
                const volatile int *q = queue + h + lane;
                e = *q;
                for (int spin = 0; e < 0 && spin < FD_QSPIN; spin++) {
                    __nanosleep(32);
                    e = *q;
                }
                if (e < 0) atomicCAS(&sh.w->status, 0, 9);   /* a claimed entry never written */
                /* an entry outside the walk's nodes ends the walk with a status instead of an access */
                const long long bound = sh.graph ? (long long)sd.g.nx * sd.g.ny * sd.g.nz : (long long)sh.n;
                if (e >= bound) {
                    (void)FD_OK(e, bound, 23);
                    atomicCAS(&sh.w->status, 0, 18);
                    e = -1;
                }
            }
            wfence(sh);
            warp_chunk(sd, sh, cs, ws, sh.graph ? qf : sh.face, e, false, 0.f, 0.f, dag, cn);
            chunks++;
            continue;
        }
        if (act == 2) {
            wfence(sh);
            const long long bound = sh.graph ? (long long)sd.g.nx * sd.g.ny * sd.g.nz : (long long)sh.n;
            if (h >= bound) {
                (void)FD_OK(h, bound, 24);
                if (lane == 0) atomicCAS(&sh.w->status, 0, 18);
                h = -1;
            }
            if (h >= 0) {
                if (sh.graph)
                    resume_graph(sd, sh, cs, ws, h, cn);
                else
                    resume_waiter(sd, sh, cs, ws, h, dag, cn);
            }
            continue;
        }
        __nanosleep(64);
    }
    if (lane == 0 && chunks) atomicAdd(reinterpret_cast<unsigned long long *>(&sh.w->rounds), (unsigned long long)chunks);
}

/* reset the walk counters (thread 0) */
__device__ void walk_reset(Shared &sh, int nq, int rqcap)
{
    sh.w->nq = nq;
    for (int k = 0; k < 6; k++) { sh.w->qhead[k] = 0; sh.w->qtail[k] = 0; sh.w->qcap[k] = 0; sh.w->qbase[k] = 0; }
    sh.w->rqhead = sh.w->rqtail = sh.w->idle = sh.w->ndone = sh.w->npark = 0;
    sh.w->rqcap = rqcap;
    sh.w->exitkey = 0ull;
}

/* Walk the current face (parameters in sh) in dependency order. */
__device__ void face_walk(const fd_station_dev &sd, Shared &sh, CtaSmem &cs, WarpSmem &ws, unsigned char *dag,
                          Counters cn)
{
    const int n = sh.n, nuf = sh.nuf, nvf = n / nuf;
    const int tid = threadIdx.x;
    const float *T = sd.T;
    const fdn_frame fr = frame_of(sh.face);
    unsigned char *emask = dag + sh.n_pad;
    int *queue = sd.scr.queue;
    FD_TIC(t0);
    /* keys: time of the inner-layer neighbour, then fill index */
    for (int i = tid; i < n; i += blockDim.x) {
        int x, y, z;
        place(fr, sh.ulo + i % nuf, sh.vlo + i / nuf, sh.layer + fr.inner, x, y, z);
        const float tin = T[((long long)z * sd.g.ny + y) * sd.g.nx + x];
        sd.scr.key[i] = ((unsigned long long)okey32(tin) << 32) | (unsigned)i;
        sd.scr.pst[i] = -1;
        queue[i] = -1;
        sd.scr.rq[2 * i] = -1;
        sd.scr.rq[2 * i + 1] = -1;
    }
    if (tid == 0) {
        walk_reset(sh, 1, 2 * n);
        sh.w->qcap[0] = n;
        sh.graph = 0;
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
        if (em == 0) enqueue_to(queue, sh.w->qtail[0], sh.w->qcap[0], sh, i);
    }
    __syncthreads();
    FD_TOC(0, t0);
    FD_TIC(tw);
    run_walk(sd, sh, cs, ws, n, dag, cn);
    __syncthreads();
    FD_TOC(4, tw);
    if (tid == 0) {
        if (sh.w->exitkey) {
            const float2 r = sd.scr.rec[(int)(sh.w->exitkey & 0xffffffffu)];
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

/* One sweep (the radius loop of src/sphfd.c:1018-5566) as one dependency graph.  Leaves walls,
 * flags, radius and the stencil-state carry as the radius loop would. */
__device__ void graph_sweep(const fd_station_dev &sd, Shared &sh, CtaSmem &cs, WarpSmem &ws, Counters cn)
{
    const int tid = threadIdx.x;
    /* the station's threads over all its CTAs, for loops over nodes */
    const int gt = sh.rank * blockDim.x + tid, gstride = sh.cs * blockDim.x;
    const bool lead = sh.rank == 0;
    const int nx = sd.g.nx, ny = sd.g.ny, nz = sd.g.nz;
    GraphSmem &gs = gsmem(sh);
    FD_TIC(t0);
    for (int k = tid; k < FDN_NFACE * FD_LMAX; k += blockDim.x) (&gs.lay2inst[0][0])[k] = -1;
    __syncthreads();
    /* the sweep's face instances, as the radius loop visits them */
    if (tid == 0) {
        const int cap = sd.scr.ginst_cap < FD_IMAX ? sd.scr.ginst_cap : FD_IMAX;
        int ninst = 0;
        long long M = 0, per_face[6] = {0, 0, 0, 0, 0, 0};
        unsigned faces = 0;
        bool over = false;
        while (sh.rad0 && (sh.dflag[0] || sh.dflag[1] || sh.dflag[2] || sh.dflag[3] || sh.dflag[4] || sh.dflag[5])) {
            for (int face = 0; face < 6; face++) {
                for (int ig = 1; ig <= sd.grow[face]; ig++) {
                    if (!sh.dflag[face]) continue;
                    setup_face(sd, sh, face);
                    if (sh.n > 0) {
                        if (ninst >= cap) { over = true; break; }
                        if (lead) {
                            fd_ginst &gi = sd.scr.ginst[ninst];
                            gi.face = face; gi.layer = sh.layer;
                            gi.ulo = sh.ulo; gi.uhi = sh.uhi; gi.vlo = sh.vlo; gi.vhi = sh.vhi;
                            gi.nuf = sh.nuf; gi.n = sh.n;
                            gi.nkeyed = 0; gi.ndone = 0; gi.evwait = 0; gi.pad = 0; gi.exitkey = 0ull;
                        }
                        GRect &gr = gs.rect[ninst];
                        gr.face = (short)face; gr.layer = (short)sh.layer;
                        gr.ulo = (short)sh.ulo; gr.uhi = (short)sh.uhi; gr.vlo = (short)sh.vlo; gr.vhi = (short)sh.vhi;
                        gr.nuf = (short)sh.nuf; gr.pad = 0;
                        gs.lay2inst[face][sh.layer] = (short)ninst;
                        ninst++;
                        M += sh.n;
                        per_face[face] += sh.n;
                        faces |= 1u << face;
                    }
                    /* move the wall outward (e.g. src/sphfd.c:1762-1764) */
                    const int inner = frame_of(face).inner;
                    const int nmax = face < 2 ? nz : face < 4 ? nx : ny;
                    const bool limit = inner > 0 ? (sh.wall[face] == 0) : (sh.wall[face] == nmax - 1);
                    if (limit) sh.dflag[face] = 0;
                    sh.wall[face] -= inner;
                }
            }
            sh.radius++;
            if (sh.radius == sd.maxrad) sh.rad0 = 0;
            if (over) break;
        }
        sh.ninst = ninst;
        sh.gfaces = faces;
        sh.single = __popc(faces) == 1;
        sh.nodefer = 0;
        sh.graph = 1;
        sh.gM = M;
        if (lead) {
            if (over) sh.w->status = 13;
            walk_reset(sh, 6, FD_GRQ_CAP);
            sh.w->nwait = 0;
            long long b = 0;
            for (int f = 0; f < 6; f++) { sh.w->qbase[f] = (int)b; sh.w->qcap[f] = (int)per_face[f]; b += per_face[f]; }
        }
    }
    csync(sh, 1);
    const int ninst = sh.ninst;
    const long long M = sh.gM;
    if (sh.single) {
        /* One face, every time below 1e9: every corner guard inside the grid passes, so each point
         * calls a corner stencil before its 2-D trials and none needs an earlier point's state;
         * the exception is the EAST corner whose guard tests the node above for being non-zero
         * (src/sphfd.c:2544), which fails only next to a zero time. */
        const int f = __ffs(sh.gfaces) - 1;
        const long long nxyz = (long long)nx * ny * nz;
        int bad = 0;
        for (long long q = tid; q < nxyz; q += blockDim.x) {
            const float t = __ldcg(&sd.T[q]);
            if (!(t < 1.e9f)) bad = 1;
            else if (f == 2 && t == 0.0f && (q / nx) % ny == 0 && q / ((long long)nx * ny) == 1) bad = 1;
        }
        bad = __syncthreads_or(bad);
        if (tid == 0) sh.nodefer = !bad;
        __syncthreads();
    }
    if (M > 0 && sh.stat == 0) {
        for (long long k = gt; k < M; k += gstride) sd.scr.gqueue[k] = -1;
        /* dependency counters */
        for (int I = 0; I < ninst; I++) {
            const GRect r = gs.rect[I];
            const fdn_frame fr = frame_of(r.face);
            const int n = rect_n(r), nvf = r.vhi - r.vlo + 1;
            const unsigned myctx = sh.ctxm[r.face], myinn = sh.innm[r.face];
            const bool prev = sh.single && I > 0 && gs.rect[I - 1].layer == r.layer + fr.inner;
            for (int j = gt; j < n; j += gstride) {
                const long long p = inst_node(sd, r, j);
                if (!FD_OK(p, (long long)nx * ny * nz, 25)) continue;
                unsigned cin = 0, c2 = 0, cx = 0;
                if (sh.single) {
                    /* one face: the same-instance neighbours and the previous plane's inner block */
                    const int iu = j % r.nuf, iv = j / r.nuf;
                    c2 = (unsigned)__popc(inrect_mask(iu, iv, r.nuf, nvf));
                    if (prev) {
                        const GRect &rp = gs.rect[I - 1];
                        const int u0 = r.ulo + iu, v0 = r.vlo + iv;
                        for (int dv = -1; dv <= 1; dv++)
                            for (int du = -1; du <= 1; du++)
                                if (u0 + du >= rp.ulo && u0 + du <= rp.uhi && v0 + dv >= rp.vlo && v0 + dv <= rp.vhi) cin++;
                    }
                } else {
                    const int pi = (int)p, pxy = pi / nx;
                    const int x = pi - pxy * nx, y = pxy % ny, z = pxy / ny;
                    for (int k = 0; k < 27; k++) {
                        if (k == 13) continue;
                        const int qx = x + k % 3 - 1, qy = y + (k / 3) % 3 - 1, qz = z + k / 9 - 1;
                        if (qx < 0 || qx >= nx || qy < 0 || qy >= ny || qz < 0 || qz >= nz) continue;
                        const int w = owner_near(gs, sh.gfaces, r.face, qx, qy, qz);
                        if (w < 0 || own_inst(w) > I) continue;
                        if (own_inst(w) == I) { c2++; continue; }
                        if (!((myctx >> k) & 1u) && !((sh.ctxm[own_face(w)] >> (26 - k)) & 1u)) continue;
                        if ((myinn >> k) & 1u) cin++; else cx++;
                    }
                }
                sd.scr.gcnt[p] = cin | (c2 << 8) | (cx << 16);
            }
        }
        csync(sh, 2);
        /* nodes whose inner block is final take their key now */
        for (int I = 0; I < ninst; I++) {
            const GRect r = gs.rect[I];
            const int n = rect_n(r);
            for (int j = gt; j < n; j += gstride) {
                const long long p = inst_node(sd, r, j);
                if ((sd.scr.gcnt[p] & 0xFFu) == 0u && ready_word(key_event(sd, sh, I, j, p))) graph_ready(sd, sh, r.face, p);
            }
        }
        csync(sh, 3);
        FD_TOC(0, t0);
        FD_TIC(tw);
        run_walk(sd, sh, cs, ws, (int)M, nullptr, cn);
        csync(sh, 4);
        FD_TOC(4, tw);
    }
    /* the small tables back to their empty state for the next sweep */
    {
        const int nw = min(vload(sh.w->nwait), FD_GWAIT_CAP), np = min(vload(sh.w->npark), FD_GPARK_CAP);
        const int nr = min(vload(sh.w->rqtail), FD_GRQ_CAP);
        for (int k = gt; k < nw; k += gstride) sd.scr.gwait[k] = make_int2(-1, -1);
        for (int k = gt; k < np; k += gstride) sd.scr.gpark[k] = make_int2(-1, -2);
        for (int k = gt; k < nr; k += gstride) sd.scr.grq[k] = -1;
    }
    if (tid == 0) {
        /* the stencil state after the sweep: the record of its last writer */
        for (int I = ninst - 1; I >= 0; I--) {
            const unsigned long long ek = vload(sd.scr.ginst[I].exitkey);
            if (ek && FD_OK((long long)(ek & 0xffffffffu), rect_n(gs.rect[I]), 26)) {
                const float2 r = __ldcg(&sd.scr.grec[inst_node(sd, gs.rect[I], (int)(ek & 0xffffffffu))]);
                sh.carry_t0 = r.x;
                sh.carry_t4 = r.y;
                break;
            }
        }
        sh.faces += ninst;
        sh.node_updates += M;
        sh.gsweeps++;
        sh.graph = 0;
    }
    csync(sh, 5);
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

/* The solve of one station by this CTA, or by this cluster of csz CTAs (csz > 1 only for sweep
 * graphs: face walks run in one CTA).  sd is the station record in this CTA's shared memory. */
__device__ __forceinline__ void solve_station(const fd_station_dev &sd, int dag_smem_bytes, int csz, Shared &sh)
{
    extern __shared__ __align__(16) unsigned char fd_dyn_smem[];
    CtaSmem &cs = *reinterpret_cast<CtaSmem *>(fd_dyn_smem);
    WarpSmem &ws = reinterpret_cast<WarpSmem *>(fd_dyn_smem + kCtaSmemBytes)[threadIdx.x >> 5];
    const int tid = threadIdx.x;
    const int rank = csz > 1 ? (int)cooperative_groups::this_cluster().block_rank() : 0;
    unsigned long long t_start = 0;
    if (tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    /* the dependency bytes of the station's largest face go to shared memory when they fit */
    unsigned char *dag = 2ll * sd.max_face_pad <= dag_smem_bytes ? fd_dyn_smem + kSmemBase : sd.scr.dag;
    const int gdim = sd.g.nx > sd.g.ny ? (sd.g.nx > sd.g.nz ? sd.g.nx : sd.g.nz) : (sd.g.ny > sd.g.nz ? sd.g.ny : sd.g.nz);
    const bool gok = sd.scr.gcnt && gdim <= FD_LMAX && (int)sizeof(GraphSmem) <= dag_smem_bytes;
    /* without sweep graphs the first CTA solves alone (the launcher does not ask for more) */
    if (!gok && rank > 0) return;
    sh.cs = gok ? csz : 1;
    sh.rank = rank;
    sh.w = sh.cs > 1 ? cooperative_groups::this_cluster().map_shared_rank(&sh.wl, 0) : &sh.wl;
    if (tid == 0 && rank == 0) sh.wl.bar_count = 0;
    if (tid == 0) sh.stat = 0;
    /* once, before any CTA touches another's shared memory: every CTA of the cluster has started and
     * the barrier counter is set; every CTA reaches this line */
    if (sh.cs > 1) cooperative_groups::this_cluster().sync();
    if (rank == 0) {
        if (gok) {
            /* the sweep-graph tables start empty */
            for (int k = tid; k < FD_GWAIT_CAP; k += blockDim.x) sd.scr.gwait[k] = make_int2(-1, -1);
            for (int k = tid; k < FD_GPARK_CAP; k += blockDim.x) sd.scr.gpark[k] = make_int2(-1, -2);
            for (int k = tid; k < FD_GRQ_CAP; k += blockDim.x) sd.scr.grq[k] = -1;
        }
        if (sd.init_mode == 0) init_field(sd);
    }
    for (int k = tid; k < FDN_NFACE * FDN_NTRIAL; k += blockDim.x) (&cs.desc[0][0])[k] = c_desc[k];
    if (tid == 0) {
        for (int f = 0; f < 6; f++) { sh.wall[f] = sd.wall[f]; sh.dflag[f] = sd.dflag[f]; }
        sh.radius = sd.radius;
        sh.rad0 = 1;
        sh.reverse = sd.reverse;
        sh.headpref = sd.headpref;
        sh.carry_t0 = sd.carry_t0;
        sh.carry_t4 = sd.carry_t4;
        if (rank == 0) {
            sh.w->status = 0;
            sh.w->rounds = sh.w->deferred = 0;
            for (int k = 0; k < 5; k++) sh.w->st[k] = 0;
            sh.w->nwait = 0;
            sh.w->npark = 0;
        }
        sh.faces = sh.node_updates = 0;
        sh.sweeps = 0;
        for (int k = 0; k < 8; k++) sh.restart_wall[k] = 0;
        for (int k = 0; k < 6; k++) sh.cyc[k] = 0;
        sh.graph = 0;
        sh.gsweeps = 0;
        for (int f = 0; f < 6; f++) relation_masks(f, sh.ctxm[f], sh.innm[f]);
        sh.gsm = fd_dyn_smem + kSmemBase;
        sh.gok = gok;
        sh.single = 0;
        sh.nodefer = 0;
        sh.gfaces = 0;
    }
    csync(sh, 6);
    if ((tid & 31) < 6) ws.cnt[tid & 31] = 0ull;
    __syncwarp();
    Counters cn;
    cn.n = ws.cnt;
    const int nx = sd.g.nx, ny = sd.g.ny, nz = sd.g.nz;
    int guard_sweeps = 0;
    while (sh.reverse > -1 && sh.stat == 0) {
        if (tid == 0 && rank == 0) for (int k = 0; k < 8; k++) sh.w->headw[k] = 0;
        csync(sh, 7);
        FD_TIC(tsweep);
        const bool as_graph = sh.gok && (FD_GRAPH_FORWARD || sh.sweeps > 0);
        if (as_graph) graph_sweep(sd, sh, cs, ws, cn);
        while (!as_graph && sh.rad0
               && (sh.dflag[0] || sh.dflag[1] || sh.dflag[2] || sh.dflag[3] || sh.dflag[4] || sh.dflag[5])
               && sh.stat == 0) {
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
            csync(sh, 10);
        }
        if (tid == 0) {
            if (sh.sweeps == 0) FD_TOC(5, tsweep);   /* profiling builds: the first sweep's cycles */
            sh.sweeps++;
            /* restart test (src/sphfd.c:5570-5676) */
            const int *hw = sh.w->headw;
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
        /* every CTA has read this sweep's head-wave counts before the next sweep clears them */
        csync(sh, 8);
        if (++guard_sweeps > 1000000) { if (tid == 0 && rank == 0) sh.w->status = 4; break; }
    }
    /* statistics */
    __syncwarp();
    if ((tid & 31) < 5) atomicAdd(&sh.w->st[tid & 31], ws.cnt[tid & 31]);
    csync(sh, 9);
    if (tid == 0 && rank == 0 && sd.stats) {
        fd_station_stats *o = sd.stats;
        o->status = sh.w->status;
        o->sweeps = sh.sweeps;
        o->node_updates = sh.node_updates;
        o->faces = sh.faces;
        o->rounds = sh.w->rounds;
        o->deferred = sh.w->deferred;
        for (int k = 0; k < 5; k++) o->stencils[k] = (int64_t)sh.w->st[k];
        for (int k = 0; k < 8; k++) o->restart_wall[k] = sh.restart_wall[k];
        for (int k = 0; k < 6; k++) o->phase_cycles[k] = sh.cyc[k];
        unsigned long long t_end;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
        o->t_start_ns = (int64_t)t_start;
        o->t_end_ns = (int64_t)t_end;
        o->pipelined_sweeps = (int32_t)sh.gsweeps;
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        o->sm = (int32_t)smid;
    }
    /* no CTA leaves while another may still read the first CTA's shared memory; every wait before
     * this line is bounded, so every CTA reaches it */
    if (sh.cs > 1) cooperative_groups::this_cluster().sync();
}

/* a station record copied into shared memory by the whole CTA; cache-volatile loads, because a
 * serving session rewrites a record slot between the requests this SM reads from it */
__device__ __forceinline__ void load_record(fd_station_dev &dst, const fd_station_dev *src)
{
    static_assert(sizeof(fd_station_dev) % 4 == 0, "record size");
    const unsigned *s = reinterpret_cast<const unsigned *>(src);
    unsigned *d = reinterpret_cast<unsigned *>(&dst);
    for (int k = threadIdx.x; k < (int)(sizeof(fd_station_dev) / 4); k += blockDim.x) d[k] = __ldcv(s + k);
}

__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_sys(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

/* Thread 0 claims the next published request of a serving session: its entry, or -1 when the host
 * has asked idle CTAs to stop, or -2 after q.idle_ns with nothing to claim (the host normally
 * stops the grid long before; the bound only ends a loop whose host has gone away). */
__device__ int serve_claim(const fd_serve_queue &q, unsigned long long *gen)
{
    unsigned long long t0, now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    /* Idle CTAs back off between looks, to 2 us on SM 0 and ~60 us on the last SM: a burst of
     * requests is claimed mostly by the low-numbered SMs, the ones a batch launch of as many CTAs
     * fills first (a 64-station batch lands on SMs 0-59 and 148-151).  Packed that way the same
     * stations solved 14 % faster than spread over both dies. */
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    const unsigned cap_ns = 2000u + 400u * smid;
    unsigned sleep_ns = 500;
    for (;;) {
        const unsigned long long h = *(volatile const unsigned long long *)q.head;
        const unsigned long long t = ld_acquire_sys(q.tail);
        if (h < t) {
            if (atomicCAS(q.head, h, h + 1) == h) {
                const int e = *(volatile const int *)(q.order + (h % (unsigned long long)q.ring));
                *gen = *(volatile const unsigned long long *)(q.gen + e);
                return e;
            }
            continue;
        }
        if (*(volatile const int *)q.stop) return -1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
        if ((long long)(now - t0) > q.idle_ns) return -2;
        __nanosleep(sleep_ns);
        if (sleep_ns < cap_ns) sleep_ns = sleep_ns * 2 < cap_ns ? sleep_ns * 2 : cap_ns;
    }
}

/* Batch mode (q == nullptr): station blockIdx.x / csz of `stations`, one launch per batch.
 * Serving mode: a long-running grid of one CTA per SM; each CTA solves the requests it claims from
 * q one after another (csz 1), and writes exitf[cta_id0 + blockIdx.x] when it leaves. */
__global__ void __launch_bounds__(FD_BLOCK, 1) fd_solve(const fd_station_dev *stations, int nst, int dag_smem_bytes,
                                                       int csz, const fd_serve_queue *q, int cta_id0)
{
    __shared__ Shared sh;
    __shared__ fd_station_dev rec;
    __shared__ int entry;
    __shared__ unsigned long long gen;
    const int station = (int)blockIdx.x / csz;
    if (!q && station >= nst) return;   /* a whole cluster: its CTAs are consecutive */
    for (;;) {
        if (q) {
            if (threadIdx.x == 0) entry = serve_claim(*q, &gen);
            __syncthreads();
            if (entry < 0) break;
        }
        load_record(rec, q ? q->desc + entry : stations + station);
        __syncthreads();
        solve_station(rec, dag_smem_bytes, q ? 1 : csz, sh);
        if (!q) return;
        /* every thread's field writes, then the statistics, then the flag the host waits for */
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence_system();
            st_release_sys(q->done + entry, gen);
        }
    }
    if (threadIdx.x == 0) {
        __threadfence_system();
        *(volatile int *)(q->exitf + cta_id0 + blockIdx.x) = 1;
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

/* shared memory per CTA that the dynamic part must leave: fd_solve's static shared memory, rounded
 * up to 1 KB */
static size_t dyn_smem_limit_margin()
{
    static size_t margin = 0;
    if (!margin) {
        cudaFuncAttributes a;
        margin = cudaFuncGetAttributes(&a, fdk::fd_solve) == cudaSuccess ? ((a.sharedSizeBytes + 1023) & ~(size_t)1023)
                                                                          : 4096;
    }
    return margin;
}

/* cluster: CTAs per station; 0 picks more than one when the stations alone would leave SMs idle,
 * up to 8 (1 keeps every station on one CTA).  Reduced until every cluster of the launch is
 * co-resident. */
/* Launch shape of a batch: dynamic shared memory (the warp areas, plus the sweep-graph tables or the
 * face's dependency bytes, whichever is larger and fits) and CTAs per station; sets the kernel's
 * shared-memory limit.  Host calls only (no stream work): done once per batch, outside any capture. */
extern "C" cudaError_t fdk_solve_config(int nst, long long max_face_pad, int cluster, long long *bytes_out,
                                        int *csz_out)
{
    int dev = 0, optin = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long room = optin - (long long)dyn_smem_limit_margin();
    const long long base = (long long)fdk::kSmemBase;
    const long long graph = (long long)sizeof(fdk::GraphSmem);
    const long long dagb = 2 * max_face_pad > graph ? 2 * max_face_pad : graph;
    const long long bytes = base + dagb <= room ? base + dagb : (base + graph <= room ? base + graph : base);
    /* the attribute is an upper bound shared by every launch of the kernel (a serving session may
     * launch it from another thread): always the largest */
    cudaError_t e = cudaFuncSetAttribute(fdk::fd_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room);
    if (e != cudaSuccess) return e;
    /* CTAs per station: with clusters of 2 any two SMs of a GPC serve; clusters of 4 and 8 are taken
     * only with room to spare, so that every cluster of the launch is co-resident (launches whose
     * clusters of 8 ran in several waves faulted once on this GPU; they are not made) */
    auto fits = [&](int c) {
        const long long ctas = (long long)nst * c;
        return c == 1 || (c == 2 && ctas <= sms) || (c == 4 && 4 * ctas <= 3ll * sms) || (c == 8 && 2 * ctas <= sms);
    };
    int cs = cluster;
    if (cs <= 0) {
        cs = 1;
        while (cs < 8 && fits(cs * 2) && (long long)nst * cs * 2 <= sms) cs *= 2;
    }
    while (cs > 1 && !fits(cs)) cs /= 2;
    if (cs > FD_MAX_CLUSTER) cs = FD_MAX_CLUSTER;
    if (bytes - base < graph) cs = 1;   /* no room for the sweep-graph tables: face walks, one CTA */
    *bytes_out = bytes;
    *csz_out = cs;
    return cudaSuccess;
}

/* One launch of a configured batch: queues the kernel only (capturable in a CUDA graph). */
extern "C" cudaError_t fdk_solve_launch(const fd_station_dev *stations, int nst, long long bytes, int cs,
                                        cudaStream_t stream)
{
    if (nst <= 0) return cudaSuccess;
    const long long base = (long long)fdk::kSmemBase;
    if (cs == 1) {
        fdk::fd_solve<<<nst, FD_BLOCK, (size_t)bytes, stream>>>(stations, nst, (int)(bytes - base), 1, nullptr, 0);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nst * cs));
    cfg.blockDim = dim3(FD_BLOCK);
    cfg.dynamicSmemBytes = (size_t)bytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fdk::fd_solve, stations, nst, (int)(bytes - base), cs,
                                             static_cast<const fd_serve_queue *>(nullptr), 0);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

extern "C" cudaError_t fdk_launch_solve(const fd_station_dev *stations, int nst, long long max_face_pad, int cluster,
                                        cudaStream_t stream)
{
    if (nst <= 0) return cudaSuccess;
    long long bytes = 0;
    int cs = 1;
    const cudaError_t e = fdk_solve_config(nst, max_face_pad, cluster, &bytes, &cs);
    return e != cudaSuccess ? e : fdk_solve_launch(stations, nst, bytes, cs, stream);
}

/* The long-running grid of a serving session: nctas CTAs (one per SM), numbered cta_id0 onward in
 * q->exitf, with the largest dynamic shared memory a CTA can have (every request then finds the
 * sweep-graph tables and, when they fit, its face's dependency bytes in shared memory). */
extern "C" cudaError_t fdk_launch_serve(const fd_serve_queue *q, int nctas, int cta_id0, cudaStream_t stream)
{
    if (nctas <= 0) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const long long bytes = optin - (long long)dyn_smem_limit_margin();
    const long long base = (long long)fdk::kSmemBase;
    if (bytes - base < (long long)sizeof(fdk::GraphSmem)) return cudaErrorInvalidConfiguration;
    /* the same bound as every other launch of the kernel */
    cudaError_t e = cudaFuncSetAttribute(fdk::fd_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    fdk::fd_solve<<<nctas, FD_BLOCK, (size_t)bytes, stream>>>(nullptr, 0, (int)(bytes - base), 1, q, cta_id0);
    return cudaGetLastError();
}

/* dynamic shared memory a launch of fd_solve needs in the serving loop */
extern "C" long long fdk_serve_smem_bytes(void)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return optin - (long long)dyn_smem_limit_margin();
}

#ifdef FD_SELFCHECK
/* the index-check record of FD_SELFCHECK builds: count, first site, first index; cleared after reading */
extern "C" cudaError_t fdk_selfcheck_read(unsigned long long *out)
{
    cudaError_t e = cudaMemcpyFromSymbol(out, fd_selfcheck_words, sizeof(unsigned long long) * 3);
    if (e == cudaSuccess) {
        const unsigned long long z[3] = {0, 0, 0};
        e = cudaMemcpyToSymbol(fd_selfcheck_words, z, sizeof z);
    }
    return e;
}
#endif

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
