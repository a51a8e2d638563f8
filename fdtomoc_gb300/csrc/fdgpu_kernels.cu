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
#include "fdgpu_layout.h"

#define FD_BLOCK 256
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
    int face, layer, ulo, uhi, vlo, vhi, nuf, n;
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

/* Evaluate face point i (fill index) of the current face with template face F.  Returns false if
 * the point needs an inherited (t0,t4) it was not given. */
template <int F>
__device__ bool eval_point(const fd_station_dev &sd, Shared &sh, int i, bool have_inherit, float it0, float it4,
                           Counters &cn)
{
    using FT = FaceT<F>;
    const fd_geo_dev &g = sd.g;
    PointCtx p;
    p.u = sh.ulo + i % sh.nuf;
    p.v = sh.vlo + i / sh.nuf;
    p.nu = sh.nu;
    p.nv = sh.nv;
    p.ulo = sh.ulo; p.uhi = sh.uhi; p.vlo = sh.vlo; p.vhi = sh.vhi;
    int xyz[3];
    xyz[FT::AU] = p.u;
    xyz[FT::AV] = p.v;
    xyz[FT::AN] = sh.layer;
    p.z = xyz[2];
    p.y = xyz[1];
    const long long nx = g.nx, nxy = (long long)g.nx * g.ny;
    p.pT = (long long)xyz[2] * nxy + (long long)xyz[1] * nx + xyz[0];
    const long long pS = (long long)xyz[2] * sd.s_sz + (long long)xyz[1] * sd.s_sy + xyz[0];
#pragma unroll
    for (int w = 0; w < 2; w++)
#pragma unroll
        for (int dv = -1; dv <= 1; dv++)
#pragma unroll
            for (int du = -1; du <= 1; du++) {
                const int uu = p.u + du, vv = p.v + dv;
                const bool in = uu >= 0 && uu < p.nu && vv >= 0 && vv < p.nv;
                float tv = 0.f, sv = 0.f;
                if (in) {
                    tv = sd.T[p.pT + du * sh.su + dv * sh.sv + (long long)(w * FT::IN) * sh.sn];
                    sv = __ldg(&sd.S[pS + du * sh.ssu + dv * sh.ssv + (long long)(w * FT::IN) * sh.ssn]);
                }
                p.t[w][dv + 1][du + 1] = tv;
                p.s[w][dv + 1][du + 1] = sv;
            }
    EvalState st;
    const float told = p.t[0][1][1];
    st.guess = f2d(told);
    st.fhead = 0.0;
    st.t0 = it0;
    st.t4 = it4;
    st.writers = 0;
    st.gate = false;
    st.have_inherit = have_inherit;
    st.defer = false;
    st.n3d = st.nne = st.n2d = st.nnf = st.n1d = 0;
    run_trials<F, 0>(g, p, st);
    if (st.defer) return false;
    cn.n[0] += st.n3d; cn.n[1] += st.nne; cn.n[2] += st.n2d; cn.n[3] += st.nnf; cn.n[4] += st.n1d;
    if (st.guess < f2d(told)) {
        sd.T[p.pT] = __double2float_rn(st.guess);
        if (st.fhead > FD_HEADTEST) atomicAdd(&sh.headw[FT::HW], 1);
    }
    if (st.writers) {
        sd.scr.rec[i] = make_float2(st.t0, st.t4);
        atomicMax(&sh.exitkey, sd.scr.key[i]);
    } else {
        sd.scr.rec[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    }
    return true;
}

__device__ __forceinline__ bool eval_dispatch(const fd_station_dev &sd, Shared &sh, int i, bool hi, float t0, float t4,
                                              Counters &cn)
{
    switch (sh.face) {
    case 0: return eval_point<0>(sd, sh, i, hi, t0, t4, cn);
    case 1: return eval_point<1>(sd, sh, i, hi, t0, t4, cn);
    case 2: return eval_point<2>(sd, sh, i, hi, t0, t4, cn);
    case 3: return eval_point<3>(sd, sh, i, hi, t0, t4, cn);
    case 4: return eval_point<4>(sd, sh, i, hi, t0, t4, cn);
    default: return eval_point<5>(sd, sh, i, hi, t0, t4, cn);
    }
}

/* mark point i done and release its later in-face neighbours into list `out` */
__device__ __forceinline__ void release(const fd_station_dev &sd, Shared &sh, int i, int out)
{
    const unsigned long long ki = sd.scr.key[i];
    sd.scr.indeg[i] = -1;
    const int iu = i % sh.nuf, iv = i / sh.nuf;
    const int nvf = sh.n / sh.nuf;
#pragma unroll
    for (int dv = -1; dv <= 1; dv++)
#pragma unroll
        for (int du = -1; du <= 1; du++) {
            if (du == 0 && dv == 0) continue;
            const int ju = iu + du, jv = iv + dv;
            if (ju < 0 || ju >= sh.nuf || jv < 0 || jv >= nvf) continue;
            const int j = jv * sh.nuf + ju;
            if (sd.scr.key[j] > ki) {
                if (atomicSub(&sd.scr.indeg[j], 1) == 1) {
                    const int pos = atomicAdd(&sh.cnt[out], 1);
                    sd.scr.wl[out][pos] = j;
                }
            }
        }
}

/* Walk the current face (parameters in sh) in dependency order. */
__device__ void face_walk(const fd_station_dev &sd, Shared &sh, Counters &cn)
{
    const int n = sh.n, nuf = sh.nuf, nvf = n / nuf;
    const int tid = threadIdx.x;
    const float *T = sd.T;
    /* keys: time of the inner-layer neighbour, then fill index */
    const fdn_frame fr = frame_of(sh.face);
    const int IN = fr.inner;
    for (int i = tid; i < n; i += FD_BLOCK) {
        const int u = sh.ulo + i % nuf, v = sh.vlo + i / nuf;
        int xyz[3];
        xyz[fr.axis_u] = u;
        xyz[fr.axis_v] = v;
        xyz[fr.axis_n] = sh.layer + IN;
        const float tin = T[(long long)xyz[2] * sd.g.nx * sd.g.ny + (long long)xyz[1] * sd.g.nx + xyz[0]];
        sd.scr.key[i] = ((unsigned long long)okey32(tin) << 32) | (unsigned)i;
    }
    if (tid == 0) { sh.cnt[0] = 0; sh.cnt[1] = 0; sh.ndef = 0; sh.exitkey = 0ull; }
    __syncthreads();
    for (int i = tid; i < n; i += FD_BLOCK) {
        const unsigned long long ki = sd.scr.key[i];
        const int iu = i % nuf, iv = i / nuf;
        int c = 0;
        for (int dv = -1; dv <= 1; dv++)
            for (int du = -1; du <= 1; du++) {
                if (du == 0 && dv == 0) continue;
                const int ju = iu + du, jv = iv + dv;
                if (ju < 0 || ju >= nuf || jv < 0 || jv >= nvf) continue;
                c += sd.scr.key[jv * nuf + ju] < ki;
            }
        sd.scr.indeg[i] = c;
        if (c == 0) sd.scr.wl[0][atomicAdd(&sh.cnt[0], 1)] = i;
    }
    int cur = 0;
    long long rounds = 0;
    const long long max_rounds = 2ll * n + 8;
    for (;;) {
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
            for (int j = tid; j < ndef; j += FD_BLOCK) {
                const unsigned long long k = sd.scr.key[sd.scr.deferred[j]];
                lm = k < lm ? k : lm;
            }
            const unsigned long long dmin = block_min_u64(lm, sh);
            /* the last writer before it in sort order */
            unsigned long long lw = 0ull;
            for (int i = tid; i < n; i += FD_BLOCK) {
                const unsigned long long k = sd.scr.key[i];
                if (k < dmin && sd.scr.indeg[i] < 0 && !isnan(sd.scr.rec[i].x)) lw = k > lw ? k : lw;
            }
            const unsigned long long wkey = block_max_u64(lw, sh);
            if (tid == 0) {
                const int d = (int)(dmin & 0xffffffffu);
                float t0 = sh.carry_t0, t4 = sh.carry_t4;
                if (wkey) {
                    const float2 r = sd.scr.rec[(int)(wkey & 0xffffffffu)];
                    t0 = r.x;
                    t4 = r.y;
                }
                eval_dispatch(sd, sh, d, true, t0, t4, cn);
                release(sd, sh, d, cur);
                for (int j = 0; j < sh.ndef; j++)
                    if (sd.scr.deferred[j] == d) { sd.scr.deferred[j] = sd.scr.deferred[sh.ndef - 1]; break; }
                sh.ndef--;
                sh.deferred++;
            }
            continue;
        }
        if (tid == 0) { sh.cnt[cur ^ 1] = 0; sh.rounds++; }
        __syncthreads();
        for (int j = tid; j < ncur; j += FD_BLOCK) {
            const int i = sd.scr.wl[cur][j];
            if (eval_dispatch(sd, sh, i, false, 0.f, 0.f, cn)) {
                release(sd, sh, i, cur ^ 1);
            } else {
                sd.scr.deferred[atomicAdd(&sh.ndef, 1)] = i;
            }
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

/* ---------------------------------------------------------------------------------------------- */
/* source box (src/sphfd.c:724-825)                                                                */

__device__ void init_field(const fd_station_dev &sd)
{
    const long long nxyz = (long long)sd.g.nx * sd.g.ny * sd.g.nz;
    float4 *T4 = reinterpret_cast<float4 *>(sd.T);
    const float u = 1.0e10f;
    for (long long i = threadIdx.x; i < nxyz / 4; i += blockDim.x) T4[i] = make_float4(u, u, u, u);
    for (long long i = (nxyz / 4) * 4 + threadIdx.x; i < nxyz; i += blockDim.x) sd.T[i] = u;
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

__global__ void __launch_bounds__(FD_BLOCK) fd_solve(const fd_station_dev *stations, int nst)
{
    __shared__ Shared sh;
    if ((int)blockIdx.x >= nst) return;
    const fd_station_dev &sd = stations[blockIdx.x];
    const int tid = threadIdx.x;
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
        while (sh.rad0 && (sh.dflag[0] || sh.dflag[1] || sh.dflag[2] || sh.dflag[3] || sh.dflag[4] || sh.dflag[5])
               && sh.status == 0) {
            for (int face = 0; face < 6; face++) {
                for (int ig = 1; ig <= sd.grow[face]; ig++) {
                    if (!sh.dflag[face]) continue;
                    if (tid == 0) {
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
                    }
                    __syncthreads();
                    if (sh.n > 0) face_walk(sd, sh, cn);
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

extern "C" cudaError_t fdk_launch_solve(const fd_station_dev *stations, int nst, cudaStream_t stream)
{
    if (nst <= 0) return cudaSuccess;
    fdk::fd_solve<<<nst, FD_BLOCK, 0, stream>>>(stations, nst);
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
