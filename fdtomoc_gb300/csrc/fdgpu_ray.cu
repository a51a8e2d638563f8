/* sphrayderv's per-observation work on the device: residual and hypocentre derivatives at the event,
 * the ray traced back from the event down the travel-time gradient to the station, and the ray's
 * slowness derivatives on the coarse metagrid (reference src/sphrayderv.c:1054-2232,
 * lib/sphrayderv/dfind.c, pmin.c), against travel-time fields already on the device.
 *
 * One thread traces one ray: a ray is a chain of dependent cell crossings, and the observations of
 * a run are independent.  Every intermediate keeps the C type the reference gives it (the type
 * decides the rounding), the build has no fused multiply-add contraction, and sin/cos/atan2 are the
 * double-double functions of fd_trig.h, so the results are bit-identical to the oracle's
 * double-double mode.  A ray's derivatives go to its own list of (coarse node, value) in the order
 * the segments add them, which gives each node the same float sum the reference's dense array
 * gets; the list is sorted by node at the end, as the reference scans its array.
 *
 * A second kernel packs the lists into the caller's arrays. */
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/fdgpu.h"
#include "fd_trig.h"
#include "fdgpu_device.h"

extern "C" int fdh_ctx_device(const fdgpu_ctx *ctx);
extern "C" void *fdh_ctx_stream(const fdgpu_ctx *ctx);
extern "C" int fdh_ctx_fail(fdgpu_ctx *ctx, int cuda_error, const char *what);

namespace {

constexpr int kRayBlock = 64;
constexpr float kRearth = 6371.0f;   /* src/sphrayderv.c:87 */

struct RayGridDev {
    int nx, ny, nz, nxc, nyc, nzc;
    double x0, y0, z0, h, dq, df;
};

struct RayObsDev {
    double ex, ey, ez, xs, ys, zs;
    const float *t;
    float obstime, pwt, tc;
    int out;              /* the observation's index in the caller's arrays */
};

/* (int) of a double as x86-64 converts it: truncation, INT_MIN for NaN and out-of-range values */
__device__ __forceinline__ int trunc_i(double v)
{
    if (!(v > -2147483649.0 && v < 2147483648.0)) return INT_MIN;
    return (int)v;
}

__device__ __forceinline__ double pmin(double d1, double d2)
{
    if (d1 >= 0) return (d2 >= 0) ? (d1 < d2 ? d1 : d2) : d1;
    return d2 >= 0 ? d2 : -1e20;
}

__device__ __forceinline__ void dfind(const double dd[3], double *d, int *md, double tolmin, double tolmax)
{
    int mn, mid, mx;
    const double a0 = fabs(dd[0]), a1 = fabs(dd[1]), a2 = fabs(dd[2]);
    if (a0 <= a1 && a0 <= a2) {
        mn = 0;
        if (a1 <= a2) { mid = 1; mx = 2; } else { mid = 2; mx = 1; }
    } else if (a1 <= a2) {
        mn = 1;
        if (a0 <= a2) { mid = 0; mx = 2; } else { mid = 2; mx = 0; }
    } else {
        mn = 2;
        if (a0 <= a1) { mid = 0; mx = 1; } else { mid = 1; mx = 0; }
    }
    *d = dd[mn];
    *md = mn;
    if (dd[mn] < tolmin) {
        if (dd[mid] < tolmin) {
            if (dd[mx] < tolmax) { *d = dd[mx]; *md = mx; }
            else { *d = dd[mid]; *md = mid; }
        } else if (dd[mid] < tolmax) {
            *d = dd[mid];
            *md = mid;
        }
    }
}

/* corner indices of fine cell (ie, je, ke); false if one falls outside the field */
__device__ __forceinline__ bool corners(const RayGridDev &g, int ie, int je, int ke, long long ipt[8])
{
    const long long nxy = (long long)g.nx * g.ny, n = nxy * g.nz;
    const long long nk = nxy * ke, nj = (long long)g.nx * je, nk2 = nxy * ((long long)ke + 1),
                    nj2 = (long long)g.nx * ((long long)je + 1);
    ipt[0] = nk + nj + ie;
    ipt[1] = nk + nj + ie + 1;
    ipt[2] = nk + nj2 + ie;
    ipt[3] = nk + nj2 + ie + 1;
    ipt[4] = nk2 + nj + ie;
    ipt[5] = nk2 + nj + ie + 1;
    ipt[6] = nk2 + nj2 + ie;
    ipt[7] = nk2 + nj2 + ie + 1;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 8; q++) ok = ok && ipt[q] >= 0 && ipt[q] < n;
    return ok;
}

/* the ray's derivative list: li/lv hold n entries, at most cap.  A ray crosses several fine cells
 * per coarse cell, and every segment in one coarse cell adds to the same eight nodes: their list
 * positions are kept (pos, for coarse cell `cell`) so that those segments add without a search. */
struct RayList {
    int *li;
    float *lv;
    int n, cap;
    bool over;
    int cell;
    int pos[8];

    /* list position of node `index` (appended if new); -1 when the list is full */
    __device__ __forceinline__ int find(int index)
    {
        for (int q = n - 1; q >= 0; q--)   /* the latest segments touch the latest nodes */
            if (li[q] == index) return q;
        if (n >= cap) return -1;
        li[n] = index;
        lv[n] = 0.0f;
        return n++;
    }

    __device__ __forceinline__ void add_at(int q, double v)
    {
        if (q < 0) {
            over = true;
            return;
        }
        lv[q] = (float)((double)lv[q] + v);
    }
};

/* sin and cos of the cell-wall angles a ray meets: rows y(j) = dq j + y0 and y(j) + dq, columns
 * x(i) = df i + x0 and x(i) + df, for j in [0, ny], i in [0, nx]; the same double-double functions
 * as everywhere else, so a table entry equals a direct call bit for bit */
struct WallTrig {
    const double4 *row;   /* (sin y, cos y, sin(y + dq), cos(y + dq)) */
    const double4 *col;   /* (sin x, cos x, sin(x + df), cos(x + df)) */
};

__global__ void ray_wall_trig(RayGridDev g, double4 *row, double4 *col)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    fdt_dd s, c, s2, c2;
    if (k <= g.ny) {
        const double yj = g.dq * k + g.y0;
        fdt_sincos_full(yj, &s, &c);
        fdt_sincos_full(yj + g.dq, &s2, &c2);
        row[k] = make_double4(s.hi + s.lo, c.hi + c.lo, s2.hi + s2.lo, c2.hi + c2.lo);
    }
    if (k <= g.nx) {
        const double xi = g.df * k + g.x0;
        fdt_sincos_full(xi, &s, &c);
        fdt_sincos_full(xi + g.df, &s2, &c2);
        col[k] = make_double4(s.hi + s.lo, c.hi + c.lo, s2.hi + s2.lo, c2.hi + c2.lo);
    }
}

/* (sin, cos) of y(je) (second = 0) or y(je) + dq (second = 1); a direct call off the table */
__device__ __forceinline__ void row_trig(const RayGridDev &g, const WallTrig &w, int je, int second, double *sn,
                                         double *cs)
{
    if (je >= 0 && je <= g.ny) {
        const double4 v = w.row[je];
        *sn = second ? v.z : v.x;
        *cs = second ? v.w : v.y;
        return;
    }
    const double yj = g.dq * je + g.y0;
    fdt_dd s, c;
    fdt_sincos_full(second ? yj + g.dq : yj, &s, &c);
    *sn = s.hi + s.lo;
    *cs = c.hi + c.lo;
}

__device__ __forceinline__ void col_trig(const RayGridDev &g, const WallTrig &w, int ie, int second, double *sn,
                                         double *cs)
{
    if (ie >= 0 && ie <= g.nx) {
        const double4 v = w.col[ie];
        *sn = second ? v.z : v.x;
        *cs = second ? v.w : v.y;
        return;
    }
    const double xi = g.df * ie + g.x0;
    fdt_dd s, c;
    fdt_sincos_full(second ? xi + g.df : xi, &s, &c);
    *sn = s.hi + s.lo;
    *cs = c.hi + c.lo;
}

/* one segment of length dlen with midpoint (xm, ym, zm) onto the coarse grid; false if the
 * midpoint is beyond it (where the reference asserts) */
__device__ bool add_segment(const RayGridDev &g, const float *gx, const float *gy, const float *gz, float xm, float ym,
                            float zm, double dlen, RayList &L)
{
    int i1 = -1, j1 = -1, k1 = -1;
    for (int q = 1; q < g.nxc; q++)
        if (xm < gx[q]) { i1 = q; break; }
    if (i1 < 0) return false;
    for (int q = 1; q < g.nyc; q++)
        if (ym < gy[q]) { j1 = q; break; }
    if (j1 < 0) return false;
    for (int q = 1; q < g.nzc; q++)
        if (zm < gz[q]) { k1 = q; break; }
    if (k1 < 0) return false;
    const float hx = gx[i1] - gx[i1 - 1];
    const float hy = gy[j1] - gy[j1 - 1];
    const float hz = gz[k1] - gz[k1 - 1];
    const double fx = (xm - gx[i1 - 1]) / hx;
    const double fy = (ym - gy[j1 - 1]) / hy;
    const double fz = (zm - gz[k1 - 1]) / hz;
    float ds[8];
    ds[0] = (1.f - fz) * (1.f - fy) * (1.f - fx);
    ds[1] = (1.f - fz) * (1.f - fy) * fx;
    ds[2] = (1.f - fz) * fy * (1.f - fx);
    ds[3] = (1.f - fz) * fy * fx;
    ds[4] = fz * (1.f - fy) * (1.f - fx);
    ds[5] = fz * (1.f - fy) * fx;
    ds[6] = fz * fy * (1.f - fx);
    ds[7] = fz * fy * fx;
    /* corner indices start at column i1, as the reference writes them (src/sphrayderv.c:2195-2205) */
    const int nxyc = g.nxc * g.nyc, nxyzc = nxyc * g.nzc;
    const int nk = nxyc * (k1 - 1), nj = g.nxc * (j1 - 1), nk2 = nxyc * k1, nj2 = g.nxc * j1;
    int jpt[8];
    jpt[0] = nk + nj + i1;
    jpt[1] = nk + nj + i1 + 1;
    jpt[2] = nk + nj2 + i1;
    jpt[3] = nk + nj2 + i1 + 1;
    jpt[4] = nk2 + nj + i1;
    jpt[5] = nk2 + nj + i1 + 1;
    jpt[6] = nk2 + nj2 + i1;
    jpt[7] = nk2 + nj2 + i1 + 1;
    const int cell = (k1 * g.nyc + j1) * g.nxc + i1;
    if (cell != L.cell) {
        for (int q = 0; q < 8; q++) L.pos[q] = jpt[q] < nxyzc ? L.find(jpt[q]) : -2;
        L.cell = cell;
    }
    for (int q = 0; q < 8; q++)
        if (L.pos[q] != -2) L.add_at(L.pos[q], ds[q] * dlen);
    return true;
}

__global__ void __launch_bounds__(kRayBlock) ray_trace(RayGridDev g, WallTrig wt, const float *__restrict__ coarse,
                                                       const RayObsDev *__restrict__ obs, int nobs, int max_seg,
                                                       int cap, fdgpu_ray_result *__restrict__ res,
                                                       int *__restrict__ lidx, float *__restrict__ lval)
{
    extern __shared__ float s_coarse[];
    const int ncoarse = g.nxc + g.nyc + g.nzc;
    for (int q = threadIdx.x; q < ncoarse; q += blockDim.x) s_coarse[q] = coarse[q];
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nobs) return;
    const float *gx = s_coarse, *gy = s_coarse + g.nxc, *gz = s_coarse + g.nxc + g.nyc;
    const RayObsDev ob = obs[k];
    const int o = ob.out;
    const float *t = ob.t;
    fdgpu_ray_result r;
    memset(&r, 0, sizeof r);
    RayList L;
    L.li = lidx + (size_t)o * cap;
    L.lv = lval + (size_t)o * cap;
    L.n = 0;
    L.cap = cap;
    L.over = false;
    L.cell = -1;

    const double x0 = g.x0, y0 = g.y0, z0 = g.z0, h = g.h, dq = g.dq, df = g.df;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double tolmin = h * 1.E-6f, tolmax = h * 6.0f;
    const double xs = ob.xs, ys = ob.ys, zs = ob.zs;
    const int is = (int)round((xs - x0) / df), js = (int)round((ys - y0) / dq), ks = (int)round((zs - z0) / h);
    const int iscell = trunc_i((xs - x0) / df), jscell = trunc_i((ys - y0) / dq), kscell = trunc_i((zs - z0) / h);
    const double ex = ob.ex, ey = ob.ey, ez = ob.ez;
    const int ies = trunc_i((ex - x0) / df), jes = trunc_i((ey - y0) / dq), kes = trunc_i((ez - z0) / h);
    const float xis = df * ies + x0, yjs = dq * jes + y0, zks = h * kes + z0;

    double xx = ex, yy = ey, zz = ez;
    int ie = ies, je = jes, ke = kes;
    double xi = xis, yj = yjs, zk = zks;
    long long ipt[8];
    int nseg = 0;
    do {
        if (!corners(g, ie, je, ke, ipt)) { r.status = FDGPU_RAY_OUTSIDE; break; }
        bool notime = false;
        for (int q = 0; q < 8; q++) notime = notime || t[ipt[q]] > 1.E9;
        if (notime) { r.status = FDGPU_RAY_NOTIME; break; }

        /* residual and hypocentre derivatives at the event (src/sphrayderv.c:1366-1441) */
        {
            const double fx = (xx - xi) / df, fy = (yy - yj) / dq, fz = (zz - zk) / h;
            float ds[8];
            ds[0] = (1.f - fz) * (1.f - fy) * (1.f - fx);
            ds[1] = (1.f - fz) * (1.f - fy) * fx;
            ds[2] = (1.f - fz) * fy * (1.f - fx);
            ds[3] = (1.f - fz) * fy * fx;
            ds[4] = fz * (1.f - fy) * (1.f - fx);
            ds[5] = fz * (1.f - fy) * fx;
            ds[6] = fz * fy * (1.f - fx);
            ds[7] = fz * fy * fx;
            float tc8[8];
            for (int q = 0; q < 8; q++) tc8[q] = t[ipt[q]];
            double dt = 0;
            for (int q = 0; q < 8; q++) dt += ds[q] * tc8[q];
            dt += 0.0f;
            dt += ob.tc;
            dt = ob.obstime - dt;
            r.dt = dt;
            r.resmin = (float)dt;
            float dsdx[8], dsdy[8], dsdz[8];
            dsdx[0] = -(1.f - fz) * (1.f - fy);
            dsdx[1] = (1.f - fz) * (1.f - fy);
            dsdx[2] = -(1.f - fz) * fy;
            dsdx[3] = (1.f - fz) * fy;
            dsdx[4] = -fz * (1.f - fy);
            dsdx[5] = fz * (1.f - fy);
            dsdx[6] = -fz * fy;
            dsdx[7] = fz * fy;
            dsdy[0] = -(1.f - fz) * (1.f - fx);
            dsdy[1] = -(1.f - fz) * fx;
            dsdy[2] = (1.f - fz) * (1.f - fx);
            dsdy[3] = (1.f - fz) * fx;
            dsdy[4] = -fz * (1.f - fx);
            dsdy[5] = -fz * fx;
            dsdy[6] = fz * (1.f - fx);
            dsdy[7] = fz * fx;
            dsdz[0] = -(1.f - fy) * (1.f - fx);
            dsdz[1] = -(1.f - fy) * fx;
            dsdz[2] = -fy * (1.f - fx);
            dsdz[3] = -fy * fx;
            dsdz[4] = (1.f - fy) * (1.f - fx);
            dsdz[5] = (1.f - fy) * fx;
            dsdz[6] = fy * (1.f - fx);
            dsdz[7] = fy * fx;
            float dtdx = 0, dtdy = 0, dtdz = 0;
            for (int q = 0; q < 8; q++) {
                dtdx += dsdx[q] * tc8[q];
                dtdy += dsdy[q] * tc8[q];
                dtdz += dsdz[q] * tc8[q];
            }
            dtdx /= df;
            dtdy /= dq;
            dtdz /= h;
            const float wet = sqrtf(ob.pwt);
            r.wet = wet;
            r.am[0] = wet;
            r.am[1] = dtdx * wet;
            r.am[2] = dtdy * wet;
            r.am[3] = dtdz * wet;
        }

        /* the station in the cartesian frame, for the last cells (src/sphrayderv.c:1812-1817) */
        float x2, y2, z2;
        {
            const double rr = kRearth - zs;
            fdt_dd sdd, cdd;
            fdt_sincos_full(xs, &sdd, &cdd);
            const double sxs = sdd.hi + sdd.lo, cxs = cdd.hi + cdd.lo;
            fdt_sincos_full(ys, &sdd, &cdd);
            const double sys_ = sdd.hi + sdd.lo, cys = cdd.hi + cdd.lo;
            x2 = rr * sys_ * cxs;
            y2 = rr * sys_ * sxs;
            z2 = rr * cys;
        }

        /* the ray (src/sphrayderv.c:1444-2232) */
        int iseg = 0, isegm1 = 0, isegm2 = 0;
        for (;;) {
            xi = df * ie + x0;
            yj = dq * je + y0;
            zk = h * ke + z0;
            const float dxs = xx - xs, dys = yy - ys, dzs = zz - zs;
            const float rs = kRearth - zz;
            const float dqs = rs * dys;
            fdt_dd sdd, cdd;
            fdt_sincos_full(yy, &sdd, &cdd);
            double sinq = sdd.hi + sdd.lo, cosq = cdd.hi + cdd.lo;
            const float dfs = rs * sinq * dxs;
            const float float_dlen = sqrtf(dfs * dfs + dqs * dqs + dzs * dzs);
            double dlen = float_dlen;
            if ((ie == iscell && je == jscell && ke == kscell) || (dlen < (h / 1000.f))) {
                const float xm = xx - dxs * 0.5f, ym = yy - dys * 0.5f, zm = zz - dzs * 0.5f;
                r.status = add_segment(g, gx, gy, gz, xm, ym, zm, dlen, L) ? FDGPU_RAY_OK : FDGPU_RAY_COARSE;
                break;
            }
            if (nseg >= max_seg) { r.status = FDGPU_RAY_STEPS; break; }
            if (!corners(g, ie, je, ke, ipt)) { r.status = FDGPU_RAY_OUTSIDE; break; }
            float tv[8];
            for (int q = 0; q < 8; q++) tv[q] = t[ipt[q]];
            const double r1 = kRearth - zk, r2 = r1 - h;
            double sq1, cq1, sq2, cq2;
            row_trig(g, wt, je, 0, &sq1, &cq1);   /* q1 = yj */
            row_trig(g, wt, je, 1, &sq2, &cq2);   /* q2 = yj + dq */
            double gradt[3];
            gradt[0] = ((tv[1] - tv[0]) / (r1 * sq1) + (tv[3] - tv[2]) / (r1 * sq2) + (tv[5] - tv[4]) / (r2 * sq1)
                        + (tv[7] - tv[6]) / (r2 * sq2)) / (4 * df);
            gradt[1] = ((tv[2] + tv[3] - tv[0] - tv[1]) / r1 + (tv[6] + tv[7] - tv[4] - tv[5]) / r2) / (4 * dq);
            gradt[2] = (tv[4] + tv[5] + tv[6] + tv[7] - tv[0] - tv[1] - tv[2] - tv[3]) / (4 * h);
            gradt[0] = gradt[0] * -1;
            gradt[1] = gradt[1] * -1;

            fdt_sincos_full(xx, &sdd, &cdd);
            double sinf_ = sdd.hi + sdd.lo, cosf_ = cdd.hi + cdd.lo;
            double ro = kRearth - zz;
            const double xo = ro * sinq * cosf_, yo = ro * sinq * sinf_, zo = ro * cosq;
            double sx, sy, sz;
            if (ie >= (is - 2) && ie < (is + 2) && je >= (js - 2) && je < (js + 2) && ke >= (ks - 2)
                && ke < (ks + 2)) {
                const double dx = x2 - xo, dy = y2 - yo, dz = z2 - zo;
                const double dl = sqrt(dx * dx + dy * dy + dz * dz);
                sx = dx / dl;
                sy = dy / dl;
                sz = dz / dl;
            } else {
                const double gradtm = sqrt(gradt[0] * gradt[0] + gradt[1] * gradt[1] + gradt[2] * gradt[2]);
                const double sf = gradt[0] / gradtm, sq = gradt[1] / gradtm, sr = gradt[2] / gradtm;
                sx = -sinf_ * sf + cosq * cosf_ * sq + sinq * cosf_ * sr;
                sy = cosf_ * sf + cosq * sinf_ * sq + sinq * sinf_ * sr;
                sz = -sinq * sq + cosq * sr;
                const float smag = sqrtf((float)(sx * sx + sy * sy + sz * sz));
                sx /= smag;
                sy /= smag;
                sz /= smag;
            }

            double dd[3];
            double a, b, c, quad;
            dd[2] = -1e20;
            if (gradt[2] != 0) {
                ro = gradt[2] > 0 ? kRearth - zk : kRearth - zk - h;
                b = xo * sx + yo * sy + zo * sz;
                c = xo * xo + yo * yo + zo * zo - ro * ro;
                quad = b * b - c;
                if (quad >= 0) {
                    const float d1 = -b + sqrt(quad);
                    const float d2 = -b - sqrt(quad);
                    dd[2] = pmin(d1, d2);
                }
            }
            dd[1] = -1e20;
            if (gradt[1] != 0) {
                if (gradt[1] < 0) {
                    sinq = sq1;
                    cosq = cq1;
                } else {
                    sinq = sq2;
                    cosq = cq2;
                }
                if (fabs(cosq) > fabs(sinq)) {
                    const double tanq = sinq / cosq, tansq = tanq * tanq;
                    a = sx * sx + sy * sy - sz * sz * tansq;
                    b = xo * sx + yo * sy - zo * sz * tansq;
                    c = xo * xo + yo * yo - zo * zo * tansq;
                } else {
                    const double ctanq = cosq / sinq, ctansq = ctanq * ctanq;
                    a = (sx * sx + sy * sy) * ctansq - sz * sz;
                    b = (xo * sx + yo * sy) * ctansq - zo * sz;
                    c = (xo * xo + yo * yo) * ctansq - zo * zo;
                }
                quad = b * b - a * c;
                if (quad >= 0) {
                    const float d1 = (-b + sqrt(quad)) / a;
                    const float d2 = (-b - sqrt(quad)) / a;
                    dd[1] = pmin(d1, d2);
                }
            }
            dd[0] = -1e20;
            if (gradt[0] != 0) {
                col_trig(g, wt, ie, gradt[0] < 0 ? 0 : 1, &sinf_, &cosf_);
                float d1;
                if (fabs(cosf_) > fabs(sinf_)) {
                    const double tanf_ = sinf_ / cosf_;
                    d1 = (xo * tanf_ - yo) / (sy - sx * tanf_);
                } else {
                    const double ctanf_ = cosf_ / sinf_;
                    d1 = (yo * ctanf_ - xo) / (sx - sy * ctanf_);
                }
                if (d1 > 0) dd[0] = d1;
            }

            const int back3 = iseg + isegm1 + isegm2;
            if (gradt[0] < 0) {
                if (dd[0] < h / 1000 && (iseg == 1 || (back3 == 1 && nseg >= 3))) { gradt[0] = 0.; dd[0] = -1e20; }
            } else if (gradt[0] > 0) {
                if (dd[0] < h / 1000 && (iseg == -1 || (back3 == -1 && nseg >= 3))) { gradt[0] = 0; dd[0] = -1e20; }
            } else {
                dd[0] = -1e20;
            }
            if (gradt[1] < 0) {
                if (dd[1] < h / 1000 && (iseg == 20 || (back3 == 20 && nseg >= 3))) { gradt[1] = 0.; dd[1] = -1e20; }
            } else if (gradt[1] > 0) {
                if (dd[1] < h / 1000 && (iseg == -20 || (back3 == -20 && nseg >= 3))) { gradt[1] = 0; dd[1] = -1e20; }
            } else {
                dd[1] = -1e20;
            }
            if (gradt[2] > 0) {
                if (dd[2] < h / 1000 && (iseg == 300 || (back3 == 300 && nseg >= 3))) { gradt[2] = 0.; dd[2] = -1e20; }
            } else if (gradt[2] < 0) {
                if (dd[2] < h / 1000 && (iseg == -300 || (back3 == -300 && nseg >= 3))) { gradt[2] = 0; dd[2] = -1e20; }
            } else {
                dd[2] = -1e20;
            }

            double d;
            int md;
            dfind(dd, &d, &md, tolmin, tolmax);
            dlen = d;
            const double xold = xx, yold = yy, zold = zz;
            const double xn = xo + d * sx, yn = yo + d * sy, zn = zo + d * sz;
            xx = fdt_atan2(yn, xn);
            yy = fdt_atan2(sqrt(xn * xn + yn * yn), zn);
            zz = kRearth - sqrt(xn * xn + yn * yn + zn * zn);
            nseg++;
            isegm2 = isegm1;
            isegm1 = iseg;
            bool left = false;
            if (md == 0) {
                je = trunc_i((yy - y0) / dq);
                ke = trunc_i((zz - z0) / h);
                if (gradt[0] < 0) {
                    if (ie < 0) left = true; else { ie--; iseg = -1; }
                } else {
                    if (ie >= nx - 1) left = true; else { ie++; iseg = 1; }
                }
            } else if (md == 1) {
                if (gradt[1] < 0) {
                    if (je < 0) left = true; else { je--; iseg = -20; }
                } else {
                    if (je >= ny - 1) left = true; else { je++; iseg = 20; }
                }
                if (!left) {
                    ie = trunc_i((xx - x0) / df);
                    ke = trunc_i((zz - z0) / h);
                }
            } else {
                if (gradt[2] > 0) {
                    if (ke < 0) left = true; else { ke--; iseg = -300; }
                } else {
                    if (ke >= nz - 1) left = true; else { ke++; iseg = 300; }
                }
                if (!left) {
                    ie = trunc_i((xx - x0) / df);
                    je = trunc_i((yy - y0) / dq);
                }
            }
            if (left || (xx < x0 || ie >= nx) || (yy < y0 || je >= ny) || (zz < z0 || ke >= nz)) {
                r.status = FDGPU_RAY_LEFT;
                break;
            }
            const float xm = (xx + xold) * 0.5, ym = (yy + yold) * 0.5, zm = (zz + zold) * 0.5;
            if (!add_segment(g, gx, gy, gz, xm, ym, zm, dlen, L)) { r.status = FDGPU_RAY_COARSE; break; }
        }
    } while (false);
    r.nseg = nseg;
    if (r.status == FDGPU_RAY_OK && L.over) r.status = FDGPU_RAY_STEPS;
    int nnz = 0;
    if (r.status == FDGPU_RAY_OK) {
        /* ascending node order, zero sums dropped (src/sphrayderv.c:1548-1552) */
        for (int q = 1; q < L.n; q++) {
            const int ki = L.li[q];
            const float kv = L.lv[q];
            int p = q - 1;
            while (p >= 0 && L.li[p] > ki) {
                L.li[p + 1] = L.li[p];
                L.lv[p + 1] = L.lv[p];
                p--;
            }
            L.li[p + 1] = ki;
            L.lv[p + 1] = kv;
        }
        for (int q = 0; q < L.n; q++)
            if (L.lv[q] != 0) {
                L.li[nnz] = L.li[q];
                L.lv[nnz] = L.lv[q];
                nnz++;
            }
    }
    r.nnz = nnz;
    res[o] = r;
}

/* the rays' lists into the packed arrays: one warp per ray */
__global__ void ray_pack(const fdgpu_ray_result *__restrict__ res, const long long *__restrict__ off, int nobs,
                         int cap, const int *__restrict__ lidx, const float *__restrict__ lval, int *__restrict__ idx,
                         float *__restrict__ du)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nobs) return;
    const int n = res[w].nnz;
    const long long base = off[w];
    for (int q = lane; q < n; q += 32) {
        idx[base + q] = lidx[(size_t)w * cap + q];
        du[base + q] = lval[(size_t)w * cap + q];
    }
}

struct Arena {
    std::vector<void *> ptrs;
    cudaStream_t s;
    explicit Arena(cudaStream_t st) : s(st) {}
    ~Arena()
    {
        for (void *p : ptrs) cudaFreeAsync(p, s);
    }
    template <class T> cudaError_t get(T **out, size_t n)
    {
        void *p = nullptr;
        const cudaError_t e = cudaMallocAsync(&p, sizeof(T) * (n ? n : 1), s);
        if (e == cudaSuccess) ptrs.push_back(p);
        *out = static_cast<T *>(p);
        return e;
    }
};

}  // namespace

#define RAY_CU(call)                                                        \
    do {                                                                    \
        const cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return fdh_ctx_fail(ctx, (int)e_, #call);    \
    } while (0)

extern "C" int fdgpu_ray_default_limits(const fdgpu_ray_grid *g, int *max_seg, int *cap)
{
    if (!g) return FDGPU_EINVAL;
    if (max_seg) *max_seg = 16 * (g->nx + g->ny + g->nz) + 256;
    if (cap) *cap = 8 * (g->nx + g->ny + g->nz) + 64;
    return FDGPU_OK;
}

extern "C" int fdgpu_raytrace(fdgpu_ctx *ctx, const fdgpu_ray_grid *g, const float *const *d_fields, int nfields,
                              int nobs, const fdgpu_ray_obs *obs, int max_seg, int cap, fdgpu_ray_result *res,
                              long long *off, int *idx, float *du, long long total_cap, void *stream)
{
    if (!ctx || !g || nobs < 0 || nobs > (1 << 24) || (nobs > 0 && (!d_fields || !obs || !res || !off)))
        return FDGPU_EINVAL;
    if (g->nx < 2 || g->ny < 2 || g->nz < 2 || g->nxc < 2 || g->nyc < 2 || g->nzc < 2 || !g->gx || !g->gy || !g->gz
        || !(g->h > 0) || !(g->dq > 0) || !(g->df > 0))
        return FDGPU_EINVAL;
    if ((long long)g->nx * g->ny * g->nz >= (1ll << 31) || (long long)g->nxc * g->nyc * g->nzc >= (1ll << 30)
        || g->nxc + g->nyc + g->nzc > 8192)
        return FDGPU_EINVAL;
    int dseg = 0, dcap = 0;
    fdgpu_ray_default_limits(g, &dseg, &dcap);
    if (max_seg <= 0) max_seg = dseg;
    if (cap <= 0) cap = dcap;
    for (int k = 0; k < nobs; k++)
        if (obs[k].field < 0 || obs[k].field >= nfields || !d_fields[obs[k].field]) return FDGPU_EINVAL;
    off[0] = 0;
    if (nobs == 0) return FDGPU_OK;
    FdDeviceScope dev_(fdh_ctx_device(ctx));
    if (dev_.err) return FDGPU_ENODEV;
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)fdh_ctx_stream(ctx);

    /* launch order: longest rays first (cells between event and station), so that a warp's rays end
     * together; each result goes back to its observation's slot */
    std::vector<int> order(nobs);
    std::vector<double> span(nobs);
    for (int k = 0; k < nobs; k++) {
        const fdgpu_ray_obs &o = obs[k];
        span[k] = std::fabs((o.ex - o.xs) / g->df) + std::fabs((o.ey - o.ys) / g->dq) + std::fabs((o.ez - o.zs) / g->h);
        if (!(span[k] == span[k])) span[k] = 0;
        order[k] = k;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return span[a] > span[b]; });
    std::vector<RayObsDev> hobs(nobs);
    for (int q = 0; q < nobs; q++) {
        const fdgpu_ray_obs &o = obs[order[q]];
        hobs[q] = RayObsDev{o.ex, o.ey, o.ez, o.xs, o.ys, o.zs, d_fields[o.field], o.obstime, o.pwt, o.tc, order[q]};
    }
    const int ncoarse = g->nxc + g->nyc + g->nzc;
    std::vector<float> hc(ncoarse);
    std::memcpy(hc.data(), g->gx, sizeof(float) * g->nxc);
    std::memcpy(hc.data() + g->nxc, g->gy, sizeof(float) * g->nyc);
    std::memcpy(hc.data() + g->nxc + g->nyc, g->gz, sizeof(float) * g->nzc);

    Arena mem(st);
    RayObsDev *dobs;
    float *dcoarse, *lval, *ddu;
    int *lidx, *didx;
    fdgpu_ray_result *dres;
    long long *doff;
    double4 *drow, *dcol;
    RAY_CU(mem.get(&dobs, nobs));
    RAY_CU(mem.get(&drow, (size_t)g->ny + 1));
    RAY_CU(mem.get(&dcol, (size_t)g->nx + 1));
    RAY_CU(mem.get(&dcoarse, ncoarse));
    RAY_CU(mem.get(&dres, nobs));
    RAY_CU(mem.get(&lidx, (size_t)nobs * cap));
    RAY_CU(mem.get(&lval, (size_t)nobs * cap));
    RAY_CU(mem.get(&doff, nobs + 1));
    RAY_CU(cudaMemcpyAsync(dobs, hobs.data(), sizeof(RayObsDev) * nobs, cudaMemcpyHostToDevice, st));
    RAY_CU(cudaMemcpyAsync(dcoarse, hc.data(), sizeof(float) * ncoarse, cudaMemcpyHostToDevice, st));
    const RayGridDev G{g->nx, g->ny, g->nz, g->nxc, g->nyc, g->nzc, g->x0, g->y0, g->z0, g->h, g->dq, g->df};
    const int nwall = (g->nx > g->ny ? g->nx : g->ny) + 1;
    ray_wall_trig<<<(nwall + 127) / 128, 128, 0, st>>>(G, drow, dcol);
    RAY_CU(cudaGetLastError());
    ray_trace<<<(nobs + kRayBlock - 1) / kRayBlock, kRayBlock, sizeof(float) * ncoarse, st>>>(
        G, WallTrig{drow, dcol}, dcoarse, dobs, nobs, max_seg, cap, dres, lidx, lval);
    RAY_CU(cudaGetLastError());
    RAY_CU(cudaMemcpyAsync(res, dres, sizeof(fdgpu_ray_result) * nobs, cudaMemcpyDeviceToHost, st));
    RAY_CU(cudaStreamSynchronize(st));
    for (int k = 0; k < nobs; k++) off[k + 1] = off[k] + res[k].nnz;
    const long long total = off[nobs];
    if (total > total_cap || (total > 0 && (!idx || !du))) return FDGPU_ETOOBIG;
    if (total == 0) return FDGPU_OK;
    RAY_CU(mem.get(&didx, (size_t)total));
    RAY_CU(mem.get(&ddu, (size_t)total));
    RAY_CU(cudaMemcpyAsync(doff, off, sizeof(long long) * (nobs + 1), cudaMemcpyHostToDevice, st));
    ray_pack<<<(nobs * 32 + 255) / 256, 256, 0, st>>>(dres, doff, nobs, cap, lidx, lval, didx, ddu);
    RAY_CU(cudaGetLastError());
    RAY_CU(cudaMemcpyAsync(idx, didx, sizeof(int) * total, cudaMemcpyDeviceToHost, st));
    RAY_CU(cudaMemcpyAsync(du, ddu, sizeof(float) * total, cudaMemcpyDeviceToHost, st));
    RAY_CU(cudaStreamSynchronize(st));
    return FDGPU_OK;
}
