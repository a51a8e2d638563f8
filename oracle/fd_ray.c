/* Oracle for sphrayderv's ray tracing and derivatives (test infrastructure only; see fd_ray.h).
 *
 * Every intermediate keeps the C type the reference gives it, because the type decides the
 * rounding: the reference's globals xx, yy, zz, xi, gradt, sx, dlen, dt, fx ... are double, its
 * xm/ym/zm, ds[], smag, d1/d2, x2/y2/z2 and the per-observation sums dtdx... are float, and the
 * event cell's corner xis/yjs/zks is float (src/sphrayderv.c:89-100, :880, :1278-1279). */
#include "fd_ray.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../fdtomoc_gb300/csrc/fd_trig.h"

static const float kRearth = 6371.0f;   /* :87 */

static double t_sin(int m, double x) { return m ? fdt_sin(x) : sin(x); }
static double t_cos(int m, double x) { return m ? fdt_cos(x) : cos(x); }
static double t_atan2(int m, double y, double x) { return m ? fdt_atan2(y, x) : atan2(y, x); }

double fdr_trig(int trig_mode, int which, double y, double x)
{
    return which == 0 ? t_sin(trig_mode, y) : which == 1 ? t_cos(trig_mode, y) : t_atan2(trig_mode, y, x);
}

/* (int) of a double as x86-64 converts it: truncation, INT_MIN for NaN and out-of-range values */
static int trunc_i(double v)
{
    if (!(v > -2147483649.0 && v < 2147483648.0)) return INT_MIN;
    return (int)v;
}

/* lib/sphrayderv/pmin.c: the smaller non-negative of two, else -1e20 */
static double pmin(double d1, double d2)
{
    if (d1 >= 0) return (d2 >= 0) ? (d1 < d2 ? d1 : d2) : d1;
    return d2 >= 0 ? d2 : -1e20;
}

/* lib/sphrayderv/dfind.c: order the three candidate steps by magnitude; take the smallest unless it
 * is below tolmin, then the middle one (if below tolmax) or the largest */
static void dfind(const double dd[3], double *d, int *md, double tolmin, double tolmax)
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

/* the eight corners of fine cell (ie, je, ke) as linear indices; 0 if one falls outside the field */
static int corners(const fdr_grid *g, int ie, int je, int ke, long long ipt[8])
{
    const long long nxy = (long long)g->nx * g->ny, n = nxy * g->nz;
    const long long nk = nxy * ke, nj = (long long)g->nx * je, nk2 = nxy * ((long long)ke + 1),
                    nj2 = (long long)g->nx * ((long long)je + 1);
    ipt[0] = nk + nj + ie;
    ipt[1] = nk + nj + ie + 1;
    ipt[2] = nk + nj2 + ie;
    ipt[3] = nk + nj2 + ie + 1;
    ipt[4] = nk2 + nj + ie;
    ipt[5] = nk2 + nj + ie + 1;
    ipt[6] = nk2 + nj2 + ie;
    ipt[7] = nk2 + nj2 + ie + 1;
    for (int q = 0; q < 8; q++)
        if (ipt[q] < 0 || ipt[q] >= n) return 0;
    return 1;
}

/* add a segment of length dlen whose midpoint is (xm, ym, zm) to du on the coarse grid
 * (:1481-1540 for the station segment, :2155-2225 for the others); 0 if the midpoint is beyond it */
static int add_segment(const fdr_grid *g, float xm, float ym, float zm, double dlen, float *du)
{
    int i1 = -1, j1 = -1, k1 = -1;
    for (int q = 1; q < g->nxc; q++)
        if (xm < g->gx[q]) { i1 = q; break; }
    if (i1 < 0) return 0;
    for (int q = 1; q < g->nyc; q++)
        if (ym < g->gy[q]) { j1 = q; break; }
    if (j1 < 0) return 0;
    for (int q = 1; q < g->nzc; q++)
        if (zm < g->gz[q]) { k1 = q; break; }
    if (k1 < 0) return 0;
    const float hx = g->gx[i1] - g->gx[i1 - 1];
    const float hy = g->gy[j1] - g->gy[j1 - 1];
    const float hz = g->gz[k1] - g->gz[k1 - 1];
    const double fx = (xm - g->gx[i1 - 1]) / hx;   /* float arithmetic, kept as double */
    const double fy = (ym - g->gy[j1 - 1]) / hy;
    const double fz = (zm - g->gz[k1 - 1]) / hz;
    float ds[8];
    ds[0] = (1.f - fz) * (1.f - fy) * (1.f - fx);
    ds[1] = (1.f - fz) * (1.f - fy) * fx;
    ds[2] = (1.f - fz) * fy * (1.f - fx);
    ds[3] = (1.f - fz) * fy * fx;
    ds[4] = fz * (1.f - fy) * (1.f - fx);
    ds[5] = fz * (1.f - fy) * fx;
    ds[6] = fz * fy * (1.f - fx);
    ds[7] = fz * fy * fx;
    /* the reference's corner indices start at column i1, not i1 - 1 (:2195-2205) */
    const int nxyc = g->nxc * g->nyc, nxyzc = nxyc * g->nzc;
    const int nk = nxyc * (k1 - 1), nj = g->nxc * (j1 - 1), nk2 = nxyc * k1, nj2 = g->nxc * j1;
    int jpt[8];
    jpt[0] = nk + nj + i1;
    jpt[1] = nk + nj + i1 + 1;
    jpt[2] = nk + nj2 + i1;
    jpt[3] = nk + nj2 + i1 + 1;
    jpt[4] = nk2 + nj + i1;
    jpt[5] = nk2 + nj + i1 + 1;
    jpt[6] = nk2 + nj2 + i1;
    jpt[7] = nk2 + nj2 + i1 + 1;
    for (int q = 0; q < 8; q++)
        if (jpt[q] < nxyzc)   /* index nxyzc is cleared but never read back (:1614) */
            du[jpt[q]] += ds[q] * dlen;
    return 1;
}

static void trace_one(const fdr_grid *g, const float *t, const fdr_obs *o, int m, int max_seg, int cap,
                      fdr_result *r, int *idx, float *duo, float *du)
{
    const double x0 = g->x0, y0 = g->y0, z0 = g->z0, h = g->h, dq = g->dq, df = g->df;
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double tolmin = h * 1.E-6f, tolmax = h * 6.0f;   /* :521-522 */
    memset(r, 0, sizeof(*r));
    const double xs = o->xs, ys = o->ys, zs = o->zs;
    const int is = (int)round((xs - x0) / df), js = (int)round((ys - y0) / dq), ks = (int)round((zs - z0) / h);
    const int iscell = trunc_i((xs - x0) / df), jscell = trunc_i((ys - y0) / dq), kscell = trunc_i((zs - z0) / h);

    /* the event's cell (:930-937) and its corner, float as the reference keeps it */
    const double ex = o->ex, ey = o->ey, ez = o->ez;
    const int ies = trunc_i((ex - x0) / df), jes = trunc_i((ey - y0) / dq), kes = trunc_i((ez - z0) / h);
    const float xis = df * ies + x0, yjs = dq * jes + y0, zks = h * kes + z0;

    double xx = ex, yy = ey, zz = ez;
    int ie = ies, je = jes, ke = kes;
    double xi = xis, yj = yjs, zk = zks;
    long long ipt[8];
    if (!corners(g, ie, je, ke, ipt)) { r->status = FDR_OUTSIDE; return; }
    for (int q = 0; q < 8; q++)
        if (t[ipt[q]] > 1.E9) { r->status = FDR_NOTIME; return; }

    /* residual and hypocentre derivatives at the event (:1366-1441) */
    double fx = (xx - xi) / df, fy = (yy - yj) / dq, fz = (zz - zk) / h;
    {
        float ds[8];
        ds[0] = (1.f - fz) * (1.f - fy) * (1.f - fx);
        ds[1] = (1.f - fz) * (1.f - fy) * fx;
        ds[2] = (1.f - fz) * fy * (1.f - fx);
        ds[3] = (1.f - fz) * fy * fx;
        ds[4] = fz * (1.f - fy) * (1.f - fx);
        ds[5] = fz * (1.f - fy) * fx;
        ds[6] = fz * fy * (1.f - fx);
        ds[7] = fz * fy * fx;
        double dt = 0;
        for (int q = 0; q < 8; q++) dt += ds[q] * t[ipt[q]];
        dt += 0.0f;        /* ttel: 0 for a local event */
        dt += o->tc;
        dt = o->obstime - dt;
        r->dt = dt;
        r->resmin = (float)dt;
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
            dtdx += dsdx[q] * t[ipt[q]];
            dtdy += dsdy[q] * t[ipt[q]];
            dtdz += dsdz[q] * t[ipt[q]];
        }
        dtdx /= df;
        dtdy /= dq;
        dtdz /= h;
        const float wet = sqrtf(o->pwt);
        r->wet = wet;
        r->am[0] = wet;
        r->am[1] = dtdx * wet;
        r->am[2] = dtdy * wet;
        r->am[3] = dtdz * wet;
    }

    /* the ray, from the event back to the station (:1444-2232) */
    int nseg = 0, iseg = 0, isegm1 = 0, isegm2 = 0;
    const int nxyzc = g->nxc * g->nyc * g->nzc;
    for (;;) {
        xi = df * ie + x0;
        yj = dq * je + y0;
        zk = h * ke + z0;
        const float dxs = xx - xs, dys = yy - ys, dzs = zz - zs;
        const float rs = kRearth - zz;
        const float dqs = rs * dys;
        const float dfs = rs * t_sin(m, yy) * dxs;
        const float float_dlen = sqrtf(dfs * dfs + dqs * dqs + dzs * dzs);
        double dlen = float_dlen;
        if ((ie == iscell && je == jscell && ke == kscell) || (dlen < (h / 1000.f))) {
            /* last segment: to the station (:1470-1545) */
            const float xm = xx - dxs * 0.5f, ym = yy - dys * 0.5f, zm = zz - dzs * 0.5f;
            if (!add_segment(g, xm, ym, zm, dlen, du)) { r->status = FDR_COARSE; break; }
            r->status = FDR_OK;
            break;
        }
        if (nseg >= max_seg) { r->status = FDR_STEPS; break; }
        if (!corners(g, ie, je, ke, ipt)) { r->status = FDR_OUTSIDE; break; }
        const double r1 = kRearth - zk, r2 = r1 - h, q1 = yj, q2 = q1 + dq;
        double gradt[3];
        gradt[0] = ((t[ipt[1]] - t[ipt[0]]) / (r1 * t_sin(m, q1)) + (t[ipt[3]] - t[ipt[2]]) / (r1 * t_sin(m, q2))
                    + (t[ipt[5]] - t[ipt[4]]) / (r2 * t_sin(m, q1)) + (t[ipt[7]] - t[ipt[6]]) / (r2 * t_sin(m, q2)))
                   / (4 * df);
        gradt[1] = ((t[ipt[2]] + t[ipt[3]] - t[ipt[0]] - t[ipt[1]]) / r1
                    + (t[ipt[6]] + t[ipt[7]] - t[ipt[4]] - t[ipt[5]]) / r2) / (4 * dq);
        gradt[2] = (t[ipt[4]] + t[ipt[5]] + t[ipt[6]] + t[ipt[7]] - t[ipt[0]] - t[ipt[1]] - t[ipt[2]] - t[ipt[3]])
                   / (4 * h);
        gradt[0] = gradt[0] * -1;
        gradt[1] = gradt[1] * -1;

        double sinf_ = t_sin(m, xx), cosf_ = t_cos(m, xx), sinq = t_sin(m, yy), cosq = t_cos(m, yy);
        double ro = kRearth - zz;
        const double xo = ro * sinq * cosf_, yo = ro * sinq * sinf_, zo = ro * cosq;
        double sx, sy, sz;
        if (ie >= (is - 2) && ie < (is + 2) && je >= (js - 2) && je < (js + 2) && ke >= (ks - 2) && ke < (ks + 2)) {
            /* near the station: straight to it (:1812-1826) */
            const double rr = kRearth - zs;
            const float x2 = rr * t_sin(m, ys) * t_cos(m, xs);
            const float y2 = rr * t_sin(m, ys) * t_sin(m, xs);
            const float z2 = rr * t_cos(m, ys);
            const double dx = x2 - xo, dy = y2 - yo, dz = z2 - zo;
            const double dl = sqrt(dx * dx + dy * dy + dz * dz);
            sx = dx / dl;
            sy = dy / dl;
            sz = dz / dl;
        } else {
            /* down the gradient, rotated to the cartesian frame (:1827-1851) */
            const double gradtm = sqrt(gradt[0] * gradt[0] + gradt[1] * gradt[1] + gradt[2] * gradt[2]);
            const double sf = gradt[0] / gradtm, sq = gradt[1] / gradtm, sr = gradt[2] / gradtm;
            sx = -sinf_ * sf + cosq * cosf_ * sq + sinq * cosf_ * sr;
            sy = cosf_ * sf + cosq * sinf_ * sq + sinq * sinf_ * sr;
            sz = -sinq * sq + cosq * sr;
            const float smag = sqrtf(sx * sx + sy * sy + sz * sz);
            sx /= smag;
            sy /= smag;
            sz /= smag;
        }

        /* distances to the cell's walls along the ray (:1860-1930) */
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
                sinq = t_sin(m, yj);
                cosq = t_cos(m, yj);
            } else {
                sinq = t_sin(m, yj + dq);
                cosq = t_cos(m, yj + dq);
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
            if (gradt[0] < 0) {
                sinf_ = t_sin(m, xi);
                cosf_ = t_cos(m, xi);
            } else {
                sinf_ = t_sin(m, xi + df);
                cosf_ = t_cos(m, xi + df);
            }
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

        /* no step straight back into the cell just left, nor round a loop of four (:1932-2000) */
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

        /* step (:2002-2140) */
        double d;
        int md;
        dfind(dd, &d, &md, tolmin, tolmax);
        dlen = d;
        const double xold = xx, yold = yy, zold = zz;
        const double xn = xo + d * sx, yn = yo + d * sy, zn = zo + d * sz;
        xx = t_atan2(m, yn, xn);
        yy = t_atan2(m, sqrt(xn * xn + yn * yn), zn);
        zz = kRearth - sqrt(xn * xn + yn * yn + zn * zn);
        nseg++;
        isegm2 = isegm1;
        isegm1 = iseg;
        int left = 0;
        if (md == 0) {
            je = trunc_i((yy - y0) / dq);
            ke = trunc_i((zz - z0) / h);
            if (gradt[0] < 0) {
                if (ie < 0) left = 1; else { ie--; iseg = -1; }
            } else {
                if (ie >= nx - 1) left = 1; else { ie++; iseg = 1; }
            }
        } else if (md == 1) {
            if (gradt[1] < 0) {
                if (je < 0) left = 1; else { je--; iseg = -20; }
            } else {
                if (je >= ny - 1) left = 1; else { je++; iseg = 20; }
            }
            if (!left) {
                ie = trunc_i((xx - x0) / df);
                ke = trunc_i((zz - z0) / h);
            }
        } else {
            if (gradt[2] > 0) {
                if (ke < 0) left = 1; else { ke--; iseg = -300; }
            } else {
                if (ke >= nz - 1) left = 1; else { ke++; iseg = 300; }
            }
            if (!left) {
                ie = trunc_i((xx - x0) / df);
                je = trunc_i((yy - y0) / dq);
            }
        }
        if (left || (xx < x0 || ie >= nx) || (yy < y0 || je >= ny) || (zz < z0 || ke >= nz)) {
            r->status = FDR_LEFT;
            break;
        }
        const float xm = (xx + xold) * 0.5, ym = (yy + yold) * 0.5, zm = (zz + zold) * 0.5;
        if (!add_segment(g, xm, ym, zm, dlen, du)) { r->status = FDR_COARSE; break; }
    }
    r->nseg = nseg;
    /* the nonzero derivatives, ascending (:1548-1560), and du cleared for the next observation */
    int n = 0;
    for (int jb = 0; jb < nxyzc; jb++) {
        if (du[jb] != 0) {
            if (r->status == FDR_OK) {
                if (n < cap) {
                    idx[n] = jb;
                    duo[n] = du[jb];
                }
                n++;
            }
            du[jb] = 0;
        }
    }
    if (r->status == FDR_OK && n > cap) r->status = FDR_STEPS;
    r->nnz = r->status == FDR_OK ? n : 0;
}

int fdr_trace(const fdr_grid *g, const float *const *fields, int nobs, const fdr_obs *obs, int trig_mode,
              int max_seg, int cap, fdr_result *res, int *idx, float *du)
{
    const int nxyzc = g->nxc * g->nyc * g->nzc;
    float *dense = (float *)calloc((size_t)nxyzc + 1, sizeof(float));
    if (!dense) return -1;
    for (int o = 0; o < nobs; o++)
        trace_one(g, fields[obs[o].field], &obs[o], trig_mode, max_seg, cap, &res[o], idx + (size_t)o * cap,
                  du + (size_t)o * cap, dense);
    free(dense);
    return 0;
}
