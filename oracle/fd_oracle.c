/*
 * fd_oracle.c — CPU restatement of FDtomoC's sphfd travel-time solver (reference: src/sphfd.c).
 *
 * TEST INFRASTRUCTURE: the checker for the GPU library.  Only the tests, the smoke check and the
 * CPU-baseline leg of bench.py load it; the product never links it.
 *
 * Every function cites the reference lines it restates.  Floating-point expressions keep the
 * reference's operand order (left-to-right products and sums), because the GPU library is held to
 * bit-for-bit agreement with the reference and this file is the proof of the arithmetic.  Build
 * with -ffp-contract=off (no fused multiply-add), as the reference's -std=c99 build is on x86.
 */
#define _POSIX_C_SOURCE 200809L
#include "fd_oracle.h"
#include "../fdtomoc_gb300/csrc/fd_face_table.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Literal constants of the reference (src/sphfd.c:128-136). */
#define FDO_PI 3.141592654
#define FDO_HPI 1.570796327
#define FDO_REARTH 6371.0
#define FDO_DEGRAD (FDO_PI / 180.0)
#define FDO_UNSET 1.0e10f
#define FDO_HEADTEST 1.e-3

/* ------------------------------------------------------------------------------------------ */
/* Geometry: rc/qc (src/sphfd.c:154-156) and WGS84 glath (src/sphfd.c:5836-5893).               */

static inline double fdo_rc(const fdo_grid *g, int z) { return g->z0r - g->h * (double)z; }
static inline double fdo_qc(const fdo_grid *g, int y) { return g->y0 + g->dq * (double)y; }

double fdo_glath(double hlat, double depth_km, double *radius_km)
{
    const double ap = 6378137.0;
    const double esq = 0.00669437978616733379;
    const double hm = -depth_km * 1000.0;
    const double sinxl = sin(hlat);
    const double anu = ap / sqrt(1.0 - esq * sinxl * sinxl);
    const double xp = (anu + hm) * cos(hlat);
    const double zp = ((1.0 - esq) * anu + hm) * sinxl;
    *radius_km = sqrt(xp * xp + zp * zp) / 1000.0;
    return atan2(zp, xp);
}

/* ------------------------------------------------------------------------------------------ */
/* The four stencils (src/sphfd.c:5906-6184), same operand order as the reference.              */

/* fdsph3d: 8-node spherical transmission stencil, point = slot 7 (src/sphfd.c:5906-6013). */
static double fdo_st3d(const double t[8], const double s[8], const double r[8], const double q[8],
                       const int g[8], const int n[8], const int m[8], double h, double dq, double df)
{
    double slo = 0.0;
    for (int i = 0; i < 8; i++) slo += s[i];
    slo = 0.125 * slo;
    const double hsq = h * h, dqsq = dq * dq, dfsq = df * df;
    const double dfs7 = df * sin(q[7]);
    const double df2s7 = df * dfs7;
    const double a = 1.0 / hsq + (1.0 / dqsq + 1. / (dfs7 * dfs7)) / (r[7] * r[7]);
    double b = 0.0;
    for (int i = 0; i < 7; i++)
        b += t[i] * ((double)(g[7] * g[i]) / hsq
                     + ((double)(n[7] * n[i]) / dqsq + (double)(m[7] * m[i]) / (df2s7 * sin(q[i])))
                       / (r[7] * r[i]));
    b = 2.0 * b;
    double c = 0.0;
    for (int i = 0; i < 7; i++) {
        const double dfsi = df * sin(q[i]);
        c += t[i] * t[i] * (1. / hsq + (1. / dqsq + 1. / (dfsi * dfsi)) / (r[i] * r[i]));
    }
    for (int i = 0; i < 6; i++) {
        double c2 = 0.0;
        const double df2si = dfsq * sin(q[i]);
        for (int j = i + 1; j < 7; j++)
            c2 += t[j] * ((double)(g[i] * g[j]) / hsq
                          + ((double)(n[i] * n[j]) / dqsq + (double)(m[i] * m[j]) / (df2si * sin(q[j])))
                            / (r[i] * r[j]));
        c += 2.0 * c2 * t[i];
    }
    c = c - 16.0 * slo * slo;
    const double rad = b * b - 4.0 * a * c;
    if (!(rad >= 0.)) return 1.e11;
    const double x1 = (-b + sqrt(rad)) / (2.0 * a);
    const double x2 = (-b - sqrt(rad)) / (2.0 * a);
    int bad1 = 0, bad2 = 0;
    for (int i = 0; i < 7; i++) { bad1 |= x1 < t[i]; bad2 |= x2 < t[i]; }
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return (x1 < x2) ? x1 : x2;
}

/* fdsphne: new-edge stencil, point = slot 5 (src/sphfd.c:6016-6074). */
static double fdo_stne(const double t[8], const double s[8], double d01, double d12, double d14,
                       double d25, double d45)
{
    const double slo = .25 * (s[1] + s[2] + s[4] + s[5]);
    const double dt1 = (t[4] - t[1]) / d14 - t[2] / d25;
    const double dt2 = (t[2] - t[1]) / d12 - t[4] / d45;
    const double dt3 = (t[0] - t[3]) / d01;
    const double a = 1. / (d25 * d25) + 1. / (d45 * d45);
    const double b = 2 * (dt1 / d25 + dt2 / d45);
    const double c = dt1 * dt1 + dt2 * dt2 + dt3 * dt3 - 4 * slo * slo;
    const double rad = b * b - 4.0 * a * c;
    if (!(rad >= 0.)) return 1.e11;
    const double x1 = (-b + sqrt(rad)) / (2 * a);
    const double x2 = (-b - sqrt(rad)) / (2 * a);
    int bad1 = 0, bad2 = 0;
    for (int i = 0; i < 5; i++) { bad1 |= x1 < t[i]; bad2 |= x2 < t[i]; }
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return (x2 < x1) ? x2 : x1;
}

/* fdsph2d: cell-face stencil, point = slot 0; t[0], t[4] are stale state (src/sphfd.c:6077-6143). */
static double fdo_st2d(const double t[8], const double s[8], double d01, double d02, double d13,
                       double d23)
{
    const double slo = .25 * (s[0] + s[1] + s[2] + s[3]);
    const double d01sq = d01 * d01, d02sq = d02 * d02;
    const double t1mt3 = t[1] - t[3], t2mt3 = t[2] - t[3];
    const double t1t3t2 = t1mt3 / d13 - t[2] / d02;
    const double t2t3t1 = t2mt3 / d23 - t[1] / d01;
    const double a = (1.0 / d01sq + 1. / d02sq);
    const double b = 2.0 * (t1t3t2 / d02 + t2t3t1 / d01);
    const double c = t1t3t2 * t1t3t2 + t2t3t1 * t2t3t1 - 4 * slo * slo;
    const double rad = b * b - 4.0 * a * c;
    if (!(rad >= 0.)) return 1.e11;
    const double x1 = (-b + sqrt(rad)) / (2 * a);
    const double x2 = (-b - sqrt(rad)) / (2 * a);
    int bad1 = 0, bad2 = 0;
    for (int i = 0; i < 5; i++) { bad1 |= x1 < t[i]; bad2 |= x2 < t[i]; }
    if (bad1) return bad2 ? 1.e11 : x2;
    if (bad2) return x1;
    return (x2 < x1) ? x2 : x1;
}

/* fdsphnf: new-face stencil, point = slot 5 (src/sphfd.c:6146-6184). */
static double fdo_stnf(const double t[8], const double s[8], double d02, double d12, double d25)
{
    const double slo = .5 * (s[5] + s[2]);
    const double t4t0 = (t[4] - t[0]) / d02;
    const double t1t3 = (t[1] - t[3]) / d12;
    double x = slo * slo - 0.25 * (t4t0 * t4t0 + t1t3 * t1t3);
    if (!(x >= 0.)) return 1.e11;
    x = t[2] + d25 * sqrt(x);
    if (x < t[0] || x < t[1] || x < t[3] || x < t[4]) return 1.e11;
    return x;
}

/* ------------------------------------------------------------------------------------------ */
/* Per-cell 3-D coefficient tables (FAST mode only).  A fdsph3d coefficient depends on the two  */
/* nodes' radii, colatitudes and whether they share a longitude column, so for the cell whose   */
/* smallest indices are (yc, zc) every coefficient the reference computes is one of: 4 diagonal */
/* values diag[ri][qi], 32 point-row values prow[r7][q7][ri][qi][same-x] and 32 pair values     */
/* pair[ri][qi][rj][qj][same-x], each computed with the reference's formula.                    */

typedef struct { double diag[2][2]; double prow[2][2][2][2][2]; double pair[2][2][2][2][2]; } fdo_cell;

static void fdo_cell_fill(const fdo_grid *g, int yc, int zc, fdo_cell *c)
{
    const double hsq = g->h * g->h, dqsq = g->dq * g->dq, dfsq = g->df * g->df, df = g->df;
    double rr[2] = {fdo_rc(g, zc), fdo_rc(g, zc + 1)};
    double sq[2] = {sin(fdo_qc(g, yc)), sin(fdo_qc(g, yc + 1))};
    for (int ri = 0; ri < 2; ri++)
        for (int qi = 0; qi < 2; qi++) {
            const double dfsi = df * sq[qi];
            c->diag[ri][qi] = 1. / hsq + (1. / dqsq + 1. / (dfsi * dfsi)) / (rr[ri] * rr[ri]);
        }
    for (int r7 = 0; r7 < 2; r7++)
        for (int q7 = 0; q7 < 2; q7++)
            for (int ri = 0; ri < 2; ri++)
                for (int qi = 0; qi < 2; qi++)
                    for (int sx = 0; sx < 2; sx++) {
                        const double gg = (r7 == ri) ? 1.0 : -1.0, nn = (q7 == qi) ? 1.0 : -1.0,
                                     mm = sx ? 1.0 : -1.0;
                        const double df2s7 = df * (df * sq[q7]);
                        c->prow[r7][q7][ri][qi][sx] =
                            gg / hsq + (nn / dqsq + mm / (df2s7 * sq[qi])) / (rr[r7] * rr[ri]);
                    }
    for (int ri = 0; ri < 2; ri++)
        for (int qi = 0; qi < 2; qi++)
            for (int rj = 0; rj < 2; rj++)
                for (int qj = 0; qj < 2; qj++)
                    for (int sx = 0; sx < 2; sx++) {
                        const double gg = (ri == rj) ? 1.0 : -1.0, nn = (qi == qj) ? 1.0 : -1.0,
                                     mm = sx ? 1.0 : -1.0;
                        const double df2si = dfsq * sq[qi];
                        c->pair[ri][qi][rj][qj][sx] =
                            gg / hsq + (nn / dqsq + mm / (df2si * sq[qj])) / (rr[ri] * rr[rj]);
                    }
}

/* ------------------------------------------------------------------------------------------ */
/* Face walk.                                                                                   */

typedef struct {
    const fdo_grid *g;
    const float *slow;
    float *time;
    int face;
    int layer;          /* grid index of the face layer along the normal */
    int ulo, uhi, vlo, vhi;  /* face rectangle (inclusive) */
    int nu, nv;         /* grid extents along u and v */
    long su, sv, sn;    /* index strides along u, v and the normal */
    int mode;
    fdo_cell *cells;    /* FAST mode: (ny-1)*(nz-1) cells indexed [zc*(ny-1)+yc] */
    fdo_stats *st;
} fdo_face;

static inline void fdo_node_xyz(const fdo_face *F, int u, int v, fdn_node nd, int xyz[3])
{
    const fdn_frame fr = fd_face_frame[F->face];
    xyz[fr.axis_u] = u + nd.du;
    xyz[fr.axis_v] = v + nd.dv;
    xyz[fr.axis_n] = F->layer + nd.w * fr.inner;
}

static inline long fdo_node_index(const fdo_face *F, int u, int v, fdn_node nd)
{
    const fdn_frame fr = fd_face_frame[F->face];
    return (long)(u + nd.du) * F->su + (long)(v + nd.dv) * F->sv
           + (long)(F->layer + nd.w * fr.inner) * F->sn;
}

static double fdo_chain(const fdo_face *F, int u, int v, const fdn_chain *c, float s_point)
{
    double acc = 0.0;
    for (int k = 0; k < c->n; k++) {
        const fdn_factor fa = c->f[k];
        double x;
        int xyz[3];
        switch (fa.kind) {
        case FDN_H: x = F->g->h; break;
        case FDN_DQ: x = F->g->dq; break;
        case FDN_DF: x = F->g->df; break;
        case FDN_R: fdo_node_xyz(F, u, v, fa.at, xyz); x = fdo_rc(F->g, xyz[2]); break;
        case FDN_S: fdo_node_xyz(F, u, v, fa.at, xyz); x = sin(fdo_qc(F->g, xyz[1])); break;
        default: x = (double)s_point; break;
        }
        acc = (k == 0) ? x : acc * x;
    }
    return acc;
}

/* The body run for one face point (e.g. TOP: src/sphfd.c:1034-1761), table-driven.  Returns the
 * number of writer calls (3-D / new-edge / new-face) the point made.  carry is the stale (t0,t4). */
static int fdo_point(fdo_face *F, int u, int v, fdo_carry *carry, int *headw)
{
    const fdo_grid *g = F->g;
    float *T = F->time;
    const float *S = F->slow;
    const long ip = fdo_node_index(F, u, v, (fdn_node){0, 0, 0});
    const float s_point = S[ip];
    double guess = T[ip];
    double fhead = 0.;
    int writers = 0, writers_before_2d = 0, saw_2d = 0;
    double t[8] = {0}, s[8] = {0};
    t[0] = carry->t0;
    t[4] = carry->t4;
    const int fast = (F->mode == FDO_MODE_FAST);

    int gate = 0;
    for (int k = 0; k < FDN_NTRIAL; k++) {
        const fdn_trial *tr = &fd_face_trials[F->face][k];
        /* the first-contact test guards a whole block of trials and is made once on entry
         * (e.g. src/sphfd.c:1375 for the four new-edge trials, :1698 for the new-face trial) */
        if (tr->big_guess) {
            if (k == 0 || fd_face_trials[F->face][k - 1].kind != tr->kind) gate = (guess > 1.0e9);
            if (!gate) continue;
        }
        if ((tr->need & FDN_NEED_UM) && !(u > 0)) continue;
        if ((tr->need & FDN_NEED_UP) && !(u < F->nu - 1)) continue;
        if ((tr->need & FDN_NEED_VM) && !(v > 0)) continue;
        if ((tr->need & FDN_NEED_VP) && !(v < F->nv - 1)) continue;
        if ((tr->inside & FDN_IN_ULO) && !(u > F->ulo)) continue;
        if ((tr->inside & FDN_IN_UHI) && !(u < F->uhi)) continue;
        if ((tr->inside & FDN_IN_VLO) && !(v > F->vlo)) continue;
        if ((tr->inside & FDN_IN_VHI) && !(v < F->vhi)) continue;
        int ok = 1;
        for (int c = 0; c < tr->nchk && ok; c++) {
            const float tv = T[fdo_node_index(F, u, v, tr->chk[c])];
            ok = ((tr->chk_nonzero >> c) & 1) ? (tv != 0.0f) : (tv < 1.e9);
        }
        if (!ok) continue;

        double try_ = 1.e11;
        int evaluated = 1;
        switch (tr->kind) {
        case FDN_3D: {
            double r[8], q[8];
            int gs[8], ns[8], ms[8], xyz[8][3];
            for (int i = 0; i < 7; i++) {
                const long ix = fdo_node_index(F, u, v, tr->t[i]);
                t[i] = T[ix];
                s[i] = S[ix];
                fdo_node_xyz(F, u, v, tr->t[i], xyz[i]);
            }
            s[7] = s_point;
            fdo_node_xyz(F, u, v, (fdn_node){0, 0, 0}, xyz[7]);
            int xmax = xyz[0][0], ymax = xyz[0][1], zmin = xyz[0][2];
            for (int i = 1; i < 8; i++) {
                if (xyz[i][0] > xmax) xmax = xyz[i][0];
                if (xyz[i][1] > ymax) ymax = xyz[i][1];
                if (xyz[i][2] < zmin) zmin = xyz[i][2];
            }
            for (int i = 0; i < 8; i++) {
                r[i] = fdo_rc(g, xyz[i][2]);
                q[i] = fdo_qc(g, xyz[i][1]);
                gs[i] = (xyz[i][2] == zmin) ? 1 : -1;
                ns[i] = (xyz[i][1] == ymax) ? 1 : -1;
                ms[i] = (xyz[i][0] == xmax) ? 1 : -1;
            }
            writers++;
            double tmax = t[0];
            for (int i = 1; i < 7; i++) tmax = t[i] > tmax ? t[i] : tmax;
            if (fast && tmax >= guess && guess <= 1.e11) { evaluated = 0; break; }
            if (!fast) {
                try_ = fdo_st3d(t, s, r, q, gs, ns, ms, g->h, g->dq, g->df);
            } else {
                /* same value from the per-cell tables */
                const int yc = ymax - 1, zc = zmin;
                const fdo_cell *C = &F->cells[(long)zc * (g->ny - 1) + yc];
                int ri[8], qi[8];
                for (int i = 0; i < 8; i++) { ri[i] = xyz[i][2] - zc; qi[i] = xyz[i][1] - yc; }
                double slo = 0.0;
                for (int i = 0; i < 8; i++) slo += s[i];
                slo = 0.125 * slo;
                const double a = C->diag[ri[7]][qi[7]];
                double b = 0.0;
                for (int i = 0; i < 7; i++)
                    b += t[i] * C->prow[ri[7]][qi[7]][ri[i]][qi[i]][xyz[i][0] == xyz[7][0]];
                b = 2.0 * b;
                double cc = 0.0;
                for (int i = 0; i < 7; i++) cc += t[i] * t[i] * C->diag[ri[i]][qi[i]];
                for (int i = 0; i < 6; i++) {
                    double c2 = 0.0;
                    for (int j = i + 1; j < 7; j++)
                        c2 += t[j] * C->pair[ri[i]][qi[i]][ri[j]][qi[j]][xyz[i][0] == xyz[j][0]];
                    cc += 2.0 * c2 * t[i];
                }
                cc = cc - 16.0 * slo * slo;
                const double rad = b * b - 4.0 * a * cc;
                if (!(rad >= 0.)) { try_ = 1.e11; break; }
                const double x1 = (-b + sqrt(rad)) / (2.0 * a);
                const double x2 = (-b - sqrt(rad)) / (2.0 * a);
                const int bad1 = x1 < tmax, bad2 = x2 < tmax;
                try_ = bad1 ? (bad2 ? 1.e11 : x2) : (bad2 ? x1 : ((x1 < x2) ? x1 : x2));
            }
            break;
        }
        case FDN_NE: {
            for (int i = 0; i < 5; i++) {
                const long ix = fdo_node_index(F, u, v, tr->t[i]);
                t[i] = T[ix];
                s[i] = S[ix];
            }
            s[5] = s_point;
            writers++;
            double tmax = t[0];
            for (int i = 1; i < 5; i++) tmax = t[i] > tmax ? t[i] : tmax;
            if (fast && tmax >= guess && guess <= 1.e11) { evaluated = 0; break; }
            const double d01 = fdo_chain(F, u, v, &tr->d[0], s_point);
            const double d12 = fdo_chain(F, u, v, &tr->d[1], s_point);
            const double d14 = fdo_chain(F, u, v, &tr->d[2], s_point);
            const double d25 = fdo_chain(F, u, v, &tr->d[3], s_point);
            const double d45 = fdo_chain(F, u, v, &tr->d[4], s_point);
            try_ = fdo_stne(t, s, d01, d12, d14, d25, d45);
            break;
        }
        case FDN_2D: {
            if (!saw_2d) {
                saw_2d = 1;
                writers_before_2d = writers;
                if (writers == 0 && F->st) F->st->inherit_points++;
            }
            s[0] = s_point;
            for (int i = 1; i < 4; i++) {
                const long ix = fdo_node_index(F, u, v, tr->t[i]);
                t[i] = T[ix];
                s[i] = S[ix];
            }
            double tmax = t[0];
            for (int i = 1; i < 5; i++) tmax = t[i] > tmax ? t[i] : tmax;
            const double d01 = fdo_chain(F, u, v, &tr->d[0], s_point);
            if (fast && tmax >= guess && guess <= 1.e11) { evaluated = 0; break; }
            const double d02 = fdo_chain(F, u, v, &tr->d[1], s_point);
            const double d13 = fdo_chain(F, u, v, &tr->d[2], s_point);
            const double d23 = fdo_chain(F, u, v, &tr->d[3], s_point);
            try_ = fdo_st2d(t, s, d01, d02, d13, d23);
            if (tr->head && try_ < guess) {
                fhead = (guess - try_) / (d01 * (double)s_point);
                guess = try_;
            }
            break;
        }
        case FDN_NF: {
            for (int i = 0; i < 5; i++) {
                const long ix = fdo_node_index(F, u, v, tr->t[i]);
                t[i] = T[ix];
                s[i] = S[ix];
            }
            s[5] = s_point;
            writers++;
            double tmax = t[0];
            for (int i = 1; i < 5; i++) tmax = t[i] > tmax ? t[i] : tmax;
            if (fast && tmax >= guess && guess <= 1.e11) { evaluated = 0; break; }
            const double d02 = fdo_chain(F, u, v, &tr->d[0], s_point);
            const double d12 = fdo_chain(F, u, v, &tr->d[1], s_point);
            const double d25 = fdo_chain(F, u, v, &tr->d[2], s_point);
            try_ = fdo_stnf(t, s, d02, d12, d25);
            break;
        }
        default: { /* FDN_1D */
            const long ix = fdo_node_index(F, u, v, tr->t[0]);
            const float ssum = s_point + S[ix];
            double x = .5 * (double)ssum;
            const fdn_chain *c = &tr->d[0];
            for (int k2 = 0; k2 < c->n; k2++) {
                const fdn_chain one = {1, {c->f[k2]}};
                x = x * fdo_chain(F, u, v, &one, s_point);
            }
            try_ = (double)T[ix] + x;
            if (tr->head && try_ < guess) {
                fhead = (guess - try_) / fdo_chain(F, u, v, &tr->hd, s_point);
                guess = try_;
            }
            break;
        }
        }
        if (F->st) {
            if (evaluated) F->st->calls[tr->kind]++;
            else F->st->skipped[tr->kind]++;
        }
        if (!tr->head && evaluated && try_ < guess) guess = try_;
#ifdef FDO_TRACE
        if (evaluated) fprintf(stderr, "T %d %.17g\n", k, try_);
#endif
    }
#ifdef FDO_TRACE
    fprintf(stderr, "P %ld %.17g %.17g\n", ip, guess, fhead);
#endif
    (void)writers_before_2d;
    if (guess < T[ip]) {
        T[ip] = (float)guess;
        if (fhead > FDO_HEADTEST) headw[fd_face_frame[F->face].headw]++;
        if (F->st && F->st->sweeps < 64) F->st->changed_per_sweep[F->st->sweeps]++;
    }
    carry->t0 = t[0];
    carry->t4 = t[4];
    return writers;
}

typedef struct { float key; int idx; } fdo_sortent;

static int fdo_sort_cmp(const void *a, const void *b)
{
    const fdo_sortent *x = (const fdo_sortent *)a, *y = (const fdo_sortent *)b;
    if (x->key > y->key) return 1;
    if (y->key > x->key) return -1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

/* Gather (time of inner neighbour, fill order) — e.g. TOP src/sphfd.c:1024-1033 — then run the
 * points in ascending time, ties in fill order (glibc's qsort is a stable merge sort). */
static void fdo_run_face(fdo_face *F, fdo_sortent *buf, fdo_carry *carry, int *headw)
{
    const int nu = F->uhi - F->ulo + 1, nvv = F->vhi - F->vlo + 1;
    if (nu <= 0 || nvv <= 0) return;
    int n = 0;
    for (int v = F->vlo; v <= F->vhi; v++)
        for (int u = F->ulo; u <= F->uhi; u++) {
            buf[n].key = F->time[fdo_node_index(F, u, v, (fdn_node){0, 0, 1})];
            buf[n].idx = n;
            n++;
        }
    qsort(buf, n, sizeof(fdo_sortent), fdo_sort_cmp);
    for (int i = 0; i < n; i++) {
        const int u = F->ulo + buf[i].idx % nu, v = F->vlo + buf[i].idx / nu;
        fdo_point(F, u, v, carry, headw);
    }
    if (F->st) {
        F->st->node_updates += n;
        F->st->faces++;
        if (F->st->sweeps < 64) {
            /* dependency depth: level = 1 + max level of earlier in-face neighbours, in sort order */
            int *lev = (int *)calloc((size_t)n, sizeof(int)), *pos = (int *)malloc(sizeof(int) * (size_t)n);
            for (int i = 0; i < n; i++) pos[buf[i].idx] = i;
            int depth = 0;
            for (int i = 0; i < n; i++) {
                const int id = buf[i].idx, iu = id % nu, iv = id / nu;
                int l = 1;
                for (int dv = -1; dv <= 1; dv++)
                    for (int du = -1; du <= 1; du++) {
                        const int ju = iu + du, jv = iv + dv;
                        if ((du || dv) && ju >= 0 && ju < nu && jv >= 0 && jv < nvv && pos[jv * nu + ju] < i)
                            if (lev[jv * nu + ju] + 1 > l) l = lev[jv * nu + ju] + 1;
                    }
                lev[id] = l;
                if (l > depth) depth = l;
            }
            F->st->depth_per_sweep[F->st->sweeps] += depth;
            F->st->updates_per_sweep[F->st->sweeps] += n;
            free(lev);
            free(pos);
        }
    }
}

int fdo_headpref(const fdo_grid *g, const fdo_box *b, int headpref)
{
    /* src/sphfd.c:977-1003 */
    if (headpref <= 0) return headpref;
    long head = (long)g->nx * g->ny * g->nz;
    if (g->nx > 5 && b->x2 <= head) { headpref = 2; head = b->x2; }
    if (g->nx > 5 && (g->nx - 1 - b->x1) <= head) { headpref = 1; head = g->nx - 1 - b->x1; }
    if (g->ny > 5 && b->y2 <= head) { headpref = 4; head = b->y2; }
    if (g->ny > 5 && (g->ny - 1 - b->y1) <= head) { headpref = 3; head = g->ny - 1 - b->y1; }
    if (g->nz > 5 && b->z2 <= head) { headpref = 6; head = b->z2; }
    if (g->nz > 5 && (g->nz - 1 - b->z1) <= head) { headpref = 5; head = g->nz - 1 - b->z1; }
    return headpref;
}

/* Box walls for a restart from one whole model wall (src/sphfd.c:5623-5674; same layout as the
 * srctype 2/3 set-up at :877-926). */
static void fdo_wall_box(const fdo_grid *g, int srcwall, fdo_box *b)
{
    b->dx1 = b->dx2 = b->dy1 = b->dy2 = b->dz1 = b->dz2 = 1;
    b->radius = 1;
    if (srcwall == 1) b->x2 = 1; else { b->x2 = g->nx; b->dx2 = 0; }
    if (srcwall == 2) b->x1 = g->nx - 2; else { b->x1 = -1; b->dx1 = 0; }
    if (srcwall == 3) b->y2 = 1; else { b->y2 = g->ny; b->dy2 = 0; }
    if (srcwall == 4) b->y1 = g->ny - 2; else { b->y1 = -1; b->dy1 = 0; }
    if (srcwall == 5) b->z2 = 1; else { b->z2 = g->nz; b->dz2 = 0; }
    if (srcwall == 6) b->z1 = g->nz - 2; else { b->z1 = -1; b->dz1 = 0; }
}

/* The sweep loop: BIGGER LOOP / BIG LOOP of src/sphfd.c:1008-5678. */
int fdo_propagate(const fdo_grid *g, const float *slow, float *time, fdo_box b, fdo_sweep sw,
                  fdo_carry *carry, int mode, fdo_stats *st)
{
    const long nxy = (long)g->nx * g->ny;
    long maxface = (long)g->nx * g->ny;
    if ((long)g->nx * g->nz > maxface) maxface = (long)g->nx * g->nz;
    if ((long)g->ny * g->nz > maxface) maxface = (long)g->ny * g->nz;
    fdo_sortent *buf = (fdo_sortent *)malloc(sizeof(fdo_sortent) * (size_t)maxface);
    fdo_cell *cells = NULL;
    if (mode == FDO_MODE_FAST) {
        cells = (fdo_cell *)malloc(sizeof(fdo_cell) * (size_t)(g->ny - 1) * (size_t)(g->nz - 1));
        for (int zc = 0; zc < g->nz - 1; zc++)
            for (int yc = 0; yc < g->ny - 1; yc++) fdo_cell_fill(g, yc, zc, &cells[(long)zc * (g->ny - 1) + yc]);
    }
    fdo_carry local = {0.0, 0.0};
    if (!carry) carry = &local;
    int reverse = sw.reverse, rad0 = 1;
    fdo_face F;
    memset(&F, 0, sizeof F);
    F.g = g; F.slow = slow; F.time = time; F.mode = mode; F.cells = cells; F.st = st;
    while (reverse > -1) {
        int headw[7] = {0, 0, 0, 0, 0, 0, 0};
        while (rad0 && (b.dx1 || b.dx2 || b.dy1 || b.dy2 || b.dz1 || b.dz2)) {
            /* TOP, BOTTOM, EAST, WEST, NORTH, SOUTH (src/sphfd.c:1021, 1770, 2506, 3275, 4035, 4800) */
            for (int face = 0; face < 6; face++) {
                int *flag, *wall, grow, limit_hit;
                switch (face) {
                case 0: flag = &b.dz1; wall = &b.z1; grow = sw.kminus; break;
                case 1: flag = &b.dz2; wall = &b.z2; grow = sw.kplus; break;
                case 2: flag = &b.dx2; wall = &b.x2; grow = sw.iplus; break;
                case 3: flag = &b.dx1; wall = &b.x1; grow = sw.iminus; break;
                case 4: flag = &b.dy1; wall = &b.y1; grow = sw.jminus; break;
                default: flag = &b.dy2; wall = &b.y2; grow = sw.jplus; break;
                }
                for (int igrow = 1; igrow <= grow; igrow++) {
                    if (!*flag) continue;
                    F.face = face;
                    F.layer = *wall;
                    switch (face) {
                    case 0: case 1:
                        F.ulo = b.x1 + 1; F.uhi = b.x2 - 1; F.vlo = b.y1 + 1; F.vhi = b.y2 - 1;
                        F.nu = g->nx; F.nv = g->ny; F.su = 1; F.sv = g->nx; F.sn = nxy; break;
                    case 2: case 3:
                        F.ulo = b.y1 + 1; F.uhi = b.y2 - 1; F.vlo = b.z1 + 1; F.vhi = b.z2 - 1;
                        F.nu = g->ny; F.nv = g->nz; F.su = g->nx; F.sv = nxy; F.sn = 1; break;
                    default:
                        F.ulo = b.x1 + 1; F.uhi = b.x2 - 1; F.vlo = b.z1 + 1; F.vhi = b.z2 - 1;
                        F.nu = g->nx; F.nv = g->nz; F.su = 1; F.sv = nxy; F.sn = g->nx; break;
                    }
                    fdo_run_face(&F, buf, carry, headw);
                    /* move the wall outward (e.g. src/sphfd.c:1762-1764) */
                    const int inner = fd_face_frame[face].inner;   /* +1: wall moves toward 0 */
                    const int nmax = (face < 2) ? g->nz : (face < 4) ? g->nx : g->ny;
                    limit_hit = (inner > 0) ? (*wall == 0) : (*wall == nmax - 1);
                    if (limit_hit) *flag = 0;
                    *wall -= inner;
                }
            }
            b.radius++;
            if (b.radius == sw.maxrad) rad0 = 0;
        }
        if (st) st->sweeps++;
        /* restart test (src/sphfd.c:5570-5676) */
        if (!headw[1] && !headw[2] && !headw[3] && !headw[4] && !headw[5] && !headw[6]) {
            reverse = 0;
        } else {
            int head = 0, srcwall = 0;
            for (int w = 1; w <= 6; w++)
                if (headw[w] > 0 && headw[w] > head) { head = headw[w]; srcwall = w; }
            if (sw.headpref > 0 && headw[sw.headpref] > 0) srcwall = sw.headpref;
            fdo_wall_box(g, srcwall, &b);
            rad0 = 1;
            if (st && reverse > 0) st->restarts[srcwall]++;
        }
        reverse--;
    }
    free(buf);
    free(cells);
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Point source box (src/sphfd.c:724-825).                                                      */

void fdo_point_source(const fdo_grid *g, const float *slow, float *time, int xs, int ys, int zs,
                      const double src_geo[3], int ncube, fdo_box *box)
{
    const long nx = g->nx, nxy = (long)g->nx * g->ny;
    const double fxss = src_geo[0], fyss = src_geo[1], fzss = src_geo[2];
    const double x1p = fzss * cos(fyss);
    const double y1p = fzss * sin(fyss) * cos(fxss);
    const double z1p = fzss * sin(fyss) * sin(fxss);
    const float s000 = slow[nxy * zs + nx * ys + xs];
    for (int zz = zs - ncube; zz <= zs + ncube; zz++) {
        if (zz < 0 || zz >= g->nz) continue;
        for (int yy = ys - ncube; yy <= ys + ncube; yy++) {
            if (yy < 0 || yy >= g->ny) continue;
            for (int xx = xs - ncube; xx <= xs + ncube; xx++) {
                if (xx < 0 || xx >= g->nx) continue;
                const double fx1 = g->x0 + g->df * (double)xx;
                const double qy1 = fdo_qc(g, yy);
                const double rz1 = fdo_rc(g, zz);
                const double x2p = rz1 * cos(qy1);
                const double y2p = rz1 * sin(qy1) * cos(fx1);
                const double z2p = rz1 * sin(qy1) * sin(fx1);
                const double dist = sqrt((x1p - x2p) * (x1p - x2p) + (y1p - y2p) * (y1p - y2p)
                                         + (z1p - z2p) * (z1p - z2p));
                time[nxy * zz + nx * yy + xx] = (float)(s000 * dist);
            }
        }
    }
    box->radius = ncube;
    box->dx1 = box->dx2 = box->dy1 = box->dy2 = box->dz1 = box->dz2 = 1;
    if (xs > ncube) box->x1 = xs - (ncube + 1); else { box->x1 = -1; box->dx1 = 0; }
    if (xs < g->nx - (ncube + 1)) box->x2 = xs + (ncube + 1); else { box->x2 = g->nx; box->dx2 = 0; }
    if (ys > ncube) box->y1 = ys - (ncube + 1); else { box->y1 = -1; box->dy1 = 0; }
    if (ys < g->ny - (ncube + 1)) box->y2 = ys + (ncube + 1); else { box->y2 = g->ny; box->dy2 = 0; }
    if (zs > ncube) box->z1 = zs - (ncube + 1); else { box->z1 = -1; box->dz1 = 0; }
    if (zs < g->nz - (ncube + 1)) box->z2 = zs + (ncube + 1); else { box->z2 = g->nz; box->dz2 = 0; }
}

/* ------------------------------------------------------------------------------------------ */
/* Parameter list with getpar semantics (src/sphfd.c:6267-6766): name=value tokens, '#' comment */
/* at token start, quotes, par=<file> recursion; the LAST definition of a name wins.            */

typedef struct { char name[64]; char value[256]; } fdo_kv;
typedef struct { fdo_kv *e; int n, cap; } fdo_plist;

static void fdo_plist_add(fdo_plist *p, const char *name, const char *value)
{
    if (p->n == p->cap) {
        p->cap = p->cap ? 2 * p->cap : 64;
        p->e = (fdo_kv *)realloc(p->e, sizeof(fdo_kv) * (size_t)p->cap);
    }
    snprintf(p->e[p->n].name, sizeof p->e[p->n].name, "%s", name);
    snprintf(p->e[p->n].value, sizeof p->e[p->n].value, "%s", value);
    p->n++;
}

static int fdo_plist_file(fdo_plist *p, const char *fname, int level);

static int fdo_plist_entry(fdo_plist *p, const char *tok, int level)
{
    char name[64] = {0};
    const char *eq = strchr(tok, '=');
    if (!eq) return 0;
    size_t ln = (size_t)(eq - tok);
    if (ln >= sizeof name) ln = sizeof name - 1;
    memcpy(name, tok, ln);
    fdo_plist_add(p, name, eq + 1);
    if (strcmp(name, "par") == 0) return fdo_plist_file(p, eq + 1, level + 1);
    return 0;
}

static int fdo_plist_file(fdo_plist *p, const char *fname, int level)
{
    if (level > 20) return -2;
    FILE *fp = fopen(fname, "r");
    if (!fp) return -3;
    char line[1024];
    while (fgets(line, sizeof line, fp)) {
        char *pl = line;
        for (;;) {
            while (*pl == ' ' || *pl == '\t') pl++;
            if (*pl == '\0' || *pl == '\n' || *pl == '#') break;
            char name[64], value[256];
            int nn = 0, nv = 0;
            while (*pl != '=' && *pl != '\0' && *pl != ' ' && *pl != '\t' && *pl != '\n') {
                if (nn < 63) name[nn++] = *pl;
                pl++;
            }
            name[nn] = 0;
            if (*pl == '=') pl++;
            char t1 = ' ', t2 = '\t';
            if (*pl == '"' || *pl == '\'') { t1 = t2 = *pl++; }
            while (*pl != t1 && *pl != t2 && *pl != '\0' && *pl != '\n') {
                if (nv < 255) value[nv++] = *pl;
                pl++;
            }
            value[nv] = 0;
            if (*pl == '"' || *pl == '\'') pl++;
            fdo_plist_add(p, name, value);
            if (strcmp(name, "par") == 0) {
                int rc = fdo_plist_file(p, value, level + 1);
                if (rc) { fclose(fp); return rc; }
            }
        }
    }
    fclose(fp);
    return 0;
}

static const char *fdo_plist_get(const fdo_plist *p, const char *name)
{
    for (int i = p->n - 1; i >= 0; i--)
        if (strcmp(p->e[i].name, name) == 0) return p->e[i].value;
    return NULL;
}

static int fdo_get_i(const fdo_plist *p, const char *n, int *v)
{ const char *s = fdo_plist_get(p, n); if (!s) return 0; *v = atoi(s); return 1; }
static int fdo_get_d(const fdo_plist *p, const char *n, double *v)
{ const char *s = fdo_plist_get(p, n); if (!s) return 0; *v = atof(s); return 1; }
static int fdo_get_f(const fdo_plist *p, const char *n, float *v)
{ const char *s = fdo_plist_get(p, n); if (!s) return 0; *v = (float)atof(s); return 1; }
static int fdo_get_s(const fdo_plist *p, const char *n, char *v, size_t cap)
{ const char *s = fdo_plist_get(p, n); if (!s) return 0; snprintf(v, cap, "%s", s); return 1; }

/* ------------------------------------------------------------------------------------------ */
/* 232-byte header (include/common/vhead.h:4-11).                                               */

typedef struct {
    char header[120];
    double fxs, fys, fzs, clat, clon, cz, x0, y0, z0, dx, dy, dz;
    float az;
    int nx, ny, nz;
} fdo_vhead;
typedef char fdo_vhead_is_232_bytes[(sizeof(fdo_vhead) == 232) ? 1 : -1];

static void fdo_swap4(void *p) { unsigned char *b = (unsigned char *)p, t; t = b[0]; b[0] = b[3]; b[3] = t; t = b[1]; b[1] = b[2]; b[2] = t; }
static void fdo_swap8(void *p) { unsigned char *b = (unsigned char *)p, t; for (int i = 0; i < 4; i++) { t = b[i]; b[i] = b[7 - i]; b[7 - i] = t; } }
static void fdo_swap_head(fdo_vhead *h, int with_src)
{
    fdo_swap4(&h->az); fdo_swap4(&h->nx); fdo_swap4(&h->ny); fdo_swap4(&h->nz);
    fdo_swap8(&h->clat); fdo_swap8(&h->clon); fdo_swap8(&h->cz);
    fdo_swap8(&h->x0); fdo_swap8(&h->y0); fdo_swap8(&h->z0);
    fdo_swap8(&h->dx); fdo_swap8(&h->dy); fdo_swap8(&h->dz);
    if (with_src) { fdo_swap8(&h->fxs); fdo_swap8(&h->fys); fdo_swap8(&h->fzs); }
}

/* ------------------------------------------------------------------------------------------ */
/* Whole-station driver: src/sphfd.c:260-5803 with errors returned instead of aborting.         */

int fdo_sphfd(int ac, char **av, const char *timedir, int mode, fdo_stats *stats)
{
    fdo_plist P = {0};
    int rc = 0;
    for (int i = 1; i < ac && !rc; i++) rc = fdo_plist_entry(&P, av[i], 0);
    if (rc) { free(P.e); return rc; }

    int nx, ny, nz, iplus = 1, iminus = 1, jplus = 1, jminus = 1, kplus = 1, kminus = 1;
    int srctype = 1, floatsrc = 1, ncube = 2, reverse = 1, headpref = 6, parse = 1, fill = 0;
    int invh = 0, invq = 0, invf = 0, invx0 = 0, invy0 = 0, invz0 = 0, swab = 0, srcwall = 0;
    int xs = 0, ys = 0, zs = 0;
    double h, dq = 0, df = 0, y0 = 90, x0 = 0, z0 = 0, fxs = 0, fys = 0, fzs = 0;
    float maxoff = -1.f;
    char ttmp[160], velfile[256], oldtfile[256], wallfile[256], boxfile[256];
    if (!fdo_get_i(&P, "nx", &nx) || !fdo_get_i(&P, "ny", &ny) || !fdo_get_i(&P, "nz", &nz)
        || !fdo_get_d(&P, "h", &h)) { free(P.e); return -10; }
    fdo_get_d(&P, "dq", &dq); fdo_get_d(&P, "df", &df);
    fdo_get_i(&P, "iminus", &iminus); fdo_get_i(&P, "iplus", &iplus);
    fdo_get_i(&P, "jminus", &jminus); fdo_get_i(&P, "jplus", &jplus);
    fdo_get_i(&P, "kminus", &kminus); fdo_get_i(&P, "kplus", &kplus);
    fdo_get_i(&P, "floatsrc", &floatsrc); fdo_get_i(&P, "srctype", &srctype);
    fdo_get_i(&P, "NCUBE", &ncube); fdo_get_i(&P, "reverse", &reverse);
    fdo_get_i(&P, "headpref", &headpref); fdo_get_f(&P, "maxoff", &maxoff);
    fdo_get_d(&P, "x0", &x0); fdo_get_d(&P, "y0", &y0); fdo_get_d(&P, "z0", &z0);
    fdo_get_i(&P, "parse", &parse); fdo_get_i(&P, "fill", &fill);
    fdo_get_i(&P, "invh", &invh); fdo_get_i(&P, "invf", &invf); fdo_get_i(&P, "invq", &invq);
    fdo_get_i(&P, "invx0", &invx0); fdo_get_i(&P, "invy0", &invy0); fdo_get_i(&P, "invz0", &invz0);
    fdo_get_i(&P, "swab", &swab);
    if (invh == 1) h = 1. / h;
    if (invq == 1 && dq != 0) dq = 1. / dq;
    if (invf == 1 && df != 0) df = 1. / df;
    if (invx0 == 1 && x0 != 0) x0 = 1. / x0;
    if (invy0 == 1 && y0 != 0) y0 = 1. / y0;
    if (invz0 == 1 && z0 != 0) z0 = 1. / z0;
    const double x0_save = x0, y0_save = y0;

    fdo_grid g;
    g.nx = nx; g.ny = ny; g.nz = nz; g.h = h;
    y0 *= FDO_DEGRAD;
    y0 = FDO_HPI - fdo_glath(y0, z0, &g.z0r);
    x0 *= FDO_DEGRAD;
    dq *= FDO_DEGRAD;
    df *= FDO_DEGRAD;
    if (dq == 0) dq = h / FDO_REARTH;
    if (df == 0) df = fabs(h / (FDO_REARTH * sin(y0)));
    g.x0 = x0; g.y0 = y0; g.dq = dq; g.df = df;

    double fxss = 0, fyss = 0, fzss = 0;
    if (srctype == 1) {
        if (floatsrc == 0) {
            if (!fdo_get_i(&P, "xs", &xs) || !fdo_get_i(&P, "ys", &ys) || !fdo_get_i(&P, "zs", &zs)) { free(P.e); return -10; }
            fxss = x0 + df * (double)xs; fyss = fdo_qc(&g, ys); fzss = fdo_rc(&g, zs);
        } else {
            if (!fdo_get_d(&P, "fxs", &fxs) || !fdo_get_d(&P, "fys", &fys) || !fdo_get_d(&P, "fzs", &fzs)) { free(P.e); return -10; }
            double rcent;
            fxs *= FDO_DEGRAD;
            fys *= FDO_DEGRAD;
            fys = FDO_HPI - fdo_glath(fys, fzs, &rcent);
            fxss = fxs; fyss = fys; fzss = rcent;
            fxs = (fxs - x0) / df;
            fys = (fys - y0) / dq;
            fzs = (g.z0r - rcent) / h;
            xs = (int)(fxs + 0.5);
            ys = (int)(fys + 0.5);
            zs = (int)(fzs + 0.5);
        }
    } else if (srctype == 2) {
        if (!fdo_get_i(&P, "srcwall", &srcwall) || !fdo_get_s(&P, "wallfile", wallfile, sizeof wallfile)) { free(P.e); return -10; }
    } else if (srctype == 3) {
        if (!fdo_get_i(&P, "srcwall", &srcwall) || !fdo_get_s(&P, "oldtfile", oldtfile, sizeof oldtfile)) { free(P.e); return -10; }
    } else { free(P.e); return -11; }
    if (fill == 1 && !fdo_get_s(&P, "boxfile", boxfile, sizeof boxfile)) { free(P.e); return -10; }
    if (!fdo_get_s(&P, "timefile", ttmp, sizeof ttmp) || !fdo_get_s(&P, "velfile", velfile, sizeof velfile)) { free(P.e); return -10; }
    free(P.e);
    /* src/sphfd.c:533-538: the reference checks the (possibly uninitialised) node even for walls */
    if (srctype == 1 && (xs < 0 || ys < 0 || zs < 0 || xs > nx - 1 || ys > ny - 1 || zs > nz - 1)) return -12;
    const int maxrad = (maxoff > 0.) ? (int)(maxoff / h + 1) : 99999999;

    const long nxyz = (long)nx * ny * nz, nxy = (long)nx * ny;
    char timefile[600];
    snprintf(timefile, sizeof timefile, "%s/%s", timedir, ttmp);
    FILE *vf = fopen(velfile, "rb");
    if (!vf) return -13;
    float *slow = (float *)malloc(4 * (size_t)nxyz), *time = (float *)malloc(4 * (size_t)nxyz);
    fdo_vhead hin;
    memset(&hin, 0, sizeof hin);
    if (fread(&hin, 1, 232, vf) != 232 || strncmp(hin.header, "HEAD", 4) != 0) {
        /* src/sphfd.c:614-665: no header — synthesise one and read the file from its start */
        hin.x0 = x0_save; hin.y0 = y0_save; hin.z0 = z0; hin.dx = df; hin.dy = dq; hin.dz = h;
        hin.nx = nx; hin.ny = ny; hin.nz = nz; hin.az = 0.f;
        hin.clat = y0_save; hin.clon = x0_save; hin.cz = z0;
        memset(hin.header, ' ', 120);
        memcpy(hin.header, "HEADFINESPHRVPMDNOFLsphfd", 25);
        hin.header[25] = 0;
        rewind(vf);
    }
    size_t got = fread(slow, 4, (size_t)nxyz, vf);
    fclose(vf);
    if (got != (size_t)nxyz) { free(slow); free(time); return -14; }
    if (swab == 1 || swab == 3) {
        fdo_swap_head(&hin, 0);
        for (long i = 0; i < nxyz; i++) fdo_swap4(&slow[i]);
    }
    for (long i = 0; i < nxyz; i++) slow[i] = 1 / slow[i];
    for (long i = 0; i < nxyz; i++) time[i] = FDO_UNSET;

    fdo_box box;
    memset(&box, 0, sizeof box);
    if (srctype == 1) {
        const double geo[3] = {fxss, fyss, fzss};
        fdo_point_source(&g, slow, time, xs, ys, zs, geo, ncube, &box);
        if (fill == 1) {
            /* src/sphfd.c:697-722, 761-764: box times from boxfile in z,y,x order */
            FILE *bf = fopen(boxfile, "rb");
            if (!bf) { free(slow); free(time); return -13; }
            int bx1 = xs - ncube < 0 ? 0 : xs - ncube, bx2 = xs + ncube > nx - 1 ? nx - 1 : xs + ncube;
            int by1 = ys - ncube < 0 ? 0 : ys - ncube, by2 = ys + ncube > ny - 1 ? ny - 1 : ys + ncube;
            int bz1 = zs - ncube < 0 ? 0 : zs - ncube, bz2 = zs + ncube > nz - 1 ? nz - 1 : zs + ncube;
            long nbox = (long)(bx2 - bx1 + 1) * (by2 - by1 + 1) * (bz2 - bz1 + 1);
            float *box0 = (float *)malloc(4 * (size_t)nbox);
            fdo_vhead hb;
            if (fread(&hb, 1, 232, bf) != 232 || fread(box0, 4, (size_t)nbox, bf) != (size_t)nbox) { fclose(bf); free(box0); free(slow); free(time); return -14; }
            fclose(bf);
            long ii = 0;
            for (int zz = bz1; zz <= bz2; zz++)
                for (int yy = by1; yy <= by2; yy++)
                    for (int xx = bx1; xx <= bx2; xx++) time[nxy * zz + (long)nx * yy + xx] = box0[ii++];
            free(box0);
        }
    } else if (srctype == 2) {
        /* src/sphfd.c:826-926: six walls, each applied if its first value > -1e-20 */
        long nwall = (nx <= ny && nx <= nz) ? (long)ny * nz : (ny <= nx && ny <= nz) ? (long)nx * nz : nxy;
        float *wall = (float *)malloc(4 * (size_t)nwall);
        FILE *wf = fopen(wallfile, "rb");
        if (!wf) { free(wall); free(slow); free(time); return -13; }
        for (int w = 0; w < 6; w++) {
            if (fread(wall, 4, (size_t)nwall, wf) != (size_t)nwall) break;
            if (!(wall[0] > -1.e-20)) continue;
            long ii = 0;
            if (w < 2) { int x = w == 0 ? 0 : nx - 1; for (int k = 0; k < nz; k++) for (int j = 0; j < ny; j++) time[nxy * k + (long)nx * j + x] = wall[ii++]; }
            else if (w < 4) { int y = w == 2 ? 0 : ny - 1; for (int k = 0; k < nz; k++) for (int i = 0; i < nx; i++) time[nxy * k + (long)nx * y + i] = wall[ii++]; }
            else { int z = w == 4 ? 0 : nz - 1; for (int j = 0; j < ny; j++) for (int i = 0; i < nx; i++) time[nxy * z + (long)nx * j + i] = wall[ii++]; }
        }
        fclose(wf);
        free(wall);
        fdo_wall_box(&g, srcwall, &box);
    } else {
        FILE *of = fopen(oldtfile, "rb");
        if (!of) { free(slow); free(time); return -13; }
        if (fread(time, 4, (size_t)nxyz, of) != (size_t)nxyz) { /* the reference reads what is there */ }
        fclose(of);
        fdo_wall_box(&g, srcwall, &box);
    }

    fdo_sweep sw;
    sw.reverse = reverse; sw.maxrad = maxrad;
    sw.kminus = kminus; sw.kplus = kplus; sw.iplus = iplus; sw.iminus = iminus; sw.jminus = jminus; sw.jplus = jplus;
    sw.headpref = fdo_headpref(&g, &box, headpref);
    fdo_carry carry = {0.0, 0.0};
    fdo_propagate(&g, slow, time, box, sw, &carry, mode, stats);

    /* output (src/sphfd.c:5702-5803) */
    int nxp = nx, nyp = ny, nzp = nz;
    long nout = nxyz;
    if (parse > 1) {
        long ii = 0;
        nzp = 0;
        for (int k = 0; k < nz; k += parse) {
            nzp++;
            for (int j = 0; j < ny; j += parse)
                for (int i = 0; i < nx; i += parse) time[ii++] = time[i + (long)j * nx + (long)k * nxy];
        }
        nxp = 0; nyp = 0;
        for (int j = 0; j < ny; j += parse) nyp++;
        for (int i = 0; i < nx; i += parse) nxp++;
        nout = ii;
    }
    fdo_vhead hout;
    memset(&hout, 0, sizeof hout);
    memcpy(hout.header, hin.header, 120);
    hout.clat = hin.clat; hout.clon = hin.clon; hout.cz = hin.cz; hout.az = hin.az;
    hout.x0 = hin.x0; hout.y0 = hin.y0; hout.z0 = hin.z0;
    hout.dx = hin.dx * parse; hout.dy = hin.dy * parse; hout.dz = hin.dz * parse;
    hout.nx = nxp; hout.ny = nyp; hout.nz = nzp;
    {
        /* strncpy(120) then "PTIM" at 12..15 via strcpy (each writes a NUL after it), then
         * strcpy(&out[i], &in[i]) for i = 16..119 (src/sphfd.c:5744-5767) */
        char tmp[121];
        size_t l = strnlen(hin.header, 120);
        memset(hout.header, 0, 120);
        memcpy(hout.header, hin.header, l);
        hout.header[12] = 'P'; hout.header[13] = 'T'; hout.header[14] = 'I'; hout.header[15] = 'M';
        if (l < 16) hout.header[16] = 0;
        for (int i = 16; i < 120; i++) {
            size_t li = strnlen(hin.header + i, 120 - i);
            memcpy(tmp, hin.header + i, li);
            tmp[li] = 0;
            memcpy(hout.header + i, tmp, (i + li < 120) ? li + 1 : li);
        }
    }
    hout.fxs = fxss; hout.fys = fyss; hout.fzs = fzss;
    if (swab == 2 || swab == 3) {
        fdo_swap_head(&hout, 1);
        for (long i = 0; i < nout; i++) fdo_swap4(&time[i]);
    }
    FILE *tf = fopen(timefile, "wb");
    if (!tf) { free(slow); free(time); return -15; }
    fwrite(&hout, 1, 232, tf);
    fwrite(time, 4, (size_t)nout, tf);
    fclose(tf);
    free(slow);
    free(time);
    return 0;
}
