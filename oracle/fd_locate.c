/*
 * fd_locate.c — CPU oracle of sphfdloc's grid-search location (see fd_locate.h).
 *
 * TEST INFRASTRUCTURE ONLY.  A restatement of the reference's per-event search, in its operation
 * order (float statistics, double positions and trilinear weights), compiled with
 * -ffp-contract=off like the reference's build (x86-64 without FMA contraction).
 */
#include "fd_locate.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* the reference's constants are float literals widened to double (src/sphfdloc.c:74-75) */
static const double kHpi = 1.570796f;
static const double kDegrad = 0.017453292f;
static const double kRearth = 6371.0;   /* :71 */

double fdo_loc_hpi(void) { return kHpi; }
double fdo_loc_degrad(void) { return kDegrad; }

/* WGS84 geodetic latitude and depth to geocentric latitude and radius (lib/common/geographic_method.c
 * glath, the version sphfdloc links) */
static double loc_glath(double xlat, double depth, double *r)
{
    const double ap = 6378137.0;
    const double esq = 6.69437978616733379 * 0.001;
    const double s = sin(xlat);
    const double hm = -depth * 1000.0;
    const double anu = ap / sqrt(1.0 - esq * s * s);
    const double x = (anu + hm) * cos(xlat);
    const double z = ((1.0 - esq) * anu + hm) * s;
    *r = sqrt(x * x + z * z) / 1000.0;
    return atan2(z, x);
}

/* the inverse, five fixed-point steps (lib/common/geographic_method.c glathinv) */
double fdo_glathinv(double xcent, double r, double *h)
{
    const double ap = 6378137.0;
    const double esq = 6.69437978616733379 * 0.001;
    const double rm = r * 1000.0;
    double lat = xcent;
    const double x = rm * cos(lat);
    const double z = rm * sin(lat);
    double anu = 0.0;
    for (int it = 0; it < 5; it++) {
        const double s = sin(lat);
        anu = ap / sqrt(1.0 - esq * s * s);
        const double hb = x / cos(lat) - anu;
        const double zp = z / (1.0 - esq * (anu / (anu + hb)));
        lat = atan2(zp, x);
    }
    *h = x / cos(lat) - anu;
    *h = -*h / 1000.0;
    return lat;
}

static int leap(int y) { return ((y % 4 == 0 && y % 100 != 0) || y % 400 == 0) ? 1 : 0; }

/* epoch seconds of (year, day of year, hour, minute, seconds) (lib/common/time_process.c htoe,
 * dtoepoch) */
double fdo_htoe(int iyear, int iday, int ihour, int imin, double sec)
{
    int days = 0;
    if (iyear > 1970)
        for (int y = 1970; y < iyear; y++) days += 365 + leap(y);
    else if (iyear < 1970)
        for (int y = iyear; y <= 1969; y++) days -= 365 + leap(y);
    days += iday - 1;
    double e = (double)(days * 24 * 60 * 60);
    return e + 3600.0 * ihour + 60.0 * imin + sec;
}

/* and back (lib/common/time_process.c etoh) */
void fdo_etoh(double epoch, int *iyear, int *iday, int *ihour, int *imin, double *sec)
{
    int doy = (int)(epoch / 86400.0);
    double left = fmod(epoch, 86400.0);
    int hour = 0, minute = 0;
    double second = 0.0;
    if (left != 0.0) {
        if (left < 0) {
            doy -= 1;
            left += 86400;
        }
        hour = (int)(left / 3600);
        left = fmod(left, 3600.0);
        minute = (int)(left / 60);
        second = fmod(left, 60.0);
    }
    int year;
    if (doy >= 0) {
        year = 1970;
        while (doy >= 365 + leap(year)) {
            doy -= 365 + leap(year);
            year++;
        }
    } else {
        year = 1969;
        while (doy < 0) {
            doy += 365 + leap(year);
            year--;
        }
    }
    *iyear = year;
    *iday = doy + 1;
    *ihour = hour;
    *imin = minute;
    *sec = second;
}

void fdo_loc_grid_from_spec(fdo_loc_grid *g, int nx, int ny, int nz, double x0_deg, double y0_deg, double z0,
                            double h)
{
    memset(g, 0, sizeof *g);
    g->nx = nx;
    g->ny = ny;
    g->nz = nz;
    g->h = h;
    g->z0 = z0;
    /* :384-394: geocentric colatitude of the north edge; dq, df from h (the spec has no dq/df) */
    const double ylat = y0_deg * kDegrad;
    g->y0 = kHpi - loc_glath(ylat, z0, &g->z0r);
    g->x0 = x0_deg * kDegrad;
    g->dq = h / kRearth;
    g->df = fabs(h / (kRearth * sin(g->y0)));
    /* :455-457 */
    g->xmax = (float)(g->x0 + (nx - 1) * g->df);
    g->ymax = (float)(g->y0 + (ny - 1) * g->dq);
    g->zmax = (float)(g->z0 + (nz - 1) * g->h);
    /* defaults of :104-136 */
    g->kmin = 2;
    g->ndiv = 20;
    g->ndiv2 = 20;
    g->ivs = 1;
    g->vpvs = 1.78f;
    g->nthres = 8;
    g->resthres = .5f;
    g->resthrep = 5.0f;
    g->stdmax = 15.0f;
}

/* trilinear time at (x lon, yy colat, z depth) from the cell that contains it, clamped to the grid
 * (find_time, src/sphfdloc.c:1305-1345) */
static double find_time(const fdo_loc_grid *g, const float *t, double x, double yy, double z)
{
    int i = (int)((x - g->x0) / g->df);
    int j = (int)((yy - g->y0) / g->dq);
    int k = (int)((z - g->z0) / g->h);
    if (i < 0) i = 0;
    if (j < 0) j = 0;
    if (k < 0) k = 0;
    if (i > g->nx - 2) i = g->nx - 2;
    if (j > g->ny - 2) j = g->ny - 2;
    if (k > g->nz - 2) k = g->nz - 2;
    const double xi = g->x0 + g->df * i, yj = g->y0 + g->dq * j, zk = g->z0 + g->h * k;
    const int a = g->nx * g->ny * k, b = g->nx * j, a2 = g->nx * g->ny * (k + 1), b2 = g->nx * (j + 1);
    const double fx = (x - xi) / g->df, fy = (yy - yj) / g->dq, fz = (z - zk) / g->h;
    double tp = (1.0 - fx) * (1.0 - fy) * (1.0 - fz) * t[a + b + i];
    tp = tp + fx * (1.0 - fy) * (1.0 - fz) * t[a + b + i + 1];
    tp = tp + (1.0 - fx) * fy * (1.0 - fz) * t[a + b2 + i];
    tp = tp + (1.0 - fx) * (1.0 - fy) * fz * t[a2 + b + i];
    tp = tp + fx * fy * (1.0 - fz) * t[a + b2 + i + 1];
    tp = tp + fx * (1.0 - fy) * fz * t[a2 + b + i + 1];
    tp = tp + (1.0 - fx) * fy * fz * t[a2 + b2 + i];
    tp = tp + fx * fy * fz * t[a2 + b2 + i + 1];
    return tp;
}

/* the search state of one event: the running minimum and the residuals where it was found */
typedef struct {
    float stdmin, avrmin;
    int nxx, nyy, nzz;
    double exm, eym, ezm;
} Best;

/* residual statistics of one trial point from its phases' times tp (:737-771); returns the
 * standard deviation, and the weighted mean residual in *avres_facs */
static float trial(const fdo_loc_grid *g, int nobs, const fdo_loc_obs *obs, const double *tp, int ngood,
                   float *res, float *mean)
{
    float avres = 0.0f, rsq = 0.0f, facs = 0.0f;
    for (int is = 0; is < nobs; is++) {
        double t = tp[is];
        if (g->ivs == 0 && obs[is].phase == 'S') t *= g->vpvs;
        res[is] = obs[is].obstime - t;
        const float wt = obs[is].pwt;
        if (obs[is].good) {
            const float r1 = res[is] * wt;
            const float r2 = r1 * res[is];
            avres += r1;
            rsq += r2;
            facs += wt;
        }
    }
    const float avwt = facs / ngood;
    const float deb = (rsq - avres * avres / facs) / ((ngood - 4) * avwt);
    const float dsum = fabs(deb);
    *mean = avres / facs;
    return sqrtf(dsum);
}

/* a new minimum (:772-785): strictly smaller only, so the first point in loop order wins ties */
static void take(Best *b, float std, float mean, int i, int j, int k, int nobs, const fdo_loc_obs *obs,
                 const float *res, float *resmin, float *tps)
{
    b->stdmin = std;
    b->avrmin = mean;
    b->nxx = i;
    b->nyy = j;
    b->nzz = k;
    for (int q = 0; q < nobs; q++) {
        resmin[q] = res[q];
        tps[q] = obs[q].obstime - res[q];
    }
}

int fdo_locate(const fdo_loc_grid *g, const float *const *fields, int nobs, fdo_loc_obs *obs, float *resmin,
               float *tps, fdo_loc_result *r)
{
    if (!g || !fields || nobs < 1 || !obs || !resmin || !tps || !r) return -1;
    double *tp = (double *)malloc(sizeof(double) * nobs);
    float *res = (float *)malloc(sizeof(float) * nobs);
    if (!tp || !res) {
        free(tp);
        free(res);
        return -2;
    }
    memset(resmin, 0, sizeof(float) * nobs);
    memset(tps, 0, sizeof(float) * nobs);
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    int ngood = nobs;   /* :686, before any outlier check: every phase, flagged or not */
    int iretry = 0, passes = 0, status = 0;
    const int maxretry = 1;
    Best b;
    for (;;) {
        passes++;
        /* coarse search over the grid nodes from depth index kmin (:729-794) */
        b.nxx = b.nyy = b.nzz = 0;
        b.stdmin = (float)DBL_MAX;   /* +inf as a float */
        b.avrmin = 0.0f;
        for (int k = g->kmin; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    const int n = nx * ny * k + nx * j + i;
                    for (int is = 0; is < nobs; is++) tp[is] = fields[obs[is].field][n];
                    float mean;
                    const float std = trial(g, nobs, obs, tp, ngood, res, &mean);
                    if (std < b.stdmin) take(&b, std, mean, i, j, k, nobs, obs, res, resmin, tps);
                }
        b.exm = g->x0 + b.nxx * g->df;
        b.eym = g->y0 + b.nyy * g->dq;
        b.ezm = g->z0 + b.nzz * g->h;

        /* first refinement: ndiv steps per cell around the best node (:840-895) */
        int n1 = g->ndiv + 1, n2 = n1 + g->ndiv;
        const double dh = g->h / g->ndiv, ddq = g->dq / g->ndiv, ddf = g->df / g->ndiv;
        int iz0 = b.nzz - 1, nsz = n2;
        if (iz0 < g->kmin) { iz0 = b.nzz; nsz = n1; }
        if (b.nzz == nz - 1) nsz = n1 - 1;
        int iy0 = b.nyy - 1, nsy = n2;
        if (iy0 < 0) { iy0 = b.nyy; nsy = n1; }
        if (b.nyy == ny - 1) nsy = n1 - 1;
        int ix0 = b.nxx - 1, nsx = n2;
        if (ix0 < 0) { ix0 = b.nxx; nsx = n1; }
        if (b.nxx == nx - 1) nsx = n1 - 1;
        double z0i = g->z0 + g->h * iz0, y0i = g->y0 + g->dq * iy0, x0i = g->x0 + g->df * ix0;
        for (int k = 0; k < nsz; k++) {
            const double zp = z0i + dh * k;
            for (int j = 0; j < nsy; j++) {
                const double yp = y0i + ddq * j;
                for (int i = 0; i < nsx; i++) {
                    const double xp = x0i + ddf * i;
                    for (int is = 0; is < nobs; is++) tp[is] = find_time(g, fields[obs[is].field], xp, yp, zp);
                    float mean;
                    const float std = trial(g, nobs, obs, tp, ngood, res, &mean);
                    if (std < b.stdmin) {
                        take(&b, std, mean, i, j, k, nobs, obs, res, resmin, tps);
                        b.exm = xp;
                        b.eym = yp;
                        b.ezm = zp;
                    }
                }
            }
        }

        /* second refinement: ndiv2 steps per first-refinement step around the best point (:967-1056) */
        n1 = g->ndiv2 + 1;
        n2 = n1 + g->ndiv2;
        const double ddh = dh / g->ndiv2, dddq = ddq / g->ndiv2, dddf = ddf / g->ndiv2;
        z0i = b.ezm - dh;
        nsz = n2;
        if (z0i <= g->z0 + g->kmin * g->h) { z0i = b.ezm; nsz = n1; }
        if (b.ezm + dh > g->zmax) nsz = n1 - 1;
        y0i = b.eym - ddq;
        nsy = n2;
        if (y0i <= g->y0) { y0i = b.eym; nsy = n1; }
        if (b.eym + ddq > g->ymax) nsy = n1 - 1;
        x0i = b.exm - ddf;
        nsx = n2;
        if (x0i <= g->x0) { x0i = b.exm; nsx = n1; }
        if (b.exm + ddf > g->xmax) nsx = n1 - 1;
        for (int k = 0; k < nsz; k++) {
            const double zp = z0i + ddh * k;
            for (int j = 0; j < nsy; j++) {
                const double yp = y0i + dddq * j;
                for (int i = 0; i < nsx; i++) {
                    const double xp = x0i + dddf * i;
                    for (int is = 0; is < nobs; is++) tp[is] = find_time(g, fields[obs[is].field], xp, yp, zp);
                    float mean;
                    const float std = trial(g, nobs, obs, tp, ngood, res, &mean);
                    if (std < b.stdmin) {
                        take(&b, std, mean, i, j, k, nobs, obs, res, resmin, tps);
                        b.exm = xp;
                        b.eym = yp;
                        b.ezm = zp;
                    }
                }
            }
        }

        /* outliers and recovered phases (:1086-1128) */
        ngood = 0;
        int redo = 0;
        for (int i = 0; i < nobs; i++) {
            if (!obs[i].good) continue;
            const float absres = fabs(resmin[i] - b.avrmin);
            const float perc = 100.0f * absres / tps[i];
            if (absres <= g->resthres || perc <= g->resthrep)
                ngood++;
            else {
                obs[i].good = 0;
                redo = 1;
            }
        }
        if (ngood < g->nthres) {
            status = 1;
            break;
        }
        if (redo) continue;
        if (iretry < maxretry) {
            iretry++;
            redo = 0;
            for (int i = 0; i < nobs; i++) {
                if (obs[i].good) continue;
                const float absres = fabs(resmin[i] - b.avrmin);
                const float perc = 100.0f * absres / tps[i];
                if (absres <= g->resthres || perc <= g->resthrep) {
                    ngood++;
                    obs[i].good = 1;
                    redo = 1;
                }
            }
            if (redo) continue;
        }
        status = b.stdmin <= g->stdmax ? 0 : 2;
        break;
    }
    r->status = status;
    r->ngood = ngood;
    r->nxx = b.nxx;
    r->nyy = b.nyy;
    r->nzz = b.nzz;
    r->passes = passes;
    r->exm = b.exm;
    r->eym = b.eym;
    r->ezm = b.ezm;
    r->stdmin = b.stdmin;
    r->avrmin = b.avrmin;
    free(tp);
    free(res);
    return 0;
}
