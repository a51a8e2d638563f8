/* Oracle for sphrayderv's per-observation work (test infrastructure only): the residual and
 * hypocentre derivatives at the event, the ray traced back down the travel-time gradient to the
 * station, and the ray's derivative with respect to slowness on the coarse "metagrid".  Restates
 * reference src/sphrayderv.c:1054-1700 (one observation of one local event) and
 * lib/sphrayderv/dfind.c, pmin.c. */
#ifndef FD_RAY_H
#define FD_RAY_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;           /* fine grid */
    int nxc, nyc, nzc;        /* coarse grid */
    double x0, y0, z0;        /* origin: longitude (rad), geocentric colatitude (rad), depth (km) */
    double h, dq, df;         /* km, rad, rad */
    const float *gx, *gy, *gz;   /* coarse node coordinates as the reference stores them (float) */
} fdr_grid;

typedef struct {
    double ex, ey, ez;        /* event: longitude, colatitude (rad), depth (km) */
    double xs, ys, zs;        /* station: longitude, colatitude (rad), -elevation (km) */
    int field;                /* which time field (station-phase) */
    int phase;                /* 0 P, 1 S */
    float obstime;            /* arrival minus origin (s) */
    float pwt;                /* 1 / rwt^2 */
    float tc;                 /* station correction */
    int pad;
} fdr_obs;

/* status of one observation */
enum {
    FDR_OK = 0,          /* ray reached the station: derivatives valid */
    FDR_NOTIME = 1,      /* a corner of the event's cell has no time (> 1e9) (:1357-1364) */
    FDR_LEFT = 2,        /* ray left the model (:2037-2140, label a150) */
    FDR_STEPS = 3,       /* ray took more than max_seg segments (the reference has no limit) */
    FDR_COARSE = 4,      /* a segment midpoint lies beyond the coarse grid (the reference asserts) */
    FDR_OUTSIDE = 5,     /* a cell corner index falls outside the field (the reference reads past it) */
};

typedef struct {
    int status;
    int nseg;
    double dt;                /* residual obstime - (t + tc), double as the reference keeps it */
    float resmin;             /* the same, as float */
    float wet;                /* sqrt(pwt) */
    float am[4];              /* wet, dt/dx wet, dt/dy wet, dt/dz wet */
    int nnz;                  /* coarse nodes with a nonzero derivative (ascending index) */
    int pad;
} fdr_result;

/* Trace nobs observations.  fields[i] is time field i (nz*ny*nx floats).  For observation o the
 * nonzero coarse derivatives (raw du, before the sqrt(pwt) weight) go to idx[o*cap ..] / du[o*cap ..]
 * in ascending coarse index, at most cap of them (status FDR_STEPS if more).  trig_mode 0: the C
 * library's sin/cos/atan2 (as the reference); 1: the double-double functions the device uses. */
int fdr_trace(const fdr_grid *g, const float *const *fields, int nobs, const fdr_obs *obs, int trig_mode,
              int max_seg, int cap, fdr_result *res, int *idx, float *du);

/* one call of the trig functions, for tests: which 0 sin, 1 cos, 2 atan2(y, x) */
double fdr_trig(int trig_mode, int which, double y, double x);

#ifdef __cplusplus
}
#endif
#endif
