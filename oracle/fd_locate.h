/*
 * fd_locate.h — CPU oracle of sphfdloc's grid-search location (reference src/sphfdloc.c).
 *
 * TEST INFRASTRUCTURE ONLY: the location tests and the benchmark's CPU leg use it as the checker of
 * the GPU location path.  Nothing in the product calls it.
 *
 * It restates, per event, the coarse search over grid nodes (:729-794), the two subgrid refinements
 * with trilinear time lookups (:840-1056, find_time :1305-1345), and the outlier / recovery loop
 * that repeats the search (:1086-1128).  Pinned against the reference's own sphfdloc binary (built
 * from its sources into _ref/) by tests/golden/make_loc_golden.py.
 */
#ifndef FD_LOCATE_H
#define FD_LOCATE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;
    double x0, y0, z0;      /* longitude of x = 0 (rad), geocentric colatitude of y = 0 (rad), depth of z = 0 (km) */
    double h, dq, df;       /* depth step (km), colatitude and longitude steps (rad) */
    float xmax, ymax, zmax; /* far grid edges, stored as floats by the reference (:455-457) */
    double z0r;             /* radius of z = 0 (km), for the hypocentre's depth */
    int kmin;               /* first depth index of the coarse search (spec kmin - 1) */
    int ndiv, ndiv2;        /* subdivisions of the first and second refinements */
    int ivs;                /* 0: S times are the P field times vpvs */
    float vpvs;
    int nthres;             /* least number of accepted phases */
    float resthres, resthrep, stdmax;
} fdo_loc_grid;

typedef struct {
    int field;      /* index of this phase's time field */
    float obstime;  /* arrival minus the event's catalogue origin time, s */
    float pwt;      /* weight 1/(rwt*rwt) */
    char phase;     /* 'P' or 'S' */
    int good;       /* in: 0 for a phase marked '*'; out: the final flag */
} fdo_loc_obs;

typedef struct {
    int status;             /* 0 accepted, 1 too few phases (ngood < nthres), 2 stdmin > stdmax */
    int ngood;
    int nxx, nyy, nzz;      /* loop indices of the last improvement (0-based) */
    int passes;             /* searches run (1 + redos) */
    double exm, eym, ezm;   /* hypocentre: longitude (rad), colatitude (rad), depth (km) */
    float stdmin, avrmin;
} fdo_loc_result;

/* grid of a sphfdloc spec (:382-395, :455-457): degrees and km in, radians out */
void fdo_loc_grid_from_spec(fdo_loc_grid *g, int nx, int ny, int nz, double x0_deg, double y0_deg, double z0,
                            double h);

/* locate one event: resmin, tps (nobs each) receive the residuals and computed times at the final
 * point; obs[].good receives the final flags */
int fdo_locate(const fdo_loc_grid *g, const float *const *fields, int nobs, fdo_loc_obs *obs, float *resmin,
               float *tps, fdo_loc_result *r);

/* helpers of the reference's output: epoch seconds from a date (htoe), the inverse (etoh), and the
 * geodetic latitude of a geocentric colatitude (glathinv) */
double fdo_htoe(int iyear, int iday, int ihour, int imin, double sec);
void fdo_etoh(double epoch, int *iyear, int *iday, int *ihour, int *imin, double *sec);
double fdo_glathinv(double xcent, double r, double *h);
double fdo_loc_hpi(void);
double fdo_loc_degrad(void);

#ifdef __cplusplus
}
#endif
#endif
