/*
 * fd_c2f.h — CPU oracle of c2f, the coarse-to-fine model interpolation (reference src/c2f.c).
 *
 * TEST INFRASTRUCTURE ONLY: the c2f tests use it as the checker of the GPU path.  Nothing in the
 * product calls it.  Pinned against the reference's own c2f binary (built from its sources into
 * _ref/) by tests/golden/make_c2f_golden.py.
 */
#ifndef FD_C2F_H
#define FD_C2F_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nxc, nyc, nzc;           /* coarse nodes per axis */
    const int *igridx, *igridy, *igridz;   /* fine steps between coarse nodes (nxc-1, ...) */
    double x0, y0, z0, h;        /* origin and fine spacing (the spec's x0, y0, z0, h) */
} fdo_c2f_grid;

/* fine dimensions of a coarse grid */
void fdo_c2f_dims(const fdo_c2f_grid *g, int *nx, int *ny, int *nz);

/* coarse (P then S velocities, nxc*nyc*nzc each, x fastest) to fine (P then S, nx*ny*nz each) */
int fdo_c2f(const fdo_c2f_grid *g, const float *coarse, float *fine);

#ifdef __cplusplus
}
#endif
#endif
