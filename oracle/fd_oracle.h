/*
 * fd_oracle.h — CPU restatement of FDtomoC's sphfd travel-time solver (reference: src/sphfd.c).
 *
 * TEST INFRASTRUCTURE.  This is the checker that the GPU library is compared against: only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The product
 * library never includes, links or calls anything in this directory.
 *
 * Parity pin: on the reference's own fixture (verification/cmod/tempvel -> M001.ptimes) and on the
 * synthetic cases in tests/golden, this restatement reproduces the reference binary bit-for-bit.
 */
#ifndef FD_ORACLE_H
#define FD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Grid geometry after sphfd's parameter conversion (src/sphfd.c:415-455): angles in radians, y0 as
 * geocentric colatitude, z0r the radius of the grid's top layer in km. */
typedef struct {
    int nx, ny, nz;
    double h, dq, df;
    double x0, y0, z0r;
} fdo_grid;

/* The expanding box (src/sphfd.c:766-825): walls x1..z2 lie one node outside the computed region;
 * d* are 1 while the wall can still move outward. */
typedef struct {
    int x1, x2, y1, y2, z1, z2;
    int dx1, dx2, dy1, dy2, dz1, dz2;
    int radius;
} fdo_box;

/* Sweep controls (src/sphfd.c:388-413, 546-552, 977-1003). */
typedef struct {
    int reverse;    /* up to reverse+1 sweeps */
    int headpref;   /* preferred restart wall (1..6), <= 0 for none; already resolved by fdo_headpref */
    int maxrad;     /* radius at which the box stops growing (99999999 = unlimited) */
    int kminus, kplus, iplus, iminus, jminus, jplus;
} fdo_sweep;

typedef struct {
    int64_t node_updates;     /* face-point bodies executed */
    int64_t calls[5];         /* stencil evaluations by kind: 3d ne 2d nf 1d (after pruning in fast mode) */
    int64_t skipped[5];       /* evaluations pruned as unable to lower the running minimum (fast mode) */
    int64_t inherit_points;   /* points whose 2-D trials used (t0,t4) left by an earlier point */
    int64_t faces;
    int sweeps;
    int restarts[7];          /* restart wall chosen after each sweep, by wall number (count) */
    int64_t changed_per_sweep[64];
    int64_t depth_per_sweep[64];  /* sum over the sweep's faces of the face's dependency depth (longest
                                     chain of in-face neighbours in sort order) */
    int64_t updates_per_sweep[64];
} fdo_stats;

/* Stale stencil state: the (t[0], t[4]) pair that fdsph2d reads but no 2-D call site assigns. */
typedef struct { double t0, t4; } fdo_carry;

enum { FDO_MODE_LITERAL = 0, FDO_MODE_FAST = 1 };

/* Solve on an already-initialised time field (source box filled, box walls set).
 * slow: nx*ny*nz slownesses; time: in/out.  mode FAST prunes stencils that cannot lower the running
 * minimum and reads 3-D coefficients from per-cell tables — both exact; used to validate the GPU
 * design on the CPU.  Returns 0. */
int fdo_propagate(const fdo_grid *g, const float *slow, float *time, fdo_box box, fdo_sweep sw,
                  fdo_carry *carry, int mode, fdo_stats *st);

/* headpref resolution from the initial box (src/sphfd.c:977-1003). */
int fdo_headpref(const fdo_grid *g, const fdo_box *b, int headpref);

/* Point-source set-up (src/sphfd.c:724-825): fills the (2*ncube+1)^3 box with straight-ray times
 * at the source-node slowness and returns the initial walls.  src_geo = geocentric source
 * (lon rad, colat rad, radius km); (xs,ys,zs) = nearest node. */
void fdo_point_source(const fdo_grid *g, const float *slow, float *time, int xs, int ys, int zs,
                      const double src_geo[3], int ncube, fdo_box *box);

/* Whole-station driver with the reference's par-file semantics (src/sphfd.c:260-5803): parses
 * "par=<file>" style arguments, reads the velocity file, solves, writes <timedir>/<timefile>.
 * Returns 0 on success, a negative code on error (never aborts).  stats may be NULL. */
int fdo_sphfd(int ac, char **av, const char *timedir, int mode, fdo_stats *stats);

/* WGS84 geodetic -> geocentric (src/sphfd.c:5836-5893).  Returns geocentric latitude (rad). */
double fdo_glath(double hlat, double depth_km, double *radius_km);

#ifdef __cplusplus
}
#endif
#endif
