/*
 * fd_c2f.c — CPU oracle of c2f (see fd_c2f.h).  TEST INFRASTRUCTURE ONLY.
 *
 * Restates src/c2f.c: coarse node coordinates accumulated in float (:265-287), velocities turned to
 * slowness in double and stored as float (:545-548), every fine node's slowness trilinearly
 * interpolated in float from the coarse cell found by a linear scan (find_vel, :673-727), and the
 * result turned back to velocity (:561-572).  Compiled with -ffp-contract=off.
 */
#include "fd_c2f.h"

#include <stdlib.h>

void fdo_c2f_dims(const fdo_c2f_grid *g, int *nx, int *ny, int *nz)
{
    *nx = *ny = *nz = 1;
    for (int i = 1; i < g->nxc; i++) *nx += g->igridx[i - 1];
    for (int i = 1; i < g->nyc; i++) *ny += g->igridy[i - 1];
    for (int i = 1; i < g->nzc; i++) *nz += g->igridz[i - 1];
}

/* coordinates of the coarse nodes, each step added in double and stored as float */
static void coords(float *c, int n, double o, double h, const int *ig)
{
    c[0] = (float)o;
    for (int i = 1; i < n; i++) c[i] = (float)(c[i - 1] + h * ig[i - 1]);
}

/* index of the coarse cell holding v: the first node past it, less one, kept inside the grid */
static int cell(const float *c, int n, float v)
{
    int i;
    for (i = 1; i < n; i++)
        if (c[i] > v) break;
    if (i == n) i--;
    return i - 1;
}

int fdo_c2f(const fdo_c2f_grid *g, const float *coarse, float *fine)
{
    const int nxc = g->nxc, nyc = g->nyc, nzc = g->nzc;
    const int nxyzc = nxc * nyc * nzc;
    int nx, ny, nz;
    fdo_c2f_dims(g, &nx, &ny, &nz);
    float *gx = malloc(sizeof(float) * nxc), *gy = malloc(sizeof(float) * nyc), *gz = malloc(sizeof(float) * nzc);
    float *s = malloc(sizeof(float) * 2 * (size_t)nxyzc);
    if (!gx || !gy || !gz || !s) {
        free(gx); free(gy); free(gz); free(s);
        return -1;
    }
    coords(gx, nxc, g->x0, g->h, g->igridx);
    coords(gy, nyc, g->y0, g->h, g->igridy);
    coords(gz, nzc, g->z0, g->h, g->igridz);
    for (int i = 0; i < 2 * nxyzc; i++) s[i] = (float)(1. / coarse[i]);
    long long ij = 0;
    for (int ph = 0; ph < 2; ph++) {
        const float *sp = s + (size_t)ph * nxyzc;
        for (int k = 0; k < nz; k++) {
            const float z = (float)(g->z0 + k * g->h);
            for (int j = 0; j < ny; j++) {
                const float y = (float)(g->y0 + j * g->h);
                for (int i = 0; i < nx; i++) {
                    const float x = (float)(g->x0 + i * g->h);
                    const int ci = cell(gx, nxc, x), cj = cell(gy, nyc, y), ck = cell(gz, nzc, z);
                    const float fx = (x - gx[ci]) / (gx[ci + 1] - gx[ci]);
                    const float fy = (y - gy[cj]) / (gy[cj + 1] - gy[cj]);
                    const float fz = (z - gz[ck]) / (gz[ck + 1] - gz[ck]);
                    const int a = nxc * nyc * ck, b = nxc * cj, a2 = nxc * nyc * (ck + 1), b2 = nxc * (cj + 1);
                    float t = (1.f - fx) * (1.f - fy) * (1.f - fz) * sp[a + b + ci];
                    t = t + fx * (1.f - fy) * (1.f - fz) * sp[a + b + ci + 1];
                    t = t + (1.f - fx) * fy * (1.f - fz) * sp[a + b2 + ci];
                    t = t + (1.f - fx) * (1.f - fy) * fz * sp[a2 + b + ci];
                    t = t + fx * fy * (1.f - fz) * sp[a + b2 + ci + 1];
                    t = t + fx * (1.f - fy) * fz * sp[a2 + b + ci + 1];
                    t = t + (1.f - fx) * fy * fz * sp[a2 + b2 + ci];
                    t = t + fx * fy * fz * sp[a2 + b2 + ci + 1];
                    fine[ij++] = 1.f / t;
                }
            }
        }
    }
    free(gx); free(gy); free(gz); free(s);
    return 0;
}
