/*
 * fdgpu_locate.cu — event location on device-resident travel-time fields: the grid search of
 * FDtomoC's sphfdloc (reference src/sphfdloc.c), for many events per call, with results
 * bit-identical to the reference's.
 *
 * Per event the reference runs (a) a coarse search over the grid nodes from depth index kmin
 * (:729-794), (b) a refinement with ndiv steps per cell around the best node (:840-895), (c) a second
 * refinement with ndiv2 steps per first-refinement step around the best point (:967-1056), each
 * trial point scored by the standard deviation of its weighted residuals, then (d) drops outliers or
 * recovers phases and repeats (a)-(c) if that changed the phase set (:1086-1128).
 *
 * GPU form: one thread per trial point and event, every event of the batch in the same launch
 * (grid.y).  Each thread keeps the reference's sequential per-phase accumulation, so the statistics
 * match bit for bit; the "first strictly smaller" scan over trial points becomes an atomicMin on
 * (float bits of the deviation << 32 | trial index in loop order), which picks the same point.  A
 * one-thread-per-event kernel between stages takes the minimum, updates the event's best point the
 * way the sequential scan would, and lays out the next stage's window; a last one recomputes the
 * residuals at the final point and runs the outlier / recovery step.  The host repeats the stages
 * for the events that asked for another pass.
 *
 * Arithmetic: statistics in float, positions and trilinear weights in double, as the reference;
 * compiled with --fmad=false and IEEE float division and square root.  At grid nodes the residual
 * obstime - t of two floats is formed in float: the reference forms it in double and rounds to
 * float, and the two agree for all finite floats (when the exponents differ by 29 or less the double
 * difference is exact, so one rounding happens in both; beyond that the smaller operand is below a
 * half unit of the larger and both give the larger).
 */
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "fdgpu.h"
#include "fdgpu_device.h"

namespace {

constexpr int kLocBlock = 256;
constexpr int kMaxObs = 800;   /* the reference's maxobs (include/common/parameter.h) */

enum { kActive = 0, kAccepted = 1, kTooFew = 2, kStdHigh = 3, kRedo = 4 };

struct LocEvent {
    int obs0, nobs;
    int ngood, iretry, passes, state;
    float stdmin, avrmin;
    int nxx, nyy, nzz;
    int wstage;                 /* stage of the last new minimum: 0 coarse, 1, 2 */
    double exm, eym, ezm;
    double x0i, y0i, z0i, sx, sy, sz;   /* current refinement window: origin and steps */
    int nsx, nsy, nsz;
    unsigned long long best;    /* (deviation bits << 32) | trial index; ~0: none */
};

struct LocObsDev {
    const float *field;
    float obstime, pwt;
    int s_scaled;   /* S phase whose time is the P field times vpvs (ivs 0) */
};

__device__ __forceinline__ unsigned long long trial_key(float std, unsigned idx)
{
    /* only deviations that can win: finite (the running minimum starts at +inf, and NaN never
     * compares smaller) */
    if (!(std < INFINITY)) return ~0ull;
    return ((unsigned long long)__float_as_uint(std) << 32) | idx;
}

/* The cell containing (x, yy, z), clamped to the grid, and its eight trilinear weights, as find_time
 * forms them (:1305-1345).  All fields share the grid, so a trial point computes these once for all
 * its phases; each weight is the same product, in the same order, that the reference multiplies by
 * the corner's time. */
struct Cell {
    long long a, b, a2, b2;
    int i;
    double w[8];
};

__device__ __forceinline__ void find_cell(const fdgpu_loc_grid &g, double x, double yy, double z, Cell &c)
{
    int i = (int)((x - g.x0) / g.df);
    int j = (int)((yy - g.y0) / g.dq);
    int k = (int)((z - g.z0) / g.h);
    i = i < 0 ? 0 : i;
    j = j < 0 ? 0 : j;
    k = k < 0 ? 0 : k;
    i = i > g.nx - 2 ? g.nx - 2 : i;
    j = j > g.ny - 2 ? g.ny - 2 : j;
    k = k > g.nz - 2 ? g.nz - 2 : k;
    const double xi = g.x0 + g.df * i, yj = g.y0 + g.dq * j, zk = g.z0 + g.h * k;
    c.a = (long long)g.nx * g.ny * k;
    c.b = (long long)g.nx * j;
    c.a2 = (long long)g.nx * g.ny * (k + 1);
    c.b2 = (long long)g.nx * (j + 1);
    c.i = i;
    const double fx = (x - xi) / g.df, fy = (yy - yj) / g.dq, fz = (z - zk) / g.h;
    c.w[0] = (1.0 - fx) * (1.0 - fy) * (1.0 - fz);
    c.w[1] = fx * (1.0 - fy) * (1.0 - fz);
    c.w[2] = (1.0 - fx) * fy * (1.0 - fz);
    c.w[3] = (1.0 - fx) * (1.0 - fy) * fz;
    c.w[4] = fx * fy * (1.0 - fz);
    c.w[5] = fx * (1.0 - fy) * fz;
    c.w[6] = (1.0 - fx) * fy * fz;
    c.w[7] = fx * fy * fz;
}

/* the trilinear time of one field in that cell: the reference's sum, term by term */
__device__ __forceinline__ double cell_time(const Cell &c, const float *t)
{
    const int i = c.i;
    double tp = c.w[0] * (double)t[c.a + c.b + i];
    tp = tp + c.w[1] * (double)t[c.a + c.b + i + 1];
    tp = tp + c.w[2] * (double)t[c.a + c.b2 + i];
    tp = tp + c.w[3] * (double)t[c.a2 + c.b + i];
    tp = tp + c.w[4] * (double)t[c.a + c.b2 + i + 1];
    tp = tp + c.w[5] * (double)t[c.a2 + c.b + i + 1];
    tp = tp + c.w[6] * (double)t[c.a2 + c.b2 + i];
    tp = tp + c.w[7] * (double)t[c.a2 + c.b2 + i + 1];
    return tp;
}

/* one phase's residual at a trial point whose time is tp (double) */
__device__ __forceinline__ float residual_d(const LocObsDev &o, double tp, float vpvs)
{
    if (o.s_scaled) tp *= (double)vpvs;
    return (float)((double)o.obstime - tp);
}

/* the accumulation of :750-770 for one phase */
__device__ __forceinline__ void accumulate(float res, float wt, bool good, float &avres, float &rsq, float &facs)
{
    if (good) {
        const float r1 = res * wt;
        const float r2 = r1 * res;
        avres += r1;
        rsq += r2;
        facs += wt;
    }
}

/* :771-777 */
__device__ __forceinline__ float deviation(float avres, float rsq, float facs, int ngood)
{
    const float avwt = facs / (float)ngood;
    const float deb = (rsq - avres * avres / facs) / ((float)(ngood - 4) * avwt);
    return sqrtf(fabsf(deb));
}

/* the block's smallest key into the event's minimum */
__device__ __forceinline__ void reduce_key(unsigned long long key, unsigned long long *dst)
{
    __shared__ unsigned long long red[kLocBlock / 32];
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
        key = other < key ? other : key;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = key;
    __syncthreads();
    if (threadIdx.x < 32) {
        key = threadIdx.x < kLocBlock / 32 ? red[threadIdx.x] : ~0ull;
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
            key = other < key ? other : key;
        }
        if (threadIdx.x == 0 && key != ~0ull) atomicMin(dst, key);
    }
}

/* the event's phases in shared memory */
struct ObsTile {
    const float *field[kMaxObs];
    float obstime[kMaxObs], pwt[kMaxObs];
    unsigned char good[kMaxObs], s_scaled[kMaxObs];
};

__device__ void load_obs(ObsTile &ot, const LocObsDev *obs, const unsigned char *good, const LocEvent &ev)
{
    for (int q = threadIdx.x; q < ev.nobs; q += blockDim.x) {
        const LocObsDev o = obs[ev.obs0 + q];
        ot.field[q] = o.field;
        ot.obstime[q] = o.obstime;
        ot.pwt[q] = o.pwt;
        ot.s_scaled[q] = (unsigned char)o.s_scaled;
        ot.good[q] = good[ev.obs0 + q];
    }
    __syncthreads();
}

/* (a) coarse search: trial c is grid node nx*ny*kmin + c, in the reference's loop order */
__global__ void __launch_bounds__(kLocBlock) loc_coarse(fdgpu_loc_grid g, const LocObsDev *obs,
                                                          const unsigned char *good, LocEvent *evs,
                                                          const int *active, long long ncand)
{
    __shared__ ObsTile ot;
    LocEvent &ev = evs[active[blockIdx.y]];
    if ((long long)blockIdx.x * kLocBlock >= ncand) return;
    load_obs(ot, obs, good, ev);
    const long long c = (long long)blockIdx.x * kLocBlock + threadIdx.x;
    unsigned long long key = ~0ull;
    if (c < ncand) {
        const long long n = (long long)g.nx * g.ny * g.kmin + c;
        float avres = 0.0f, rsq = 0.0f, facs = 0.0f;
        /* the phases' times are loaded eight at a time, so that eight loads are in flight, and then
         * accumulated in phase order */
        constexpr int kBatch = 8;
        for (int q0 = 0; q0 < ev.nobs; q0 += kBatch) {
            float tv[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) tv[u] = q0 + u < ev.nobs ? ot.field[q0 + u][n] : 0.0f;
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int q = q0 + u;
                if (q >= ev.nobs) break;
                const float t = tv[u];
                const float res = ot.s_scaled[q] ? (float)((double)ot.obstime[q] - (double)t * (double)g.vpvs)
                                                 : ot.obstime[q] - t;
                accumulate(res, ot.pwt[q], ot.good[q] != 0, avres, rsq, facs);
            }
        }
        key = trial_key(deviation(avres, rsq, facs, ev.ngood), (unsigned)c);
    }
    reduce_key(key, &ev.best);
}

/* (b), (c) refinements: trial c = (k * nsy + j) * nsx + i of the event's window */
__global__ void __launch_bounds__(kLocBlock) loc_refine(fdgpu_loc_grid g, const LocObsDev *obs,
                                                          const unsigned char *good, LocEvent *evs,
                                                          const int *active)
{
    __shared__ ObsTile ot;
    LocEvent &ev = evs[active[blockIdx.y]];
    const long long ncand = (long long)ev.nsx * ev.nsy * ev.nsz;
    if ((long long)blockIdx.x * kLocBlock >= ncand) return;
    load_obs(ot, obs, good, ev);
    const long long c = (long long)blockIdx.x * kLocBlock + threadIdx.x;
    unsigned long long key = ~0ull;
    if (c < ncand) {
        const int i = (int)(c % ev.nsx), j = (int)((c / ev.nsx) % ev.nsy), k = (int)(c / ((long long)ev.nsx * ev.nsy));
        const double zp = ev.z0i + ev.sz * k, yp = ev.y0i + ev.sy * j, xp = ev.x0i + ev.sx * i;
        Cell cell;
        find_cell(g, xp, yp, zp, cell);
        float avres = 0.0f, rsq = 0.0f, facs = 0.0f;
        for (int q = 0; q < ev.nobs; q++) {
            const LocObsDev o{ot.field[q], ot.obstime[q], ot.pwt[q], ot.s_scaled[q]};
            const float res = residual_d(o, cell_time(cell, o.field), g.vpvs);
            accumulate(res, ot.pwt[q], ot.good[q] != 0, avres, rsq, facs);
        }
        key = trial_key(deviation(avres, rsq, facs, ev.ngood), (unsigned)c);
    }
    reduce_key(key, &ev.best);
}

/* Take the stage's minimum (stage 0 coarse, 1, 2) and lay out the next window. */
__global__ void loc_plan(fdgpu_loc_grid g, LocEvent *evs, const int *active, int nact, int stage)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nact) return;
    LocEvent &ev = evs[active[a]];
    const unsigned long long key = ev.best;
    ev.best = ~0ull;
    const float std = __uint_as_float((unsigned)(key >> 32));
    const unsigned idx = (unsigned)key;
    if (stage == 0) {
        ev.nxx = ev.nyy = ev.nzz = 0;
        ev.stdmin = INFINITY;
        ev.wstage = 0;
        if (key != ~0ull) {
            const long long n = (long long)g.nx * g.ny * g.kmin + idx;
            ev.nxx = (int)(n % g.nx);
            ev.nyy = (int)((n / g.nx) % g.ny);
            ev.nzz = (int)(n / ((long long)g.nx * g.ny));
            ev.stdmin = std;
        }
        ev.exm = g.x0 + ev.nxx * g.df;
        ev.eym = g.y0 + ev.nyy * g.dq;
        ev.ezm = g.z0 + ev.nzz * g.h;
        /* first refinement window (:840-877) */
        const int n1 = g.ndiv + 1, n2 = n1 + g.ndiv;
        int iz0 = ev.nzz - 1, nsz = n2;
        if (iz0 < g.kmin) { iz0 = ev.nzz; nsz = n1; }
        if (ev.nzz == g.nz - 1) nsz = n1 - 1;
        int iy0 = ev.nyy - 1, nsy = n2;
        if (iy0 < 0) { iy0 = ev.nyy; nsy = n1; }
        if (ev.nyy == g.ny - 1) nsy = n1 - 1;
        int ix0 = ev.nxx - 1, nsx = n2;
        if (ix0 < 0) { ix0 = ev.nxx; nsx = n1; }
        if (ev.nxx == g.nx - 1) nsx = n1 - 1;
        ev.z0i = g.z0 + g.h * iz0;
        ev.y0i = g.y0 + g.dq * iy0;
        ev.x0i = g.x0 + g.df * ix0;
        ev.sz = g.h / g.ndiv;
        ev.sy = g.dq / g.ndiv;
        ev.sx = g.df / g.ndiv;
        ev.nsx = nsx;
        ev.nsy = nsy;
        ev.nsz = nsz;
        return;
    }
    if (key != ~0ull && std < ev.stdmin) {
        const int i = (int)(idx % (unsigned)ev.nsx), j = (int)((idx / (unsigned)ev.nsx) % (unsigned)ev.nsy);
        const int k = (int)(idx / ((unsigned)ev.nsx * (unsigned)ev.nsy));
        ev.nxx = i;
        ev.nyy = j;
        ev.nzz = k;
        ev.ezm = ev.z0i + ev.sz * k;
        ev.eym = ev.y0i + ev.sy * j;
        ev.exm = ev.x0i + ev.sx * i;
        ev.stdmin = std;
        ev.wstage = stage;
    }
    if (stage == 1) {
        /* second refinement window (:967-999) */
        const double dh = g.h / g.ndiv, ddq = g.dq / g.ndiv, ddf = g.df / g.ndiv;
        const int n1 = g.ndiv2 + 1, n2 = n1 + g.ndiv2;
        double z0i = ev.ezm - dh;
        int nsz = n2;
        if (z0i <= g.z0 + g.kmin * g.h) { z0i = ev.ezm; nsz = n1; }
        if (ev.ezm + dh > (double)g.zmax) nsz = n1 - 1;
        double y0i = ev.eym - ddq;
        int nsy = n2;
        if (y0i <= g.y0) { y0i = ev.eym; nsy = n1; }
        if (ev.eym + ddq > (double)g.ymax) nsy = n1 - 1;
        double x0i = ev.exm - ddf;
        int nsx = n2;
        if (x0i <= g.x0) { x0i = ev.exm; nsx = n1; }
        if (ev.exm + ddf > (double)g.xmax) nsx = n1 - 1;
        ev.z0i = z0i;
        ev.y0i = y0i;
        ev.x0i = x0i;
        ev.sz = dh / g.ndiv2;
        ev.sy = ddq / g.ndiv2;
        ev.sx = ddf / g.ndiv2;
        ev.nsx = nsx;
        ev.nsy = nsy;
        ev.nsz = nsz;
    }
}

/* Residuals at the final point, then the outlier / recovery step (:1086-1128). */
__global__ void loc_finish(fdgpu_loc_grid g, const LocObsDev *obs, unsigned char *good, LocEvent *evs,
                           const int *active, int nact, float *resmin, float *tps)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nact) return;
    LocEvent &ev = evs[active[a]];
    float avres = 0.0f, rsq = 0.0f, facs = 0.0f;
    const bool found = ev.stdmin < INFINITY;
    const long long node = (long long)g.nx * g.ny * ev.nzz + (long long)g.nx * ev.nyy + ev.nxx;
    Cell cell;
    find_cell(g, ev.exm, ev.eym, ev.ezm, cell);
    for (int q = 0; q < ev.nobs; q++) {
        const int o = ev.obs0 + q;
        const LocObsDev d = obs[o];
        float res;
        if (ev.wstage == 0)
            res = d.s_scaled ? (float)((double)d.obstime - (double)d.field[node] * (double)g.vpvs) : d.obstime - d.field[node];
        else
            res = residual_d(d, cell_time(cell, d.field), g.vpvs);
        accumulate(res, d.pwt, good[o] != 0, avres, rsq, facs);
        /* where no trial became the minimum in this pass the reference keeps the previous pass's
         * values (zero before the first) */
        if (found) {
            resmin[o] = res;
            tps[o] = d.obstime - res;
        }
    }
    ev.avrmin = found ? avres / facs : 0.0f;
    int ngood = 0, redo = 0;
    for (int q = 0; q < ev.nobs; q++) {
        const int o = ev.obs0 + q;
        if (!good[o]) continue;
        const float absres = fabsf(resmin[o] - ev.avrmin);
        const float perc = 100.0f * absres / tps[o];
        if (absres <= g.resthres || perc <= g.resthrep)
            ngood++;
        else {
            good[o] = 0;
            redo = 1;
        }
    }
    ev.ngood = ngood;
    if (ngood < g.nthres) {
        ev.state = kTooFew;
        return;
    }
    if (redo) {
        ev.state = kRedo;
        return;
    }
    if (ev.iretry < 1) {
        ev.iretry++;
        for (int q = 0; q < ev.nobs; q++) {
            const int o = ev.obs0 + q;
            if (good[o]) continue;
            const float absres = fabsf(resmin[o] - ev.avrmin);
            const float perc = 100.0f * absres / tps[o];
            if (absres <= g.resthres || perc <= g.resthrep) {
                ngood++;
                good[o] = 1;
                redo = 1;
            }
        }
        ev.ngood = ngood;
        if (redo) {
            ev.state = kRedo;
            return;
        }
    }
    ev.state = ev.stdmin <= g.stdmax ? kAccepted : kStdHigh;
}

__global__ void loc_init(LocEvent *evs, const int *offs, int nev)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nev) return;
    LocEvent &ev = evs[e];
    ev.obs0 = offs[e];
    ev.nobs = offs[e + 1] - offs[e];
    ev.ngood = ev.nobs;   /* :686: every phase, flagged or not, before the first check */
    ev.iretry = 0;
    ev.passes = 0;
    ev.state = kActive;
    ev.best = ~0ull;
}

__global__ void loc_begin_pass(LocEvent *evs, const int *active, int nact)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nact) return;
    LocEvent &ev = evs[active[a]];
    ev.passes++;
    ev.state = kActive;
    ev.best = ~0ull;
}

__global__ void loc_results(const LocEvent *evs, int nev, fdgpu_loc_result *out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nev) return;
    const LocEvent &ev = evs[e];
    fdgpu_loc_result r;
    r.status = ev.state == kAccepted ? 0 : ev.state == kTooFew ? 1 : 2;
    r.ngood = ev.ngood;
    r.nxx = ev.nxx;
    r.nyy = ev.nyy;
    r.nzz = ev.nzz;
    r.passes = ev.passes;
    r.exm = ev.exm;
    r.eym = ev.eym;
    r.ezm = ev.ezm;
    r.stdmin = ev.stdmin;
    r.avrmin = ev.avrmin;
    out[e] = r;
}

__global__ void loc_states(const LocEvent *evs, int nev, int *state)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nev) state[e] = evs[e].state;
}

}  // namespace

/* ---- host side -------------------------------------------------------------------------------- */

#include <cmath>
#include <cstring>
#include <vector>

extern "C" int fdh_ctx_device(const fdgpu_ctx *ctx);
extern "C" void *fdh_ctx_stream(const fdgpu_ctx *ctx);
extern "C" int fdh_ctx_fail(fdgpu_ctx *ctx, int cuda_error, const char *what);

namespace {

constexpr double kHpi = 1.570796f;          /* src/sphfdloc.c:74-75: float literals */
constexpr double kDegrad = 0.017453292f;

struct DevArena {
    std::vector<void *> ptrs;
    cudaStream_t s;
    explicit DevArena(cudaStream_t st) : s(st) {}
    ~DevArena()
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

extern "C" void fdgpu_loc_grid_from_spec(fdgpu_loc_grid *g, int nx, int ny, int nz, double x0_deg, double y0_deg,
                                         double z0_km, double h_km)
{
    if (!g) return;
    std::memset(g, 0, sizeof *g);
    g->nx = nx;
    g->ny = ny;
    g->nz = nz;
    g->h = h_km;
    g->z0 = z0_km;
    /* WGS84 geocentric colatitude of the north edge and radius of z = 0, as sphfdloc links it
     * (lib/common/geographic_method.c glath; src/sphfdloc.c:384-394) */
    const double ap = 6378137.0, esq = 6.69437978616733379 * 0.001;
    const double lat = y0_deg * kDegrad;
    const double s = std::sin(lat);
    const double hm = -z0_km * 1000.0;
    const double anu = ap / std::sqrt(1.0 - esq * s * s);
    const double x = (anu + hm) * std::cos(lat);
    const double z = ((1.0 - esq) * anu + hm) * s;
    g->z0r = std::sqrt(x * x + z * z) / 1000.0;
    g->y0 = kHpi - std::atan2(z, x);
    g->x0 = x0_deg * kDegrad;
    g->dq = h_km / 6371.0;
    g->df = std::fabs(h_km / (6371.0 * std::sin(g->y0)));
    g->xmax = (float)(g->x0 + (nx - 1) * g->df);
    g->ymax = (float)(g->y0 + (ny - 1) * g->dq);
    g->zmax = (float)(g->z0 + (nz - 1) * g->h);
    g->kmin = 2;
    g->ndiv = 20;
    g->ndiv2 = 20;
    g->ivs = 1;
    g->vpvs = 1.78f;
    g->nthres = 8;
    g->resthres = 0.5f;
    g->resthrep = 5.0f;
    g->stdmax = 15.0f;
}

#define LOC_CU(call)                                                        \
    do {                                                                    \
        const cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return fdh_ctx_fail(ctx, (int)e_, #call);    \
    } while (0)

extern "C" int fdgpu_locate(fdgpu_ctx *ctx, const fdgpu_loc_grid *g, const float *const *d_fields, int nfields,
                            int nev, const int *obs_offset, fdgpu_loc_obs *obs, float *resmin, float *tps,
                            fdgpu_loc_result *results, void *stream)
{
    if (!ctx || !g || nev < 0 || (nev > 0 && (!d_fields || !obs_offset || !obs || !resmin || !tps || !results)))
        return FDGPU_EINVAL;
    if (nev == 0) return FDGPU_OK;
    if (g->nx < 2 || g->ny < 2 || g->nz < 2 || g->ndiv < 1 || g->ndiv2 < 1 || g->ndiv > 1000 || g->ndiv2 > 1000
        || g->kmin < 0 || !(g->h > 0) || !(g->dq > 0) || !(g->df > 0))
        return FDGPU_EINVAL;
    if ((long long)g->nx * g->ny * g->nz >= (1ll << 31)) return FDGPU_EINVAL;
    if (obs_offset[0] != 0) return FDGPU_EINVAL;
    for (int e = 0; e < nev; e++) {
        const int n = obs_offset[e + 1] - obs_offset[e];
        if (n < 1 || n > kMaxObs) return FDGPU_EINVAL;
    }
    const int nobs = obs_offset[nev];
    for (int k = 0; k < nobs; k++) {
        const fdgpu_loc_obs &o = obs[k];
        if (o.field < 0 || o.field >= nfields || !d_fields[o.field]) return FDGPU_EINVAL;
        if (o.phase != 'P' && o.phase != 'S') return FDGPU_EINVAL;
    }
    FdDeviceScope dev_(fdh_ctx_device(ctx));
    if (dev_.err) return FDGPU_ENODEV;
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)fdh_ctx_stream(ctx);

    std::vector<LocObsDev> hobs(nobs);
    std::vector<unsigned char> hgood(nobs);
    for (int k = 0; k < nobs; k++) {
        hobs[k].field = d_fields[obs[k].field];
        hobs[k].obstime = obs[k].obstime;
        hobs[k].pwt = obs[k].pwt;
        hobs[k].s_scaled = (g->ivs == 0 && obs[k].phase == 'S') ? 1 : 0;
        hgood[k] = obs[k].good ? 1 : 0;
    }
    DevArena mem(st);
    LocObsDev *dobs;
    unsigned char *dgood;
    LocEvent *devs;
    int *doffs, *dact, *dstate;
    float *dres, *dtps;
    fdgpu_loc_result *dout;
    LOC_CU(mem.get(&dobs, nobs));
    LOC_CU(mem.get(&dgood, nobs));
    LOC_CU(mem.get(&devs, nev));
    LOC_CU(mem.get(&doffs, nev + 1));
    LOC_CU(mem.get(&dact, nev));
    LOC_CU(mem.get(&dstate, nev));
    LOC_CU(mem.get(&dres, nobs));
    LOC_CU(mem.get(&dtps, nobs));
    LOC_CU(mem.get(&dout, nev));
    LOC_CU(cudaMemcpyAsync(dobs, hobs.data(), sizeof(LocObsDev) * nobs, cudaMemcpyHostToDevice, st));
    LOC_CU(cudaMemcpyAsync(dgood, hgood.data(), nobs, cudaMemcpyHostToDevice, st));
    LOC_CU(cudaMemcpyAsync(doffs, obs_offset, sizeof(int) * (nev + 1), cudaMemcpyHostToDevice, st));
    LOC_CU(cudaMemsetAsync(dres, 0, sizeof(float) * nobs, st));
    LOC_CU(cudaMemsetAsync(dtps, 0, sizeof(float) * nobs, st));
    loc_init<<<(nev + 127) / 128, 128, 0, st>>>(devs, doffs, nev);
    LOC_CU(cudaGetLastError());

    const fdgpu_loc_grid G = *g;
    const long long ncoarse = g->kmin < g->nz ? (long long)(g->nz - g->kmin) * g->nx * g->ny : 0;
    const long long nwin1 = (long long)(2 * g->ndiv + 1) * (2 * g->ndiv + 1) * (2 * g->ndiv + 1);
    const long long nwin2 = (long long)(2 * g->ndiv2 + 1) * (2 * g->ndiv2 + 1) * (2 * g->ndiv2 + 1);
    std::vector<int> act(nev), state(nev);
    for (int e = 0; e < nev; e++) act[e] = e;
    for (int pass = 0; !act.empty(); pass++) {
        if (pass > 2 * kMaxObs + 4) return FDGPU_ESCHED;   /* each redo drops or recovers a phase */
        const int nact = (int)act.size();
        LOC_CU(cudaMemcpyAsync(dact, act.data(), sizeof(int) * nact, cudaMemcpyHostToDevice, st));
        const int tb = (nact + 127) / 128;
        loc_begin_pass<<<tb, 128, 0, st>>>(devs, dact, nact);
        /* grid.y carries the events; more than 65535 go in slices */
        for (int a0 = 0; a0 < nact; a0 += 65535) {
            const int na = nact - a0 < 65535 ? nact - a0 : 65535;
            if (ncoarse > 0)
                loc_coarse<<<dim3((unsigned)((ncoarse + kLocBlock - 1) / kLocBlock), na), kLocBlock, 0, st>>>(
                    G, dobs, dgood, devs, dact + a0, ncoarse);
        }
        loc_plan<<<tb, 128, 0, st>>>(G, devs, dact, nact, 0);
        for (int a0 = 0; a0 < nact; a0 += 65535) {
            const int na = nact - a0 < 65535 ? nact - a0 : 65535;
            loc_refine<<<dim3((unsigned)((nwin1 + kLocBlock - 1) / kLocBlock), na), kLocBlock, 0, st>>>(
                G, dobs, dgood, devs, dact + a0);
        }
        loc_plan<<<tb, 128, 0, st>>>(G, devs, dact, nact, 1);
        for (int a0 = 0; a0 < nact; a0 += 65535) {
            const int na = nact - a0 < 65535 ? nact - a0 : 65535;
            loc_refine<<<dim3((unsigned)((nwin2 + kLocBlock - 1) / kLocBlock), na), kLocBlock, 0, st>>>(
                G, dobs, dgood, devs, dact + a0);
        }
        loc_plan<<<tb, 128, 0, st>>>(G, devs, dact, nact, 2);
        loc_finish<<<tb, 128, 0, st>>>(G, dobs, dgood, devs, dact, nact, dres, dtps);
        loc_states<<<(nev + 127) / 128, 128, 0, st>>>(devs, nev, dstate);
        LOC_CU(cudaGetLastError());
        LOC_CU(cudaMemcpyAsync(state.data(), dstate, sizeof(int) * nev, cudaMemcpyDeviceToHost, st));
        LOC_CU(cudaStreamSynchronize(st));
        std::vector<int> next;
        for (int e : act)
            if (state[e] == kRedo) next.push_back(e);
        act.swap(next);
    }
    loc_results<<<(nev + 127) / 128, 128, 0, st>>>(devs, nev, dout);
    LOC_CU(cudaGetLastError());
    LOC_CU(cudaMemcpyAsync(results, dout, sizeof(fdgpu_loc_result) * nev, cudaMemcpyDeviceToHost, st));
    LOC_CU(cudaMemcpyAsync(resmin, dres, sizeof(float) * nobs, cudaMemcpyDeviceToHost, st));
    LOC_CU(cudaMemcpyAsync(tps, dtps, sizeof(float) * nobs, cudaMemcpyDeviceToHost, st));
    LOC_CU(cudaMemcpyAsync(hgood.data(), dgood, nobs, cudaMemcpyDeviceToHost, st));
    LOC_CU(cudaStreamSynchronize(st));
    for (int k = 0; k < nobs; k++) obs[k].good = hgood[k];
    return FDGPU_OK;
}
