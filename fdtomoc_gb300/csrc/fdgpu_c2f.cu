/*
 * fdgpu_c2f.cu — coarse-to-fine model interpolation on the device: FDtomoC's c2f (reference
 * src/c2f.c), which turns the inversion's coarse P and S velocity nodes into the fine model sphfd
 * reads.  Results are bit-identical to the reference's.
 *
 * The reference places the coarse nodes at float coordinates accumulated step by step (:265-287),
 * turns the coarse velocities into slowness (:545-548), and for every fine node (x, y, z) = (x0 + i h,
 * ...) rounded to float scans for the coarse cell that holds it and interpolates the slowness
 * trilinearly in float (find_vel, :673-727), writing back 1/slowness (:561-572).
 *
 * GPU form: the cell and fractional offset along each axis depend only on that axis's fine index, so
 * the host forms them once per axis with the reference's float operations (nx + ny + nz entries), a
 * first kernel forms the coarse slowness, and the main kernel gives each fine node one thread that
 * combines the three axes' entries into the eight weights, in the reference's order, and writes the
 * velocity.  The slowness 1/v of the reference is computed in double and stored as float; float
 * division gives the same value (a double has more than twice a float's precision plus two bits, so
 * rounding the double quotient to float is the correctly rounded float quotient).  The main kernel
 * writes 8 bytes per fine node (P and S) and reads a coarse model that stays in L2: it is bound by
 * HBM writes.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "fdgpu.h"
#include "fdgpu_device.h"

namespace {

struct Axis {
    int cell;    /* coarse cell index */
    float f;     /* (v - g[cell]) / (g[cell+1] - g[cell]) */
    float omf;   /* 1 - f */
};

__global__ void c2f_slowness(const float *v, float *s, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s[i] = 1.f / v[i];
}

/* Rows (phase, z, y) of the fine model go to warps, grid-stride; a warp's lanes take x = lane,
 * lane + 32, ..., so each store instruction writes 128 contiguous bytes.  The grid is one resident
 * wave of blocks: the work is 2 nz ny rows of nx nodes, far too many short blocks otherwise. */
constexpr int kC2fBlock = 256;

__global__ void __launch_bounds__(kC2fBlock) c2f_interp(const float *__restrict__ slow, const Axis *__restrict__ ax,
                                                        const Axis *__restrict__ ay, const Axis *__restrict__ az,
                                                        int nx, int ny, int nz, int nxc, int nyc, int nzc,
                                                        float *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const long long rows = 2ll * nz * ny;
    const long long nwarps = (long long)gridDim.x * (kC2fBlock / 32);
    const long long ncoarse = (long long)nxc * nyc * nzc;
    for (long long r = (long long)blockIdx.x * (kC2fBlock / 32) + (threadIdx.x >> 5); r < rows; r += nwarps) {
        const int j = (int)(r % ny);
        const int pk = (int)(r / ny);
        const int ph = pk / nz, k = pk - ph * nz;
        const Axis Y = ay[j], Z = az[k];
        const float *sp = slow + ph * ncoarse;
        const int a = nxc * nyc * Z.cell, b = nxc * Y.cell, a2 = nxc * nyc * (Z.cell + 1), b2 = nxc * (Y.cell + 1);
        const float fy = Y.f, fz = Z.f, gy = Y.omf, gz = Z.omf;
        float *row = out + r * nx;
        for (int i = lane; i < nx; i += 32) {
            const Axis X = ax[i];
            const int ci = X.cell;
            const float fx = X.f, gx = X.omf;
            float t = gx * gy * gz * sp[a + b + ci];
            t = t + fx * gy * gz * sp[a + b + ci + 1];
            t = t + gx * fy * gz * sp[a + b2 + ci];
            t = t + gx * gy * fz * sp[a2 + b + ci];
            t = t + fx * fy * gz * sp[a + b2 + ci + 1];
            t = t + fx * gy * fz * sp[a2 + b + ci + 1];
            t = t + gx * fy * fz * sp[a2 + b2 + ci];
            t = t + fx * fy * fz * sp[a2 + b2 + ci + 1];
            row[i] = 1.f / t;
        }
    }
}

/* the per-axis entries: node coordinates accumulated as the reference does, fine positions rounded
 * to float, the first node past each position less one (kept inside), and the offset */
void axis_table(int nc, const int *ig, double o, double h, int nfine, std::vector<Axis> &out)
{
    std::vector<float> g(nc);
    g[0] = (float)o;
    for (int i = 1; i < nc; i++) g[i] = (float)(g[i - 1] + h * ig[i - 1]);
    out.resize(nfine);
    for (int i = 0; i < nfine; i++) {
        const float v = (float)(o + i * h);
        int c;
        for (c = 1; c < nc; c++)
            if (g[c] > v) break;
        if (c == nc) c--;
        c--;
        const float f = (v - g[c]) / (g[c + 1] - g[c]);
        out[i].cell = c;
        out[i].f = f;
        out[i].omf = 1.f - f;
    }
}

int kind_of(const void *p, int device, bool *on_device)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        *on_device = false;
        return FDGPU_OK;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        if (a.device != device) return FDGPU_EINVAL;
        *on_device = true;
    } else {
        *on_device = false;
    }
    return FDGPU_OK;
}

}  // namespace

extern "C" int fdh_ctx_device(const fdgpu_ctx *ctx);
extern "C" void *fdh_ctx_stream(const fdgpu_ctx *ctx);
extern "C" int fdh_ctx_fail(fdgpu_ctx *ctx, int cuda_error, const char *what);

extern "C" int fdgpu_c2f_dims(const fdgpu_c2f_grid *g, int *nx, int *ny, int *nz)
{
    if (!g || !nx || !ny || !nz || g->nxc < 2 || g->nyc < 2 || g->nzc < 2 || !g->igridx || !g->igridy || !g->igridz)
        return FDGPU_EINVAL;
    long long x = 1, y = 1, z = 1;
    for (int i = 1; i < g->nxc; i++) { if (g->igridx[i - 1] < 1) return FDGPU_EINVAL; x += g->igridx[i - 1]; }
    for (int i = 1; i < g->nyc; i++) { if (g->igridy[i - 1] < 1) return FDGPU_EINVAL; y += g->igridy[i - 1]; }
    for (int i = 1; i < g->nzc; i++) { if (g->igridz[i - 1] < 1) return FDGPU_EINVAL; z += g->igridz[i - 1]; }
    if (x * y * z >= (1ll << 31) || (long long)g->nxc * g->nyc * g->nzc >= (1ll << 30)) return FDGPU_EINVAL;
    *nx = (int)x;
    *ny = (int)y;
    *nz = (int)z;
    return FDGPU_OK;
}

struct fdgpu_c2f_plan {
    fdgpu_ctx *ctx = nullptr;
    int device = 0;
    int nx = 0, ny = 0, nz = 0, nxc = 0, nyc = 0, nzc = 0;
    int sms = 0, per_sm = 1;   /* SMs, and interpolation blocks resident per SM */
    char *mem = nullptr;   /* slowness (2 x coarse), axis tables */
    float *slow = nullptr;
    Axis *ax = nullptr, *ay = nullptr, *az = nullptr;
};

extern "C" int fdgpu_c2f_plan_create(fdgpu_ctx *ctx, const fdgpu_c2f_grid *g, fdgpu_c2f_plan **out)
{
    if (!ctx || !out) return FDGPU_EINVAL;
    *out = nullptr;
    int nx, ny, nz;
    int rc = fdgpu_c2f_dims(g, &nx, &ny, &nz);
    if (rc) return rc;
    if (!(g->h > 0)) return FDGPU_EINVAL;
    const int dev = fdh_ctx_device(ctx);
    FdDeviceScope dev_(dev);
    if (dev_.err) return FDGPU_ENODEV;
    std::vector<Axis> ax, ay, az;
    axis_table(g->nxc, g->igridx, g->x0, g->h, nx, ax);
    axis_table(g->nyc, g->igridy, g->y0, g->h, ny, ay);
    axis_table(g->nzc, g->igridz, g->z0, g->h, nz, az);
    auto *p = new (std::nothrow) fdgpu_c2f_plan;
    if (!p) return FDGPU_ENOMEM;
    p->ctx = ctx;
    p->device = dev;
    p->nx = nx; p->ny = ny; p->nz = nz;
    p->nxc = g->nxc; p->nyc = g->nyc; p->nzc = g->nzc;
    if (cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || p->sms < 1) p->sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p->per_sm, c2f_interp, kC2fBlock, 0) != cudaSuccess
        || p->per_sm < 1)
        p->per_sm = 1;
    const size_t nc2 = 2 * (size_t)g->nxc * g->nyc * g->nzc;
    const size_t o_x = (sizeof(float) * nc2 + 255) & ~(size_t)255;
    const size_t o_y = o_x + ((sizeof(Axis) * nx + 255) & ~(size_t)255);
    const size_t o_z = o_y + ((sizeof(Axis) * ny + 255) & ~(size_t)255);
    const size_t total = o_z + sizeof(Axis) * nz;
    cudaError_t e = cudaMalloc((void **)&p->mem, total);
    if (!e) e = cudaMemcpy(p->mem + o_x, ax.data(), sizeof(Axis) * nx, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(p->mem + o_y, ay.data(), sizeof(Axis) * ny, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(p->mem + o_z, az.data(), sizeof(Axis) * nz, cudaMemcpyHostToDevice);
    if (e) {
        rc = fdh_ctx_fail(ctx, (int)e, "c2f plan");
        if (p->mem) cudaFree(p->mem);
        delete p;
        return rc;
    }
    p->slow = reinterpret_cast<float *>(p->mem);
    p->ax = reinterpret_cast<Axis *>(p->mem + o_x);
    p->ay = reinterpret_cast<Axis *>(p->mem + o_y);
    p->az = reinterpret_cast<Axis *>(p->mem + o_z);
    *out = p;
    return FDGPU_OK;
}

extern "C" int fdgpu_c2f_run(fdgpu_c2f_plan *p, const float *d_coarse, float *d_fine, void *stream)
{
    if (!p || !d_coarse || !d_fine) return FDGPU_EINVAL;
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)fdh_ctx_stream(p->ctx);
    FdDeviceScope dev_(p->device);
    if (dev_.err) return FDGPU_ENODEV;
    const int nc2 = 2 * p->nxc * p->nyc * p->nzc;
    c2f_slowness<<<(nc2 + 255) / 256 < 1024 ? (nc2 + 255) / 256 : 1024, 256, 0, st>>>(d_coarse, p->slow, nc2);
    const long long rows = 2ll * p->nz * p->ny;
    const long long want = (rows + kC2fBlock / 32 - 1) / (kC2fBlock / 32);
    const long long resident = (long long)p->sms * p->per_sm;   /* one wave: rows go to resident warps */
    const int blocks = (int)(want < resident ? want : resident);
    c2f_interp<<<blocks, kC2fBlock, 0, st>>>(p->slow, p->ax, p->ay, p->az, p->nx, p->ny, p->nz, p->nxc, p->nyc,
                                              p->nzc, d_fine);
    const cudaError_t e = cudaGetLastError();
    return e ? fdh_ctx_fail(p->ctx, (int)e, "c2f launch") : FDGPU_OK;
}

extern "C" void fdgpu_c2f_plan_destroy(fdgpu_c2f_plan *p)
{
    if (!p) return;
    FdDeviceScope dev_(p->device);
    if (p->mem) {
        cudaDeviceSynchronize();
        cudaFree(p->mem);
    }
    delete p;
}

extern "C" int fdgpu_c2f(fdgpu_ctx *ctx, const fdgpu_c2f_grid *g, const float *coarse, float *fine, void *stream)
{
    if (!ctx || !coarse || !fine) return FDGPU_EINVAL;
    fdgpu_c2f_plan *p = nullptr;
    int rc = fdgpu_c2f_plan_create(ctx, g, &p);
    if (rc) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)fdh_ctx_stream(ctx);
    bool cin = false, cout = false;
    const long long nxyz = (long long)p->nx * p->ny * p->nz;
    const size_t nc2 = 2 * (size_t)p->nxc * p->nyc * p->nzc;
    float *dc = nullptr, *df = nullptr;
    cudaError_t e = cudaSuccess;
    if (kind_of(coarse, p->device, &cin) || kind_of(fine, p->device, &cout)) {
        fdgpu_c2f_plan_destroy(p);
        return FDGPU_EINVAL;
    }
    if (!cin) {
        e = cudaMallocAsync((void **)&dc, sizeof(float) * nc2, st);
        if (!e) e = cudaMemcpyAsync(dc, coarse, sizeof(float) * nc2, cudaMemcpyHostToDevice, st);
    }
    if (!e && !cout) e = cudaMallocAsync((void **)&df, sizeof(float) * 2 * (size_t)nxyz, st);
    if (!e) rc = fdgpu_c2f_run(p, cin ? coarse : dc, cout ? fine : df, st);
    if (!e && !rc && !cout) e = cudaMemcpyAsync(fine, df, sizeof(float) * 2 * (size_t)nxyz, cudaMemcpyDeviceToHost, st);
    if (dc) cudaFreeAsync(dc, st);
    if (df) cudaFreeAsync(df, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (!e) e = e2;
    if (e && !rc) rc = fdh_ctx_fail(ctx, (int)e, "c2f");
    fdgpu_c2f_plan_destroy(p);
    return rc;
}
