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

/* one thread per fine node and phase; blockIdx.y = phase */
__global__ void __launch_bounds__(256) c2f_interp(const float *slow, const Axis *ax, const Axis *ay, const Axis *az,
                                                  int nx, int ny, int nz, int nxc, int nyc, int nzc, float *out)
{
    const long long nxyz = (long long)nx * ny * nz;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nxyz) return;
    const int ph = blockIdx.y;
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((long long)nx * ny));
    const Axis X = ax[i], Y = ay[j], Z = az[k];
    const float *sp = slow + (long long)ph * nxc * nyc * nzc;
    const int a = nxc * nyc * Z.cell, b = nxc * Y.cell, a2 = nxc * nyc * (Z.cell + 1), b2 = nxc * (Y.cell + 1);
    const int ci = X.cell;
    const float fx = X.f, fy = Y.f, fz = Z.f, gx = X.omf, gy = Y.omf, gz = Z.omf;
    float t = gx * gy * gz * sp[a + b + ci];
    t = t + fx * gy * gz * sp[a + b + ci + 1];
    t = t + gx * fy * gz * sp[a + b2 + ci];
    t = t + gx * gy * fz * sp[a2 + b + ci];
    t = t + fx * fy * gz * sp[a + b2 + ci + 1];
    t = t + fx * gy * fz * sp[a2 + b + ci + 1];
    t = t + gx * fy * fz * sp[a2 + b2 + ci];
    t = t + fx * fy * fz * sp[a2 + b2 + ci + 1];
    out[(long long)ph * nxyz + n] = 1.f / t;
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

#define C2F_CU(call)                                                        \
    do {                                                                    \
        const cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) { rc = fdh_ctx_fail(ctx, (int)e_, #call); goto done; } \
    } while (0)

extern "C" int fdgpu_c2f(fdgpu_ctx *ctx, const fdgpu_c2f_grid *g, const float *coarse, float *fine, void *stream)
{
    int nx, ny, nz;
    if (!ctx || !coarse || !fine) return FDGPU_EINVAL;
    int rc = fdgpu_c2f_dims(g, &nx, &ny, &nz);
    if (rc) return rc;
    if (!(g->h > 0)) return FDGPU_EINVAL;
    const int dev = fdh_ctx_device(ctx);
    if (cudaSetDevice(dev) != cudaSuccess) return FDGPU_ENODEV;
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)fdh_ctx_stream(ctx);
    bool cin = false, cout = false;
    if (kind_of(coarse, dev, &cin) || kind_of(fine, dev, &cout)) return FDGPU_EINVAL;
    const long long nxyz = (long long)nx * ny * nz;
    const int nc2 = 2 * g->nxc * g->nyc * g->nzc;
    std::vector<Axis> ax, ay, az;
    axis_table(g->nxc, g->igridx, g->x0, g->h, nx, ax);
    axis_table(g->nyc, g->igridy, g->y0, g->h, ny, ay);
    axis_table(g->nzc, g->igridz, g->z0, g->h, nz, az);
    /* one scratch allocation: coarse velocities (if on the host), slowness, axis tables, and the fine
     * output (if on the host) */
    const size_t off_v = 0, off_s = off_v + ((sizeof(float) * nc2 + 255) & ~(size_t)255);
    const size_t off_x = off_s + ((sizeof(float) * nc2 + 255) & ~(size_t)255);
    const size_t off_y = off_x + ((sizeof(Axis) * nx + 255) & ~(size_t)255);
    const size_t off_z = off_y + ((sizeof(Axis) * ny + 255) & ~(size_t)255);
    const size_t off_o = off_z + ((sizeof(Axis) * nz + 255) & ~(size_t)255);
    const size_t total = off_o + (cout ? 0 : sizeof(float) * 2 * (size_t)nxyz);
    char *mem = nullptr;
    const float *vsrc;
    float *dst;
    C2F_CU(cudaMallocAsync((void **)&mem, total, st));
    vsrc = cin ? coarse : reinterpret_cast<float *>(mem + off_v);
    dst = cout ? fine : reinterpret_cast<float *>(mem + off_o);
    if (!cin) C2F_CU(cudaMemcpyAsync(mem + off_v, coarse, sizeof(float) * nc2, cudaMemcpyHostToDevice, st));
    C2F_CU(cudaMemcpyAsync(mem + off_x, ax.data(), sizeof(Axis) * nx, cudaMemcpyHostToDevice, st));
    C2F_CU(cudaMemcpyAsync(mem + off_y, ay.data(), sizeof(Axis) * ny, cudaMemcpyHostToDevice, st));
    C2F_CU(cudaMemcpyAsync(mem + off_z, az.data(), sizeof(Axis) * nz, cudaMemcpyHostToDevice, st));
    c2f_slowness<<<(nc2 + 255) / 256 < 1024 ? (nc2 + 255) / 256 : 1024, 256, 0, st>>>(
        vsrc, reinterpret_cast<float *>(mem + off_s), nc2);
    c2f_interp<<<dim3((unsigned)((nxyz + 255) / 256), 2), 256, 0, st>>>(
        reinterpret_cast<const float *>(mem + off_s), reinterpret_cast<const Axis *>(mem + off_x),
        reinterpret_cast<const Axis *>(mem + off_y), reinterpret_cast<const Axis *>(mem + off_z), nx, ny, nz, g->nxc,
        g->nyc, g->nzc, dst);
    C2F_CU(cudaGetLastError());
    if (!cout) C2F_CU(cudaMemcpyAsync(fine, dst, sizeof(float) * 2 * (size_t)nxyz, cudaMemcpyDeviceToHost, st));
    C2F_CU(cudaStreamSynchronize(st));
done:
    if (mem) {
        cudaFreeAsync(mem, st);
        cudaStreamSynchronize(st);
    }
    return rc;
}
