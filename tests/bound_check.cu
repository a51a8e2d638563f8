/*
 * bound_check.cu — test harness: the single-precision lower bound of a 2-D stencil value
 * (lower_2d) against the exact FP64 value the solver computes (eval_2d and the causality
 * selection), on random and near-degenerate inputs over a real geometry.
 *
 * Built by tests/test_gpu_bound.py with nvcc into a temporary directory; it includes the kernel
 * translation unit so that it uses the same tables, descriptors and evaluators as the solver.
 */
#include "../fdtomoc_gb300/csrc/fdgpu_kernels.cu"

#include <cmath>
#include <vector>

namespace {
using namespace fdk;

__device__ __forceinline__ unsigned long long mix(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ float unif(unsigned long long &s)
{
    s = mix(s);
    return (float)((s >> 40) & 0xffffff) * (1.0f / 16777216.0f);
}

/* per sample: face F, 2-D trial K, a node (z,y) away from the edges, 18 times and slownesses */
__global__ void bound_kernel(fd_geo_dev g, unsigned long long seed, long long n, unsigned long long *out)
{
    unsigned long long viol = 0, tight = 0, usable = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long s = seed ^ (unsigned long long)i * 0x2545f4914f6cdd1dull;
        const int F = (int)(unif(s) * 6.f) % 6;
        const int K = TK_2D0 + (int)(unif(s) * 8.f) % 8;
        const fdk::TrialDesc &d = fdk::c_desc[F * FDN_NTRIAL + K];
        const int z = 1 + (int)(unif(s) * (float)(g.nz - 3));
        const int y = 1 + (int)(unif(s) * (float)(g.ny - 3));
        float t18[NB_PAD], s18[NB_PAD];
        /* a base time, a gradient of random size and direction, jitter; sometimes near-equal times */
        const float base = unif(s) < 0.1f ? unif(s) * 0.05f : unif(s) * 80.f;
        const float slow = 0.1f + 0.25f * unif(s);
        const float gsz = slow * (unif(s) < 0.5f ? 1.f : 2.5f * unif(s));
        const float gu = gsz * (2.f * unif(s) - 1.f), gv = gsz * (2.f * unif(s) - 1.f), gw = gsz * (2.f * unif(s) - 1.f);
        const float jit = unif(s) < 0.3f ? 0.f : 0.05f * unif(s) * slow;
        for (int nb = 0; nb < NB_N; nb++) {
            const int w = nb / 9, dv = (nb / 3) % 3 - 1, du = nb % 3 - 1;
            t18[nb] = fmaxf(0.f, base + 0.5f * (gu * du + gv * dv + gw * w) + jit * (2.f * unif(s) - 1.f));
            s18[nb] = slow * (1.f + 0.05f * (2.f * unif(s) - 1.f));
        }
        double x1, x2;
        fdk::eval_2d(d, t18, s18, g, z, y, x1, x2);
        const float fl = fmaxf(fmaxf(t18[d.slot[1]], t18[d.slot[2]]), t18[d.slot[3]]);
        double v;
        if (x1 != x1) {
            v = 1.e11;
        } else {
            const double f = fdk::f2d(fl);
            const bool bad1 = fdk::lt(x1, f), bad2 = fdk::lt(x2, f);
            v = bad1 ? (bad2 ? 1.e11 : x2) : (bad2 ? x1 : (fdk::lt(x2, x1) ? x2 : x1));
        }
        const float lo = fdk::lower_2d(d, t18, s18, g, z, y, fl);
        if (lo == lo && (double)lo > v) viol++;
        if (v < 1.e11 && lo == lo) {
            usable++;
            if ((double)lo >= v * (1.0 - 1e-4)) tight++;
        }
    }
    atomicAdd(&out[0], viol);
    atomicAdd(&out[1], tight);
    atomicAdd(&out[2], usable);
}

}  // namespace

/* 0 on success; counts[0] bound violations, [1] accepted values bounded within 1e-4, [2] accepted values */
extern "C" int bound_check(int nx, int ny, int nz, double h, double dq, double df, double z0r, double y0, long long n,
                           unsigned long long seed, unsigned long long *counts)
{
    std::vector<double> ys(ny);
    for (int y = 0; y < ny; y++) ys[y] = std::sin(y0 + dq * (double)y);
    double *ysin = nullptr, *zrow = nullptr, *node = nullptr, *cell = nullptr;
    unsigned long long *out = nullptr;
    if (cudaMalloc(&ysin, sizeof(double) * ny) || cudaMalloc(&zrow, sizeof(double) * FD_Z_N * nz)
        || cudaMalloc(&node, sizeof(double) * FD_N_N * (size_t)nz * ny)
        || cudaMalloc(&cell, sizeof(double) * FD_C_N * (size_t)(nz - 1) * (ny - 1))
        || cudaMalloc(&out, 3 * sizeof(unsigned long long)))
        return 1;
    cudaMemcpy(ysin, ys.data(), sizeof(double) * ny, cudaMemcpyHostToDevice);
    cudaMemset(out, 0, 3 * sizeof(unsigned long long));
    fdk_launch_geo_build(nx, ny, nz, h, dq, df, z0r, ysin, zrow, node, cell, 0);
    fd_geo_dev g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.h = h; g.inv_h = 1.0 / h; g.dq = dq; g.df = df; g.is_h = 1.0 / (h * h);
    g.zrow = zrow; g.ysin = ysin; g.node = node; g.cell = cell;
    bound_kernel<<<152 * 4, 256>>>(g, seed, n, out);
    const cudaError_t e = cudaMemcpy(counts, out, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(ysin); cudaFree(zrow); cudaFree(node); cudaFree(cell); cudaFree(out);
    return e == cudaSuccess ? 0 : 2;
}
