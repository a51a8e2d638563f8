/*
 * fdgpu_noalloc.cu — one station solve that allocates no device memory.
 *
 * Some callers cannot let a library call cudaMalloc or cudaFree.
 *   - A serving loop that must not stall other streams: cudaFree synchronises the whole device,
 *     and cudaMalloc can.
 *   - An application whose device memory is owned by another allocator, for example a framework's
 *     caching pool that has already reserved the GPU.  A library-side cudaMalloc there either fails
 *     or escapes that allocator's accounting.
 * fdgpu_solve_noalloc serves them.  The caller passes the slowness and the output field (device
 * buffers it owns), and every other buffer the solve needs comes from one file-scope device array
 * of FDGPU_NOALLOC_SCRATCH_BYTES.  The array holds the station descriptor, its statistics, the
 * geometry tables and the face-walk scratch.  Each GPU that loads the library holds the array until
 * the process exits.
 *
 * Set-up: the first call on a device looks up the array's device address with
 * cudaGetSymbolAddress (host code cannot use the array's name as a device pointer) and caches it
 * for that device.  Make that first call before any stream capture on the device.
 *
 * Sharing: every call uses the same array, so two calls that overlap on one GPU (for example from
 * two host threads on two streams) corrupt each other's scratch.  Callers must serialise calls per
 * device.  Each call completes its work before returning.  The array keeps the last call's
 * contents: the only part that must start at zero, the statistics record, is cleared by every call,
 * and the kernels write every other part before reading it.
 */
#include "fdgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "fdgpu_layout.h"

extern "C" cudaError_t fdk_launch_geo_build(int nx, int ny, int nz, double h, double dq, double df, double z0r,
                                            const double *ysin, double *zrow, double *node, double *cell,
                                            cudaStream_t stream);
extern "C" cudaError_t fdk_launch_solve(const fd_station_dev *stations, int nst, long long max_face_pad, int cluster,
                                        cudaStream_t stream);

static __device__ __align__(256) unsigned char fd_noalloc_scratch[FDGPU_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_addr_lock;
unsigned char *g_addr[kMaxDevices];

/* device address of the scratch array on the current device, looked up once per device */
int scratch_address(int dev, unsigned char **out)
{
    if (dev < 0 || dev >= kMaxDevices) return FDGPU_EINVAL;
    std::lock_guard<std::mutex> lk(g_addr_lock);
    if (!g_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, fd_noalloc_scratch);
        if (e != cudaSuccess || !p) return FDGPU_ECUDA;
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return FDGPU_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* same checks as the allocating entry points (src/sphfd.c:533-538 for the source) */
int check(const fdgpu_station &s)
{
    if (s.nx < 2 || s.ny < 2 || s.nz < 2 || !(s.h > 0) || !(s.dq != 0) || !(s.df != 0)) return FDGPU_EINVAL;
    if (s.srctype != 1) return FDGPU_EINVAL;   /* point sources only: no starting field is supplied */
    if (s.xs < 0 || s.ys < 0 || s.zs < 0 || s.xs > s.nx - 1 || s.ys > s.ny - 1 || s.zs > s.nz - 1)
        return FDGPU_ESOURCE;
    if (s.ncube < 0 || s.ncube > 64) return FDGPU_EINVAL;
    return FDGPU_OK;
}

struct Plan {
    size_t station, stats, trig, ysin, zrow, node, cell, face, end;
    long long max_face, max_face_pad;
};

Plan plan(const fdgpu_station &s)
{
    Plan p;
    const long long mf = std::max({(long long)s.nx * s.ny, (long long)s.nx * s.nz, (long long)s.ny * s.nz});
    const int w = 2 * s.ncube + 1;
    size_t o = 0;
    p.station = o; o += align256(sizeof(fd_station_dev));
    p.stats = o;   o += align256(sizeof(fd_station_stats));
    p.trig = o;    o += align256(sizeof(double) * 4 * (size_t)w);
    p.ysin = o;    o += align256(sizeof(double) * (size_t)s.ny);
    p.zrow = o;    o += align256(sizeof(double) * FD_Z_N * (size_t)s.nz);
    p.node = o;    o += align256(sizeof(double) * FD_N_N * (size_t)s.nz * s.ny);
    p.cell = o;    o += align256(sizeof(double) * FD_C_N * (size_t)(s.nz - 1) * (s.ny - 1));
    p.face = o;    o += align256((size_t)(mf + 16) * 34);
    p.end = o;
    p.max_face = mf;
    p.max_face_pad = (mf + 15) & ~15LL;
    return p;
}

}  // namespace

extern "C" int fdgpu_solve_noalloc(const fdgpu_station *st, const float *d_slowness, long long s_sy, long long s_sz,
                                   float *d_time, fdgpu_stats *stats, void *stream)
{
    if (!st || !d_slowness || !d_time) return FDGPU_EINVAL;
    if (((uintptr_t)d_slowness & 3u) || ((uintptr_t)d_time & 3u)) return FDGPU_EINVAL;
    const fdgpu_station &s = *st;
    int rc = check(s);
    if (rc) return rc;
    const Plan p = plan(s);
    if (p.end > (size_t)FDGPU_NOALLOC_SCRATCH_BYTES) return FDGPU_ETOOBIG;   /* before any CUDA call */

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FDGPU_ENODEV;
    unsigned char *base = nullptr;
    rc = scratch_address(dev, &base);
    if (rc) return rc;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);

    /* sin(colatitude) of every row, evaluated by the C library as the reference does; staged
     * through a small stack buffer (pageable copies return once the buffer may be reused) */
    double buf[256];
    for (int y0 = 0; y0 < s.ny; y0 += 256) {
        const int n = std::min(256, s.ny - y0);
        for (int k = 0; k < n; k++) buf[k] = std::sin(s.y0 + s.dq * (double)(y0 + k));
        if (cudaMemcpyAsync(base + p.ysin + sizeof(double) * y0, buf, sizeof(double) * n, cudaMemcpyHostToDevice,
                            cs) != cudaSuccess)
            return FDGPU_ECUDA;
    }
    double *ysin = reinterpret_cast<double *>(base + p.ysin);
    double *zrow = reinterpret_cast<double *>(base + p.zrow);
    double *node = reinterpret_cast<double *>(base + p.node);
    double *cell = reinterpret_cast<double *>(base + p.cell);
    if (fdk_launch_geo_build(s.nx, s.ny, s.nz, s.h, s.dq, s.df, s.z0r, ysin, zrow, node, cell, cs) != cudaSuccess)
        return FDGPU_ECUDA;

    /* the station descriptor, as the allocating path builds it */
    fd_station_dev d;
    std::memset(&d, 0, sizeof d);
    d.g.nx = s.nx; d.g.ny = s.ny; d.g.nz = s.nz;
    d.g.h = s.h; d.g.inv_h = 1.0 / s.h; d.g.dq = s.dq; d.g.df = s.df; d.g.is_h = 1.0 / (s.h * s.h);
    d.g.zrow = zrow; d.g.ysin = ysin; d.g.node = node; d.g.cell = cell;
    d.T = d_time;
    d.S = d_slowness + (long long)s.oz * s_sz + (long long)s.oy * s_sy + s.ox;
    d.s_sy = s_sy; d.s_sz = s_sz;
    /* initial box of the point source (src/sphfd.c:766-825), walls in face order z1 z2 x2 x1 y1 y2 */
    const int nc = s.ncube;
    for (int f = 0; f < 6; f++) d.dflag[f] = 1;
    if (s.xs > nc) d.wall[3] = s.xs - (nc + 1); else { d.wall[3] = -1; d.dflag[3] = 0; }
    if (s.xs < s.nx - (nc + 1)) d.wall[2] = s.xs + (nc + 1); else { d.wall[2] = s.nx; d.dflag[2] = 0; }
    if (s.ys > nc) d.wall[4] = s.ys - (nc + 1); else { d.wall[4] = -1; d.dflag[4] = 0; }
    if (s.ys < s.ny - (nc + 1)) d.wall[5] = s.ys + (nc + 1); else { d.wall[5] = s.ny; d.dflag[5] = 0; }
    if (s.zs > nc) d.wall[0] = s.zs - (nc + 1); else { d.wall[0] = -1; d.dflag[0] = 0; }
    if (s.zs < s.nz - (nc + 1)) d.wall[1] = s.zs + (nc + 1); else { d.wall[1] = s.nz; d.dflag[1] = 0; }
    const int grow[6] = {s.kminus, s.kplus, s.iplus, s.iminus, s.jminus, s.jplus};
    for (int f = 0; f < 6; f++) d.grow[f] = grow[f];
    d.radius = nc;
    d.reverse = s.reverse;
    /* preferred restart wall (src/sphfd.c:977-1003) */
    int hp = s.headpref;
    if (hp > 0) {
        const int x1 = d.wall[3], x2 = d.wall[2], y1 = d.wall[4], y2 = d.wall[5], z1 = d.wall[0], z2 = d.wall[1];
        long long head = (long long)s.nx * s.ny * s.nz;
        if (s.nx > 5 && x2 <= head) { hp = 2; head = x2; }
        if (s.nx > 5 && (s.nx - 1 - x1) <= head) { hp = 1; head = s.nx - 1 - x1; }
        if (s.ny > 5 && y2 <= head) { hp = 4; head = y2; }
        if (s.ny > 5 && (s.ny - 1 - y1) <= head) { hp = 3; head = s.ny - 1 - y1; }
        if (s.nz > 5 && z2 <= head) { hp = 6; head = z2; }
        if (s.nz > 5 && (s.nz - 1 - z1) <= head) { hp = 5; head = s.nz - 1 - z1; }
    }
    d.headpref = hp;
    d.maxrad = s.maxrad;
    d.init_mode = 0;
    d.xs = s.xs; d.ys = s.ys; d.zs = s.zs; d.ncube = nc;
    const double fxss = s.src_geo[0], fyss = s.src_geo[1], fzss = s.src_geo[2];
    d.src_xyz[0] = fzss * std::cos(fyss);
    d.src_xyz[1] = fzss * std::sin(fyss) * std::cos(fxss);
    d.src_xyz[2] = fzss * std::sin(fyss) * std::sin(fxss);
    const int w = 2 * nc + 1;
    double trig[4 * 129];
    for (int j = 0; j < w; j++) {
        const double q = s.y0 + s.dq * (double)(s.ys - nc + j), f = s.x0 + s.df * (double)(s.xs - nc + j);
        trig[2 * j] = std::cos(q);
        trig[2 * j + 1] = std::sin(q);
        trig[2 * w + 2 * j] = std::cos(f);
        trig[2 * w + 2 * j + 1] = std::sin(f);
    }
    d.box_trig = reinterpret_cast<const double *>(base + p.trig);
    const size_t m = (size_t)p.max_face;
    unsigned char *fb = base + p.face;
    d.scr.key = reinterpret_cast<unsigned long long *>(fb);
    d.scr.rec = reinterpret_cast<float2 *>(fb + 8 * m);
    d.scr.pst = reinterpret_cast<int *>(fb + 16 * m);
    d.scr.queue = reinterpret_cast<int *>(fb + 20 * m);
    d.scr.rq = reinterpret_cast<int *>(fb + 24 * m);
    d.scr.dag = fb + 32 * m;
    d.max_face_pad = p.max_face_pad;
    d.stats = reinterpret_cast<fd_station_stats *>(base + p.stats);

    if (cudaMemcpyAsync(base + p.trig, trig, sizeof(double) * 4 * (size_t)w, cudaMemcpyHostToDevice, cs) != cudaSuccess
        || cudaMemsetAsync(base + p.stats, 0, sizeof(fd_station_stats), cs) != cudaSuccess
        || cudaMemcpyAsync(base + p.station, &d, sizeof d, cudaMemcpyHostToDevice, cs) != cudaSuccess)
        return FDGPU_ECUDA;
    if (fdk_launch_solve(reinterpret_cast<const fd_station_dev *>(base + p.station), 1, p.max_face_pad, 1, cs)
        != cudaSuccess)
        return FDGPU_ECUDA;
    fd_station_stats hs;
    if (cudaMemcpyAsync(&hs, base + p.stats, sizeof hs, cudaMemcpyDeviceToHost, cs) != cudaSuccess
        || cudaStreamSynchronize(cs) != cudaSuccess)
        return FDGPU_ECUDA;
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        stats->status = hs.status ? FDGPU_ESCHED : FDGPU_OK;
        stats->sweeps = hs.sweeps;
        stats->node_updates = hs.node_updates;
        stats->faces = hs.faces;
        stats->rounds = hs.rounds;
        stats->deferred = hs.deferred;
        for (int j = 0; j < 5; j++) stats->stencils[j] = hs.stencils[j];
        for (int j = 0; j < 8; j++) stats->restart_wall[j] = hs.restart_wall[j];
        stats->t_start_ns = hs.t_start_ns;
        stats->t_end_ns = hs.t_end_ns;
        stats->pipelined_sweeps = hs.pipelined_sweeps;
        stats->detail = hs.status;
    }
    return hs.status ? FDGPU_ESCHED : FDGPU_OK;
}
