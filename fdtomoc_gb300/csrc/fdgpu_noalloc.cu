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
 * for that device.  The call cannot be captured in a CUDA graph: it waits for its solve and copies
 * the statistics to the host.  Its first call on a device may also load the module, which a stream
 * capture in global mode elsewhere in the process would reject, so make that first call while no
 * stream is capturing.  The cached
 * address belongs to the device's primary context: after cudaDeviceReset it is stale, and the
 * entry point must not be called again in that process.
 *
 * Device: the call works on the calling thread's current device; a stream of another device is
 * refused with FDGPU_EINVAL before any work is queued.
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
#include "fdgpu_station.h"

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

using fdh::align256;

/* the checks of the allocating entry points, and point sources only (no starting field is
 * supplied) */
int check(const fdgpu_station &s)
{
    const int rc = fdh::check_station(s);
    if (rc) return rc;
    return s.srctype == 1 ? FDGPU_OK : FDGPU_EINVAL;
}

struct Plan {
    size_t station, stats, trig, ysin, face, end;
    long long max_face, max_face_pad;
};

Plan plan(const fdgpu_station &s)
{
    Plan p;
    size_t o = 0;
    p.station = o; o += align256(sizeof(fd_station_dev));
    p.stats = o;   o += align256(sizeof(fd_station_stats));
    p.trig = o;    o += align256(sizeof(double) * (size_t)fdh::box_trig_count(s));
    p.ysin = o;    o += fdh::geo_bytes(s.ny, s.nz);   /* ysin | zrow | node | cell */
    p.face = o;    o += fdh::face_bytes(s);
    p.end = o;
    p.max_face = fdh::max_face(s);
    p.max_face_pad = (p.max_face + 15) & ~15LL;
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
    if (stream) {
        int sdev = -1;
        if (cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev) != cudaSuccess || sdev != dev)
            return FDGPU_EINVAL;
    }
    unsigned char *base = nullptr;
    rc = scratch_address(dev, &base);
    if (rc) return rc;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);

    /* sin(colatitude) of every row, evaluated by the C library as the reference does; staged
     * through a small stack buffer (pageable copies return once the buffer may be reused) */
    const fdh::GeoPtrs g = fdh::geo_carve(reinterpret_cast<char *>(base + p.ysin), s.ny, s.nz);
    double buf[256];
    for (int y0 = 0; y0 < s.ny; y0 += 256) {
        const int n = std::min(256, s.ny - y0);
        for (int k = 0; k < n; k++) buf[k] = std::sin(fdh::qc(s, y0 + k));
        if (cudaMemcpyAsync(g.ysin + y0, buf, sizeof(double) * n, cudaMemcpyHostToDevice, cs) != cudaSuccess)
            return FDGPU_ECUDA;
    }
    if (fdk_launch_geo_build(s.nx, s.ny, s.nz, s.h, s.dq, s.df, s.z0r, g.ysin, g.zrow, g.node, g.cell, cs)
        != cudaSuccess)
        return FDGPU_ECUDA;

    /* the station descriptor, as the allocating path builds it, without sweep-graph arrays */
    fd_station_dev d;
    fdh::fill_station(d, s, g, d_time, d_slowness, s_sy, s_sz, 0, reinterpret_cast<char *>(base + p.face), nullptr,
                      reinterpret_cast<const double *>(base + p.trig),
                      reinterpret_cast<fd_station_stats *>(base + p.stats));
    const int w = 2 * s.ncube + 1;
    double trig[4 * 129];
    fdh::box_trig(s, trig);

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
    if (stats) fdh::copy_stats(*stats, hs);
    return hs.status ? FDGPU_ESCHED : FDGPU_OK;
}
