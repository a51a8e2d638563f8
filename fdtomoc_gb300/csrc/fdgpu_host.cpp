/*
 * fdgpu_host.cpp — host runtime of libfdgpu: set-up of station solves, device memory, launches,
 * and the drop-in sphfd() file front end.
 *
 * Host arithmetic that feeds the GPU (geocentric conversion, source placement, sin/cos of grid
 * colatitudes and longitudes) uses the C library exactly as the reference does and is compiled
 * with -ffp-contract=off, so the doubles handed to the kernels are the reference's.
 */
#include "fdgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "fdgpu_device.h"
#include "fdgpu_layout.h"
#include "fdgpu_station.h"

extern "C" cudaError_t fdk_launch_geo_build(int nx, int ny, int nz, double h, double dq, double df, double z0r,
                                            const double *ysin, double *zrow, double *node, double *cell,
                                            cudaStream_t stream);
extern "C" cudaError_t fdk_launch_solve(const fd_station_dev *stations, int nst, long long max_face_pad, int cluster,
                                        cudaStream_t stream);
extern "C" cudaError_t fdk_launch_v2s(const float *v, float *s, long long n, cudaStream_t stream);
extern "C" cudaError_t fdk_solve_config(int nst, long long max_face_pad, int cluster, long long *bytes_out,
                                        int *csz_out);
extern "C" cudaError_t fdk_solve_launch(const fd_station_dev *stations, int nst, long long bytes, int cs,
                                        cudaStream_t stream);
extern "C" cudaError_t fdk_probe_fp64(double *scratch, int blocks, int threads, int iters, float *ms, cudaStream_t s);

namespace {

/* literal constants of the reference (src/sphfd.c:128-136) */
constexpr double kPi = 3.141592654;
constexpr double kHalfPi = 1.570796327;
constexpr double kRearth = 6371.0;
constexpr double kDegrad = kPi / 180.0;

/* ---- device buffers ---------------------------------------------------------------------- */

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

/* geometry tables of one grid geometry (see fdgpu_layout.h) */
struct Geo {
    DevBuf ysin, zrow, node, cell;
    int ny = 0, nz = 0;
};

using GeoKey = std::tuple<int, int, uint64_t, uint64_t, uint64_t, uint64_t, uint64_t>;

/* Device buffers of one prepared batch: scratch, station records, statistics, box trig tables. */
struct BatchBufs {
    DevBuf scratch, stations, stats, trig;
};

uint64_t bits(double x)
{
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
}

}  // namespace

struct fdgpu_ctx {
    int device = 0;
    int cluster = 0;   /* CTAs per station: 0 automatic */
    long long wait_cycles = 0, walk_cycles = 0;   /* bounds of the solver's waits, 0: built-in */
    /* measured solve time (ns) of each station this context has solved, keyed by the station's
     * record (fdgpu_station bytes): the launch-order table */
    std::map<std::string, long long> solve_ns;
    cudaStream_t stream = nullptr;
    std::map<GeoKey, std::unique_ptr<Geo>> geos;
    BatchBufs batch;   /* the buffers of fdgpu_solve_device, kept for the next call */
    DevBuf model, fields;
    std::string err;
};

namespace {

int cuda_fail(fdgpu_ctx *ctx, cudaError_t e, const char *what)
{
    if (ctx) ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
    return FDGPU_ECUDA;
}

#define FD_CU(ctx, call)                                                \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);      \
    } while (0)

/* WGS84 geodetic -> geocentric (src/sphfd.c:5836-5893) */
double glath(double hlat, double depth_km, double *radius_km)
{
    const double ap = 6378137.0;
    const double esq = 0.00669437978616733379;
    const double hm = -depth_km * 1000.0;
    const double sinxl = std::sin(hlat);
    const double anu = ap / std::sqrt(1.0 - esq * sinxl * sinxl);
    const double xp = (anu + hm) * std::cos(hlat);
    const double zp = ((1.0 - esq) * anu + hm) * sinxl;
    *radius_km = std::sqrt(xp * xp + zp * zp) / 1000.0;
    return std::atan2(zp, xp);
}

using fdh::qc;
using fdh::fc;
double rc(const fdgpu_station &s, int z) { return s.z0r - s.h * (double)z; }

Geo *geometry(fdgpu_ctx *ctx, const fdgpu_station &s, int *status)
{
    const GeoKey key{s.ny, s.nz, bits(s.h), bits(s.dq), bits(s.df), bits(s.z0r), bits(s.y0)};
    auto it = ctx->geos.find(key);
    if (it != ctx->geos.end()) return it->second.get();
    auto g = std::make_unique<Geo>();
    std::vector<double> ys(s.ny);
    fdh::ysin_table(s, ys.data());
    cudaError_t e;
    if ((e = g->ysin.ensure(sizeof(double) * s.ny)) || (e = g->zrow.ensure(sizeof(double) * FD_Z_N * s.nz))
        || (e = g->node.ensure(sizeof(double) * FD_N_N * (size_t)s.nz * s.ny))
        || (e = g->cell.ensure(sizeof(double) * FD_C_N * (size_t)std::max(1, s.nz - 1) * std::max(1, s.ny - 1)))) {
        *status = cuda_fail(ctx, e, "geometry alloc");
        return nullptr;
    }
    if ((e = cudaMemcpyAsync(g->ysin.p, ys.data(), sizeof(double) * s.ny, cudaMemcpyHostToDevice, ctx->stream))
        || (e = fdk_launch_geo_build(s.nx, s.ny, s.nz, s.h, s.dq, s.df, s.z0r, g->ysin.as<double>(),
                                     g->zrow.as<double>(), g->node.as<double>(), g->cell.as<double>(), ctx->stream))
        || (e = cudaStreamSynchronize(ctx->stream))) {
        *status = cuda_fail(ctx, e, "geometry build");
        return nullptr;
    }
    g->ny = s.ny;
    g->nz = s.nz;
    Geo *raw = g.get();
    ctx->geos.emplace(key, std::move(g));
    return raw;
}

using fdh::check_station;
using fdh::max_face;

}  // namespace

/* ------------------------------------------------------------------------------------------ */

extern "C" int fdgpu_create(int device, fdgpu_ctx **out)
{
    if (!out) return FDGPU_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) return FDGPU_ENODEV;
    FdDeviceScope dev_(device);
    if (dev_.err) return FDGPU_ENODEV;
    auto *ctx = new (std::nothrow) fdgpu_ctx;
    if (!ctx) return FDGPU_ENOMEM;
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return FDGPU_ECUDA;
    }
    *out = ctx;
    return FDGPU_OK;
}

extern "C" void fdgpu_destroy(fdgpu_ctx *ctx)
{
    if (!ctx) return;
    FdDeviceScope dev_(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStream_t s = ctx->stream;
    delete ctx;   /* frees every device buffer it holds */
    cudaStreamDestroy(s);
}

extern "C" const char *fdgpu_strerror(int s)
{
    switch (s) {
    case FDGPU_OK: return "ok";
    case FDGPU_EINVAL: return "invalid argument";
    case FDGPU_ENOMEM: return "out of memory";
    case FDGPU_ECUDA: return "CUDA error";
    case FDGPU_EIO: return "file I/O error";
    case FDGPU_EPAR: return "missing or invalid par parameter";
    case FDGPU_ESOURCE: return "source outside the grid";
    case FDGPU_ESCHED: return "a schedule check of the solve failed (fdgpu_stats.detail says which)";
    case FDGPU_ENODEV: return "no CUDA device";
    case FDGPU_ETOOBIG: return "problem exceeds the memory the entry point may use";
    case FDGPU_ETIMEDOUT: return "time limit passed before the wait ended";
    default: return "unknown status";
    }
}

extern "C" const char *fdgpu_last_error(const fdgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

extern "C" int fdgpu_probe_fp64(fdgpu_ctx *ctx, double *gops)
{
    if (!ctx || !gops) return FDGPU_EINVAL;
    FdDeviceScope dev_(ctx->device);
    FD_CU(ctx, dev_.err);
    int sms = 0;
    FD_CU(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int blocks = sms * 8, threads = 256, iters = 2048;
    DevBuf buf;
    FD_CU(ctx, buf.ensure(sizeof(double) * (size_t)blocks * threads));
    float ms = 0.f;
    FD_CU(ctx, fdk_probe_fp64(buf.as<double>(), blocks, threads, iters, &ms, ctx->stream));
    *gops = (double)blocks * threads * iters * 8 / (ms * 1e-3) / 1e9;   /* FP64 instructions per second */
    return FDGPU_OK;
}

/* context access for the library's other translation units */
extern "C" int fdh_ctx_device(const fdgpu_ctx *ctx) { return ctx->device; }
extern "C" void *fdh_ctx_stream(const fdgpu_ctx *ctx) { return (void *)ctx->stream; }
extern "C" int fdh_ctx_fail(fdgpu_ctx *ctx, int cuda_error, const char *what)
{
    return cuda_fail(ctx, (cudaError_t)cuda_error, what);
}

extern "C" int fdgpu_velocity_to_slowness(fdgpu_ctx *ctx, const float *v, float *s, long long n, void *stream)
{
    if (!ctx || (!v && n) || (!s && n) || n < 0) return FDGPU_EINVAL;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    FdDeviceScope dev_(ctx->device);
    FD_CU(ctx, dev_.err);
    FD_CU(ctx, fdk_launch_v2s(v, s, n, st));
    return FDGPU_OK;
}

extern "C" int fdgpu_set_cluster(fdgpu_ctx *ctx, int ctas_per_station)
{
    if (!ctx || ctas_per_station < 0 || ctas_per_station > 8 || (ctas_per_station & (ctas_per_station - 1)))
        return FDGPU_EINVAL;
    ctx->cluster = ctas_per_station;
    return FDGPU_OK;
}

/* the launch-order table on disk: "FDGPUORD", a record count, then per station its key length,
 * key and solve time (ns), all little-endian as written by this machine */
extern "C" int fdgpu_order_save(const fdgpu_ctx *ctx, const char *path)
{
    if (!ctx || !path) return FDGPU_EINVAL;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return FDGPU_EIO;
    bool ok = std::fwrite("FDGPUORD", 1, 8, fp) == 8;
    const long long n = (long long)ctx->solve_ns.size();
    ok = ok && std::fwrite(&n, sizeof n, 1, fp) == 1;
    for (const auto &kv : ctx->solve_ns) {
        const int len = (int)kv.first.size();
        ok = ok && std::fwrite(&len, sizeof len, 1, fp) == 1 && std::fwrite(kv.first.data(), 1, len, fp) == (size_t)len
             && std::fwrite(&kv.second, sizeof kv.second, 1, fp) == 1;
    }
    ok = std::fclose(fp) == 0 && ok;
    return ok ? FDGPU_OK : FDGPU_EIO;
}

extern "C" int fdgpu_order_load(fdgpu_ctx *ctx, const char *path)
{
    if (!ctx || !path) return FDGPU_EINVAL;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return FDGPU_EIO;
    char magic[8];
    long long n = 0;
    int rc = FDGPU_OK;
    if (std::fread(magic, 1, 8, fp) != 8 || std::memcmp(magic, "FDGPUORD", 8) != 0 || std::fread(&n, sizeof n, 1, fp) != 1
        || n < 0 || n > (1ll << 24))
        rc = FDGPU_EIO;
    std::map<std::string, long long> got;
    for (long long k = 0; rc == FDGPU_OK && k < n; k++) {
        int len = 0;
        long long ns = 0;
        if (std::fread(&len, sizeof len, 1, fp) != 1 || len <= 0 || len > 4096) { rc = FDGPU_EIO; break; }
        std::string key((size_t)len, '\0');
        if (std::fread(&key[0], 1, (size_t)len, fp) != (size_t)len || std::fread(&ns, sizeof ns, 1, fp) != 1) {
            rc = FDGPU_EIO;
            break;
        }
        got[key] = ns;
    }
    std::fclose(fp);
    if (rc == FDGPU_OK)
        for (auto &kv : got) ctx->solve_ns[kv.first] = kv.second;
    return rc;
}

extern "C" int fdgpu_set_wait_limits(fdgpu_ctx *ctx, long long wait_cycles, long long walk_cycles)
{
    if (!ctx || wait_cycles < 0 || walk_cycles < 0) return FDGPU_EINVAL;
    ctx->wait_cycles = wait_cycles;
    ctx->walk_cycles = walk_cycles;
    return FDGPU_OK;
}

namespace {

/* a station's key in the launch-order table: its fields' bytes, member by member (the struct's
 * padding is not part of it) */
std::string station_key(const fdgpu_station &s)
{
    std::string k;
    auto put = [&k](const void *p, size_t n) { k.append(reinterpret_cast<const char *>(p), n); };
    const int iv[] = {s.nx, s.ny, s.nz, s.srctype, s.xs, s.ys, s.zs, s.ncube, s.reverse, s.headpref, s.maxrad,
                      s.kminus, s.kplus, s.iplus, s.iminus, s.jminus, s.jplus, s.srcwall, s.ox, s.oy, s.oz};
    const double dv[] = {s.h, s.dq, s.df, s.x0, s.y0, s.z0r, s.src_geo[0], s.src_geo[1], s.src_geo[2]};
    put(iv, sizeof iv);
    put(dv, sizeof dv);
    return k;
}

/* Check the stations and lay out their records in bufs (queued on cs): everything a launch of
 * fd_solve reads, except the fields and the slowness it points at.  *max_pad: the largest face. */
int prepare_batch(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *slowness, long long s_sy,
                  long long s_sz, float *const *d_times, int times_initialised, BatchBufs &bufs, cudaStream_t cs,
                  long long *max_pad_out)
{
    if (((uintptr_t)slowness & 3u) != 0) return FDGPU_EINVAL;
    for (int k = 0; k < n; k++) {
        const int c = check_station(st[k]);
        if (c) return c;
        if (!d_times[k] || ((uintptr_t)d_times[k] & 3u) != 0) return FDGPU_EINVAL;
        if (st[k].srctype != 1 && !times_initialised) return FDGPU_EINVAL;
    }
    /* scratch and per-station records: per station, face scratch, then the sweep-graph arrays */
    std::vector<size_t> off(n + 1, 0);
    for (int k = 0; k < n; k++) off[k + 1] = off[k] + fdh::face_bytes(st[k]) + fdh::graph_bytes(st[k]);
    FD_CU(ctx, bufs.scratch.ensure(off[n]));
    FD_CU(ctx, bufs.stations.ensure(sizeof(fd_station_dev) * n));
    FD_CU(ctx, bufs.stats.ensure(sizeof(fd_station_stats) * n));
    int maxt = 0;
    for (int k = 0; k < n; k++) maxt = std::max(maxt, fdh::box_trig_count(st[k]));
    FD_CU(ctx, bufs.trig.ensure(sizeof(double) * (size_t)maxt * n + 8));
    std::vector<fd_station_dev> hs(n);
    long long max_pad = 16;
    std::vector<double> trig((size_t)maxt * n, 0.0);
    for (int k = 0; k < n; k++) {
        const fdgpu_station &s = st[k];
        int status = 0;
        Geo *g = geometry(ctx, s, &status);
        if (!g) return status;
        const fdh::GeoPtrs gp{g->ysin.as<double>(), g->zrow.as<double>(), g->node.as<double>(), g->cell.as<double>()};
        fdh::box_trig(s, trig.data() + (size_t)maxt * k);
        char *base = bufs.scratch.as<char>() + off[k];
        fdh::fill_station(hs[k], s, gp, d_times[k], slowness, s_sy, s_sz,
                          (s.srctype == 1 && !times_initialised) ? 0 : 1, base, base + fdh::face_bytes(s),
                          bufs.trig.as<double>() + (size_t)maxt * k, bufs.stats.as<fd_station_stats>() + k);
        hs[k].wait_cycles = ctx->wait_cycles;
        hs[k].walk_cycles = ctx->walk_cycles;
        max_pad = std::max(max_pad, hs[k].max_face_pad);
    }
    /* Launch order: largest grids first.  CTA i solves record i, and CTAs beyond the resident ones
     * start as earlier ones finish, so a batch of uneven windows ends sooner when the long solves
     * start first (longest-processing-time order).  Each record keeps its own statistics slot, so
     * the caller's order is unaffected. */
    std::vector<long long> known(n, -1);
    bool all_known = true;
    for (int k = 0; k < n; k++) {
        auto it = ctx->solve_ns.find(station_key(st[k]));
        if (it != ctx->solve_ns.end()) known[k] = it->second; else all_known = false;
    }
    if (all_known) {
        /* every station has a measured solve time in this context: longest first */
        const fd_station_stats *sbase = bufs.stats.as<fd_station_stats>();
        std::stable_sort(hs.begin(), hs.end(), [&](const fd_station_dev &a, const fd_station_dev &b) {
            return known[a.stats - sbase] > known[b.stats - sbase];
        });
    } else {
        std::stable_sort(hs.begin(), hs.end(), [](const fd_station_dev &a, const fd_station_dev &b) {
            return (long long)a.g.nx * a.g.ny * a.g.nz > (long long)b.g.nx * b.g.ny * b.g.nz;
        });
    }
    FD_CU(ctx, cudaMemcpyAsync(bufs.trig.p, trig.data(), sizeof(double) * trig.size(), cudaMemcpyHostToDevice, cs));
    FD_CU(ctx, cudaMemcpyAsync(bufs.stations.p, hs.data(), sizeof(fd_station_dev) * n, cudaMemcpyHostToDevice, cs));
    /* the host vectors go away on return: the copies must have left them */
    FD_CU(ctx, cudaStreamSynchronize(cs));
    *max_pad_out = max_pad;
    return FDGPU_OK;
}

/* a station's measured solve time into the context's table: the mean of the last value and the new one,
 * so that one run's noise (a solve's time depends on what runs beside it) moves the order less */
void record_time(fdgpu_ctx *ctx, const fdgpu_station &s, long long ns)
{
    auto it = ctx->solve_ns.find(station_key(s));
    if (it == ctx->solve_ns.end()) ctx->solve_ns[station_key(s)] = ns;
    else it->second = (it->second + ns) / 2;
}

/* which run a set of statistics records comes from: the latest start among them (the GPU's global
 * timer), different for every run */
long long run_id(const std::vector<fd_station_stats> &hst)
{
    long long id = 0;
    for (const auto &x : hst) id = std::max(id, (long long)x.t_start_ns);
    return id;
}

/* Clean solves' times of one run into the context's launch-order table (st: the stations, in the
 * caller's order), once per run: *recorded (if given) holds the run last recorded. */
void record_run(fdgpu_ctx *ctx, const std::vector<fd_station_stats> &hst, const fdgpu_station *st,
                long long *recorded)
{
    const long long id = run_id(hst);
    if (!st || (recorded && *recorded == id)) return;
    if (recorded) *recorded = id;
    for (size_t k = 0; k < hst.size(); k++)
        if (!hst[k].status && hst[k].t_end_ns > hst[k].t_start_ns)
            record_time(ctx, st[k], hst[k].t_end_ns - hst[k].t_start_ns);
}

/* The public statistics of n solves from their device records (queued on cs, then waited for);
 * their times go into the launch-order table (see record_run). */
int read_stats(fdgpu_ctx *ctx, const DevBuf &stats_buf, int n, fdgpu_stats *stats, cudaStream_t cs,
               const fdgpu_station *st, long long *recorded)
{
    std::vector<fd_station_stats> hst(n);
    FD_CU(ctx, cudaMemcpyAsync(hst.data(), stats_buf.p, sizeof(fd_station_stats) * n, cudaMemcpyDeviceToHost, cs));
    FD_CU(ctx, cudaStreamSynchronize(cs));
    int rc = FDGPU_OK;
    for (int k = 0; k < n; k++) {
        if (stats) fdh::copy_stats(stats[k], hst[k]);
        if (hst[k].status && rc == FDGPU_OK) rc = FDGPU_ESCHED;
    }
    record_run(ctx, hst, st, recorded);
    return rc;
}

}  // namespace

struct fdgpu_batch {
    fdgpu_ctx *ctx = nullptr;
    int n = 0;
    std::vector<fdgpu_station> stations;   /* the caller's stations, in its order */
    long long max_pad = 16;
    long long smem_bytes = 0;   /* launch shape, fixed at creation */
    int csz = 1;
    long long recorded = -1;    /* the run whose times the order table holds (see record_run) */
    BatchBufs bufs;
};

extern "C" int fdgpu_solve_device(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *slowness,
                                  long long s_sy, long long s_sz, float *const *d_times, int times_initialised,
                                  fdgpu_stats *stats, void *stream)
{
    if (!ctx || n < 0 || (n > 0 && (!st || !slowness || !d_times))) return FDGPU_EINVAL;
    if (n == 0) return FDGPU_OK;
    FdDeviceScope dev_(ctx->device);
    FD_CU(ctx, dev_.err);
    cudaStream_t cs = stream ? (cudaStream_t)stream : ctx->stream;
    BatchBufs &bufs = ctx->batch;
    long long max_pad = 16;
    int rc = prepare_batch(ctx, n, st, slowness, s_sy, s_sz, d_times, times_initialised, bufs, cs, &max_pad);
    if (rc == FDGPU_OK) {
        const cudaError_t e = fdk_launch_solve(bufs.stations.as<fd_station_dev>(), n, max_pad, ctx->cluster, cs);
        rc = e ? cuda_fail(ctx, e, "fdk_launch_solve") : read_stats(ctx, bufs.stats, n, stats, cs, st, nullptr);
    }
    return rc;
}

extern "C" int fdgpu_batch_create(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *slowness,
                                  long long s_sy, long long s_sz, float *const *d_times, int times_initialised,
                                  fdgpu_batch **out)
{
    if (!out) return FDGPU_EINVAL;
    *out = nullptr;
    if (!ctx || n < 1 || !st || !slowness || !d_times) return FDGPU_EINVAL;
    FdDeviceScope dev_(ctx->device);
    FD_CU(ctx, dev_.err);
    auto *b = new (std::nothrow) fdgpu_batch;
    if (!b) return FDGPU_ENOMEM;
    b->ctx = ctx;
    b->n = n;
    b->stations.assign(st, st + n);
    int rc = prepare_batch(ctx, n, st, slowness, s_sy, s_sz, d_times, times_initialised, b->bufs, ctx->stream,
                           &b->max_pad);
    if (!rc) {
        const cudaError_t e = fdk_solve_config(n, b->max_pad, ctx->cluster, &b->smem_bytes, &b->csz);
        if (e) rc = cuda_fail(ctx, e, "fdk_solve_config");
    }
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return FDGPU_OK;
}

extern "C" int fdgpu_batch_run(fdgpu_batch *b, void *stream)
{
    if (!b) return FDGPU_EINVAL;
    fdgpu_ctx *ctx = b->ctx;
    cudaStream_t cs = stream ? (cudaStream_t)stream : ctx->stream;
    FdDeviceScope dev_(ctx->device);   /* switches nothing when the device is already current */
    FD_CU(ctx, dev_.err);
    FD_CU(ctx, fdk_solve_launch(b->bufs.stations.as<fd_station_dev>(), b->n, b->smem_bytes, b->csz, cs));
    return FDGPU_OK;
}

extern "C" int fdgpu_batch_stats(fdgpu_batch *b, fdgpu_stats *stats, void *stream)
{
    if (!b) return FDGPU_EINVAL;
    fdgpu_ctx *ctx = b->ctx;
    return read_stats(ctx, b->bufs.stats, b->n, stats, stream ? (cudaStream_t)stream : ctx->stream,
                      b->stations.data(), &b->recorded);
}

namespace {

/* the batch's records as they sit on the device, in launch order, with the caller's index of each
 * (its statistics slot) */
int batch_records(fdgpu_batch *b, std::vector<fd_station_dev> &rec, std::vector<int> &idx, cudaStream_t cs)
{
    fdgpu_ctx *ctx = b->ctx;
    rec.resize(b->n);
    idx.resize(b->n);
    FD_CU(ctx, cudaMemcpyAsync(rec.data(), b->bufs.stations.p, sizeof(fd_station_dev) * b->n, cudaMemcpyDeviceToHost, cs));
    FD_CU(ctx, cudaStreamSynchronize(cs));
    const fd_station_stats *base = b->bufs.stats.as<fd_station_stats>();
    for (int k = 0; k < b->n; k++) idx[k] = (int)(rec[k].stats - base);
    return FDGPU_OK;
}

}  // namespace

extern "C" int fdgpu_batch_order(fdgpu_batch *b, int *order, void *stream)
{
    if (!b || !order) return FDGPU_EINVAL;
    std::vector<fd_station_dev> rec;
    std::vector<int> idx;
    const int rc = batch_records(b, rec, idx, stream ? (cudaStream_t)stream : b->ctx->stream);
    if (rc) return rc;
    for (int k = 0; k < b->n; k++) order[k] = idx[k];
    return FDGPU_OK;
}

extern "C" int fdgpu_batch_set_order(fdgpu_batch *b, const int *order, void *stream)
{
    if (!b || !order) return FDGPU_EINVAL;
    fdgpu_ctx *ctx = b->ctx;
    cudaStream_t cs = stream ? (cudaStream_t)stream : ctx->stream;
    std::vector<char> seen(b->n, 0);
    for (int k = 0; k < b->n; k++) {
        if (order[k] < 0 || order[k] >= b->n || seen[order[k]]) return FDGPU_EINVAL;
        seen[order[k]] = 1;
    }
    std::vector<fd_station_dev> rec, out(b->n);
    std::vector<int> idx;
    int rc = batch_records(b, rec, idx, cs);
    if (rc) return rc;
    std::vector<int> at(b->n);
    for (int k = 0; k < b->n; k++) at[idx[k]] = k;
    for (int k = 0; k < b->n; k++) out[k] = rec[at[order[k]]];
    FD_CU(ctx, cudaMemcpyAsync(b->bufs.stations.p, out.data(), sizeof(fd_station_dev) * b->n, cudaMemcpyHostToDevice, cs));
    FD_CU(ctx, cudaStreamSynchronize(cs));
    return FDGPU_OK;
}

extern "C" int fdgpu_batch_tune_order(fdgpu_batch *b, void *stream)
{
    if (!b) return FDGPU_EINVAL;
    fdgpu_ctx *ctx = b->ctx;
    cudaStream_t cs = stream ? (cudaStream_t)stream : ctx->stream;
    std::vector<fd_station_stats> hst(b->n);
    FD_CU(ctx, cudaMemcpyAsync(hst.data(), b->bufs.stats.p, sizeof(fd_station_stats) * b->n, cudaMemcpyDeviceToHost, cs));
    FD_CU(ctx, cudaStreamSynchronize(cs));
    for (int k = 0; k < b->n; k++)
        if (hst[k].t_end_ns <= hst[k].t_start_ns || hst[k].status) return FDGPU_EINVAL;   /* no clean run yet */
    /* the last run's times into the context's table (blended with earlier ones, unless
     * fdgpu_batch_stats already put them there), then longest first by the table; equal times keep
     * the current order */
    record_run(ctx, hst, b->stations.data(), &b->recorded);
    std::vector<long long> t(b->n);
    for (int k = 0; k < b->n; k++) t[k] = ctx->solve_ns[station_key(b->stations[k])];
    std::vector<fd_station_dev> rec;
    std::vector<int> idx;
    int rc = batch_records(b, rec, idx, cs);
    if (rc) return rc;
    std::vector<int> order(idx);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return t[a] > t[c]; });
    return fdgpu_batch_set_order(b, order.data(), stream);
}

extern "C" void fdgpu_batch_destroy(fdgpu_batch *b)
{
    if (!b) return;
    FdDeviceScope dev_(b->ctx->device);
    delete b;   /* frees its device buffers */
}

extern "C" int fdgpu_solve_host(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *velocity, int mnx,
                                int mny, int mnz, float *const *times, const float *const *init_times,
                                fdgpu_stats *stats)
{
    if (!ctx || n < 0 || (n > 0 && (!st || !velocity || !times)) || mnx < 1 || mny < 1 || mnz < 1) return FDGPU_EINVAL;
    if (n == 0) return FDGPU_OK;
    FdDeviceScope dev_(ctx->device);
    FD_CU(ctx, dev_.err);
    for (int k = 0; k < n; k++) {
        const fdgpu_station &s = st[k];
        if (s.ox < 0 || s.oy < 0 || s.oz < 0 || s.ox + s.nx > mnx || s.oy + s.ny > mny || s.oz + s.nz > mnz)
            return FDGPU_EINVAL;
        if (!times[k]) return FDGPU_EINVAL;
    }
    const long long nm = (long long)mnx * mny * mnz;
    /* each station's field starts on a 256-byte boundary of the shared field buffer */
    std::vector<size_t> off(n + 1, 0), len(n);
    for (int k = 0; k < n; k++) {
        len[k] = (size_t)st[k].nx * st[k].ny * st[k].nz;
        off[k + 1] = off[k] + ((len[k] + 63) & ~(size_t)63);
    }
    FD_CU(ctx, ctx->model.ensure(sizeof(float) * (size_t)nm));
    FD_CU(ctx, ctx->fields.ensure(sizeof(float) * off[n]));
    FD_CU(ctx, cudaMemcpyAsync(ctx->model.p, velocity, sizeof(float) * nm, cudaMemcpyHostToDevice, ctx->stream));
    FD_CU(ctx, fdk_launch_v2s(ctx->model.as<float>(), ctx->model.as<float>(), nm, ctx->stream));
    std::vector<float *> dt(n);
    bool any_init = false;
    for (int k = 0; k < n; k++) {
        dt[k] = ctx->fields.as<float>() + off[k];
        if (init_times && init_times[k]) {
            any_init = true;
            FD_CU(ctx, cudaMemcpyAsync(dt[k], init_times[k], sizeof(float) * len[k], cudaMemcpyHostToDevice,
                                       ctx->stream));
        }
    }
    if (any_init) {
        /* stations without a supplied field cannot be mixed into an initialised batch */
        for (int k = 0; k < n; k++)
            if (!init_times[k]) return FDGPU_EINVAL;
    }
    const int rc = fdgpu_solve_device(ctx, n, st, ctx->model.as<float>(), mnx, (long long)mnx * mny, dt.data(),
                                      any_init ? 1 : 0, stats, ctx->stream);
    if (rc) return rc;
    for (int k = 0; k < n; k++)
        FD_CU(ctx, cudaMemcpyAsync(times[k], dt[k], sizeof(float) * len[k], cudaMemcpyDeviceToHost, ctx->stream));
    FD_CU(ctx, cudaStreamSynchronize(ctx->stream));
    return FDGPU_OK;
}

/* ------------------------------------------------------------------------------------------ */
/* getpar front end (src/sphfd.c:383-552, getpar at :6267-6766)                                */

namespace {

struct ParList {
    std::vector<std::pair<std::string, std::string>> e;
    int add_file(const std::string &fname, int level);
    void add(const std::string &n, const std::string &v) { e.emplace_back(n, v); }
    int add_arg(const char *tok, int level)
    {
        const char *eq = std::strchr(tok, '=');
        if (!eq) return 0;
        std::string name(tok, eq - tok), val(eq + 1);
        add(name, val);
        if (name == "par") return add_file(val, level + 1);
        return 0;
    }
    const std::string *get(const char *name) const
    {
        for (auto it = e.rbegin(); it != e.rend(); ++it)   /* the last definition wins */
            if (it->first == name) return &it->second;
        return nullptr;
    }
    bool geti(const char *n, int *v) const { auto s = get(n); if (!s) return false; *v = std::atoi(s->c_str()); return true; }
    bool getd(const char *n, double *v) const { auto s = get(n); if (!s) return false; *v = std::atof(s->c_str()); return true; }
    bool getf(const char *n, float *v) const { auto s = get(n); if (!s) return false; *v = (float)std::atof(s->c_str()); return true; }
};

int ParList::add_file(const std::string &fname, int level)
{
    if (level > 20) return FDGPU_EPAR;
    FILE *fp = std::fopen(fname.c_str(), "r");
    if (!fp) return FDGPU_EIO;
    char line[2048];
    while (std::fgets(line, sizeof line, fp)) {
        const char *pl = line;
        for (;;) {
            while (*pl == ' ' || *pl == '\t') pl++;
            if (*pl == '\0' || *pl == '\n' || *pl == '#') break;
            std::string name, val;
            while (*pl != '=' && *pl != '\0' && *pl != ' ' && *pl != '\t' && *pl != '\n') name += *pl++;
            if (*pl == '=') pl++;
            char t1 = ' ', t2 = '\t';
            if (*pl == '"' || *pl == '\'') t1 = t2 = *pl++;
            while (*pl != t1 && *pl != t2 && *pl != '\0' && *pl != '\n') val += *pl++;
            if (*pl == '"' || *pl == '\'') pl++;
            add(name, val);
            if (name == "par") {
                const int rc = add_file(val, level + 1);
                if (rc) { std::fclose(fp); return rc; }
            }
        }
    }
    std::fclose(fp);
    return 0;
}

/* everything sphfd() reads from its par file */
struct ParSetup {
    fdgpu_station st;
    std::string velfile, timefile, boxfile, wallfile, oldtfile;
    int fill = 0, parse = 1, swab = 0, floatsrc = 1;
    double x0_save = 0, y0_save = 0, z0 = 0;
};

int setup_from_par(int ac, char **av, ParSetup &ps)
{
    ParList P;
    for (int i = 1; i < ac; i++) {
        const int rc = P.add_arg(av[i], 0);
        if (rc) return rc;
    }
    fdgpu_station &s = ps.st;
    std::memset(&s, 0, sizeof s);
    int nx, ny, nz;
    double h, dq = 0, df = 0, y0 = 90, x0 = 0, z0 = 0;
    if (!P.geti("nx", &nx) || !P.geti("ny", &ny) || !P.geti("nz", &nz) || !P.getd("h", &h)) return FDGPU_EPAR;
    int iplus = 1, iminus = 1, jplus = 1, jminus = 1, kplus = 1, kminus = 1, srctype = 1, floatsrc = 1, ncube = 2;
    int reverse = 1, headpref = 6, parse = 1, fill = 0, swab = 0;
    int invh = 0, invq = 0, invf = 0, invx0 = 0, invy0 = 0, invz0 = 0;
    float maxoff = -1.f;
    P.getd("dq", &dq); P.getd("df", &df);
    P.geti("iminus", &iminus); P.geti("iplus", &iplus); P.geti("jminus", &jminus); P.geti("jplus", &jplus);
    P.geti("kminus", &kminus); P.geti("kplus", &kplus); P.geti("floatsrc", &floatsrc); P.geti("srctype", &srctype);
    P.geti("NCUBE", &ncube); P.geti("reverse", &reverse); P.geti("headpref", &headpref); P.getf("maxoff", &maxoff);
    P.getd("x0", &x0); P.getd("y0", &y0); P.getd("z0", &z0); P.geti("parse", &parse); P.geti("fill", &fill);
    P.geti("invh", &invh); P.geti("invf", &invf); P.geti("invq", &invq);
    P.geti("invx0", &invx0); P.geti("invy0", &invy0); P.geti("invz0", &invz0); P.geti("swab", &swab);
    if (invh == 1) h = 1. / h;
    if (invq == 1 && dq != 0) dq = 1. / dq;
    if (invf == 1 && df != 0) df = 1. / df;
    if (invx0 == 1 && x0 != 0) x0 = 1. / x0;
    if (invy0 == 1 && y0 != 0) y0 = 1. / y0;
    if (invz0 == 1 && z0 != 0) z0 = 1. / z0;
    ps.x0_save = x0;
    ps.y0_save = y0;
    ps.z0 = z0;
    /* src/sphfd.c:432-455 */
    y0 *= kDegrad;
    y0 = kHalfPi - glath(y0, z0, &s.z0r);
    x0 *= kDegrad;
    dq *= kDegrad;
    df *= kDegrad;
    if (dq == 0) dq = h / kRearth;
    if (df == 0) df = std::fabs(h / (kRearth * std::sin(y0)));
    s.nx = nx; s.ny = ny; s.nz = nz; s.h = h; s.dq = dq; s.df = df; s.x0 = x0; s.y0 = y0;
    s.srctype = srctype;
    if (srctype == 1) {
        if (floatsrc == 0) {
            if (!P.geti("xs", &s.xs) || !P.geti("ys", &s.ys) || !P.geti("zs", &s.zs)) return FDGPU_EPAR;
            s.src_geo[0] = fc(s, s.xs);
            s.src_geo[1] = qc(s, s.ys);
            s.src_geo[2] = rc(s, s.zs);
        } else {
            double fxs, fys, fzs, rcent;
            if (!P.getd("fxs", &fxs) || !P.getd("fys", &fys) || !P.getd("fzs", &fzs)) return FDGPU_EPAR;
            fxs *= kDegrad;
            fys *= kDegrad;
            fys = kHalfPi - glath(fys, fzs, &rcent);
            s.src_geo[0] = fxs; s.src_geo[1] = fys; s.src_geo[2] = rcent;
            fxs = (fxs - x0) / df;
            fys = (fys - y0) / dq;
            fzs = (s.z0r - rcent) / h;
            s.xs = (int)(fxs + 0.5);
            s.ys = (int)(fys + 0.5);
            s.zs = (int)(fzs + 0.5);
        }
    } else if (srctype == 2) {
        if (!P.geti("srcwall", &s.srcwall)) return FDGPU_EPAR;
        auto w = P.get("wallfile");
        if (!w) return FDGPU_EPAR;
        ps.wallfile = *w;
    } else if (srctype == 3) {
        if (!P.geti("srcwall", &s.srcwall)) return FDGPU_EPAR;
        auto w = P.get("oldtfile");
        if (!w) return FDGPU_EPAR;
        ps.oldtfile = *w;
    } else {
        return FDGPU_EPAR;
    }
    if (fill == 1) {
        auto b = P.get("boxfile");
        if (!b) return FDGPU_EPAR;
        ps.boxfile = *b;
    }
    auto tf = P.get("timefile");
    auto vf = P.get("velfile");
    if (!tf || !vf) return FDGPU_EPAR;
    ps.timefile = *tf;
    ps.velfile = *vf;
    s.ncube = ncube;
    s.reverse = reverse;
    s.headpref = headpref;
    s.maxrad = (maxoff > 0.) ? (int)(maxoff / h + 1) : 99999999;
    s.kminus = kminus; s.kplus = kplus; s.iplus = iplus; s.iminus = iminus; s.jminus = jminus; s.jplus = jplus;
    ps.fill = fill; ps.parse = parse; ps.swab = swab; ps.floatsrc = floatsrc;
    if (srctype == 1 && (s.xs < 0 || s.ys < 0 || s.zs < 0 || s.xs > nx - 1 || s.ys > ny - 1 || s.zs > nz - 1))
        return FDGPU_ESOURCE;
    return FDGPU_OK;
}

/* 232-byte header (include/common/vhead.h:4-11) */
struct VHead {
    char header[120];
    double fxs, fys, fzs, clat, clon, cz, x0, y0, z0, dx, dy, dz;
    float az;
    int nx, ny, nz;
};
static_assert(sizeof(VHead) == 232, "vhead layout");

void swap4(void *p) { auto *b = (unsigned char *)p; std::swap(b[0], b[3]); std::swap(b[1], b[2]); }
void swap8(void *p) { auto *b = (unsigned char *)p; for (int i = 0; i < 4; i++) std::swap(b[i], b[7 - i]); }
void swap_head(VHead &h, bool src)
{
    swap4(&h.az); swap4(&h.nx); swap4(&h.ny); swap4(&h.nz);
    swap8(&h.clat); swap8(&h.clon); swap8(&h.cz); swap8(&h.x0); swap8(&h.y0); swap8(&h.z0);
    swap8(&h.dx); swap8(&h.dy); swap8(&h.dz);
    if (src) { swap8(&h.fxs); swap8(&h.fys); swap8(&h.fzs); }
}

/* velocity file (src/sphfd.c:611-686): header if it starts with "HEAD", else the data start at 0 */
int read_velocity(const ParSetup &ps, VHead &hin, std::vector<float> &v)
{
    const fdgpu_station &s = ps.st;
    const size_t n = (size_t)s.nx * s.ny * s.nz;
    FILE *fp = std::fopen(ps.velfile.c_str(), "rb");
    if (!fp) return FDGPU_EIO;
    std::memset(&hin, 0, sizeof hin);
    if (std::fread(&hin, 1, 232, fp) != 232 || std::strncmp(hin.header, "HEAD", 4) != 0) {
        /* no header: the reference builds one (it overruns the 120-byte text there; this keeps
         * the same leading text, NUL-terminated) and rereads the file from its start */
        hin.x0 = ps.x0_save; hin.y0 = ps.y0_save; hin.z0 = ps.z0;
        hin.dx = s.df; hin.dy = s.dq; hin.dz = s.h;
        hin.nx = s.nx; hin.ny = s.ny; hin.nz = s.nz; hin.az = 0.f;
        hin.clat = ps.y0_save; hin.clon = ps.x0_save; hin.cz = ps.z0;
        std::memset(hin.header, ' ', 120);
        std::memcpy(hin.header, "HEADFINESPHRVPMDNOFLsphfd", 25);
        hin.header[25] = 0;
        std::rewind(fp);
    }
    v.resize(n);
    const size_t got = std::fread(v.data(), 4, n, fp);
    std::fclose(fp);
    if (got != n) return FDGPU_EIO;
    if (ps.swab == 1 || ps.swab == 3) {
        swap_head(hin, false);
        for (auto &x : v) swap4(&x);
    }
    return FDGPU_OK;
}

/* initial field for srctype 2/3 and fill=1 (src/sphfd.c:697-722, 826-971) */
int initial_field(const ParSetup &ps, const std::vector<float> &vel, std::vector<float> &t)
{
    const fdgpu_station &s = ps.st;
    const long long nx = s.nx, ny = s.ny, nz = s.nz, nxy = nx * ny, nxyz = nxy * nz;
    t.assign((size_t)nxyz, 1.0e10f);
    if (s.srctype == 1) {
        /* constant-slowness box, then (fill=1) the boxfile values over it */
        const float s000 = 1 / vel[(size_t)(nxy * s.zs + nx * s.ys + s.xs)];
        const double fxss = s.src_geo[0], fyss = s.src_geo[1], fzss = s.src_geo[2];
        const double x1p = fzss * std::cos(fyss), y1p = fzss * std::sin(fyss) * std::cos(fxss),
                     z1p = fzss * std::sin(fyss) * std::sin(fxss);
        const int nc = s.ncube;
        for (int zz = s.zs - nc; zz <= s.zs + nc; zz++)
            for (int yy = s.ys - nc; yy <= s.ys + nc; yy++)
                for (int xx = s.xs - nc; xx <= s.xs + nc; xx++) {
                    if (zz < 0 || zz >= nz || yy < 0 || yy >= ny || xx < 0 || xx >= nx) continue;
                    const double fx1 = fc(s, xx), qy1 = qc(s, yy), rz1 = rc(s, zz);
                    const double x2p = rz1 * std::cos(qy1), y2p = rz1 * std::sin(qy1) * std::cos(fx1),
                                 z2p = rz1 * std::sin(qy1) * std::sin(fx1);
                    t[(size_t)(nxy * zz + nx * yy + xx)] = (float)(s000 * std::sqrt((x1p - x2p) * (x1p - x2p)
                        + (y1p - y2p) * (y1p - y2p) + (z1p - z2p) * (z1p - z2p)));
                }
        if (ps.fill == 1) {
            const int bx1 = std::max(0, s.xs - nc), bx2 = std::min(s.nx - 1, s.xs + nc);
            const int by1 = std::max(0, s.ys - nc), by2 = std::min(s.ny - 1, s.ys + nc);
            const int bz1 = std::max(0, s.zs - nc), bz2 = std::min(s.nz - 1, s.zs + nc);
            const size_t nbox = (size_t)(bx2 - bx1 + 1) * (by2 - by1 + 1) * (bz2 - bz1 + 1);
            std::vector<float> box(nbox);
            FILE *fp = std::fopen(ps.boxfile.c_str(), "rb");
            if (!fp) return FDGPU_EIO;
            VHead hb;
            const bool ok = std::fread(&hb, 1, 232, fp) == 232 && std::fread(box.data(), 4, nbox, fp) == nbox;
            std::fclose(fp);
            if (!ok) return FDGPU_EIO;
            size_t ii = 0;
            for (int zz = bz1; zz <= bz2; zz++)
                for (int yy = by1; yy <= by2; yy++)
                    for (int xx = bx1; xx <= bx2; xx++) t[(size_t)(nxy * zz + nx * yy + xx)] = box[ii++];
        }
    } else if (s.srctype == 2) {
        const long long nwall = (nx <= ny && nx <= nz) ? ny * nz : (ny <= nx && ny <= nz) ? nx * nz : nxy;
        std::vector<float> wall((size_t)nwall);
        FILE *fp = std::fopen(ps.wallfile.c_str(), "rb");
        if (!fp) return FDGPU_EIO;
        for (int w = 0; w < 6; w++) {
            if (std::fread(wall.data(), 4, (size_t)nwall, fp) != (size_t)nwall) break;
            if (!(wall[0] > -1.e-20)) continue;
            size_t ii = 0;
            if (w < 2) { const long long x = w == 0 ? 0 : nx - 1; for (long long k = 0; k < nz; k++) for (long long j = 0; j < ny; j++) t[(size_t)(nxy * k + nx * j + x)] = wall[ii++]; }
            else if (w < 4) { const long long y = w == 2 ? 0 : ny - 1; for (long long k = 0; k < nz; k++) for (long long i = 0; i < nx; i++) t[(size_t)(nxy * k + nx * y + i)] = wall[ii++]; }
            else { const long long z = w == 4 ? 0 : nz - 1; for (long long j = 0; j < ny; j++) for (long long i = 0; i < nx; i++) t[(size_t)(nxy * z + nx * j + i)] = wall[ii++]; }
        }
        std::fclose(fp);
    } else {
        FILE *fp = std::fopen(ps.oldtfile.c_str(), "rb");
        if (!fp) return FDGPU_EIO;
        const size_t got = std::fread(t.data(), 4, (size_t)nxyz, fp);   /* the reference reads the raw file */
        (void)got;
        std::fclose(fp);
    }
    return FDGPU_OK;
}

/* travel-time file (src/sphfd.c:5702-5803) */
int write_times(const ParSetup &ps, const VHead &hin, std::vector<float> &t, const char *outdir)
{
    const fdgpu_station &s = ps.st;
    const long long nx = s.nx, ny = s.ny, nz = s.nz, nxy = nx * ny;
    int nxp = s.nx, nyp = s.ny, nzp = s.nz;
    size_t nout = (size_t)(nxy * nz);
    const int parse = ps.parse;
    if (parse > 1) {
        size_t ii = 0;
        nzp = 0;
        for (long long k = 0; k < nz; k += parse) {
            nzp++;
            for (long long j = 0; j < ny; j += parse)
                for (long long i = 0; i < nx; i += parse) t[ii++] = t[(size_t)(i + j * nx + k * nxy)];
        }
        nxp = 0;
        nyp = 0;
        for (long long j = 0; j < ny; j += parse) nyp++;
        for (long long i = 0; i < nx; i += parse) nxp++;
        nout = ii;
    }
    VHead ho;
    std::memset(&ho, 0, sizeof ho);
    /* text: leading string of the input (up to 120 bytes, NUL padded), "PTIM" at 12..15, then
     * bytes 16..119 copied string by string (strncpy + strcpy sequence of :5744-5767) */
    const size_t l = strnlen(hin.header, 120);
    std::memcpy(ho.header, hin.header, l);
    ho.header[12] = 'P'; ho.header[13] = 'T'; ho.header[14] = 'I'; ho.header[15] = 'M';
    for (int i = 16; i < 120; i++) {
        const size_t li = strnlen(hin.header + i, 120 - i);
        std::memcpy(ho.header + i, hin.header + i, li);
        if (i + li < 120) ho.header[i + li] = 0;
    }
    ho.clat = hin.clat; ho.clon = hin.clon; ho.cz = hin.cz; ho.az = hin.az;
    ho.x0 = hin.x0; ho.y0 = hin.y0; ho.z0 = hin.z0;
    ho.dx = hin.dx * parse; ho.dy = hin.dy * parse; ho.dz = hin.dz * parse;
    ho.nx = nxp; ho.ny = nyp; ho.nz = nzp;
    ho.fxs = s.src_geo[0]; ho.fys = s.src_geo[1]; ho.fzs = s.src_geo[2];
    if (s.srctype != 1) { ho.fxs = 0; ho.fys = 0; ho.fzs = 0; }
    if (ps.swab == 2 || ps.swab == 3) {
        swap_head(ho, true);
        for (size_t i = 0; i < nout; i++) swap4(&t[i]);
    }
    const std::string path = std::string(outdir) + "/" + ps.timefile;
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) return FDGPU_EIO;
    const bool ok = std::fwrite(&ho, 1, 232, fp) == 232 && std::fwrite(t.data(), 4, nout, fp) == nout;
    std::fclose(fp);
    return ok ? FDGPU_OK : FDGPU_EIO;
}

/* Contexts of the drop-in entry points' worker threads, one per (device, position in the device
 * list), created on first use.  Like the per-thread ones below they are deliberately never
 * destroyed, so that no CUDA call runs during process teardown.  Calls that use several devices
 * must not overlap: their workers share these contexts. */
fdgpu_ctx *slot_ctx(int device, int slot, int *status)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, fdgpu_ctx *> ctxs;
    std::lock_guard<std::mutex> lk(mu);
    fdgpu_ctx *&ctx = ctxs[{device, slot}];
    if (!ctx) {
        *status = fdgpu_create(device, &ctx);
        if (*status) ctx = nullptr;
    }
    return ctx;
}

/* the calling thread's own context on a device (the single-device drop-in: concurrent callers on
 * different threads do not share one) */
fdgpu_ctx *thread_ctx(int device, int *status)
{
    thread_local std::map<int, fdgpu_ctx *> ctxs;
    fdgpu_ctx *&ctx = ctxs[device];
    if (!ctx) {
        *status = fdgpu_create(device, &ctx);
        if (*status) ctx = nullptr;
    }
    return ctx;
}

/* the calling thread's current device (the one a caller selected with cudaSetDevice; 0 if none) */
int current_device()
{
    int d = 0;
    return cudaGetDevice(&d) == cudaSuccess ? d : 0;
}

/* solve a set of parsed par files and write their time files.  Every input (par file, velocity
 * file, starting field) is read and checked before the GPU is touched: the context is created on
 * the first solve, so a run whose inputs are all bad returns their statuses without a device. */
void run_setups(std::vector<ParSetup> &ps, std::vector<int> &stat, const char *output_path,
                const std::vector<int> &devices)
{
    const int n = (int)ps.size();
    /* group stations by velocity file and grid so each model is read and uploaded once */
    std::map<std::tuple<std::string, int, int, int, int>, std::vector<int>> groups;
    for (int k = 0; k < n; k++)
        if (stat[k] == FDGPU_OK)
            groups[{ps[k].velfile, ps[k].st.nx, ps[k].st.ny, ps[k].st.nz, ps[k].swab}].push_back(k);
    for (auto &gr : groups) {
        const auto &idx = gr.second;
        VHead hin;
        std::vector<float> vel;
        int rc = read_velocity(ps[idx[0]], hin, vel);
        if (rc) { for (int k : idx) stat[k] = rc; continue; }
        /* stations that start from a supplied field run as their own batch */
        std::vector<int> plain, seeded;
        for (int k : idx) ((ps[k].st.srctype == 1 && ps[k].fill == 0) ? plain : seeded).push_back(k);
        for (int pass = 0; pass < 2; pass++) {
            const auto &sel = pass == 0 ? plain : seeded;
            if (sel.empty()) continue;
            std::vector<fdgpu_station> sts;
            std::vector<std::vector<float>> out(sel.size()), init(sel.size());
            std::vector<float *> outp;
            std::vector<const float *> initp;
            bool bad = false;
            for (size_t j = 0; j < sel.size(); j++) {
                const ParSetup &p = ps[sel[j]];
                sts.push_back(p.st);
                out[j].resize((size_t)p.st.nx * p.st.ny * p.st.nz);
                outp.push_back(out[j].data());
                if (pass == 1) {
                    rc = initial_field(p, vel, init[j]);
                    if (rc) { stat[sel[j]] = rc; bad = true; }
                    initp.push_back(init[j].data());
                }
            }
            if (bad) { for (int k : sel) if (!stat[k]) stat[k] = FDGPU_EIO; continue; }
            /* the stations of this group, dealt round-robin over the devices; one worker thread per
             * device with more than one, each with its own context */
            const int nd = (int)std::min(devices.size(), sts.size());
            auto work = [&](int d) {
                std::vector<int> mine;
                for (size_t j = d; j < sel.size(); j += nd) mine.push_back((int)j);
                std::vector<fdgpu_station> ms;
                std::vector<float *> mo;
                std::vector<const float *> mi;
                for (int j : mine) {
                    ms.push_back(sts[j]);
                    mo.push_back(outp[j]);
                    if (pass == 1) mi.push_back(initp[j]);
                }
                std::vector<fdgpu_stats> sst(ms.size());
                int rcd = FDGPU_OK;
                fdgpu_ctx *ctx = nd > 1 ? slot_ctx(devices[d], d, &rcd) : thread_ctx(devices[d], &rcd);
                if (ctx)
                    rcd = fdgpu_solve_host(ctx, (int)ms.size(), ms.data(), vel.data(), ms[0].nx, ms[0].ny, ms[0].nz,
                                           mo.data(), pass == 1 ? mi.data() : nullptr, sst.data());
                /* a failed solve is reported on stderr, as the reference reports its failures */
                if (rcd)
                    std::fprintf(stderr, "sphfd: %s: %s%s%s\n", ps[sel[0]].velfile.c_str(), fdgpu_strerror(rcd),
                                 ctx && *fdgpu_last_error(ctx) ? ": " : "", ctx ? fdgpu_last_error(ctx) : "");
                for (int j : mine) stat[sel[j]] = rcd ? rcd : write_times(ps[sel[j]], hin, out[j], output_path);
            };
            if (nd <= 1) {
                work(0);
            } else {
                std::vector<std::thread> th;
                for (int d = 0; d < nd; d++) th.emplace_back(work, d);
                for (auto &t : th) t.join();
            }
        }
    }
}

}  // namespace

extern "C" int fdgpu_station_from_par(int ac, char **av, fdgpu_station *st, char *velfile, size_t velcap,
                                      char *timefile, size_t timecap)
{
    if (!st || !av || ac < 1) return FDGPU_EINVAL;
    ParSetup ps;
    const int rc = setup_from_par(ac, av, ps);
    if (rc) return rc;
    *st = ps.st;
    if (velfile && velcap) std::snprintf(velfile, velcap, "%s", ps.velfile.c_str());
    if (timefile && timecap) std::snprintf(timefile, timecap, "%s", ps.timefile.c_str());
    return FDGPU_OK;
}

extern "C" int fdgpu_sphfd_parlist_devices(int n, char **entries, const char *output_path, int *status, int ndev,
                                           const int *devices)
{
    if (n < 0 || (n > 0 && !entries) || !output_path || ndev < 1 || !devices) return FDGPU_EINVAL;
    std::vector<int> devs(devices, devices + ndev);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) count = 0;
    for (int d : devs)
        if (d < 0 || (count > 0 && d >= count)) return FDGPU_ENODEV;
    std::vector<ParSetup> ps(n);
    std::vector<int> stat(n, FDGPU_OK);
    for (int k = 0; k < n; k++) {
        char *av[2] = {(char *)"sphfd", entries[k]};
        stat[k] = setup_from_par(2, av, ps[k]);
    }
    run_setups(ps, stat, output_path, devs);
    int first = FDGPU_OK;
    for (int k = 0; k < n; k++) {
        if (status) status[k] = stat[k];
        if (stat[k] && first == FDGPU_OK) first = stat[k];
    }
    return first;
}

extern "C" int fdgpu_sphfd_parlist(int n, char **entries, const char *output_path, int *status)
{
    const int dev = current_device();
    return fdgpu_sphfd_parlist_devices(n, entries, output_path, status, 1, &dev);
}

extern "C" int fdgpu_sphfd(int ac, char **av, const char *output_path)
{
    if (ac < 1 || !av || !output_path) return FDGPU_EINVAL;
    std::vector<ParSetup> ps(1);
    std::vector<int> stat(1, setup_from_par(ac, av, ps[0]));
    run_setups(ps, stat, output_path, {current_device()});
    return stat[0];
}
