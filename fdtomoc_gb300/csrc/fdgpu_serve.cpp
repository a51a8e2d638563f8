/*
 * fdgpu_serve.cpp — serving session: velocity models kept on the device, station requests solved
 * as they arrive by a long-running grid of solver CTAs (the fd_solve kernel in its serving mode).
 *
 * Host side, one dispatcher thread per session:
 *   admit     takes queued requests in submission order while a request slot ("entry") and the
 *             memory for its field, its scratch and its grid geometry's tables are free;
 *             starting fields of srctype 2/3 requests are copied in first ("staging");
 *   publish   writes the station record into the entry's slot of the pinned, device-mapped
 *             request table and raises the published count the CTAs watch;
 *   reap      notices the done flags the CTAs set, copies fields to host buffers, frees the
 *             request's memory and queues its result for fdgpu_serve_poll;
 *   grid      launches the solver grid when work is published and none runs, and stops it after
 *             idle_stop_us with nothing in flight.
 * Nothing the dispatcher issues waits on the solver grid in stream order: the grid runs alone on
 * its stream, copies run on a copy stream, and the session's small kernels (geometry tables,
 * velocity to slowness) run on the SMs the grid leaves free.  All device memory is taken from one
 * allocation made when the session opens, so no allocation or free (which can synchronise the
 * device) happens while the grid runs.
 */
#include "fdgpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "fdgpu_device.h"
#include "fdgpu_layout.h"
#include "fdgpu_station.h"

extern "C" cudaError_t fdk_launch_geo_build(int nx, int ny, int nz, double h, double dq, double df, double z0r,
                                            const double *ysin, double *zrow, double *node, double *cell,
                                            cudaStream_t stream);
extern "C" cudaError_t fdk_launch_serve(const fd_serve_queue *q, int nctas, int cta_id0, cudaStream_t stream);
extern "C" cudaError_t fdk_launch_v2s(const float *v, float *s, long long n, cudaStream_t stream);

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

/* First-fit allocator over the session's one device allocation; 256-byte granules, free blocks
 * kept by offset and merged with their neighbours. */
class Arena {
public:
    void init(char *base, size_t cap)
    {
        base_ = base;
        cap_ = cap;
        free_.clear();
        if (cap) free_[0] = cap;
    }
    char *alloc(size_t n)
    {
        n = fdh::align256(std::max<size_t>(n, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            used_ += n;
            peak_ = std::max(peak_, used_);
            return base_ + off;
        }
        return nullptr;
    }
    void release(char *p, size_t n)
    {
        if (!p) return;
        n = fdh::align256(std::max<size_t>(n, 1));
        used_ -= n;
        auto it = free_.emplace((size_t)(p - base_), n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t cap() const { return cap_; }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }

private:
    char *base_ = nullptr;
    size_t cap_ = 0, used_ = 0, peak_ = 0;
    std::map<size_t, size_t> free_;
};

struct ModelVer {
    char *mem = nullptr;
    size_t bytes = 0;
    int mnx = 0, mny = 0, mnz = 0;
    int version = 0;
    int refs = 0;          /* requests submitted against this version and not yet completed */
    bool current = true;   /* still the slot's version for new requests */
};

using GeoKey = std::tuple<int, int, uint64_t, uint64_t, uint64_t, uint64_t, uint64_t>;

struct GeoEntry {
    char *mem = nullptr;
    size_t bytes = 0;
    fdh::GeoPtrs p{};
    int refs = 0;
    uint64_t last_use = 0;
};

uint64_t bits(double x)
{
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
}

enum class St { Queued, Staging, Published, Copying };

enum Kind { kPageable = 0, kPinned = 1, kDevice = 2 };

struct Req {
    uint64_t id = 0, tag = 0;
    fdgpu_station st{};
    ModelVer *mv = nullptr;
    float *out = nullptr;
    int out_kind = kPageable;
    const float *init = nullptr;
    int init_kind = kPageable;
    size_t field_bytes = 0, work_bytes = 0;
    char *field = nullptr;   /* arena field (host outputs), else null */
    char *work = nullptr;    /* face scratch then sweep-graph arrays */
    GeoEntry *geo = nullptr;
    int entry = -1;
    St state = St::Queued;
    Clock::time_point t_submit, t_publish;
};

constexpr int kMaxTrig = 4 * 129;   /* box trig doubles of the largest source box (NCUBE 64) */

int pointer_kind(const void *p, int device, int *kind)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        *kind = kPageable;
        return FDGPU_OK;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        if (a.device != device) return FDGPU_EINVAL;
        *kind = kDevice;
    } else if (a.type == cudaMemoryTypeHost) {
        *kind = kPinned;
    } else {
        *kind = kPageable;
    }
    return FDGPU_OK;
}

}  // namespace

struct fdgpu_server {
    int device = 0;
    int sms = 0, nctas = 0, nent = 0, ring = 0;
    long long idle_stop_us = 2000;
    cudaStream_t kstream = nullptr, cstream = nullptr, astream = nullptr;

    /* the session's device memory */
    char *dmem = nullptr;
    Arena arena;
    fd_serve_queue *q_dev = nullptr;      /* the queue description the grid reads */
    unsigned long long *head_dev = nullptr;

    /* pinned, device-mapped request table */
    fd_station_dev *desc = nullptr;
    unsigned long long *gen = nullptr, *done = nullptr, *tail = nullptr;
    int *order = nullptr, *exitf = nullptr, *stop = nullptr;
    fd_station_stats *stats = nullptr;
    double *trig = nullptr;
    std::vector<cudaEvent_t> ev;
    std::vector<Req *> ent;               /* request holding each entry */
    std::vector<int> free_ent;
    unsigned long long published = 0;

    std::vector<std::unique_ptr<ModelVer>> versions;
    std::vector<ModelVer *> models;
    std::vector<int> model_count;
    std::map<GeoKey, GeoEntry> geos;
    uint64_t geo_clock = 0;

    std::deque<Req *> queue;
    int inflight = 0;                     /* admitted and not completed */
    int npub = 0;                         /* in state Published */
    std::deque<fdgpu_serve_result> results;

    bool grid_live = false;
    bool grid_draining = false;
    bool idle_mark = false;
    Clock::time_point idle_since, last_health;
    int launches = 0;

    /* statistics */
    uint64_t next_id = 1;
    int64_t submitted = 0, completed = 0, failed = 0, node_updates = 0;
    std::vector<double> lat_ms, solve_ms;
    int64_t hist[40] = {};
    Clock::time_point t_open, t_first_submit, t_last_done, t_close;
    bool any_submit = false;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread thr;
    bool closing = false, fatal = false;
    std::string err;

    int open(int dev, const fdgpu_serve_opts *o);
    void run();
    bool admit();
    void publish(Req *r);
    bool reap();
    void manage_grid();
    void launch_grid();
    bool stop_grid();
    void finish(Req *r, int status, const fd_station_stats *hs);
    void fail_all(const char *what, cudaError_t e);
    GeoEntry *geometry(const fdgpu_station &s, int *status);
    char *alloc_evicting(size_t n);
    void release_geo(GeoEntry *g) { if (g) g->refs--; }
    void release_model(ModelVer *mv);
    size_t model_bytes() const;
    void free_all();
};

/* ---- set-up and tear-down ------------------------------------------------------------------ */

int fdgpu_server::open(int dev, const fdgpu_serve_opts *o)
{
    device = dev;
    t_open = Clock::now();
    if (cudaSetDevice(dev) != cudaSuccess) return FDGPU_ENODEV;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FDGPU_ENODEV;
    /* at least one SM stays free: the session's own kernels must be able to run beside the grid */
    const int reserve = o && o->reserve_sms >= 0 ? std::max(1, o->reserve_sms) : 2;
    nctas = std::max(1, sms - reserve);
    nent = o && o->max_inflight > 0 ? o->max_inflight : 2 * nctas;
    ring = 2 * nent;
    idle_stop_us = o && o->idle_stop_us > 0 ? o->idle_stop_us : 2000;
    const int nmod = o && o->max_models > 0 ? o->max_models : 2;
    models.assign(nmod, nullptr);
    model_count.assign(nmod, 0);
    size_t freeb = 0, total = 0;
    if (cudaMemGetInfo(&freeb, &total) != cudaSuccess) return FDGPU_ECUDA;
    size_t cap = o && o->hbm_bytes > 0 ? (size_t)o->hbm_bytes : freeb / 2;
    cap &= ~(size_t)255;
    if (cap < (1u << 20)) return FDGPU_EINVAL;
    auto fail = [&](const char *what, cudaError_t e) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FDGPU_ENOMEM : FDGPU_ECUDA;
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&kstream, cudaStreamNonBlocking))
        || (e = cudaStreamCreateWithFlags(&cstream, cudaStreamNonBlocking))
        || (e = cudaStreamCreateWithFlags(&astream, cudaStreamNonBlocking)))
        return fail("stream", e);
    if ((e = cudaMalloc(&dmem, cap))) return fail("session memory", e);
    arena.init(dmem, cap);
    if ((e = cudaMalloc(&q_dev, sizeof(fd_serve_queue))) || (e = cudaMalloc(&head_dev, sizeof(unsigned long long)))
        || (e = cudaMemset(head_dev, 0, sizeof(unsigned long long))))
        return fail("queue", e);
    /* the request table: pinned and mapped, read and written by the grid across the host link */
    const unsigned fl = cudaHostAllocMapped | cudaHostAllocPortable;
    if ((e = cudaHostAlloc(&desc, sizeof(fd_station_dev) * nent, fl))
        || (e = cudaHostAlloc(&gen, sizeof(unsigned long long) * nent, fl))
        || (e = cudaHostAlloc(&done, sizeof(unsigned long long) * nent, fl))
        || (e = cudaHostAlloc(&tail, sizeof(unsigned long long), fl))
        || (e = cudaHostAlloc(&order, sizeof(int) * ring, fl))
        || (e = cudaHostAlloc(&exitf, sizeof(int) * nctas, fl))
        || (e = cudaHostAlloc(&stop, sizeof(int), fl))
        || (e = cudaHostAlloc(&stats, sizeof(fd_station_stats) * nent, fl))
        || (e = cudaHostAlloc(&trig, sizeof(double) * kMaxTrig * nent, fl)))
        return fail("request table", e);
    std::memset(desc, 0, sizeof(fd_station_dev) * nent);
    std::memset(gen, 0, sizeof(unsigned long long) * nent);
    std::memset(done, 0, sizeof(unsigned long long) * nent);
    *tail = 0;
    std::memset(order, 0, sizeof(int) * ring);
    std::memset(exitf, 0, sizeof(int) * nctas);
    *stop = 0;
    fd_serve_queue q{};
    void *p;
    if ((e = cudaHostGetDevicePointer(&p, desc, 0))) return fail("mapping", e);
    q.desc = static_cast<const fd_station_dev *>(p);
    if ((e = cudaHostGetDevicePointer(&p, gen, 0))) return fail("mapping", e);
    q.gen = static_cast<const unsigned long long *>(p);
    if ((e = cudaHostGetDevicePointer(&p, order, 0))) return fail("mapping", e);
    q.order = static_cast<const int *>(p);
    if ((e = cudaHostGetDevicePointer(&p, tail, 0))) return fail("mapping", e);
    q.tail = static_cast<const unsigned long long *>(p);
    if ((e = cudaHostGetDevicePointer(&p, done, 0))) return fail("mapping", e);
    q.done = static_cast<unsigned long long *>(p);
    if ((e = cudaHostGetDevicePointer(&p, exitf, 0))) return fail("mapping", e);
    q.exitf = static_cast<int *>(p);
    if ((e = cudaHostGetDevicePointer(&p, stop, 0))) return fail("mapping", e);
    q.stop = static_cast<const int *>(p);
    q.head = head_dev;
    q.ring = ring;
    q.idle_ns = 60ll * 1000 * 1000 * 1000;   /* only ends a loop whose host has gone away */
    if ((e = cudaMemcpy(q_dev, &q, sizeof q, cudaMemcpyHostToDevice))) return fail("queue", e);
    ev.assign(nent, nullptr);
    for (int k = 0; k < nent; k++)
        if ((e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming))) return fail("events", e);
    ent.assign(nent, nullptr);
    for (int k = nent - 1; k >= 0; k--) free_ent.push_back(k);
    thr = std::thread([this] { run(); });
    return FDGPU_OK;
}

void fdgpu_server::free_all()
{
    cudaSetDevice(device);
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    ev.clear();
    if (dmem) cudaFree(dmem);
    if (q_dev) cudaFree(q_dev);
    if (head_dev) cudaFree(head_dev);
    for (void *h : {(void *)desc, (void *)gen, (void *)done, (void *)tail, (void *)order, (void *)exitf, (void *)stop,
                    (void *)stats, (void *)trig})
        if (h) cudaFreeHost(h);
    for (cudaStream_t s : {kstream, cstream, astream})
        if (s) cudaStreamDestroy(s);
    dmem = nullptr;
    q_dev = nullptr;
    head_dev = nullptr;
}

size_t fdgpu_server::model_bytes() const
{
    size_t b = 0;
    for (const auto &v : versions) b += fdh::align256(v->bytes);
    return b;
}

void fdgpu_server::release_model(ModelVer *mv)
{
    if (!mv) return;
    if (--mv->refs > 0 || mv->current) return;
    arena.release(mv->mem, mv->bytes);
    for (auto it = versions.begin(); it != versions.end(); ++it)
        if (it->get() == mv) {
            versions.erase(it);
            break;
        }
}

/* arena memory, evicting geometry tables no request uses (least recently used first) */
char *fdgpu_server::alloc_evicting(size_t n)
{
    for (;;) {
        if (char *p = arena.alloc(n)) return p;
        auto victim = geos.end();
        for (auto it = geos.begin(); it != geos.end(); ++it)
            if (it->second.refs == 0 && (victim == geos.end() || it->second.last_use < victim->second.last_use))
                victim = it;
        if (victim == geos.end()) return nullptr;
        arena.release(victim->second.mem, victim->second.bytes);
        geos.erase(victim);
    }
}

/* geometry tables of a station's grid, built on the auxiliary stream when first needed */
GeoEntry *fdgpu_server::geometry(const fdgpu_station &s, int *status)
{
    *status = FDGPU_OK;
    const GeoKey key{s.ny, s.nz, bits(s.h), bits(s.dq), bits(s.df), bits(s.z0r), bits(s.y0)};
    auto it = geos.find(key);
    if (it != geos.end()) {
        it->second.last_use = ++geo_clock;
        return &it->second;
    }
    const size_t bytes = fdh::geo_bytes(s.ny, s.nz);
    char *mem = alloc_evicting(bytes);
    if (!mem) return nullptr;   /* no room now */
    GeoEntry g;
    g.mem = mem;
    g.bytes = bytes;
    g.p = fdh::geo_carve(mem, s.ny, s.nz);
    g.last_use = ++geo_clock;
    std::vector<double> ys(s.ny);
    fdh::ysin_table(s, ys.data());
    cudaError_t e;
    if ((e = cudaMemcpyAsync(g.p.ysin, ys.data(), sizeof(double) * s.ny, cudaMemcpyHostToDevice, astream))
        || (e = fdk_launch_geo_build(s.nx, s.ny, s.nz, s.h, s.dq, s.df, s.z0r, g.p.ysin, g.p.zrow, g.p.node, g.p.cell,
                                     astream))
        || (e = cudaStreamSynchronize(astream))) {
        arena.release(mem, bytes);
        err = std::string("geometry build: ") + cudaGetErrorString(e);
        *status = FDGPU_ECUDA;
        return nullptr;
    }
    return &geos.emplace(key, g).first->second;
}

/* ---- the dispatcher ------------------------------------------------------------------------- */

void fdgpu_server::fail_all(const char *what, cudaError_t e)
{
    if (!fatal) err = std::string(what) + ": " + cudaGetErrorString(e);
    fatal = true;
    for (int k = 0; k < nent; k++)
        if (ent[k]) finish(ent[k], FDGPU_ECUDA, nullptr);
    while (!queue.empty()) {
        Req *r = queue.front();
        queue.pop_front();
        finish(r, FDGPU_ECUDA, nullptr);
    }
    grid_live = false;
}

void fdgpu_server::finish(Req *r, int status, const fd_station_stats *hs)
{
    const Clock::time_point now = Clock::now();
    fdgpu_serve_result res;
    std::memset(&res, 0, sizeof res);
    res.id = r->id;
    res.tag = r->tag;
    res.model_version = r->mv ? r->mv->version : 0;
    if (hs) {
        fdh::copy_stats(res.stats, *hs);
        if (status == FDGPU_OK && hs->status) status = FDGPU_ESCHED;
        res.solve_ms = (double)(hs->t_end_ns - hs->t_start_ns) * 1e-6;
    }
    res.status = status;
    res.latency_ms = ms_between(r->t_submit, now);
    res.queue_ms = (r->state == St::Queued || r->state == St::Staging) ? res.latency_ms
                                                                       : ms_between(r->t_submit, r->t_publish);
    if (r->state == St::Published) npub--;
    if (r->entry >= 0) {
        ent[r->entry] = nullptr;
        free_ent.push_back(r->entry);
    }
    if (r->state != St::Queued) inflight--;
    arena.release(r->field, r->field_bytes);
    arena.release(r->work, r->work_bytes);
    release_geo(r->geo);
    release_model(r->mv);
    if (status == FDGPU_OK) {
        completed++;
        node_updates += res.stats.node_updates;
        lat_ms.push_back(res.latency_ms);
        solve_ms.push_back(res.solve_ms);
        int b = 0;
        for (double x = res.latency_ms * 1024.0; x >= 2.0 && b < 39; x *= 0.5) b++;
        hist[b]++;
    } else {
        failed++;
    }
    t_last_done = now;
    results.push_back(res);
    delete r;
    cv_done.notify_all();
}

/* Admit queued requests in order while an entry and memory are free. */
bool fdgpu_server::admit()
{
    bool progress = false;
    while (!queue.empty() && !free_ent.empty() && !fatal) {
        Req *r = queue.front();
        int status = FDGPU_OK;
        GeoEntry *g = geometry(r->st, &status);
        if (status) {
            queue.pop_front();
            finish(r, status, nullptr);
            progress = true;
            continue;
        }
        if (!g) break;
        g->refs++;
        char *work = alloc_evicting(r->work_bytes);
        char *field = (work && r->out_kind != kDevice) ? alloc_evicting(r->field_bytes) : nullptr;
        if (!work || (r->out_kind != kDevice && !field)) {
            arena.release(work, r->work_bytes);
            g->refs--;
            if (inflight == 0) {
                /* nothing will free memory: the request cannot fit next to the models */
                queue.pop_front();
                finish(r, FDGPU_ETOOBIG, nullptr);
                progress = true;
                continue;
            }
            break;
        }
        queue.pop_front();
        progress = true;
        r->geo = g;
        r->work = work;
        r->field = field;
        const int e = free_ent.back();
        free_ent.pop_back();
        r->entry = e;
        ent[e] = r;
        inflight++;
        float *T = r->out_kind == kDevice ? r->out : reinterpret_cast<float *>(field);
        const fdgpu_station &s = r->st;
        double *tg = trig + (size_t)kMaxTrig * e;
        fdh::box_trig(s, tg);
        void *tg_dev = nullptr, *st_dev = nullptr;
        cudaHostGetDevicePointer(&tg_dev, tg, 0);
        cudaHostGetDevicePointer(&st_dev, stats + e, 0);
        std::memset(stats + e, 0, sizeof(fd_station_stats));
        const bool init = s.srctype != 1 || r->init;
        fdh::fill_station(desc[e], s, g->p, T, reinterpret_cast<const float *>(r->mv->mem), r->mv->mnx,
                          (long long)r->mv->mnx * r->mv->mny, init ? 1 : 0, work, work + fdh::face_bytes(s),
                          static_cast<const double *>(tg_dev), static_cast<fd_station_stats *>(st_dev));
        if (r->init && r->init != T) {
            const cudaMemcpyKind kind = r->init_kind == kDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
            cudaError_t ce;
            if ((ce = cudaMemcpyAsync(T, r->init, r->field_bytes, kind, cstream))
                || (ce = cudaEventRecord(ev[e], cstream))) {
                fail_all("starting field copy", ce);
                return true;
            }
            r->state = St::Staging;
        } else {
            r->state = St::Staging;
            publish(r);
        }
    }
    return progress;
}

/* hand an admitted request to the grid: its record, generation and order slot first, then the
 * published count the CTAs watch */
void fdgpu_server::publish(Req *r)
{
    const int e = r->entry;
    gen[e] = r->id + 1;
    __atomic_store_n(&done[e], 0ull, __ATOMIC_RELAXED);
    order[published % (unsigned long long)ring] = e;
    published++;
    __atomic_store_n(tail, published, __ATOMIC_RELEASE);
    r->state = St::Published;
    r->t_publish = Clock::now();
    npub++;
}

/* Move requests along: staged ones are published, finished ones copied out and completed. */
bool fdgpu_server::reap()
{
    bool progress = false;
    for (int e = 0; e < nent && !fatal; e++) {
        Req *r = ent[e];
        if (!r) continue;
        if (r->state == St::Staging) {
            const cudaError_t q = cudaEventQuery(ev[e]);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                fail_all("starting field copy", q);
                return true;
            }
            publish(r);
            progress = true;
        } else if (r->state == St::Published) {
            if (__atomic_load_n(&done[e], __ATOMIC_ACQUIRE) != gen[e]) continue;
            npub--;
            r->state = St::Copying;
            progress = true;
            if (r->out_kind == kDevice) {
                finish(r, FDGPU_OK, &stats[e]);
                continue;
            }
            cudaError_t ce;
            if ((ce = cudaMemcpyAsync(r->out, r->field, r->field_bytes, cudaMemcpyDeviceToHost, cstream))
                || (ce = cudaEventRecord(ev[e], cstream))) {
                fail_all("field copy", ce);
                return true;
            }
        } else if (r->state == St::Copying) {
            const cudaError_t q = cudaEventQuery(ev[e]);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                fail_all("field copy", q);
                return true;
            }
            progress = true;
            finish(r, FDGPU_OK, &stats[e]);
        }
    }
    return progress;
}

void fdgpu_server::launch_grid()
{
    std::memset(exitf, 0, sizeof(int) * nctas);
    __atomic_store_n(stop, 0, __ATOMIC_RELEASE);
    const cudaError_t e = fdk_launch_serve(q_dev, nctas, 0, kstream);
    if (e != cudaSuccess) {
        fail_all("solver grid launch", e);
        return;
    }
    launches++;
    grid_live = true;
    grid_draining = false;
    idle_mark = false;
    last_health = Clock::now();
}

/* ask idle CTAs to leave and wait (bounded) until the grid has ended */
bool fdgpu_server::stop_grid()
{
    __atomic_store_n(stop, 1, __ATOMIC_RELEASE);
    const Clock::time_point t0 = Clock::now();
    for (;;) {
        const cudaError_t q = cudaStreamQuery(kstream);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) {
            fail_all("solver grid", q);
            return false;
        }
        if (ms_between(t0, Clock::now()) > 60000.0) {
            fail_all("solver grid did not stop", cudaErrorLaunchTimeout);
            return false;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    __atomic_store_n(stop, 0, __ATOMIC_RELEASE);
    grid_live = false;
    grid_draining = false;
    return true;
}

void fdgpu_server::manage_grid()
{
    if (fatal) return;
    const Clock::time_point now = Clock::now();
    if (!grid_live) {
        if (npub > 0) launch_grid();
        return;
    }
    if (ms_between(last_health, now) > 2.0) {
        last_health = now;
        const cudaError_t q = cudaStreamQuery(kstream);
        if (q == cudaSuccess) {
            grid_live = false;   /* every CTA left (idle bound); published work goes to the next grid */
            if (npub > 0) launch_grid();
            return;
        }
        if (q != cudaErrorNotReady) {
            fail_all("solver grid", q);
            return;
        }
        if (!grid_draining) {
            /* a CTA that left on its own lowers the grid's width: let the rest finish, relaunch */
            for (int c = 0; c < nctas; c++)
                if (__atomic_load_n(&exitf[c], __ATOMIC_ACQUIRE)) {
                    grid_draining = true;
                    __atomic_store_n(stop, 1, __ATOMIC_RELEASE);
                    break;
                }
        }
    }
    if (inflight == 0 && queue.empty()) {
        if (!idle_mark) {
            idle_mark = true;
            idle_since = now;
        } else if (std::chrono::duration<double, std::micro>(now - idle_since).count() > (double)idle_stop_us) {
            stop_grid();
            idle_mark = false;
        }
    } else {
        idle_mark = false;
    }
}

void fdgpu_server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool progress = false;
        progress |= reap();
        progress |= admit();
        progress |= reap();
        manage_grid();
        if (closing && ((queue.empty() && inflight == 0) || fatal)) {
            if (grid_live) stop_grid();
            break;
        }
        if (closing && ms_between(t_close, Clock::now()) > 300000.0) {
            /* outstanding work that does not finish within 5 minutes of close: give up on it */
            fail_all("close: outstanding requests did not finish", cudaErrorLaunchTimeout);
            continue;
        }
        if (progress) continue;
        if (!grid_live && queue.empty() && inflight == 0)
            cv_work.wait(lk);
        else
            cv_work.wait_for(lk, std::chrono::microseconds(inflight ? 20 : 200));
    }
    cv_done.notify_all();
}

/* ---- C ABI ---------------------------------------------------------------------------------- */

extern "C" int fdgpu_serve_open(int device, const fdgpu_serve_opts *opts, fdgpu_server **out)
{
    if (!out) return FDGPU_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return FDGPU_ENODEV;
    FdDeviceScope dev_(device);
    if (dev_.err) return FDGPU_ENODEV;
    auto *sv = new (std::nothrow) fdgpu_server;
    if (!sv) return FDGPU_ENOMEM;
    const int rc = sv->open(device, opts);
    if (rc) {
        if (sv->thr.joinable()) {
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->closing = true;
            }
            sv->cv_work.notify_all();
            sv->thr.join();
        }
        sv->free_all();
        delete sv;
        return rc;
    }
    *out = sv;
    return FDGPU_OK;
}

extern "C" int fdgpu_serve_set_model(fdgpu_server *sv, int model, const float *velocity, int mnx, int mny, int mnz,
                                     int *version)
{
    if (!sv || !velocity || model < 0 || model >= (int)sv->models.size() || mnx < 1 || mny < 1 || mnz < 1)
        return FDGPU_EINVAL;
    if (((uintptr_t)velocity & 3u) != 0) return FDGPU_EINVAL;
    FdDeviceScope dev_(sv->device);
    int kind = kPageable;
    if (pointer_kind(velocity, sv->device, &kind)) return FDGPU_EINVAL;
    const long long nm = (long long)mnx * mny * mnz;
    const size_t bytes = sizeof(float) * (size_t)nm;
    char *mem;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->fatal) return FDGPU_ECUDA;
        mem = sv->alloc_evicting(bytes);
        if (!mem) return FDGPU_ETOOBIG;
    }
    /* the copy and the conversion run on the SMs the solver grid leaves free */
    cudaError_t e = cudaSuccess;
    if (kind == kDevice) {
        e = fdk_launch_v2s(velocity, reinterpret_cast<float *>(mem), nm, sv->astream);
    } else {
        e = cudaMemcpyAsync(mem, velocity, bytes, cudaMemcpyHostToDevice, sv->astream);
        if (!e) e = fdk_launch_v2s(reinterpret_cast<float *>(mem), reinterpret_cast<float *>(mem), nm, sv->astream);
    }
    if (!e) e = cudaStreamSynchronize(sv->astream);
    std::lock_guard<std::mutex> lk(sv->mu);
    if (e) {
        sv->arena.release(mem, bytes);
        sv->err = std::string("model upload: ") + cudaGetErrorString(e);
        return FDGPU_ECUDA;
    }
    auto mv = std::make_unique<ModelVer>();
    mv->mem = mem;
    mv->bytes = bytes;
    mv->mnx = mnx;
    mv->mny = mny;
    mv->mnz = mnz;
    mv->version = ++sv->model_count[model];
    ModelVer *old = sv->models[model];
    sv->models[model] = mv.get();
    sv->versions.push_back(std::move(mv));
    if (old) {
        old->current = false;
        old->refs++;
        sv->release_model(old);   /* freed now if no request holds it */
    }
    if (version) *version = sv->model_count[model];
    return FDGPU_OK;
}

extern "C" int fdgpu_serve_submit(fdgpu_server *sv, const fdgpu_station *st, int model, float *times,
                                  const float *init_times, uint64_t tag, uint64_t *id)
{
    if (!sv || !st || !times || model < 0 || model >= (int)sv->models.size()) return FDGPU_EINVAL;
    int rc = fdh::check_station(*st);
    if (rc) return rc;
    if (((uintptr_t)times & 3u) != 0 || ((uintptr_t)init_times & 3u) != 0) return FDGPU_EINVAL;
    if (st->srctype != 1 && !init_times) return FDGPU_EINVAL;
    FdDeviceScope dev_(sv->device);
    auto r = std::make_unique<Req>();
    if (pointer_kind(times, sv->device, &r->out_kind)) return FDGPU_EINVAL;
    if (init_times && pointer_kind(init_times, sv->device, &r->init_kind)) return FDGPU_EINVAL;
    r->st = *st;
    r->tag = tag;
    r->out = times;
    r->init = init_times;
    r->field_bytes = sizeof(float) * (size_t)st->nx * st->ny * st->nz;
    r->work_bytes = fdh::face_bytes(*st) + fdh::graph_bytes(*st);
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->fatal) return FDGPU_ECUDA;
    if (sv->closing) return FDGPU_EINVAL;
    ModelVer *mv = sv->models[model];
    if (!mv) return FDGPU_EINVAL;
    if (st->ox < 0 || st->oy < 0 || st->oz < 0 || st->ox + st->nx > mv->mnx || st->oy + st->ny > mv->mny
        || st->oz + st->nz > mv->mnz)
        return FDGPU_EINVAL;
    const size_t need = fdh::align256(r->work_bytes) + (r->out_kind == kDevice ? 0 : fdh::align256(r->field_bytes))
                        + fdh::geo_bytes(st->ny, st->nz);
    if (need + sv->model_bytes() > sv->arena.cap()) return FDGPU_ETOOBIG;
    r->mv = mv;
    mv->refs++;
    r->id = sv->next_id++;
    r->t_submit = Clock::now();
    if (!sv->any_submit) {
        sv->any_submit = true;
        sv->t_first_submit = r->t_submit;
    }
    sv->submitted++;
    if (id) *id = r->id;
    sv->queue.push_back(r.release());
    sv->cv_work.notify_all();
    return FDGPU_OK;
}

extern "C" int fdgpu_serve_poll(fdgpu_server *sv, fdgpu_serve_result *out, int max, int timeout_ms, int *n)
{
    if (!sv || !n || max < 0 || (max > 0 && !out)) return FDGPU_EINVAL;
    *n = 0;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto ready = [&] { return !sv->results.empty() || (timeout_ms < 0 && sv->queue.empty() && sv->inflight == 0); };
    if (timeout_ms < 0)
        sv->cv_done.wait(lk, ready);
    else if (timeout_ms > 0)
        sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
    while (*n < max && !sv->results.empty()) {
        out[(*n)++] = sv->results.front();
        sv->results.pop_front();
    }
    return FDGPU_OK;
}

extern "C" int fdgpu_serve_drain(fdgpu_server *sv, int timeout_ms)
{
    if (!sv) return FDGPU_EINVAL;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto idle = [&] { return sv->queue.empty() && sv->inflight == 0; };
    if (timeout_ms < 0) {
        sv->cv_done.wait(lk, idle);
        return FDGPU_OK;
    }
    return sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle) ? FDGPU_OK : FDGPU_ETIMEDOUT;
}

extern "C" int fdgpu_serve_metrics_get(fdgpu_server *sv, fdgpu_serve_metrics *m)
{
    if (!sv || !m) return FDGPU_EINVAL;
    std::lock_guard<std::mutex> lk(sv->mu);
    std::memset(m, 0, sizeof *m);
    m->submitted = sv->submitted;
    m->completed = sv->completed;
    m->failed = sv->failed;
    m->queued = (int64_t)sv->queue.size();
    m->inflight = sv->inflight;
    auto pct = [](std::vector<double> v, double p) {
        if (v.empty()) return 0.0;
        const size_t k = std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5));
        std::nth_element(v.begin(), v.begin() + k, v.end());
        return v[k];
    };
    m->p50_ms = pct(sv->lat_ms, 0.50);
    m->p90_ms = pct(sv->lat_ms, 0.90);
    m->p99_ms = pct(sv->lat_ms, 0.99);
    m->max_ms = sv->lat_ms.empty() ? 0.0 : *std::max_element(sv->lat_ms.begin(), sv->lat_ms.end());
    double sum = 0;
    for (double x : sv->lat_ms) sum += x;
    m->mean_ms = sv->lat_ms.empty() ? 0.0 : sum / (double)sv->lat_ms.size();
    m->solve_p50_ms = pct(sv->solve_ms, 0.50);
    m->solve_p99_ms = pct(sv->solve_ms, 0.99);
    if (sv->completed > 0) {
        const double span = ms_between(sv->t_first_submit, sv->t_last_done) * 1e-3;
        if (span > 0) {
            m->fields_per_s = (double)sv->completed / span;
            m->node_updates_per_s = (double)sv->node_updates / span;
        }
    }
    m->node_updates = sv->node_updates;
    m->hbm_bytes = (int64_t)sv->arena.cap();
    m->hbm_used = (int64_t)sv->arena.used();
    m->hbm_peak = (int64_t)sv->arena.peak();
    m->solver_ctas = sv->nctas;
    m->grid_launches = sv->launches;
    for (int k = 0; k < 40; k++) m->hist[k] = sv->hist[k];
    return FDGPU_OK;
}

extern "C" const char *fdgpu_serve_last_error(const fdgpu_server *sv) { return sv ? sv->err.c_str() : ""; }

extern "C" int fdgpu_serve_close(fdgpu_server *sv)
{
    if (!sv) return FDGPU_EINVAL;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->closing = true;
        sv->t_close = Clock::now();
    }
    sv->cv_work.notify_all();
    if (sv->thr.joinable()) sv->thr.join();
    const int rc = sv->fatal ? FDGPU_ECUDA : FDGPU_OK;
    FdDeviceScope dev_(sv->device);
    sv->free_all();
    delete sv;
    return rc;
}
