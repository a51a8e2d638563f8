/*
 * fdgpu.h — C ABI of the GB300 sphfd travel-time solver (libfdgpu.so).
 *
 * The library replaces the solve of FDtomoC's sphfd program (reference: src/sphfd.c).  Its
 * results are bit-identical to the reference's: same travel times, same head-wave restarts.
 *
 * Two levels:
 *   1. Drop-in entry points with the reference's file interface:
 *        fdgpu_sphfd          replaces  int sphfd(int ac, char **av, char *output_path)
 *                                       (src/sphfd.c:194, body :260-5803)
 *        fdgpu_sphfd_parlist  replaces  the OpenMP loop over par files in main()
 *                                       (src/sphfd.c:247-255); all stations run on the GPU at once.
 *   2. Array entry points for callers that keep models and fields in memory (batch drivers):
 *      fdgpu_station_from_par, fdgpu_solve_host, fdgpu_solve_device, fdgpu_solve_noalloc.
 *   3. A serving session (fdgpu_serve_*): models resident on the device, requests admitted as
 *      they arrive and solved by a long-running grid, with latency statistics.
 *   4. The path's neighbours on the device: fdgpu_c2f (c2f, the model's producer), fdgpu_locate
 *      (sphfdloc's event location) and fdgpu_raytrace (sphrayderv's rays and derivatives), with
 *      fdgpu_sphfdloc and fdgpu_sphrayderv, drop-ins for those programs' main built on them.
 *   Level 2 also has prepared batches (fdgpu_batch_*) whose launch can be captured in a CUDA graph.
 *
 * Conventions: every function returns an FDGPU_* status (0 = success) and never aborts; the
 * caller owns host buffers and any device buffers it passes in; the library owns its scratch,
 * geometry tables and streams, all held in an fdgpu_ctx.  A context is not thread-safe; use one
 * per host thread.  Grids are x fastest (index nx*ny*z + nx*y + x), as in the reference.
 * Devices: a context, a batch, a c2f plan and a serving session belong to one device; their
 * calls run there and give the calling thread's current device back as they found it.  The
 * entry points without such an object (the drop-ins, fdgpu_solve_noalloc) use the calling
 * thread's current device.
 */
#ifndef FDGPU_H
#define FDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FDGPU_OK = 0,
    FDGPU_EINVAL = -1,   /* bad argument */
    FDGPU_ENOMEM = -2,   /* device or host allocation failed */
    FDGPU_ECUDA = -3,    /* a CUDA call failed (message via fdgpu_last_error) */
    FDGPU_EIO = -4,      /* a file could not be read or written */
    FDGPU_EPAR = -5,     /* a required par parameter is missing or a value is invalid */
    FDGPU_ESOURCE = -6,  /* the source is outside the grid (src/sphfd.c:533-538) */
    FDGPU_ESCHED = -7,   /* internal: a walk's schedule check failed (fdgpu_stats.detail says which) */
    FDGPU_ENODEV = -8,   /* no CUDA device */
    FDGPU_ETOOBIG = -9,  /* the problem needs more memory than the entry point may use
                            (fdgpu_solve_noalloc's static scratch, a serving session's memory) */
    FDGPU_ETIMEDOUT = -10   /* a wait's time limit passed first (fdgpu_serve_drain) */
};

typedef struct fdgpu_ctx fdgpu_ctx;

/* One station solve, as sphfd() has set it up after reading its par file (src/sphfd.c:383-552,
 * 724-825, 977-1003).  fdgpu_station_from_par fills it from par-file arguments. */
typedef struct {
    int nx, ny, nz;
    double h;              /* radial step, km */
    double dq, df;         /* colatitude / longitude steps, radians */
    double x0;             /* longitude of x = 0, radians */
    double y0;             /* geocentric colatitude of y = 0, radians */
    double z0r;            /* radius of z = 0, km */
    int srctype;           /* 1 point source; 3 restart from a supplied field (srcwall); 2 as 3 */
    int xs, ys, zs;        /* source node (srctype 1) */
    double src_geo[3];     /* geocentric source: longitude rad, colatitude rad, radius km */
    int ncube;             /* source box half-width (NCUBE) */
    int reverse;           /* up to reverse+1 sweeps */
    int headpref;          /* par value (> 0: prefer the wall opposite the source) */
    int maxrad;            /* radius limit from maxoff (99999999 = none) */
    int kminus, kplus, iplus, iminus, jminus, jplus;
    int srcwall;           /* srctype 2/3: wall holding the starting times (1..6) */
    int ox, oy, oz;        /* this grid's origin inside the slowness model it reads */
} fdgpu_station;

typedef struct {
    int32_t status;
    int32_t sweeps;          /* sweeps run (1 + restarts) */
    int64_t node_updates;    /* face-point evaluations */
    int64_t faces;
    int64_t rounds;          /* chunks of up to 32 ready nodes evaluated by one warp */
    int64_t deferred;        /* points that took the stale (t0,t4) of an earlier point */
    int64_t stencils[5];     /* stencil evaluations: 3-D, new-edge, 2-D, new-face, 1-D */
    int32_t restart_wall[8]; /* restarts per wall 1..6 */
    int64_t phase_cycles[6]; /* profiling builds only: warp cycles summed over the warps in face
                                set-up, the three evaluation phases and the face walks */
    int64_t t_start_ns, t_end_ns; /* GPU global timer (ns) at the start and end of this solve */
    int32_t pipelined_sweeps; /* sweeps walked as one plane-pipelined dependency graph */
    int32_t detail;           /* on FDGPU_ESCHED, the check that failed: 3 nodes left that nothing
                                 releases, 4 sweep bound, 6 a pipelined sweep met a point needing an
                                 earlier point's stencil state, 8 a worker waited too long, 9 a
                                 claimed queue entry was never written, 10 a node queued twice,
                                 11 a second point waiting on one point, 12 a point found no
                                 earlier point to take its stencil state from, 14 a node that no
                                 face instance owns, 15 a wait table full, 17 a walk ran past its
                                 bound, 18 a queue entry outside the walk's nodes, 100 + k a
                                 cluster barrier k gave up (several CTAs per station only) */
    int32_t sm;               /* the SM whose CTA ran the solve */
    int32_t pad;
} fdgpu_stats;

int fdgpu_create(int device, fdgpu_ctx **out);
void fdgpu_destroy(fdgpu_ctx *ctx);
const char *fdgpu_strerror(int status);
/* text of the last CUDA or I/O failure in this context ("" if none) */
const char *fdgpu_last_error(const fdgpu_ctx *ctx);

/* Parse getpar-style arguments (e.g. {"sphfd", "par=station.par"}) the way sphfd() does
 * (src/sphfd.c:383-552): geometry conversion (WGS84 geocentric colatitude), source placement,
 * box walls.  velfile/timefile receive the file names from the par file (timefile without the
 * output directory).  Replaces the set-up part of sphfd(). */
int fdgpu_station_from_par(int ac, char **av, fdgpu_station *st, char *velfile, size_t velcap,
                           char *timefile, size_t timecap);

/* Solve n stations whose velocities are in host memory: model (mnx, mny, mnz) is copied to the
 * device, converted to slowness, each station reads its window at (ox, oy, oz), and each field is
 * copied back to times[k] (nx*ny*nz floats).  init_times[k] may give the starting field for
 * srctype 2/3 stations (NULL otherwise).  stats may be NULL. */
int fdgpu_solve_host(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *velocity, int mnx, int mny,
                     int mnz, float *const *times, const float *const *init_times, fdgpu_stats *stats);

/* CTAs (one per SM) that may cooperate on each station in later solves of this context, as one
 * thread-block cluster: 0 (the default) lets the library choose, 1, 2, 4 or 8 asks for that many.
 * The library currently caps it at 1 (multi-CTA solving is disabled in this build).  Results do not
 * depend on it.  No counterpart in the reference (one OpenMP thread per station). */
int fdgpu_set_cluster(fdgpu_ctx *ctx, int ctas_per_station);

/* Bounds, in SM clock cycles, of the solver's waits in later solves of this context: a warp with
 * nothing to do for wait_cycles, or one walk (a face, or a whole sweep) running for walk_cycles,
 * ends that station's solve with FDGPU_ESCHED (fdgpu_stats.detail 8 or 17) instead of waiting on.
 * 0 keeps the built-in bounds (about 2 s and 66 s at the GB300's clock, far beyond any real solve).
 * The context stays usable after such a status.  No counterpart in the reference (its loops have
 * no waits); it exists so that a stalled schedule is reported, and so that this is testable. */
int fdgpu_set_wait_limits(fdgpu_ctx *ctx, long long wait_cycles, long long walk_cycles);

/* Same with everything already on the device: slowness (1/v, float) of a model with strides
 * (1, s_sy, s_sz), one device field per station.  Work is queued on `stream` (a cudaStream_t,
 * NULL = the context's stream); the call returns after the solve has completed. */
int fdgpu_solve_device(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *slowness, long long s_sy,
                       long long s_sz, float *const *d_times, int times_initialised, fdgpu_stats *stats,
                       void *stream);

/* The same batch prepared once and launched many times, e.g. inside a captured CUDA graph: create
 * builds the geometry tables, the scratch and the station records on the device (the context must
 * outlive the batch); run queues the solve of all n stations as one kernel launch on `stream` (NULL:
 * the context's), with no allocation and no host synchronisation, so it can be captured; stats waits
 * for `stream` and reads the statistics of the last run.  Point-source stations initialise their
 * fields in every run; stations that start from a supplied field (times_initialised) need it put
 * back before each run.  Runs of one batch share its scratch: two of them must not overlap. */
typedef struct fdgpu_batch fdgpu_batch;
int fdgpu_batch_create(fdgpu_ctx *ctx, int n, const fdgpu_station *st, const float *slowness, long long s_sy,
                       long long s_sz, float *const *d_times, int times_initialised, fdgpu_batch **out);
int fdgpu_batch_run(fdgpu_batch *batch, void *stream);
int fdgpu_batch_stats(fdgpu_batch *batch, fdgpu_stats *stats, void *stream);
void fdgpu_batch_destroy(fdgpu_batch *batch);

/* Launch order of a prepared batch (no counterpart in the reference, whose OpenMP loop takes par
 * files in list order).  CTA k solves the k-th station of the order, and CTAs beyond the resident
 * ones start as earlier ones finish, so the batch ends sooner when its longest solves start first.
 * A new batch is ordered by grid size (or by the context's measured times, see below);
 * fdgpu_batch_tune_order reorders it longest first by the solve times its last run measured, each
 * blended with the context's earlier measurement of that station (the mean of the two), so that
 * one run's noise moves the order less (an inversion loop re-solves the same stations every
 * iteration, so earlier runs' times predict the next run's).  fdgpu_batch_order reads the order (the
 * caller's station indices, in launch order) and fdgpu_batch_set_order sets one, e.g. saved from an
 * earlier process.  These copy on `stream` and wait for it: call them between runs, not while one
 * is in flight.  The order changes which CTA solves which station, never a result. */
int fdgpu_batch_order(fdgpu_batch *batch, int *order, void *stream);

/* The context's launch-order table: every clean solve of fdgpu_solve_device / fdgpu_solve_host /
 * fdgpu_batch_stats records each station's measured solve time (the mean of the new time and the
 * one recorded before; a batch run's times are recorded once, however often its statistics are
 * read or its order tuned), and a later batch whose stations all have one is launched longest first
 * (otherwise largest grid first).  order_save writes the table to a file and order_load merges one
 * into the context, so that a new process (the next inversion iteration, say) starts with the
 * order the last one measured.  Results never depend on it.  No counterpart in the reference. */
int fdgpu_order_save(const fdgpu_ctx *ctx, const char *path);
int fdgpu_order_load(fdgpu_ctx *ctx, const char *path);
int fdgpu_batch_set_order(fdgpu_batch *batch, const int *order, void *stream);
int fdgpu_batch_tune_order(fdgpu_batch *batch, void *stream);

/* velocity -> slowness on the device, slow[i] = 1/v[i] as the reference rounds it (src/sphfd.c:689) */
int fdgpu_velocity_to_slowness(fdgpu_ctx *ctx, const float *d_velocity, float *d_slowness, long long n,
                               void *stream);

/* Diagnostics: measured FP64 instruction rate of this GPU (fused multiply-adds per second / 1e9),
 * the denominator the benchmark reports the solver's FP64 throughput against.  No counterpart in
 * the reference. */
int fdgpu_probe_fp64(fdgpu_ctx *ctx, double *gops);

/* Solve one point-source station without allocating device memory.  It has no counterpart in the
 * reference: it is for callers that must not have a library call cudaMalloc / cudaFree.  Such
 * callers include loops that cannot afford the device-wide synchronisation cudaFree implies, and
 * applications whose device memory belongs to another allocator.  The caller passes the slowness
 * model (strides 1, s_sy, s_sz; the station reads its window at ox, oy, oz) and the output field
 * (nx*ny*nz floats), both device buffers it owns.  All other scratch (station descriptor,
 * statistics, geometry tables, face-walk scratch) lives in one static device array of
 * FDGPU_NOALLOC_SCRATCH_BYTES per GPU, held from library load to process exit.  A station that needs
 * more returns FDGPU_ETOOBIG before any GPU work; a 201x201x81 grid needs about 12 MiB.  The first
 * call on a device looks up the array's address; make it while no stream is capturing.  The call
 * itself cannot be captured in a CUDA graph (it waits for the solve).  That address
 * is kept for the life of the process: it does not survive cudaDeviceReset (or any other teardown
 * of the device's primary context), after which this entry point must not be called again.  The
 * call runs on the calling thread's current device, and `stream` (a cudaStream_t, NULL = the
 * default stream) must belong to that device (FDGPU_EINVAL otherwise).  Calls share the array, so
 * calls that overlap on one GPU race: serialise them per device.  The call returns when the solve
 * has finished on `stream`; results are bit-identical to fdgpu_solve_device. */
#define FDGPU_NOALLOC_SCRATCH_BYTES (16u << 20)
int fdgpu_solve_noalloc(const fdgpu_station *st, const float *d_slowness, long long s_sy, long long s_sz,
                        float *d_time, fdgpu_stats *stats, void *stream);

/* ---- Serving -------------------------------------------------------------------------------
 *
 * A serving session keeps velocity models on the device and solves station requests as they
 * arrive.  It has no counterpart in the reference, whose driver runs one sphfd() per par file
 * under OpenMP (src/sphfd.c:247-255) and reads the model from disk in every call (:586-700).
 *
 * One long-running grid of solver CTAs (one per SM, less reserve_sms) loops on the device: each
 * CTA claims the next published request, solves it and flags it done.  A host thread admits
 * requests in submission order whenever a request slot and enough of the session's device memory
 * are free (the field, the solve's scratch and the geometry tables it needs), publishes them to the
 * grid, copies finished fields to host buffers, and records latencies.  Requests that arrive while
 * others run are therefore solved alongside them, and a result does not depend on what else is in
 * flight: it is bit-identical to fdgpu_solve_device of the same station.  The grid leaves the GPU
 * after idle_stop_us with nothing in flight and comes back with the next request.
 *
 * All functions may be called from any host thread. */
typedef struct fdgpu_server fdgpu_server;

typedef struct {
    long long hbm_bytes;   /* device memory the session holds for models, geometry tables and the
                              working sets of admitted solves; 0: half the free memory at open */
    int max_inflight;      /* requests admitted at once (published, running or being copied out);
                              0: twice the number of solver CTAs */
    int reserve_sms;       /* SMs left without a solver CTA, for the session's own small kernels and
                              for other work; at least 1; -1: 2 */
    int max_models;        /* model slots, e.g. 2 for P and S; 0: 2 */
    int idle_stop_us;      /* the grid leaves after this long with nothing in flight; 0: 2000 */
} fdgpu_serve_opts;

typedef struct {
    uint64_t id;           /* as returned by fdgpu_serve_submit */
    uint64_t tag;          /* the caller's tag */
    int32_t status;        /* FDGPU_OK or the failure */
    int32_t model_version; /* version of the model slot the request was solved against */
    double queue_ms;       /* submission to publication on the device */
    double latency_ms;     /* submission to the field being in the caller's buffer */
    double solve_ms;       /* the solve on its CTA (GPU timer) */
    fdgpu_stats stats;
} fdgpu_serve_result;

typedef struct {
    int64_t submitted, completed, failed;
    int64_t queued;          /* submitted, not yet admitted */
    int64_t inflight;        /* admitted, not yet completed */
    double p50_ms, p90_ms, p99_ms, max_ms, mean_ms;   /* latency of completed requests */
    double solve_p50_ms, solve_p99_ms;                /* GPU solve time of completed requests */
    double fields_per_s;     /* completed / (last completion - first submission) */
    double node_updates_per_s;
    int64_t node_updates;
    int64_t hbm_bytes;       /* session memory */
    int64_t hbm_used, hbm_peak;   /* held now, largest held */
    int32_t solver_ctas;     /* CTAs of the solver grid */
    int32_t grid_launches;   /* times the grid was launched */
    int64_t hist[40];        /* latency histogram: hist[k] counts latencies in [2^(k-10), 2^(k-9)) ms
                                (the first and last buckets are open-ended) */
} fdgpu_serve_metrics;

int fdgpu_serve_open(int device, const fdgpu_serve_opts *opts, fdgpu_server **out);

/* Set model slot `model` to a velocity model (mnx, mny, mnz floats, x fastest; host or device
 * memory).  It is converted to slowness on the device as the reference rounds it
 * (src/sphfd.c:689).  Requests submitted afterwards use the new version; requests submitted
 * before keep the one they were submitted against, which is freed when the last of them
 * completes.  *version (may be NULL) receives the new version number (1, 2, ...). */
int fdgpu_serve_set_model(fdgpu_server *sv, int model, const float *velocity, int mnx, int mny, int mnz,
                          int *version);

/* Queue one solve of station st against model slot `model` (st->ox/oy/oz place its window).
 * times (nx*ny*nz floats) receives the field: device memory (the solve writes it in place) or host
 * memory (pinned or not; copied when the solve is done).  It must stay valid until the request's
 * result has been polled.  init_times (host or device, may be NULL) is the starting field of a
 * srctype 2/3 station.  Returns at once; *id (may be NULL) receives the request id.
 * FDGPU_ETOOBIG: the request can never fit the session's memory. */
int fdgpu_serve_submit(fdgpu_server *sv, const fdgpu_station *st, int model, float *times, const float *init_times,
                       uint64_t tag, uint64_t *id);

/* Completed requests, in completion order: up to max results into out, *n of them.  Waits up to
 * timeout_ms for the first one (0: do not wait; -1: until one completes or nothing is left
 * outstanding). */
int fdgpu_serve_poll(fdgpu_server *sv, fdgpu_serve_result *out, int max, int timeout_ms, int *n);

/* Wait until every submitted request has completed (timeout_ms -1: no limit).  FDGPU_ETIMEDOUT if
 * the limit passed first; the requests go on, and a later drain or poll collects them. */
int fdgpu_serve_drain(fdgpu_server *sv, int timeout_ms);

int fdgpu_serve_metrics_get(fdgpu_server *sv, fdgpu_serve_metrics *m);

/* text of the session's last CUDA failure ("" if none) */
const char *fdgpu_serve_last_error(const fdgpu_server *sv);

/* Complete every outstanding request, stop the grid and free the session. */
int fdgpu_serve_close(fdgpu_server *sv);

/* ---- Event location on device fields --------------------------------------------------------
 *
 * The grid search of FDtomoC's sphfdloc (src/sphfdloc.c) over travel-time fields that are already
 * on the device (e.g. the fields a batch or a serving session just wrote): per event, a search over
 * the grid nodes from depth index kmin (:729-794), two subgrid refinements with trilinear lookups
 * (:840-1056, find_time :1305-1345), and the outlier / recovery passes that repeat the search
 * (:1086-1128).  Results are bit-identical to the reference's; reading the event files and writing
 * its report files stay with the caller. */
typedef struct {
    int nx, ny, nz;          /* the fields' grid */
    double x0, y0, z0;       /* longitude of x = 0 (rad), geocentric colatitude of y = 0 (rad), depth of
                                z = 0 (km) */
    double h, dq, df;        /* depth step (km), colatitude and longitude steps (rad) */
    float xmax, ymax, zmax;  /* far edges, as floats (src/sphfdloc.c:455-457) */
    double z0r;              /* radius at z = 0 (km) */
    int kmin;                /* first depth index of the node search (the spec's kmin - 1) */
    int ndiv, ndiv2;         /* subdivisions of the two refinements */
    int ivs;                 /* 0: an S time is the P field's time times vpvs */
    float vpvs;
    int nthres;              /* least number of accepted phases */
    float resthres, resthrep, stdmax;
} fdgpu_loc_grid;

typedef struct {
    int32_t field;           /* index of the phase's time field in d_fields */
    float obstime;           /* arrival minus the event's catalogue origin time, s */
    float pwt;               /* weight 1/(rwt*rwt) */
    char phase;              /* 'P' or 'S' */
    char good;               /* in: 0 for a phase marked '*'; out: the final flag */
    char pad[2];
} fdgpu_loc_obs;

typedef struct {
    int32_t status;          /* 0 accepted, 1 fewer than nthres phases left, 2 stdmin above stdmax */
    int32_t ngood;           /* phases accepted */
    int32_t nxx, nyy, nzz;   /* loop indices of the last improvement (0-based, as the reference's) */
    int32_t passes;          /* searches run (1 + redos) */
    double exm, eym, ezm;    /* hypocentre: longitude (rad), geocentric colatitude (rad), depth (km) */
    float stdmin, avrmin;    /* deviation and mean residual there */
} fdgpu_loc_result;

/* The grid of a sphfdloc spec (src/sphfdloc.c:382-395): degrees and km in, and the reference's
 * defaults for the search parameters (kmin 2, ndiv 20, ndiv2 20, ivs 1, vpvs 1.78, nthres 8,
 * resthres 0.5, resthrep 5, stdmax 15). */
void fdgpu_loc_grid_from_spec(fdgpu_loc_grid *g, int nx, int ny, int nz, double x0_deg, double y0_deg,
                              double z0_km, double h_km);

/* Locate nev events.  d_fields: device pointers to the time fields (nx*ny*nz floats each);
 * obs_offset (nev + 1 entries, obs_offset[0] = 0): event e's phases are obs[obs_offset[e] ..
 * obs_offset[e+1]), 1 to 800 of them; obs[].good is updated; resmin and tps (one per phase) receive
 * the residuals and the computed times at the final point; results one per event.  Runs on `stream`
 * (NULL: the context's) and returns when done. */
int fdgpu_locate(fdgpu_ctx *ctx, const fdgpu_loc_grid *g, const float *const *d_fields, int nfields, int nev,
                 const int *obs_offset, fdgpu_loc_obs *obs, float *resmin, float *tps, fdgpu_loc_result *results,
                 void *stream);

/* ---- Coarse-to-fine model on the device ---------------------------------------------------------
 *
 * FDtomoC's c2f (src/c2f.c): the inversion's coarse P and S velocity nodes interpolated to the fine
 * model sphfd reads, bit-identical to the reference's, so the model can go from the inversion to the
 * solver without leaving the device. */
typedef struct {
    int nxc, nyc, nzc;                    /* coarse nodes per axis */
    const int *igridx, *igridy, *igridz;  /* fine steps between neighbouring coarse nodes (nxc-1, ...) */
    double x0, y0, z0, h;                 /* origin and fine spacing (the spec's x0, y0, z0, h) */
} fdgpu_c2f_grid;

/* fine dimensions: 1 + the sum of each axis's steps */
int fdgpu_c2f_dims(const fdgpu_c2f_grid *g, int *nx, int *ny, int *nz);

/* coarse velocities (P then S, nxc*nyc*nzc each, x fastest; host or device memory) to fine
 * velocities (P then S, nx*ny*nz each; host or device memory), as c2f writes its .pvel and .svel
 * files (src/c2f.c:541-572). */
int fdgpu_c2f(fdgpu_ctx *ctx, const fdgpu_c2f_grid *g, const float *coarse, float *fine, void *stream);

/* The same for a loop that interpolates a new coarse model onto one grid every iteration: the plan
 * holds the grid's per-axis tables and the slowness scratch; fdgpu_c2f_run takes device buffers and
 * only queues the two kernels on `stream` (NULL: the context's).  A plan is used by one stream at a
 * time. */
typedef struct fdgpu_c2f_plan fdgpu_c2f_plan;
int fdgpu_c2f_plan_create(fdgpu_ctx *ctx, const fdgpu_c2f_grid *g, fdgpu_c2f_plan **out);
int fdgpu_c2f_run(fdgpu_c2f_plan *plan, const float *d_coarse, float *d_fine, void *stream);
void fdgpu_c2f_plan_destroy(fdgpu_c2f_plan *plan);

/* ---- sphrayderv's rays on the device fields (reference src/sphrayderv.c:1054-2232) ----------
 * For each observation (an event's phase at a station): the residual and hypocentre derivatives at
 * the event (:1366-1441), the ray traced from the event back down the travel-time gradient to the
 * station (:1444-2140), and its slowness derivatives on the coarse metagrid (:2155-2232), bit-
 * identical to the oracle with correctly rounded sin/cos/atan2.  The event loop's bookkeeping and
 * the output files stay with the caller (fdtomoc_gb300/rayderv.py writes them as the reference). */
typedef struct fdgpu_ray_grid {
    int nx, ny, nz;            /* fine grid */
    int nxc, nyc, nzc;         /* coarse grid */
    double x0, y0, z0;         /* origin: longitude (rad), geocentric colatitude (rad), depth (km) */
    double h, dq, df;          /* km, rad, rad (:470-525) */
    const float *gx, *gy, *gz; /* host: coarse node coordinates as the reference stores them (:779-788) */
} fdgpu_ray_grid;

typedef struct fdgpu_ray_obs {
    double ex, ey, ez;         /* event: longitude, colatitude (rad), depth (km) (:924-927) */
    double xs, ys, zs;         /* station: longitude, colatitude (rad), -elevation (km) (:835-838) */
    int field;                 /* index into d_fields: the station-phase's time field */
    int phase;                 /* 0 P, 1 S */
    float obstime;             /* arrival minus origin (s) */
    float pwt;                 /* 1 / rwt^2 */
    float tc;                  /* station correction */
    int pad;
} fdgpu_ray_obs;

enum {
    FDGPU_RAY_OK = 0,          /* reached the station: derivatives valid */
    FDGPU_RAY_NOTIME = 1,      /* a corner of the event's cell has no time (> 1e9) (:1357-1364) */
    FDGPU_RAY_LEFT = 2,        /* the ray left the model (:2037-2140) */
    FDGPU_RAY_STEPS = 3,       /* more than max_seg segments or cap derivatives (the reference has no limit) */
    FDGPU_RAY_COARSE = 4,      /* a segment midpoint beyond the coarse grid (the reference asserts) */
    FDGPU_RAY_OUTSIDE = 5,     /* a cell corner outside the field (the reference reads past it) */
};

typedef struct fdgpu_ray_result {
    int status;
    int nseg;
    double dt;                 /* residual obstime - (t + tc) (:1397-1400) */
    float resmin;              /* the same as float */
    float wet;                 /* sqrt(pwt) */
    float am[4];               /* wet, dt/dx wet, dt/dy wet, dt/dz wet (:1600-1604) */
    int nnz;                   /* nonzero coarse derivatives */
    int pad;
} fdgpu_ray_result;

/* Default limits for a grid: segments per ray and derivative entries per ray. */
int fdgpu_ray_default_limits(const fdgpu_ray_grid *g, int *max_seg, int *cap);

/* Trace nobs observations against device fields d_fields[0..nfields) (nz*ny*nx floats each).  obs and
 * res are host arrays; observation k's nonzero derivatives (raw du before the sqrt(pwt) weight,
 * ascending coarse node) go to idx/du[off[k] .. off[k+1]), off host (nobs+1), idx/du host arrays of
 * total_cap entries (FDGPU_ETOOBIG if the run has more; off and res are filled either way).
 * max_seg, cap <= 0: the defaults. */
int fdgpu_raytrace(fdgpu_ctx *ctx, const fdgpu_ray_grid *g, const float *const *d_fields, int nfields, int nobs,
                   const fdgpu_ray_obs *obs, int max_seg, int cap, fdgpu_ray_result *res, long long *off, int *idx,
                   float *du, long long total_cap, void *stream);

/* The locator a sphfdloc run calls: fdgpu_locate's contract with host fields (the default moves them to
 * device 0 and calls fdgpu_locate). */
typedef int (*fdgpu_loc_locator)(void *user, const fdgpu_loc_grid *g, const float *const *h_fields, int nfields,
                                 int nev, const int *obs_offset, fdgpu_loc_obs *obs, float *resmin, float *tps,
                                 fdgpu_loc_result *results);

/* Drop-in sphfdloc (src/sphfdloc.c main): reads the spec, its event file (leqsfil) and the time files its
 * phases name (<timedir>/<station>.ptimes|.stimes), locates every event (locator NULL: on the GPU), and
 * writes fhedfil, fdatfil, fsumfil and outlfil as the reference writes them.  The per-event split under
 * eqkdir and the log file are not made. */
int fdgpu_sphfdloc(const char *specfile, fdgpu_loc_locator locator, void *user);

/* The tracer a sphrayderv run calls: fdgpu_raytrace's contract with host fields (the default moves them
 * to device 0 and calls fdgpu_raytrace). */
typedef int (*fdgpu_ray_tracer)(void *user, const fdgpu_ray_grid *g, const float *const *h_fields, int nfields,
                                int nobs, const fdgpu_ray_obs *obs, fdgpu_ray_result *res, long long *off, int *idx,
                                float *du, long long total_cap);

/* Drop-in sphrayderv (src/sphrayderv.c main) for local earthquakes: reads the spec file, its station
 * list, event file and time files as the reference does, traces every observation (tracer NULL: on the
 * GPU), and writes dtdsfil, resfile, dtdhfil, bookfil, sclefil and hitfile as the reference writes them.
 * spacing_rule 1 replaces dq/df below 1e-4 rad by h/rearth as the reference does (:515-518); 0 keeps
 * the spec's spacing (the spacing sphfd used for the fields).  Teleseisms, shots, ivpvs and nomat are
 * refused with FDGPU_EINVAL. */
int fdgpu_sphrayderv(const char *specfile, int spacing_rule, fdgpu_ray_tracer tracer, void *user);

/* Drop-in sphfd() (src/sphfd.c:260): ac/av as the reference's (av[1] = "par=<file>"),
 * output_path = timedir.  Reads the velocity file, solves on the GPU, writes
 * <output_path>/<timefile> byte-for-byte as the reference does.  Inputs are read and checked before
 * the GPU is touched; the solve runs on the calling thread's current device (cudaSetDevice; 0 by
 * default) in a context of that thread, created on first use. */
int fdgpu_sphfd(int ac, char **av, const char *output_path);

/* Drop-in for main()'s OpenMP loop over a par list (src/sphfd.c:231-255): every entry is
 * "par=<file>"; all stations are solved together (stations sharing a velocity file share one read
 * of it and one device copy).  status[k] receives each station's result if status is non-NULL; the
 * return value is the first failure (or 0).  Runs on the calling thread's current device. */
int fdgpu_sphfd_parlist(int n, char **par_entries, const char *output_path, int *status);

/* The same over several GPUs of this process: the stations of each velocity-file group are dealt
 * round-robin over devices[0..ndev) (a device may be listed twice: two contexts share it), solved
 * by one worker thread per listed device, and written by the workers (each station to its own
 * file).  The velocity file is read once per group on the host.  Stations are independent, so the
 * files equal the single-device ones byte for byte.  The reference's counterpart is its OpenMP
 * parallel loop over par files (src/sphfd.c:247-255), one thread per station.  Calls of this
 * function must not overlap. */
int fdgpu_sphfd_parlist_devices(int n, char **par_entries, const char *output_path, int *status, int ndev,
                                const int *devices);

#ifdef __cplusplus
}
#endif
#endif
