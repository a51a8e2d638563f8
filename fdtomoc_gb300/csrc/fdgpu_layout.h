/*
 * fdgpu_layout.h — device-side data layout shared by the host runtime and the kernels.
 *
 * One station solve = one sphfd() call (reference: src/sphfd.c:260-5803).  Its state on the GPU:
 *   T      the station's travel-time field, float32, x fastest (nx*ny*nz), also the output;
 *   S      slowness (float32, 1/v rounded as the reference does), a window into a model that
 *          may be larger than the station grid and shared by many stations;
 *   geometry tables, shared by every station with the same grid geometry (see below);
 *   face scratch for the dependency-ordered face walk (keys, in-degrees, two work lists,
 *   per-point stencil-state records), sized for the station's largest face.
 *
 * Geometry tables.  Every floating-point quantity the stencils take from the grid geometry is
 * computed once, with the reference's own formula and operand order, so that the per-point work
 * only touches travel times and slownesses:
 *   zrow[z][FD_Z*]      radius rc(z) and rc(z)*dq with its reciprocal;
 *   ysin[y]             sin(qc(y)), evaluated by the host C library (the reference calls sin());
 *   node[z][y][FD_N*]   the products r*sin(q)*df and r*df*sin(q), reciprocals, and the "a"
 *                       coefficient (with 1/(2a)) for the three distance pairs that the
 *                       new-edge and 2-D stencils use;
 *   cell[zc][yc][FD_C*] every fdsph3d coefficient for the cell with corner (yc, zc): the
 *                       quadratic's a for each of the cell's four (r,q) corners and 1/(2a),
 *                       the point-row products (doubled) and the pair products (doubled).
 */
#ifndef FDGPU_LAYOUT_H
#define FDGPU_LAYOUT_H

#include <stdint.h>

/* zrow entries */
enum { FD_Z_R = 0, FD_Z_RDQ, FD_Z_INV_RDQ, FD_Z_N };
/* node entries */
enum {
    FD_N_RSDF = 0,   /* (rc(z)*sin(qc(y)))*df */
    FD_N_INV_RSDF,   /* 1/that, correctly rounded */
    FD_N_RDFS,       /* (rc(z)*df)*sin(qc(y)) */
    FD_N_A_SH,       /* 1/RSDF^2 + 1/h^2           (each term as the reference rounds it) */
    FD_N_I2A_SH,     /* 1/(2a) */
    FD_N_A_QH,       /* 1/RDQ^2 + 1/h^2 */
    FD_N_I2A_QH,
    FD_N_A_SQ,       /* 1/RSDF^2 + 1/RDQ^2 */
    FD_N_I2A_SQ,
    FD_N_N
};
/* cell entries: diag[ri][qi] (4), inv2a[ri][qi] (4), prow2[r7][q7][ri][qi][sx] (32), pair2[ri][qi][rj][qj][sx] (32) */
#define FD_C_DIAG(ri, qi) ((ri) * 2 + (qi))
#define FD_C_I2A(ri, qi) (4 + (ri) * 2 + (qi))
#define FD_C_PROW(r7, q7, ri, qi, sx) (8 + ((((r7) * 2 + (q7)) * 2 + (ri)) * 2 + (qi)) * 2 + (sx))
#define FD_C_PAIR(ri, qi, rj, qj, sx) (40 + ((((ri) * 2 + (qi)) * 2 + (rj)) * 2 + (qj)) * 2 + (sx))
#define FD_C_N 72

typedef struct {
    int nx, ny, nz;
    double h, inv_h, dq, df;
    double is_h;             /* 1/(h*h) as the reference rounds it */
    const double *zrow;
    const double *ysin;
    const double *node;
    const double *cell;
} fd_geo_dev;

/* Per-station solve statistics (the counters the reference prints, plus schedule counters). */
typedef struct {
    int32_t status;          /* 0 ok; FDGPU_E* on failure */
    int32_t sweeps;
    int64_t node_updates;
    int64_t faces;
    int64_t rounds;          /* warp chunks over all walks */
    int64_t deferred;        /* points that waited for an earlier point's (t0,t4) */
    int64_t stencils[5];     /* stencil evaluations by kind (3d ne 2d nf 1d), after pruning */
    int32_t restart_wall[8]; /* how often each wall (1..6) was chosen for a restart */
    int64_t phase_cycles[6]; /* with FDGPU_PHASE_TIMERS: warp cycles summed over warps in face
                                set-up, phases A, B, C and the face walks (zero otherwise) */
    int64_t t_start_ns, t_end_ns; /* GPU global timer when the station's solve began and ended */
    int32_t pipelined_sweeps;
    int32_t sm;              /* the SM whose CTA ran the solve */
} fd_station_stats;

/* One face instance of a sweep graph: a face walked at one wall position, with its point
 * rectangle and its completion state. */
typedef struct {
    int face, layer, ulo, uhi, vlo, vhi, nuf, n;
    int nkeyed, ndone;             /* points whose sort key is final; points done */
    int evwait, pad;               /* bit 1: points wait for all keys, bit 2: for all points done */
    unsigned long long exitkey;    /* largest key of a point that made a writer call (0: none) */
} fd_ginst;

/* sizes of the small sweep-graph tables */
#define FD_GWAIT_CAP 65536   /* (awaited point, waiting point) pairs */
#define FD_GPARK_CAP 65536   /* points parked on an instance event, and their wait states */
#define FD_GRQ_CAP 262144    /* resume queue */

/* Face-walk scratch of one station, sized for its largest face m (34 bytes per point):
 * key 8m | rec 8m | pst 4m | queue 4m | rq 8m | dag 2m (+32). */
typedef struct {
    unsigned long long *key;   /* (time bits of the inner-layer node << 32) | fill index */
    float2 *rec;               /* (t0,t4) the point left in the stencil state; NaN if no writer */
    int *pst;                  /* -1 pending, -2 done, >= 0 pending with that point waiting on it */
    int *queue;                /* ready points, one entry per point */
    int *rq;                   /* points waiting for an earlier point's (t0,t4), 2 entries per point */
    unsigned char *dag;        /* in-degree and earlier-neighbour bytes (2 per point) when they do
                                  not fit in shared memory */
    /* sweep graphs (gcnt NULL: not available, every face is walked on its own).  Per grid node:
     * dependency counter word (inner block pending in bits 0-7, same-instance neighbours in 8-15,
     * other instances' nodes in 16-23, a point waits on it bit 29, done bit 30, sort key final
     * bit 31), ready queue, earlier-neighbour byte, stencil-state record.  Small tables: the
     * sweep's face instances, wait pairs, parked points, resume queue. */
    unsigned *gcnt;
    int *gqueue;
    unsigned char *gemask;
    float2 *grec;
    fd_ginst *ginst;
    int ginst_cap;
    int2 *gwait;
    int2 *gpark;
    int *grq;
} fd_scratch_dev;

typedef struct {
    fd_geo_dev g;
    float *T;
    const float *S;            /* slowness at the station's (0,0,0) */
    long long s_sy, s_sz;      /* slowness strides in y and z (x stride is 1) */
    /* walls and flags in face order TOP BOTTOM EAST WEST NORTH SOUTH: z1 z2 x2 x1 y1 y2 */
    int wall[6], dflag[6], grow[6];
    int radius, reverse, headpref, maxrad;
    float carry_t0, carry_t4;  /* stale (t0,t4) before the first face (0,0 at start) */
    /* point-source initialisation (init_mode 0): box filled on the device */
    int init_mode;             /* 0: point source box; 1: T already holds the initial field */
    int xs, ys, zs, ncube;
    double src_xyz[3];         /* Cartesian source point (x1p, y1p, z1p of src/sphfd.c:727-729) */
    const double *box_trig;    /* per box column: cos q, sin q (y) then cos f, sin f (x) */
    fd_scratch_dev scr;
    long long max_face_pad;    /* largest face, rounded up to 16 points */
    fd_station_stats *stats;
    /* bounds of the walk's waits in SM clock cycles (0: the built-in ones): a worker idle this long
     * without progress, and a whole walk running this long, end the solve with a status */
    long long wait_cycles, walk_cycles;
} fd_station_dev;

/* Request loop of a serving session.  The host publishes station records; each CTA of the
 * long-running solver grid claims the next one, solves it and flags it done, until the host asks
 * idle CTAs to leave.  The host-side arrays are pinned and mapped (the CTAs read and write them
 * across the host link); only the claim counter lives in device memory.
 *   desc[e], gen[e]  entry e's station record and the generation (request number + 1) it holds;
 *   order[k % ring]  the entry of the k-th published request;
 *   tail             requests published (the host raises it after writing desc, gen and order);
 *   head             requests claimed (device; a CTA claims k by moving head from k to k + 1);
 *   done[e]          set to gen[e] once entry e's solve has finished and its field is written;
 *   exitf[c]         1 once CTA c (cta_id0 + blockIdx.x) has left the loop;
 *   stop             non-zero: a CTA with nothing to claim leaves. */
typedef struct {
    const fd_station_dev *desc;
    const unsigned long long *gen;
    const int *order;
    const unsigned long long *tail;
    unsigned long long *head;
    unsigned long long *done;
    int *exitf;
    const int *stop;
    int ring;
    int pad;
    long long idle_ns;         /* a CTA with nothing to claim for this long leaves on its own */
} fd_serve_queue;

#endif
