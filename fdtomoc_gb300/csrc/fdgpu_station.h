/*
 * fdgpu_station.h — host-side set-up of one station solve, shared by the batch entry points
 * (fdgpu_host.cpp), the no-allocation entry point (fdgpu_noalloc.cu) and the serving session
 * (fdgpu_serve.cpp).
 *
 * It turns an fdgpu_station (sphfd()'s state after reading its par file) into the device record
 * fd_station_dev: the initial box and its restart preference (src/sphfd.c:766-825, :877-926,
 * :977-1003), the Cartesian source point and the box's trig values (:727-745), and the pointers
 * into the geometry tables, the slowness window, the field and the scratch.  Host arithmetic that
 * feeds the kernels uses the C library as the reference does; every file that includes this header
 * is compiled with -ffp-contract=off, so the doubles handed to the GPU are the reference's.
 */
#ifndef FDGPU_STATION_H
#define FDGPU_STATION_H

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>

#include "fdgpu.h"
#include "fdgpu_layout.h"

namespace fdh {

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* grid coordinates (src/sphfd.c:150-156) */
inline double qc(const fdgpu_station &s, int y) { return s.y0 + s.dq * (double)y; }
inline double fc(const fdgpu_station &s, int x) { return s.x0 + s.df * (double)x; }

inline long long max_face(const fdgpu_station &s)
{
    return std::max({(long long)s.nx * s.ny, (long long)s.nx * s.nz, (long long)s.ny * s.nz});
}

/* face-walk scratch per point of the largest face: key 8 | rec 8 | pst 4 | queue 4 | rq 8 | dag 2 */
constexpr size_t kFacePerPoint = 8 + 4 + 4 + 4 + 8 + 4 + 2;
inline size_t face_bytes(const fdgpu_station &s) { return align256(((size_t)max_face(s) + 16) * kFacePerPoint); }

/* sweep-graph arrays per grid node: stencil-state record, counter, queue, earlier-neighbour byte;
 * then the face instances, wait pairs, parked points and resume queue */
constexpr size_t kGraphPerNode = 8 + 4 + 4 + 1;
inline size_t graph_node_bytes(size_t nn) { return align256(nn * kGraphPerNode); }
inline int graph_instances(const fdgpu_station &s) { return s.nx + s.ny + s.nz + 8; }
inline size_t graph_bytes(const fdgpu_station &s)
{
    const size_t nn = (size_t)s.nx * s.ny * s.nz;
    return graph_node_bytes(nn) + align256((size_t)graph_instances(s) * sizeof(fd_ginst))
           + 8 * (size_t)FD_GWAIT_CAP + 8 * (size_t)FD_GPARK_CAP + 4 * (size_t)FD_GRQ_CAP;
}

/* geometry tables of one grid geometry: ysin | zrow | node | cell */
inline size_t geo_bytes(int ny, int nz)
{
    return align256(sizeof(double) * (size_t)ny) + align256(sizeof(double) * FD_Z_N * (size_t)nz)
           + align256(sizeof(double) * FD_N_N * (size_t)nz * ny)
           + align256(sizeof(double) * FD_C_N * (size_t)std::max(1, nz - 1) * std::max(1, ny - 1));
}

struct GeoPtrs {
    double *ysin, *zrow, *node, *cell;
};

inline GeoPtrs geo_carve(char *base, int ny, int nz)
{
    GeoPtrs g;
    g.ysin = reinterpret_cast<double *>(base);
    base += align256(sizeof(double) * (size_t)ny);
    g.zrow = reinterpret_cast<double *>(base);
    base += align256(sizeof(double) * FD_Z_N * (size_t)nz);
    g.node = reinterpret_cast<double *>(base);
    base += align256(sizeof(double) * FD_N_N * (size_t)nz * ny);
    g.cell = reinterpret_cast<double *>(base);
    return g;
}

/* sin(qc(y)) of every row, evaluated by the C library (the reference calls sin() per use) */
inline void ysin_table(const fdgpu_station &s, double *out)
{
    for (int y = 0; y < s.ny; y++) out[y] = std::sin(qc(s, y));
}

/* the argument checks every entry point makes (the source test is src/sphfd.c:533-538) */
inline int check_station(const fdgpu_station &s)
{
    if (s.nx < 2 || s.ny < 2 || s.nz < 2 || !(s.h > 0) || !(s.dq != 0) || !(s.df != 0)) return FDGPU_EINVAL;
    if ((long long)s.nx * s.ny > 0x7fffffffLL / 2 || max_face(s) > (1LL << 30)) return FDGPU_EINVAL;
    if (s.srctype == 1) {
        if (s.xs < 0 || s.ys < 0 || s.zs < 0 || s.xs > s.nx - 1 || s.ys > s.ny - 1 || s.zs > s.nz - 1)
            return FDGPU_ESOURCE;
        if (s.ncube < 0 || s.ncube > 64) return FDGPU_EINVAL;
    } else if (s.srctype == 2 || s.srctype == 3) {
        if (s.srcwall < 1 || s.srcwall > 6) return FDGPU_EPAR;
    } else {
        return FDGPU_EPAR;
    }
    return FDGPU_OK;
}

/* initial box of a point source (src/sphfd.c:766-825), in face order z1 z2 x2 x1 y1 y2 */
inline void point_box(const fdgpu_station &s, int wall[6], int dflag[6])
{
    const int nc = s.ncube;
    for (int f = 0; f < 6; f++) dflag[f] = 1;
    if (s.xs > nc) wall[3] = s.xs - (nc + 1); else { wall[3] = -1; dflag[3] = 0; }
    if (s.xs < s.nx - (nc + 1)) wall[2] = s.xs + (nc + 1); else { wall[2] = s.nx; dflag[2] = 0; }
    if (s.ys > nc) wall[4] = s.ys - (nc + 1); else { wall[4] = -1; dflag[4] = 0; }
    if (s.ys < s.ny - (nc + 1)) wall[5] = s.ys + (nc + 1); else { wall[5] = s.ny; dflag[5] = 0; }
    if (s.zs > nc) wall[0] = s.zs - (nc + 1); else { wall[0] = -1; dflag[0] = 0; }
    if (s.zs < s.nz - (nc + 1)) wall[1] = s.zs + (nc + 1); else { wall[1] = s.nz; dflag[1] = 0; }
}

/* box = one whole model wall (src/sphfd.c:877-926 and :5623-5674) */
inline void wall_box(const fdgpu_station &s, int srcwall, int wall[6], int dflag[6])
{
    for (int f = 0; f < 6; f++) dflag[f] = 1;
    if (srcwall == 1) wall[2] = 1; else { wall[2] = s.nx; dflag[2] = 0; }
    if (srcwall == 2) wall[3] = s.nx - 2; else { wall[3] = -1; dflag[3] = 0; }
    if (srcwall == 3) wall[5] = 1; else { wall[5] = s.ny; dflag[5] = 0; }
    if (srcwall == 4) wall[4] = s.ny - 2; else { wall[4] = -1; dflag[4] = 0; }
    if (srcwall == 5) wall[1] = 1; else { wall[1] = s.nz; dflag[1] = 0; }
    if (srcwall == 6) wall[0] = s.nz - 2; else { wall[0] = -1; dflag[0] = 0; }
}

/* preferred restart wall from the initial box (src/sphfd.c:977-1003) */
inline int resolve_headpref(const fdgpu_station &s, const int wall[6], int headpref)
{
    if (headpref <= 0) return headpref;
    const int x1 = wall[3], x2 = wall[2], y1 = wall[4], y2 = wall[5], z1 = wall[0], z2 = wall[1];
    long long head = (long long)s.nx * s.ny * s.nz;
    if (s.nx > 5 && x2 <= head) { headpref = 2; head = x2; }
    if (s.nx > 5 && (s.nx - 1 - x1) <= head) { headpref = 1; head = s.nx - 1 - x1; }
    if (s.ny > 5 && y2 <= head) { headpref = 4; head = y2; }
    if (s.ny > 5 && (s.ny - 1 - y1) <= head) { headpref = 3; head = s.ny - 1 - y1; }
    if (s.nz > 5 && z2 <= head) { headpref = 6; head = z2; }
    if (s.nz > 5 && (s.nz - 1 - z1) <= head) { headpref = 5; head = s.nz - 1 - z1; }
    return headpref;
}

/* doubles of the source box's trig table (4 per box column) */
inline int box_trig_count(const fdgpu_station &s) { return 4 * (2 * s.ncube + 1); }

/* cos/sin of the box's colatitudes then longitudes (src/sphfd.c:740-745) */
inline void box_trig(const fdgpu_station &s, double *out)
{
    const int w = 2 * s.ncube + 1;
    for (int j = 0; j < w; j++) {
        const double q = qc(s, s.ys - s.ncube + j), f = fc(s, s.xs - s.ncube + j);
        out[2 * j] = std::cos(q);
        out[2 * j + 1] = std::sin(q);
        out[2 * w + 2 * j] = std::cos(f);
        out[2 * w + 2 * j + 1] = std::sin(f);
    }
}

/* The device record of one solve.  `slowness` is the model's (0,0,0) with strides (1, s_sy, s_sz);
 * the station reads its window at (ox, oy, oz).  init_mode 0: a point source whose box the kernel
 * fills; 1: T already holds the starting field.  `face` holds face_bytes(s); `graph` holds
 * graph_bytes(s), or is null for face walks only.  box_trig points at the device copy of
 * box_trig(s). */
inline void fill_station(fd_station_dev &d, const fdgpu_station &s, const GeoPtrs &g, float *T, const float *slowness,
                         long long s_sy, long long s_sz, int init_mode, char *face, char *graph,
                         const double *box_trig_dev, fd_station_stats *stats)
{
    std::memset(&d, 0, sizeof d);
    d.g.nx = s.nx; d.g.ny = s.ny; d.g.nz = s.nz;
    d.g.h = s.h; d.g.inv_h = 1.0 / s.h; d.g.dq = s.dq; d.g.df = s.df; d.g.is_h = 1.0 / (s.h * s.h);
    d.g.zrow = g.zrow; d.g.ysin = g.ysin; d.g.node = g.node; d.g.cell = g.cell;
    d.T = T;
    d.S = slowness + (long long)s.oz * s_sz + (long long)s.oy * s_sy + s.ox;
    d.s_sy = s_sy; d.s_sz = s_sz;
    if (s.srctype == 1) point_box(s, d.wall, d.dflag);
    else wall_box(s, s.srcwall, d.wall, d.dflag);
    const int grow[6] = {s.kminus, s.kplus, s.iplus, s.iminus, s.jminus, s.jplus};
    for (int f = 0; f < 6; f++) d.grow[f] = grow[f];
    d.radius = s.srctype == 1 ? s.ncube : 1;
    d.reverse = s.reverse;
    d.headpref = resolve_headpref(s, d.wall, s.headpref);
    d.maxrad = s.maxrad;
    d.carry_t0 = 0.f; d.carry_t4 = 0.f;
    d.init_mode = init_mode;
    d.xs = s.xs; d.ys = s.ys; d.zs = s.zs; d.ncube = s.ncube;
    /* Cartesian source point (src/sphfd.c:727-729) */
    const double fxss = s.src_geo[0], fyss = s.src_geo[1], fzss = s.src_geo[2];
    d.src_xyz[0] = fzss * std::cos(fyss);
    d.src_xyz[1] = fzss * std::sin(fyss) * std::cos(fxss);
    d.src_xyz[2] = fzss * std::sin(fyss) * std::sin(fxss);
    d.box_trig = box_trig_dev;
    const size_t m = (size_t)max_face(s);
    d.scr.key = reinterpret_cast<unsigned long long *>(face);
    d.scr.rec = reinterpret_cast<float2 *>(face + 8 * m);
    d.scr.pst = reinterpret_cast<int *>(face + 16 * m);
    d.scr.queue = reinterpret_cast<int *>(face + 20 * m);
    d.scr.rq = reinterpret_cast<int *>(face + 24 * m);
    d.scr.dag = reinterpret_cast<unsigned char *>(face + 32 * m);
    if (graph) {
        /* 8-byte records first, then the 4-byte arrays, then the bytes */
        const size_t nn = (size_t)s.nx * s.ny * s.nz;
        d.scr.grec = reinterpret_cast<float2 *>(graph);
        d.scr.gcnt = reinterpret_cast<unsigned *>(graph + 8 * nn);
        d.scr.gqueue = reinterpret_cast<int *>(graph + 12 * nn);
        d.scr.gemask = reinterpret_cast<unsigned char *>(graph + 16 * nn);
        char *tb = graph + graph_node_bytes(nn);
        d.scr.ginst_cap = graph_instances(s);
        d.scr.ginst = reinterpret_cast<fd_ginst *>(tb);
        tb += align256((size_t)d.scr.ginst_cap * sizeof(fd_ginst));
        d.scr.gwait = reinterpret_cast<int2 *>(tb);
        tb += 8 * (size_t)FD_GWAIT_CAP;
        d.scr.gpark = reinterpret_cast<int2 *>(tb);
        tb += 8 * (size_t)FD_GPARK_CAP;
        d.scr.grq = reinterpret_cast<int *>(tb);
    }
    d.max_face_pad = (max_face(s) + 15) & ~15LL;
    d.stats = stats;
}

/* the public statistics of one solve from the device record */
inline void copy_stats(fdgpu_stats &o, const fd_station_stats &h)
{
    std::memset(&o, 0, sizeof o);
    o.status = h.status ? FDGPU_ESCHED : FDGPU_OK;
    o.sweeps = h.sweeps;
    o.node_updates = h.node_updates;
    o.faces = h.faces;
    o.rounds = h.rounds;
    o.deferred = h.deferred;
    for (int j = 0; j < 5; j++) o.stencils[j] = h.stencils[j];
    for (int j = 0; j < 8; j++) o.restart_wall[j] = h.restart_wall[j];
    for (int j = 0; j < 6; j++) o.phase_cycles[j] = h.phase_cycles[j];
    o.t_start_ns = h.t_start_ns;
    o.t_end_ns = h.t_end_ns;
    o.pipelined_sweeps = h.pipelined_sweeps;
    o.sm = h.sm;
    o.detail = h.status;
}

}  // namespace fdh

#endif
