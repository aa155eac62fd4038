// sm_103a kernels of the per-step particle update.
//
// One step is four launches on the handle's stream (captured in a CUDA graph by the host):
//   k_scan     exclusive scan of the cell-list counts; block bases from per-tile counts that the
//              previous step accumulated (no inter-block waiting); R extra blocks finalize the
//              previous step's order parameter per replica
//   k_scatter  counting-sort scatter: tmp[start[key] + rank] = slot (rank from atomics)
//   k_order    orders each cell's particles by particle id (so that the neighbour visiting order,
//              and every floating-point sum, is the same on every run) and writes the state in
//              that sorted order: the step kernel reads its own state coalesced and the
//              candidates of a cell run from consecutive addresses
//   k_step     fused pair sums + tangent projection + polarity update + chart advance + seam
//              wrap + face location + chart->3D map + next-step cell key/count + order partials
// (k_finalize runs the same per-replica finalize on its own before the series is read.)
// Replaces (reference): Locomotion::simulate_flight + ForceHelper + OrientationHelper
// (Locomotion.cpp:57-162, ForceHelper.cpp:34-104, OrientationHelper.cpp:29-116),
// EuclideanTiling::diagonal_seam_edges_square_border (EuclideanTiling.cpp:31-208),
// CellHelper::get_r3d (CellHelper.cpp:71-160), Validation (Validation.cpp:40-72),
// count_particle_neighbors (2DTissue.cpp:254-268), calculate_order_parameter (LinearAlgebra.cpp:90-105).
//
// State per particle (structure of arrays):
//   pos = (x, y, z, theta)  3D position and chart polarity angle
//   pol = (px, py, pz, face) unit 3D polarity normalize(J_face (cos theta, sin theta)) and the
//                            containing chart face (stored with the polarity so that a
//                            neighbour's polarity is one load)
//   uv, id, key (cell bucket)
// The step kernel writes the "unsorted" arrays (in the previous cell order); k_order writes the
// sorted copy (s-prefixed) that the next step kernel reads.
//
// Face record (16 reals, 64 bytes in FP32): [0..5] chart corners a, b, c (CCW); [6] canonical
// edge bits (bit k: edge k evaluated reversed and negated); [7] A.x; [8..13] J = dX/d(uv),
// column u = [8..10], column v = [11..13]; [14] A.y; [15] A.z (A = 3D image of a). The normal and
// the pseudo-inverse of J are derived from J where needed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tds.h"
#include "philox.cuh"

namespace tdsk {

enum : int {
    ST_NONFINITE = 1,
    ST_WRAP = 2,
    ST_LOCATE = 4,
    ST_CELL = 16,
};

constexpr int kRec = 16;          // reals per face record
constexpr int kMaxWraps = 8;      // seam wraps per particle per step
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // buckets per scan tile
constexpr int kStepThreads = 256;  // default block of k_step
constexpr int kPhiCopies = 32;    // spread the order-parameter atomics over copies

template <typename real>
struct alignas(4 * sizeof(real)) R4 {
    real x, y, z, w;
};
template <typename real>
struct alignas(2 * sizeof(real)) R2 {
    real x, y;
};

// Per-replica parameters and the replica's cell level (device copy).
template <typename real>
struct RepParams {
    real twoR, inv_twoR, k, adh_scale;  // adh_scale = k_adh / (r_max - 2R)
    real r_max2, v0, mu, inv_tau;
    real align, eta, dt, inv_h;
    real ox, oy, oz, inv_adh_w;           // cell-grid origin; 1 / (r_max - 2R)
    double phiscale;                      // order-parameter fixed point (warp sums -> int64)
    double inv_n;                         // 1 / particles in this replica
    int force_mode, base, C, gx;          // bucket base, surface cells, grid size
    int gy, gz, row_off, n;               // row table offset of the level
    int off, desc_off, pad4, pad5;        // off: global index of the replica's first particle;
                                          // desc_off: the level's descriptor offset (uint4 units)
};

// The constants of the pair force (a replica's).
template <typename real>
struct PairC {
    real r_max2, twoR, inv_twoR, k, adh_scale;
};

template <typename real>
struct StepArgs {
    const R4<real>* pos;  // state in sorted order (k_order output)
    const R4<real>* pol;
    const R2<real>* uv;
    const int* ids;
    R4<real>* pos_o;  // outputs, same order
    R4<real>* pol_o;
    R2<real>* uv_o;
    int* ids_o;
    R2<real>* vel_o;
    int* cnt_o;
    int* key_o;
    const int* key_in;  // cell bucket of each particle (sorted order)
    const uint4* desc;  // per-cell neighbour-run descriptors, all levels
    const int* start;
    int* count;
    int* tile_sum;  // [2][n_tiles]
    int n_tiles;
    const real* rec;
    const int4* adj;
    int G;
    const int* bin_start;
    const int* bin_faces;
    const int4* rows;  // row records (two int4 per grid row, see bucket_of)
    const int4* ivals;
    const RepParams<real>* reps;
    int local_bits;
    real cx, cy, cz;
    const real* noise;  // nullable: angle increments by global particle index
    unsigned long long* phi_acc;
    int* phi_pending;  // set: this step's order parameter awaits finalizing
    const long long* d_step;
    unsigned long long seed;
    int* status;
    int N;
    int single;  // every replica has the same pair constants, held in pc0
    PairC<real> pc0;
    RepParams<real> rp0;  // the replica's parameters when there is one (read from the constant bank)
    int* nbr_list;  // neighbour export (the NBR instantiation only): nbr_cap ids per particle
    int nbr_cap;
    R4<real>* sum_f;  // the pair sums by slot (the STORE instantiation only): (F, m.x)
    R2<real>* sum_m;  //   and (m.y, m.z), for the adjoint's reverse step
};

// ---------------------------------------------------------------------------------------------
// math helpers (float / double overloads)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float d_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double d_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ void d_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void d_sincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float d_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double d_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float d_floor(float x) { return floorf(x); }
__device__ __forceinline__ double d_floor(double x) { return floor(x); }
__device__ __forceinline__ float d_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double d_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float d_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double d_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float d_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double d_rsqrt(double x) { return 1.0 / sqrt(x); }

__device__ __forceinline__ bool is_finite(float x) { return isfinite(x); }
__device__ __forceinline__ bool is_finite(double x) { return isfinite(x); }
__device__ __forceinline__ float face_to_real(int f, float) { return __int_as_float(f); }
__device__ __forceinline__ double face_to_real(int f, double) { return (double)f; }
__device__ __forceinline__ int real_to_face(float v) { return __float_as_int(v); }
__device__ __forceinline__ int real_to_face(double v) { return (int)v; }

template <typename real>
__device__ __forceinline__ real kPi() {
    return (real)3.14159265358979323846;
}

// Quad k (reals 4k..4k+3) of a face record: records are 16 reals aligned to their size, so each
// is read with four vector loads instead of sixteen scalar ones.
template <typename real>
__device__ __forceinline__ R4<real> rq(const real* r, int k) {
    return reinterpret_cast<const R4<real>*>(r)[k];
}

// unit 3D polarity from the chart angle on face record g: normalize(J (cos th, sin th))
template <typename real>
__device__ __forceinline__ void polarity3(const real* g, real th, real& px, real& py, real& pz) {
    real sn, cs;
    d_sincos(th, &sn, &cs);
    const R4<real> q2 = rq(g, 2), q3 = rq(g, 3);
    const real qx = q2.x * cs + q2.w * sn, qy = q2.y * cs + q3.x * sn, qz = q2.z * cs + q3.y * sn;
    const real qn = d_sqrt(qx * qx + qy * qy + qz * qz);
    px = qx / qn, py = qy / qn, pz = qz / qn;
}

// ---------------------------------------------------------------------------------------------
// point location in the UV chart (canonical edge orientation => watertight)
// ---------------------------------------------------------------------------------------------
template <typename real>
__device__ __forceinline__ real orient(real Px, real Py, real Qx, real Qy, real px, real py) {
    return d_fma(Qx - Px, py - Py, -d_mul(Qy - Py, px - Px));
}
template <typename real>
__device__ __forceinline__ void edge_values(const real* r, real px, real py, real e[3]) {
    const R4<real> q0 = rq(r, 0), q1 = rq(r, 1);
    const int bits = (int)q1.z;
    const real P[3][2] = {{q0.x, q0.y}, {q0.z, q0.w}, {q1.x, q1.y}};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int k1 = (k + 1) % 3;
        e[k] = (bits >> k & 1) ? -orient(P[k1][0], P[k1][1], P[k][0], P[k][1], px, py)
                               : orient(P[k][0], P[k][1], P[k1][0], P[k1][1], px, py);
    }
}
template <typename real>
__device__ __forceinline__ real min_edge(const real* r, real px, real py) {
    real e[3];
    edge_values(r, px, py, e);
    return fmin(e[0], fmin(e[1], e[2]));
}
template <typename real>
__device__ __forceinline__ real face_score(const real* r, real px, real py) {
    real e[3];
    edge_values(r, px, py, e);
    const R4<real> q0 = rq(r, 0), q1 = rq(r, 1);
    const real c[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
    real s = (real)1e30;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int k1 = (k + 1) % 3;
        const real ex = c[2 * k1] - c[2 * k], ey = c[2 * k1 + 1] - c[2 * k + 1];
        s = fmin(s, e[k] / d_sqrt(ex * ex + ey * ey));
    }
    return s;
}

// Unit normal and pseudo-inverse Jp = (J^T J)^-1 J^T of a face's chart map.
template <typename real>
__device__ __forceinline__ void face_frame(const real* g, real n[3], real Jp[6]) {
    const R4<real> q2 = rq(g, 2), q3 = rq(g, 3);
    const real ux = q2.x, uy = q2.y, uz = q2.z, vx = q2.w, vy = q3.x, vz = q3.y;
    const real cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    const real ic = d_rsqrt(cx * cx + cy * cy + cz * cz);
    n[0] = cx * ic, n[1] = cy * ic, n[2] = cz * ic;
    const real g11 = ux * ux + uy * uy + uz * uz, g12 = ux * vx + uy * vy + uz * vz, g22 = vx * vx + vy * vy + vz * vz;
    const real idet = (real)1 / (g11 * g22 - g12 * g12);
    const real a11 = g22 * idet, a12 = -g12 * idet, a22 = g11 * idet;
    Jp[0] = a11 * ux + a12 * vx, Jp[1] = a11 * uy + a12 * vy, Jp[2] = a11 * uz + a12 * vz;
    Jp[3] = a12 * ux + a22 * vx, Jp[4] = a12 * uy + a22 * vy, Jp[5] = a12 * uz + a22 * vz;
}

// chart point -> 3D on face record h (multiply-adds written out: the step and the state load
// produce the same bits for the same chart point)
template <typename real>
__device__ __forceinline__ void face_map(const real* h, real u, real v, real& x, real& y, real& z) {
    const R4<real> q0 = rq(h, 0), q1 = rq(h, 1), q2 = rq(h, 2), q3 = rq(h, 3);
    const real du = u - q0.x, dv = v - q0.y;
    x = d_fma(q2.w, dv, d_fma(q2.x, du, q1.w));
    y = d_fma(q3.x, dv, d_fma(q2.y, du, q3.z));
    z = d_fma(q3.y, dv, d_fma(q2.z, du, q3.w));
}
template <typename real>
__device__ __forceinline__ int bin_coord(real x, int G) {
    int b = (int)d_floor(x * (real)G);
    return b < 0 ? 0 : (b >= G ? G - 1 : b);
}
// 1. keep f_old if strictly inside; 2. an edge-neighbour of f_old that strictly contains p;
// 3. lowest-index closed-containing face; 4. best score (nearest face).
template <typename real>
__device__ int locate(const real* rec, const int4* adj, int G, const int* bs, const int* bf, real px, real py,
                      int f_old, int& mode) {
    mode = 0;
    real e[3];
    edge_values(rec + (size_t)f_old * kRec, px, py, e);
    if (fmin(e[0], fmin(e[1], e[2])) > (real)0) return f_old;
    if (adj) {
        // the neighbour across edge k can strictly contain p only if p lies strictly outside
        // that edge (shared edges give exactly negated values), so only those are tested
        const int4 A = adj[f_old];
        const int nb[3] = {A.x, A.y, A.z};
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (e[k] < (real)0 && nb[k] >= 0 && min_edge(rec + (size_t)nb[k] * kRec, px, py) > (real)0) return nb[k];
    }
    const int bx = bin_coord(px, G), by = bin_coord(py, G);
    const int b = by * G + bx;
    const int e1 = bs[b + 1];
    for (int e = bs[b]; e < e1; ++e) {
        const int g = bf[e];
        if (min_edge(rec + (size_t)g * kRec, px, py) >= (real)0) {
            mode = 1;
            return g;
        }
    }
    int best = f_old;
    real bsc = -(real)1e30;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = bx + dx, y = by + dy;
            if (x < 0 || y < 0 || x >= G || y >= G) continue;
            const int bb = y * G + x;
            for (int e = bs[bb]; e < bs[bb + 1]; ++e) {
                const int g = bf[e];
                const real s = face_score(rec + (size_t)g * kRec, px, py);
                if (s > bsc || (s == bsc && g < best)) bsc = s, best = g;
            }
        }
    mode = 2;
    return best;
}

// ---------------------------------------------------------------------------------------------
// seam wrap on the unit-square chart (gluing maps of EuclideanTiling::processPoints,
// EuclideanTiling.cpp:112-154); first side crossed along the segment; bounded.
// ---------------------------------------------------------------------------------------------
// The chart vectors (vx, vy) (velocity) and (wx, wy) (polarity direction) are rotated with the
// gluing map's linear part; the polarity angle is atan2(wy, wx) afterwards.
template <typename real>
__device__ int seam_wrap(real sx, real sy, real& ex, real& ey, real& vx, real& vy, real& wx, real& wy, int& nw) {
    int excl = -1;
    int w = 0;
    const real one = (real)1, zero = (real)0;
    for (; w < kMaxWraps; ++w) {
        if (ex >= zero && ex <= one && ey >= zero && ey <= one) break;
        int best = -1;
        real tb = (real)1e30;
        if (excl != 0 && ex < zero) {
            const real t = sx / (sx - ex), y = sy + t * (ey - sy);
            if (y >= zero && y <= one && t < tb) tb = t, best = 0;
        }
        if (excl != 1 && ex > one) {
            const real t = (one - sx) / (ex - sx), y = sy + t * (ey - sy);
            if (y >= zero && y <= one && t < tb) tb = t, best = 1;
        }
        if (excl != 2 && ey > one) {
            const real t = (one - sy) / (ey - sy), x = sx + t * (ex - sx);
            if (x >= zero && x <= one && t < tb) tb = t, best = 2;
        }
        if (excl != 3 && ey < zero) {
            const real t = sy / (sy - ey), x = sx + t * (ex - sx);
            if (x >= zero && x <= one && t < tb) tb = t, best = 3;
        }
        if (best < 0) {
            nw = w;
            return 2;
        }
        real qx = sx + tb * (ex - sx), qy = sy + tb * (ey - sy);
        if (best == 0) qx = zero;
        if (best == 1) qx = one;
        if (best == 2) qy = one;
        if (best == 3) qy = zero;
        qx = fmin(one, fmax(zero, qx));
        qy = fmin(one, fmax(zero, qy));
        real nx, ny, vnx, vny;
        const real two = (real)2;
        if (best == 0) {
            sx = qy, sy = -qx;
            nx = ey, ny = -ex;
        } else if (best == 1) {
            sx = qy, sy = two - qx;
            nx = ey, ny = two - ex;
        } else if (best == 2) {
            sx = two - qy, sy = qx;
            nx = two - ey, ny = ex;
        } else {
            sx = -qy, sy = qx;
            nx = -ey, ny = ex;
        }
        ex = nx, ey = ny;
        if (best <= 1) {  // rotation by -90 degrees
            vnx = vy, vny = -vx;
            vx = vnx, vy = vny;
            vnx = wy, vny = -wx;
        } else {  // rotation by +90 degrees
            vnx = -vy, vny = vx;
            vx = vnx, vy = vny;
            vnx = -wy, vny = wx;
        }
        wx = vnx, wy = vny;
        excl = (best == 0) ? 3 : (best == 1) ? 2 : (best == 2) ? 1 : 0;
    }
    nw = w;
    if (!(ex >= zero && ex <= one && ey >= zero && ey <= one)) {
        ex = fmin(one, fmax(zero, ex));
        ey = fmin(one, fmax(zero, ey));
        return 1;
    }
    return 0;
}


// ---------------------------------------------------------------------------------------------
// compact surface-cell list
// ---------------------------------------------------------------------------------------------
template <typename real>
__device__ __forceinline__ void cell_coords(const RepParams<real>& rp, real x, real y, real z, int& ix, int& iy,
                                            int& iz) {
    // clamped into the grid interior so that every lookup stays in bounds (positions on the mesh
    // are at least two cells inside; NaN converts to 0 and is clamped)
    ix = min(max((int)d_floor((x - rp.ox) * rp.inv_h), 1), rp.gx - 2);
    iy = min(max((int)d_floor((y - rp.oy) * rp.inv_h), 1), rp.gy - 2);
    iz = min(max((int)d_floor((z - rp.oz) * rp.inv_h), 1), rp.gz - 2);
}
// bucket of a position: base + surface-cell id, or base + C when the cell is not a surface cell.
// Row records are two int4 per grid row (iz, iy): {x_lo, x_hi, first id, intervals} and the same for
// the second interval with the index of the row's intervals in `ivals` in place of the count. A row
// crosses the surface in at most two x-intervals on a convex or mildly bumpy surface, so the lookup
// is one 32-byte load; rows with more intervals continue in `ivals`.
template <typename real>
__device__ __forceinline__ int bucket_of(const RepParams<real>& rp, const int4* rows, const int4* ivals, real x,
                                         real y, real z, bool& lost) {
    int ix, iy, iz;
    cell_coords(rp, x, y, z, ix, iy, iz);
    const int4* R = rows + 2 * (size_t)(rp.row_off + iz * rp.gy + iy);
    const int4 A = R[0], B = R[1];
    lost = false;
    if (A.w > 0 && ix >= A.x && ix <= A.y) return rp.base + A.z + ix - A.x;
    if (A.w > 1 && ix >= B.x && ix <= B.y) return rp.base + B.z + ix - B.x;
    for (int k = 2; k < A.w; ++k) {
        const int4 I = ivals[B.w + k];
        if (ix >= I.x && ix <= I.y) return rp.base + I.z + ix - I.x;
    }
    lost = true;
    return rp.base + rp.C;
}

__device__ __forceinline__ void add_tile(int* tile_sum, int key) {
    // warp-aggregated count of keys per scan tile (keys of a warp are nearly always in one tile)
    const int tile = key / kScanTile;
    const unsigned act = __activemask();
    const int leader = __ffs(act) - 1;
    const int t0 = __shfl_sync(act, tile, leader);
    if (__all_sync(act, tile == t0)) {
        if ((int)(threadIdx.x & 31) == leader) atomicAdd(&tile_sum[tile], __popc(act));
    } else {
        const unsigned m = __match_any_sync(act, tile);
        if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(&tile_sum[tile], __popc(m));
    }
}

// ---------------------------------------------------------------------------------------------
// k_step
// ---------------------------------------------------------------------------------------------
// p[i] read through a pointer the compiler cannot see into: the load is issued where it is
// written and not merged with an earlier load of the same element, so a value that is read again
// need not be kept live (or spilled) in between
template <typename T>
__device__ __forceinline__ T reload(const T* p, int i) {
    asm volatile("" : "+l"(p));
    return p[i];
}
// One neighbour candidate: 3D chord distance test, Szabo force and polarity sums.
template <typename real>
__device__ __forceinline__ PairC<real> pair_constants(const RepParams<real>& rp) {
    PairC<real> c;
    c.r_max2 = rp.r_max2, c.twoR = rp.twoR, c.inv_twoR = rp.inv_twoR, c.k = rp.k, c.adh_scale = rp.adh_scale;
    return c;
}

// Every multiply-add is written out (d_fma / d_mul), so that each inlined copy (the step kernel's
// single-system and ensemble loops, the adjoint's recompute) rounds identically whatever the
// compiler would contract.
template <typename real>
__device__ __forceinline__ real pair_d2(const R4<real>& P, const R4<real>& Q) {
    const real dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
    return d_fma(dz, dz, d_fma(dy, dy, d_mul(dx, dx)));
}
// The term of one neighbour (pair_d2 < r_max^2, not the particle itself), QL its polarity. The
// separation is computed again from P and Q (the same bits as pair_d2's) rather than kept live
// between the distance test and the term.
template <typename real>
__device__ __forceinline__ void pair_add(const PairC<real>& rp, const R4<real>& P, const R4<real>& Q,
                                         const R4<real>& QL, real (&acc)[6], int& cnt) {
    const real dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
    const real d2 = d_fma(dz, dz, d_fma(dy, dy, d_mul(dx, dx)));
    const real rd = d_rsqrt(d2);  // 1/d (d2 > 0 unless two particles coincide)
    const real d = d_mul(d2, rd);
    const real fm = d < rp.twoR ? d_mul(d_mul(rp.k, rp.twoR - d), rp.inv_twoR) : -d_mul(rp.adh_scale, d - rp.twoR);
    if (d2 > (real)0) {
        const real c = d_mul(fm, rd);
        acc[0] = d_fma(c, dx, acc[0]);
        acc[1] = d_fma(c, dy, acc[1]);
        acc[2] = d_fma(c, dz, acc[2]);
    }
    acc[3] += QL.x;
    acc[4] += QL.y;
    acc[5] += QL.z;
    ++cnt;
}
template <typename real>
__device__ __forceinline__ void pair_term(const PairC<real>& rp, const R4<real>& P, const R4<real>& Q,
                                          const R4<real>* __restrict__ pol, int j, bool self, real (&acc)[6],
                                          int& cnt) {
    // polarity only for neighbours (about a third of candidates)
    if (pair_d2(P, Q) < rp.r_max2 && !self) pair_add(rp, P, Q, pol[j], acc, cnt);
}
template <typename real>
__device__ __forceinline__ void pair_term(const RepParams<real>& rp, const R4<real>& P, const R4<real>& Q,
                                          const R4<real>* __restrict__ pol, int j, bool self, real (&acc)[6],
                                          int& cnt) {
    pair_term(pair_constants(rp), P, Q, pol, j, self, acc, cnt);
}

// Pair sums over a particle's candidate runs in a fixed order (runs 0..8, slots ascending), two
// candidates per iteration. The run table lives in shared memory, one column per thread (entry r
// of thread t at srun[r * BLOCK]): switching runs is a shared-memory load instead of a local-memory
// (L1-cached stack) one, which took the step kernel from 142.7 to 137.0 us at 1M particles. The
// table holds the non-empty runs only, so a switch loads the next run once (stepping over empty
// runs inside the loop cost another 1.5% of the step).
// Each iteration takes both distance tests first, then issues both neighbours' polarity loads
// (independent, so they are in flight together), then adds the two terms in candidate order with
// pair_term's arithmetic (bit-identical sums). Keeping only the candidates' positions live between
// the test and the term (pair_add recomputes the separation) leaves 4 bytes of spills per thread
// at 40 registers instead of 12: the step kernel 123.0 -> 118.7 us at 1M particles.
// NBR (a test hook's instantiation): each neighbour's sorted slot is also written to list[0..cap).
// SPEC: both candidates' polarities are loaded with their positions, before the distance tests (one
// dependent load level per iteration instead of two, at the cost of loading non-neighbours'
// polarities). Used when the pair constants come from the kernel parameters (one replica, or
// replicas that share them): 1M particles 109.4 -> 107.2 us, 10,000 particles 21.5 -> 20.6 us
// per step, the 4,096-replica ensemble 559 -> 547 us; with per-replica constants from the table
// (five more live registers) the loads stay behind the tests.
template <typename real, int BLOCK, bool NBR = false, bool SPEC = false>
__device__ __forceinline__ void pair_sums_s(const PairC<real>& pc, const R4<real>& P, const R4<real>* __restrict__ pos,
                                          const R4<real>* __restrict__ pol, const int2* srun, int total, int self,
                                          real (&acc)[6], int& cnt, int* list = nullptr, int cap = 0) {
    if (total == 0) return;
    const int2* sp = srun;
    int2 x0 = *sp;
    int t = x0.x, left = x0.y;
    for (int rem = total; rem > 0; rem -= 2) {
        if (left == 0) {
            sp += BLOCK;
            const int2 x = *sp;
            t = x.x;
            left = x.y;
        }
        const int ta = t++;
        --left;
        int tb = -1;
        if (rem > 1) {
            if (left == 0) {
                sp += BLOCK;
                const int2 x = *sp;
                t = x.x;
                left = x.y;
            }
            tb = t++;
            --left;
        }
        const R4<real> Qa = pos[ta];
        const R4<real> Qb = pos[tb >= 0 ? tb : ta];
        R4<real> La, Lb;
        if (SPEC) La = pol[ta], Lb = pol[tb >= 0 ? tb : ta];
        const bool na = pair_d2(P, Qa) < pc.r_max2 && ta != self;
        const bool nb = tb >= 0 && pair_d2(P, Qb) < pc.r_max2 && tb != self;
        if (!SPEC) {
            if (na) La = pol[ta];
            if (nb) Lb = pol[tb];
        }
        if (na) {
            if (NBR && cnt < cap) list[cnt] = ta;
            pair_add(pc, P, Qa, La, acc, cnt);
        }
        if (nb) {
            if (NBR && cnt < cap) list[cnt] = tb;
            pair_add(pc, P, Qb, Lb, acc, cnt);
        }
    }
}

// Several lanes per particle (LPP = 2 or 4, a tuning choice): lane `sub` of the particle's group
// takes the candidates sub, sub + LPP, sub + 2 LPP, ... of the visiting order, one per iteration,
// and sums their terms in that order; the group's partial sums are then added over the lanes with a
// fixed butterfly, so every lane of the group holds the same totals and every run gives the same
// bits (a different rounding order from the one-lane loop, the same sums to rounding).
template <typename real, int BLOCK, int LPP>
__device__ __forceinline__ void pair_sums_lanes(const PairC<real>& pc, const R4<real>& P,
                                                const R4<real>* __restrict__ pos, const R4<real>* __restrict__ pol,
                                                const int2* srun, int total, int self, int sub, real (&acc)[6],
                                                int& cnt) {
    const int mine = total > sub ? (total - sub + LPP - 1) / LPP : 0;
    const int2* sp = srun;
    int t = 0, left = 0;
    if (total > 0) {
        const int2 x0 = *sp;
        t = x0.x, left = x0.y;
    }
    int skip = sub;
    for (int i = 0; i < mine; ++i) {
        while (skip >= left) {  // the table holds non-empty runs only; `mine` keeps this in range
            skip -= left;
            sp += BLOCK;
            const int2 x = *sp;
            t = x.x, left = x.y;
        }
        t += skip, left -= skip;
        const int j = t++;
        --left;
        skip = LPP - 1;
        const R4<real> Q = pos[j];
        if (pair_d2(P, Q) < pc.r_max2 && j != self) pair_add(pc, P, Q, pol[j], acc, cnt);
    }
}

// BLOCK: threads per block (a tuning choice: 128 or 256); the register budget is the same either
// way (6 blocks of 256, 12 of 128 per SM in FP32: 40 registers; 6 rather than 5 blocks of 256 took the
// step from 170.9 to 168.6 us at 1M particles).
// NBR: the test hook's instantiation that also exports each particle's neighbours (sorted slots,
// converted to particle indices by k_nbr_ids); the production launches use NBR = false.
// LPP: lanes per particle (1, 2 or 4; 32 / LPP particles per warp). With LPP > 1 the lanes of a
// particle split its candidates (pair_sums_lanes), then all of them run the particle's update on
// the same sums and the group's first lane ("lead") stores the results and does the atomics.
// SINGLE: a one-replica system reads its parameters from the kernel arguments (rp0, the constant
// bank: operands of the arithmetic, no loads) instead of the replica table (2.2% faster at 1M
// particles, results bit-identical).
// STORE: a step whose sorted state the adjoint keeps also stores its pair sums (force F and
// neighbour polarity sum m, by slot; with several lanes per particle the group's sums, by its first
// lane), so that the reverse step reads the forward's own values instead of running a pair loop.
template <typename real, int BLOCK, bool NBR = false, int LPP = 1, bool SINGLE = false, bool STORE = false>
__global__ void __launch_bounds__(BLOCK, (sizeof(real) == 4 ? 6 : 3) * 256 / BLOCK) k_step(const StepArgs<real> a) {
    typedef R4<real> r4;
    static_assert(LPP == 1 || LPP == 2 || LPP == 4, "1, 2 or 4 lanes per particle");
    static_assert(!(NBR && LPP > 1), "the neighbour export runs one lane per particle");
    const int q = (int)((blockIdx.x * BLOCK + threadIdx.x) / LPP);
    const int sub = LPP > 1 ? (int)(threadIdx.x % LPP) : 0;
    const bool active = q < a.N;
    const bool lead = active && sub == 0;
    int rep = -1;
    real ph[6] = {0, 0, 0, 0, 0, 0};
    int st = 0;
    if (active) {
        // pair sums over all candidates (in a fixed order); only what the loop uses is live
        // across it, the rest of the particle's state is read after it
        real acc[6] = {0, 0, 0, 0, 0, 0};
        int cnt = 0;
        {
        const r4 P = a.pos[q];
        const int id = a.ids[q];
        const int key0 = a.key_in[q];
        rep = (int)((unsigned)id >> a.local_bits);
        const RepParams<real>& rp = SINGLE ? a.rp0 : a.reps[rep];

        // candidate ranges: the 9 x-runs of the particle's cell (static 32-byte descriptors: 8 runs,
        // the own row's derived from two bits; 48-byte descriptors with the 9th run stored took the
        // step kernel 2% longer at 1M particles), as (first slot, count) pairs so that the loop
        // switches runs with one 8-byte load
        __shared__ int2 s_run[9 * BLOCK];
        int2* srun = s_run + threadIdx.x;
        int nrun = 0;
        int total = 0;
        const int id0 = key0 - rp.base;
        if (id0 < rp.C) {
            const uint4* dp = a.desc + (size_t)rp.desc_off + (size_t)id0 * 2;
            const uint4 d0 = dp[0], d1 = dp[1];
            const unsigned e[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
            const int Lb = (int)((d0.x >> 2) & 1u), Rb = (int)((d0.x >> 3) & 1u);
#pragma unroll
            for (int r = 0; r < 9; ++r) {
                const int first = r == 4 ? id0 - Lb : (int)(e[r < 4 ? r : r - 1] >> 4);
                const int len = r == 4 ? 1 + Lb + Rb : (int)(e[r < 4 ? r : r - 1] & 3u);
                const int b0 = rp.base + first;
                const int t0 = len ? a.start[b0] : 0;
                const int t1 = len ? a.start[b0 + len] : 0;
                // only non-empty runs are kept, in order: the loop never steps over an empty one
                if (t1 > t0) {
                    srun[nrun * BLOCK] = make_int2(t0, t1 - t0);
                    ++nrun;
                }
                total += t1 - t0;
            }
        }
        // a single-replica system takes the pair constants from the kernel parameters (constant
        // bank) rather than from the replica table, so the loop does not re-read them from global
        // memory
        int* list = NBR ? a.nbr_list + (size_t)(rp.off + (int)((unsigned)id & ((1u << a.local_bits) - 1u))) * a.nbr_cap
                        : nullptr;
        if (LPP == 1) {
            if (a.single)
                pair_sums_s<real, BLOCK, NBR, true>(a.pc0, P, a.pos, a.pol, srun, total, q, acc, cnt, list,
                                                    a.nbr_cap);
            else
                pair_sums_s<real, BLOCK, NBR>(pair_constants(rp), P, a.pos, a.pol, srun, total, q, acc, cnt, list,
                                              a.nbr_cap);
        } else {
            pair_sums_lanes<real, BLOCK, LPP>(a.single ? a.pc0 : pair_constants(rp), P, a.pos, a.pol, srun, total, q,
                                              sub, acc, cnt);
            const unsigned gm = ((1u << LPP) - 1u) << ((threadIdx.x & 31) & ~(unsigned)(LPP - 1));
#pragma unroll
            for (int o = 1; o < LPP; o <<= 1) {
#pragma unroll
                for (int k = 0; k < 6; ++k) acc[k] += __shfl_xor_sync(gm, acc[k], o);
                cnt += __shfl_xor_sync(gm, cnt, o);
            }
        }
        if (STORE && lead) {
            R4<real> sf;
            sf.x = acc[0], sf.y = acc[1], sf.z = acc[2], sf.w = acc[3];
            R2<real> sm;
            sm.x = acc[4], sm.y = acc[5];
            a.sum_f[q] = sf;
            a.sum_m[q] = sm;
        }
        }
        // the rest of the particle's own state, read again (an L1/L2 hit) rather than kept live
        // (spilled at 40 registers) across the pair loop: 64/104 bytes of spill stores/loads per
        // thread down to 12/12, the step kernel 123.1 -> 120.8 us at 1M particles
        const r4 PL = reload(a.pol, q);
        const R2<real> U = reload(a.uv, q);
        const int id = reload(a.ids, q);
        if (lead) {
            a.ids_o[q] = id;
            a.cnt_o[q] = cnt;
        }
        const int f = real_to_face(PL.w);
        rep = (int)((unsigned)id >> a.local_bits);
        const unsigned local = (unsigned)id & ((1u << a.local_bits) - 1u);
        const RepParams<real>& rp = SINGLE ? a.rp0 : a.reps[rep];
        const real* g = a.rec + (size_t)f * kRec;
        const real px = PL.x, py = PL.y, pz = PL.z;
        const real Fxr = acc[0], Fyr = acc[1], Fzr = acc[2];
        const real mxr = acc[3], myr = acc[4], mzr = acc[5];

        // tangent projection and velocity
        real nrm[3], Jp[6];
        face_frame(g, nrm, Jp);
        const real nx = nrm[0], ny = nrm[1], nz = nrm[2];
        const real Fn = Fxr * nx + Fyr * ny + Fzr * nz;
        const real Tx = Fxr - Fn * nx, Ty = Fyr - Fn * ny, Tz = Fzr - Fn * nz;
        real vx, vy, vz;
        if (rp.force_mode == 0) {
            vx = rp.v0 * px + rp.mu * Tx, vy = rp.v0 * py + rp.mu * Ty, vz = rp.v0 * pz + rp.mu * Tz;
        } else {
            const real t2 = Tx * Tx + Ty * Ty + Tz * Tz;
            const real sp = rp.v0 + (t2 > (real)0 ? t2 * d_rsqrt(t2) : (real)0);
            vx = sp * px, vy = sp * py, vz = sp * pz;
        }
        // polarity rotation about n: relaxation towards v, alignment with neighbours, noise
        const real vn2 = vx * vx + vy * vy + vz * vz;
        const real mn2 = mxr * mxr + myr * myr + mzr * mzr;
        const real ivn = vn2 > (real)0 ? d_rsqrt(vn2) : (real)0;
        const real imn = mn2 > (real)0 ? d_rsqrt(mn2) : (real)0;
        real omega;
        {
            const real cx = py * vz - pz * vy, cy = pz * vx - px * vz, cz = px * vy - py * vx;
            const real ex = py * mzr - pz * myr, ey = pz * mxr - px * mzr, ez = px * myr - py * mxr;
            omega = (cx * nx + cy * ny + cz * nz) * ivn * rp.inv_tau + rp.align * (ex * nx + ey * ny + ez * nz) * imn;
        }
        real xi;
        if (a.noise) {
            xi = a.noise[rp.off + (int)local];
        } else {
            const unsigned bits = tdsr::noise_bits24(a.seed, *a.d_step, local, (unsigned)rep);
            xi = rp.eta * ((real)bits * (real)(1.0 / 16777216.0) - (real)0.5);
        }
        const real delta = rp.dt * omega + xi;
        real sd, cd;
        d_sincos(delta, &sd, &cd);
        const real npx = ny * pz - nz * py, npy = nz * px - nx * pz, npz = nx * py - ny * px;
        const real p2x = cd * px + sd * npx, p2y = cd * py + sd * npy, p2z = cd * pz + sd * npz;
        // chart direction of the new polarity and chart velocity through the face's map
        real w0 = Jp[0] * p2x + Jp[1] * p2y + Jp[2] * p2z;
        real w1 = Jp[3] * p2x + Jp[4] * p2y + Jp[5] * p2z;
        real vu = Jp[0] * vx + Jp[1] * vy + Jp[2] * vz;
        real vv = Jp[3] * vx + Jp[4] * vy + Jp[5] * vz;
        real u2 = U.x + rp.dt * vu, v2 = U.y + rp.dt * vv;
        int nw = 0;
        if (seam_wrap(U.x, U.y, u2, v2, vu, vv, w0, w1, nw)) st |= ST_WRAP;
        {
            // outputs are stored as soon as they are known, so that nothing is live for them
            R2<real> vo;
            vo.x = vu, vo.y = vv;
            if (lead) a.vel_o[q] = vo;
            R2<real> uo;
            uo.x = u2, uo.y = v2;
            if (lead) a.uv_o[q] = uo;
        }
        int mode = 0;
        const int f2 = locate(a.rec, a.adj, a.G, a.bin_start, a.bin_faces, u2, v2, f, mode);
        if (mode == 2) st |= ST_LOCATE;
        const real* h = a.rec + (size_t)f2 * kRec;
        real rx, ry, rz;
        face_map(h, u2, v2, rx, ry, rz);
        // new 3D polarity: normalize(J_f2 w) (= normalize(J_f2 (cos th, sin th)))
        real qx, qy, qz;
        {
            const R4<real> h2 = rq(h, 2), h3 = rq(h, 3);
            const real ex = h2.x * w0 + h2.w * w1, ey = h2.y * w0 + h3.x * w1, ez = h2.z * w0 + h3.y * w1;
            const real ien = d_rsqrt(ex * ex + ey * ey + ez * ez);
            qx = ex * ien, qy = ey * ien, qz = ez * ien;
        }
        const real th = d_atan2(w1, w0);
        if (!(is_finite(rx) && is_finite(ry) && is_finite(rz) && is_finite(u2) && is_finite(v2) && is_finite(th)))
            st |= ST_NONFINITE;

        r4 o;
        o.x = rx, o.y = ry, o.z = rz, o.w = th;
        if (lead) a.pos_o[q] = o;
        r4 ol;
        ol.x = qx, ol.y = qy, ol.z = qz, ol.w = face_to_real(f2, (real)0);
        if (lead) a.pol_o[q] = ol;
        // next step's cell key: the surface cell of the new position (one row-record load; looking the
        // new cell up in the old cell's neighbour descriptor first took the step kernel 4 us longer
        // at 1M particles), count and scan-tile count (counting sort)
        bool lost = false;
        const int key = bucket_of(rp, a.rows, a.ivals, rx, ry, rz, lost);
        if (lost) st |= ST_CELL;
        if (lead) {
            atomicAdd(&a.count[key], 1);
            a.key_o[q] = key;
            add_tile(a.tile_sum + (size_t)((*a.d_step + 1) & 1) * a.n_tiles, key);
        }

        // order-parameter partials: normalize((r' - c) x v), v / |v|
        const real ax = rx - a.cx, ay = ry - a.cy, az = rz - a.cz;
        const real Lx = ay * vz - az * vy, Ly = az * vx - ax * vz, Lz = ax * vy - ay * vx;
        const real Ln2 = Lx * Lx + Ly * Ly + Lz * Lz;
        if (lead && Ln2 > (real)0) {
            const real iL = d_rsqrt(Ln2);
            ph[0] = Lx * iL, ph[1] = Ly * iL, ph[2] = Lz * iL;
        }
        if (lead && vn2 > (real)0) {
            ph[3] = vx * ivn, ph[4] = vy * ivn, ph[5] = vz * ivn;
        }
    }
    if (st && lead) atomicOr(a.status, st);
    if (q == 0 && sub == 0) *a.phi_pending = 1;

    // order-parameter reduction: warp sum (same replica) -> atomics on one of kPhiCopies slots
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned amask = __ballot_sync(FULL, lead);
    if (!amask) return;
    const int rep0 = __shfl_sync(FULL, rep, __ffs(amask) - 1);
    const bool same = __all_sync(FULL, !lead || rep == rep0);
    const int copy = (int)(((blockIdx.x * BLOCK + threadIdx.x) >> 5) % kPhiCopies);
    if (same) {
        // fixed butterfly over fixed lanes: the warp sum is the same on every run
#pragma unroll
        for (int k = 0; k < 6; ++k) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ph[k] += __shfl_xor_sync(FULL, ph[k], o);
        }
        if (lane < 6) {
            real v = ph[0];
#pragma unroll
            for (int k = 1; k < 6; ++k)
                if (k == lane) v = ph[k];
            const long long iv = __double2ll_rn((double)v * (SINGLE ? a.rp0.phiscale : a.reps[rep0].phiscale));
            atomicAdd(&a.phi_acc[((size_t)rep0 * kPhiCopies + copy) * 6 + lane], (unsigned long long)iv);
        }
    } else if (lead) {
        const double ps = a.reps[rep].phiscale;
#pragma unroll
        for (int k = 0; k < 6; ++k)
            atomicAdd(&a.phi_acc[((size_t)rep * kPhiCopies + copy) * 6 + k],
                      (unsigned long long)__double2ll_rn((double)ph[k] * ps));
    }
}

// ---------------------------------------------------------------------------------------------
// order parameter of a step, per replica
// ---------------------------------------------------------------------------------------------
template <typename real>
struct FinArgs {
    unsigned long long* phi_acc;  // [R][kPhiCopies][6] fixed-point sums of the step just taken
    const RepParams<real>* reps;
    int R;
    double* series;  // [cap_steps][2][R]: phi, psi by step
    long long cap_steps;
    double* phisum;  // nullable: the vector sums (sum normalize((r' - c) x v), sum v/|v|),
                     // [step - phisum_base][R][6], for the adjoint
    long long phisum_base, phisum_cap;
    int* pending;  // set by k_step, cleared by k_scatter and after a standalone finalize
};

constexpr int kFinWarps = 8;  // replicas finalized per 256-thread block (one warp each)
static_assert(kScanThreads == 32 * kFinWarps, "k_scan's extra blocks finalize one replica per warp");

// One warp: replica r's order parameter of `step` into the series; zeroes its accumulators. Lane c
// holds copy c's six components; each component is summed over the kPhiCopies copies in int64
// (exact, so the order of the additions does not matter), then converted to double once.
template <typename real>
__device__ void finalize_replica(const FinArgs<real>& f, int r, long long step) {
    const int lane = threadIdx.x & 31;
    static_assert(kPhiCopies == 32, "one copy per lane");
    unsigned long long* p = &f.phi_acc[((size_t)r * kPhiCopies + lane) * 6];
    long long x[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        x[k] = (long long)p[k];
        p[k] = 0ull;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[k] += __shfl_xor_sync(0xffffffffu, x[k], o);
    }
    if (lane == 0) {
        double v[6];
        for (int k = 0; k < 6; ++k) v[k] = (double)x[k];
        const RepParams<real>& rp = f.reps[r];
        const double inv = 1.0 / rp.phiscale;
        const double phi = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * inv * rp.inv_n;
        const double psi = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]) * inv * rp.inv_n;
        if (step >= 0 && step < f.cap_steps) {
            f.series[(size_t)step * 2 * f.R + r] = phi;
            f.series[(size_t)step * 2 * f.R + f.R + r] = psi;
        }
        const long long tp = step - f.phisum_base;
        if (f.phisum && tp >= 0 && tp < f.phisum_cap)
            for (int k = 0; k < 6; ++k) f.phisum[((size_t)tp * f.R + r) * 6 + k] = v[k] * inv;
    }
}

// ---------------------------------------------------------------------------------------------
// cell-list kernels
// ---------------------------------------------------------------------------------------------
// Exclusive scan of count[0..M) into start[0..M). Each block's base is the sum of
// the per-tile counts of the tiles before it (accumulated by the previous step), so no block
// waits on another. Also zeroes the other parity's tile counts for the step about to run.
// The R blocks past the n_tiles scan blocks finalize the previous step's order parameter (when a
// step is pending), so that it costs no launch of its own.
template <typename real>
__global__ void __launch_bounds__(kScanThreads) k_scan(int* __restrict__ count, int* __restrict__ start, long long M,
                                                       int* __restrict__ tile_sum, int n_tiles,
                                                       const long long* d_step, const FinArgs<real> fin) {
    __shared__ int s_warp[kScanThreads / 32];
    __shared__ int s_base;
    if ((int)blockIdx.x >= n_tiles) {
        if (*fin.pending == 0) return;
        const int r = ((int)blockIdx.x - n_tiles) * kFinWarps + (int)(threadIdx.x >> 5);
        if (r < fin.R) finalize_replica(fin, r, *d_step);
        return;
    }
    const int tile = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // this thread's counts, loaded first so that their latency overlaps the block-base sum
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    if (base + kScanItems <= M) {
#pragma unroll
        for (int i = 0; i < kScanItems; i += 4) {
            const int4 x = *reinterpret_cast<const int4*>(count + base + i);
            v[i] = x.x, v[i + 1] = x.y, v[i + 2] = x.z, v[i + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) v[i] = base + i < M ? count[base + i] : 0;
    }
    const int par = (int)((*d_step + 1) & 1);
    const int* ts = tile_sum + (size_t)par * n_tiles;
    // base = sum of ts[0..tile)
    int part = 0;
    for (int i = threadIdx.x; i < tile; i += kScanThreads) part += ts[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) s_warp[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        int b = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) b += s_warp[w];
        s_base = b;
        tile_sum[(size_t)(par ^ 1) * n_tiles + tile] = 0;
    }
    __syncthreads();
    int sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) sum += v[i];
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __syncthreads();
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kScanThreads / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < kScanThreads / 32) s_warp[lane] = w;
    }
    __syncthreads();
    int run = s_base + incl - sum + (warp ? s_warp[warp - 1] : 0);
    if (base + kScanItems <= M) {
#pragma unroll
        for (int i = 0; i < kScanItems; i += 4) {
            int4 o;
            o.x = run;
            run += v[i];
            o.y = run;
            run += v[i + 1];
            o.z = run;
            run += v[i + 2];
            o.w = run;
            run += v[i + 3];
            *reinterpret_cast<int4*>(start + base + i) = o;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) {
            if (base + i < M) start[base + i] = run;
            run += v[i];
        }
    }
}

// Counting-sort scatter; the cell's count is the cursor and ends at zero for the next step.
// PPT slots per thread (s, s + 256, ... of a block's 256 * PPT), their returning atomics in flight
// together.
template <int PPT>
__global__ void __launch_bounds__(256) k_scatter(const int* __restrict__ key, int* __restrict__ count,
                                                 const int* __restrict__ start, int* __restrict__ tmp, int N,
                                                 long long* d_step, int* phi_pending) {
    const int s0 = (int)blockIdx.x * 256 * PPT + (int)threadIdx.x;
    if (s0 == 0) {
        *d_step += 1;
        *phi_pending = 0;  // k_scan has finalized the previous step
    }
    int b[PPT], c[PPT], r[PPT];
#pragma unroll
    for (int i = 0; i < PPT; ++i) b[i] = s0 + i * 256 < N ? key[s0 + i * 256] : -1;
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        c[i] = b[i] >= 0 ? start[b[i]] : 0;
        r[i] = b[i] >= 0 ? atomicSub(&count[b[i]], 1) : 0;
    }
#pragma unroll
    for (int i = 0; i < PPT; ++i)
        if (b[i] >= 0) tmp[c[i] + r[i] - 1] = s0 + i * 256;
}

// Within each cell, particles in increasing particle-id order: the particle in slot s goes to
// start[b] + (number of the cell's particles with a smaller id); its state is copied there.
// PPT particles per thread (p, p + 256, ... of a block's 256 * PPT): the chains of dependent
// loads of the thread's particles (slot -> cell and id -> cell starts -> the cell's other ids)
// are interleaved, so that more of them are in flight at once.
template <typename real, int PPT>
__global__ void __launch_bounds__(256) k_order(const int* __restrict__ tmp, const int* __restrict__ key,
                                               const int* __restrict__ ids, const int* __restrict__ start,
                                               const R4<real>* __restrict__ pos, const R4<real>* __restrict__ pol,
                                               const R2<real>* __restrict__ uv, R4<real>* __restrict__ spos,
                                               R4<real>* __restrict__ spol, R2<real>* __restrict__ suv,
                                               int* __restrict__ sids, int* __restrict__ skey, int N) {
    int s[PPT], b[PPT], me[PPT], c0[PPT], c1[PPT], rank[PPT];
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        const int p = (int)blockIdx.x * 256 * PPT + i * 256 + (int)threadIdx.x;
        s[i] = p < N ? tmp[p] : -1;
    }
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        b[i] = s[i] >= 0 ? key[s[i]] : 0;
        me[i] = s[i] >= 0 ? ids[s[i]] : 0;
    }
    int len = 0;
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        c0[i] = s[i] >= 0 ? start[b[i]] : 0;
        c1[i] = s[i] >= 0 ? start[b[i] + 1] : 0;
        rank[i] = 0;
        len = max(len, c1[i] - c0[i]);
    }
    for (int k = 0; k < len; ++k) {
#pragma unroll
        for (int i = 0; i < PPT; ++i)
            if (c0[i] + k < c1[i]) rank[i] += ids[tmp[c0[i] + k]] < me[i];
    }
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        if (s[i] < 0) continue;
        const int d = c0[i] + rank[i];
        spos[d] = pos[s[i]];
        spol[d] = pol[s[i]];
        suv[d] = uv[s[i]];
        sids[d] = me[i];
        skey[d] = b[i];
    }
}

// Per-tile sums of the cell counts (one block per scan tile), written into the tile counts of the
// parity the next k_scan reads. Used after a state load, where the counts come from k_load_state.
__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const int* __restrict__ count, long long M,
                                                            int* __restrict__ tile_sum, int n_tiles,
                                                            const long long* d_step, const int* flag) {
    __shared__ int s_warp[kScanThreads / 32];
    if (flag[0]) return;  // a refused load (k_check_faces): the tile counts stay as they were
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    int sum = 0;
    if (base + kScanItems <= M) {
#pragma unroll
        for (int i = 0; i < kScanItems; i += 4) {
            const int4 x = *reinterpret_cast<const int4*>(count + base + i);
            sum += x.x + x.y + x.z + x.w;
        }
    } else {
        for (int i = 0; i < kScanItems; ++i) sum += base + i < M ? count[base + i] : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int b = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) b += s_warp[w];
        tile_sum[(size_t)((*d_step + 1) & 1) * n_tiles + blockIdx.x] = b;
    }
}

// Order parameter of the step just taken, per replica (one block per replica); zeroes the
// accumulators.
// Standalone finalize (the flush before the series is read): the same as the blocks that k_scan
// runs past its tiles, for a step that no k_scan has followed yet.
template <typename real>
__global__ void k_finalize(const FinArgs<real> f, const long long* d_step) {
    if (*f.pending == 0) return;
    const int r = (int)blockIdx.x * kFinWarps + (int)(threadIdx.x >> 5);
    if (r < f.R) finalize_replica(f, r, *d_step);
}

// State (physical order) -> id order, in two passes: k_slot_of writes each particle's slot at its
// global index (one scattered 4-byte store per particle), then k_gather_state reads each
// particle's records from its slot and writes the outputs in index order, coalesced. (Writing
// the outputs straight from the slot order scatters six partial-sector stores per particle: the
// end-to-end loop went 0.335 -> 0.295 ms per step at 1M particles with the two passes.)
template <typename real>
__global__ void k_slot_of(const int* __restrict__ ids, const RepParams<real>* __restrict__ reps, int local_bits,
                          int* __restrict__ slot, int N) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const unsigned id = (unsigned)ids[s];
    slot[reps[id >> local_bits].off + (int)(id & ((1u << local_bits) - 1u))] = s;
}
// O: double (the reference's type), or float for an FP32 state (the values as they are on the
// device, half the bytes for the host link).
template <typename real, typename O>
__global__ void k_gather_state(const R4<real>* __restrict__ pos, const R4<real>* __restrict__ pol,
                               const R2<real>* __restrict__ uv, const R2<real>* __restrict__ vel,
                               const int* __restrict__ cnt, const int* __restrict__ slot, O* o_uv, O* o_th,
                               int* o_face, O* o_r3d, O* o_vel, int* o_cnt, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int s = slot[i];
    const R4<real> P = pos[s];
    const R2<real> U = uv[s];
    const R2<real> V = vel[s];
    const int f = real_to_face(pol[s].w);
    const int c = cnt[s];
    o_uv[2 * i] = U.x, o_uv[2 * i + 1] = U.y;
    o_th[i] = P.w;
    o_face[i] = f;
    o_r3d[3 * i] = P.x, o_r3d[3 * i + 1] = P.y, o_r3d[3 * i + 2] = P.z;
    o_vel[2 * i] = V.x, o_vel[2 * i + 1] = V.y;
    o_cnt[i] = c;
}

// Neighbour export (test hook): sorted slots -> particle indices (id order), right after the step
// that wrote them (its sorted ids are still in place); unused entries stay -1.
template <typename real>
__global__ void k_nbr_ids(int* __restrict__ list, int cap, const int* __restrict__ sids,
                          const RepParams<real>* __restrict__ reps, int local_bits, long long total) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int t = list[e];
    if (t < 0) return;
    const unsigned id = (unsigned)sids[t];
    list[e] = reps[id >> local_bits].off + (int)(id & ((1u << local_bits) - 1u));
}

// State (physical order) -> the reference's Particle records in id order (tds_particle, 88 bytes:
// ten doubles and the neighbour count). The angle in degrees is (theta * 180) / pi, as the C++
// facade writes it.
template <typename real>
__global__ void k_pack_particles(const R4<real>* pos, const R2<real>* uv, const int* ids, const R2<real>* vel,
                                 const int* cnt, const RepParams<real>* reps, int local_bits, tds_particle* out, int N) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const unsigned id = (unsigned)ids[s];
    const int i = reps[id >> local_bits].off + (int)(id & ((1u << local_bits) - 1u));
    const R4<real> P = pos[s];
    const R2<real> U = uv[s], V = vel[s];
    tds_particle q;
    q.x_UV = U.x, q.y_UV = U.y;
    q.x_velocity_UV = V.x, q.y_velocity_UV = V.y;
    q.alignment_UV = __ddiv_rn(__dmul_rn((double)P.w, 180.0), 3.14159265358979323846);
    q.compass_north_pole_UV = 0.0, q.compass_south_pole_UV = 0.0;
    q.x_3D = P.x, q.y_3D = P.y, q.z_3D = P.z;
    q.neighbor_count = cnt[s];
    out[i] = q;
}

// A state load is checked on the device before anything of the current state is touched: a face
// index >= F refuses the whole load (refused, cleared before each check) and records the refusal
// for the caller (sticky, until reported); negative indices mean "locate" and are valid. The
// kernels of the load then leave the state, the cell counts and the tile counts as they were.
__global__ void k_check_faces(const int* __restrict__ face, int N, int F, int* refused, int* sticky) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool bad = i < N && face[i] >= F;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) {
        atomicOr(refused, 1);
        atomicOr(sticky, 1);
    }
}
// zeroes the cell counts and both parities of the tile counts before a load (unless refused)
__global__ void k_clear_counts(int* __restrict__ count, long long M, int* __restrict__ tile_sum, int n_tile_sum,
                               const int* __restrict__ flag) {
    if (flag[0]) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += stride) count[i] = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_tile_sum; i += stride) tile_sum[i] = 0;
}

// Loads a state given in id order (I: double, or float for an FP32 state), one thread per slot:
// slot s takes the particle it holds in the handle's current order (slot_ids: the current packed
// ids by slot, a permutation of the handle's particles from creation on). Any arrangement gives the
// same next step, whose counting sort orders the particles by cell and id; keeping the current one
// makes the writes coalesced and the face-record and cell-row reads spatially coherent (the input
// is read by particle index, from the staging the upload just wrote), and the next step's sort
// starts from a sorted order. Locates faces that are < 0, maps r3d when it is not given, derives
// the 3D polarity, and counts the particle into its cell bucket for the next step's counting sort
// (counts must be zero on entry).
template <typename real, typename I>
__global__ void k_load_state(const I* i_uv, const I* i_th, const int* i_face, const I* i_r3d,
                             int has_face, int has_r3d, const real* rec, const int4* adj, int G, const int* bs,
                             const int* bf, const RepParams<real>* reps, int local_bits, const int4* rows,
                             const int4* ivals, const int* slot_ids, R4<real>* pos, R4<real>* pol, R2<real>* uv,
                             int* ids, R2<real>* vel, int* cnt, int* key, int* count, int N, int* status,
                             const int* flag) {
    const int sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= N || flag[0]) return;
    const int id = slot_ids[sl];
    const int i = reps[(unsigned)id >> local_bits].off + (int)((unsigned)id & ((1u << local_bits) - 1u));
    const real u = (real)i_uv[2 * i], v = (real)i_uv[2 * i + 1];
    int f = has_face ? i_face[i] : -1;
    if (f < 0) {
        int mode = 0;
        f = locate<real>(rec, nullptr, G, bs, bf, u, v, 0, mode);
        if (mode == 2) atomicOr(status, ST_LOCATE);
    }
    const real* h = rec + (size_t)f * kRec;
    R4<real> P;
    if (has_r3d) {
        P.x = (real)i_r3d[3 * i], P.y = (real)i_r3d[3 * i + 1], P.z = (real)i_r3d[3 * i + 2];
    } else {
        face_map(h, u, v, P.x, P.y, P.z);
    }
    P.w = (real)i_th[i];
    pos[sl] = P;
    R4<real> L;
    polarity3(h, P.w, L.x, L.y, L.z);
    L.w = face_to_real(f, (real)0);
    pol[sl] = L;
    R2<real> U;
    U.x = u, U.y = v;
    uv[sl] = U;
    ids[sl] = id;
    R2<real> Z;
    Z.x = 0, Z.y = 0;
    vel[sl] = Z;
    cnt[sl] = 0;
    bool lost = false;
    const int k = bucket_of(reps[(unsigned)id >> local_bits], rows, ivals, P.x, P.y, P.z, lost);
    if (lost) atomicOr(status, ST_CELL);
    key[sl] = k;
    atomicAdd(&count[k], 1);
}

// Seeded placement on the device (FP64): face drawn with probability proportional to its 3D area
// (lower bound of u1 in the area CDF), uniform barycentric point (sqrt(u2), u3), polarity at angle
// 2 pi u4 from e1 = normalize(B - A) in the face's tangent frame (e2 = n x e1), as a chart angle.
// Draws: Philox4x32-10(ctr = (local index, replica, 0xFFFFFFFF, 0), key = seed), the same stream
// as the host placement. Face data per face: uv corners a, b, c (6), A (3), J (6, column u then
// v), n (3), e1 (3) = kPlaceRec doubles. Output in id order into the state-load staging.
constexpr int kPlaceRec = 21;
__global__ void k_place(const double* __restrict__ frec, const double* __restrict__ cdf, int F,
                        const int* __restrict__ packed_ids, int local_bits, unsigned long long seed, double* o_uv,
                        double* o_th, int* o_face, double* o_r3d, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const unsigned id = (unsigned)packed_ids[i];
    const uint32_t ctr[4] = {id & ((1u << local_bits) - 1u), id >> local_bits, 0xFFFFFFFFu, 0u};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    tdsr::philox10(ctr, key, o);
    const double u1 = __dmul_rn(__dadd_rn((double)(o[0] >> 11), 0.5), 1.0 / 2097152.0);  // (0, 1)
    const double u2 = __dmul_rn((double)(o[1] >> 8), 1.0 / 16777216.0);
    const double u3 = __dmul_rn((double)(o[2] >> 8), 1.0 / 16777216.0);
    const double u4 = __dmul_rn((double)(o[3] >> 8), 1.0 / 16777216.0);
    int lo = 0, hi = F;  // first face with cdf >= u1
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] < u1)
            lo = mid + 1;
        else
            hi = mid;
    }
    const int f = min(lo, F - 1);
    const double* r = frec + (size_t)f * kPlaceRec;
    const double s2 = sqrt(u2);
    const double w0 = __dadd_rn(1.0, -s2), w1 = __dmul_rn(s2, __dadd_rn(1.0, -u3)), w2 = __dmul_rn(s2, u3);
    const double pu = __dadd_rn(__dadd_rn(__dmul_rn(w0, r[0]), __dmul_rn(w1, r[2])), __dmul_rn(w2, r[4]));
    const double pv = __dadd_rn(__dadd_rn(__dmul_rn(w0, r[1]), __dmul_rn(w1, r[3])), __dmul_rn(w2, r[5]));
    o_uv[2 * (size_t)i] = pu, o_uv[2 * (size_t)i + 1] = pv;
    o_face[i] = f;
    const double du = __dadd_rn(pu, -r[0]), dv = __dadd_rn(pv, -r[1]);
    for (int k = 0; k < 3; ++k)
        o_r3d[3 * (size_t)i + k] = __dadd_rn(__dadd_rn(r[6 + k], __dmul_rn(r[9 + k], du)), __dmul_rn(r[12 + k], dv));
    const double* n = r + 15;
    const double* e1 = r + 18;
    const double e2[3] = {__dadd_rn(__dmul_rn(n[1], e1[2]), -__dmul_rn(n[2], e1[1])),
                          __dadd_rn(__dmul_rn(n[2], e1[0]), -__dmul_rn(n[0], e1[2])),
                          __dadd_rn(__dmul_rn(n[0], e1[1]), -__dmul_rn(n[1], e1[0]))};
    double sp, cp;
    sincos(__dmul_rn(6.28318530717958647692, u4), &sp, &cp);
    double p[3];
    for (int k = 0; k < 3; ++k) p[k] = __dadd_rn(__dmul_rn(cp, e1[k]), __dmul_rn(sp, e2[k]));
    // chart direction through the pseudo-inverse of J
    const double ux = r[9], uy = r[10], uz = r[11], vx = r[12], vy = r[13], vz = r[14];
    const double g11 = ux * ux + uy * uy + uz * uz, g12 = ux * vx + uy * vy + uz * vz, g22 = vx * vx + vy * vy + vz * vz;
    const double pu3 = ux * p[0] + uy * p[1] + uz * p[2], pv3 = vx * p[0] + vy * p[1] + vz * p[2];
    const double wu = g22 * pu3 - g12 * pv3, wv = g11 * pv3 - g12 * pu3;  // (J^T J)^-1 J^T p times det > 0
    o_th[i] = atan2(wv, wu);
}

// The run's loop on the device. The handle's loop graph holds k_loop_arm and two conditional WHILE
// nodes: the first one's body is a block of steps followed by k_loop_ctl, the second one's body one
// step followed by k_loop_ctl. Before the graph is launched, k_loop_set stores the number of blocks
// and of single steps; k_loop_arm sets each loop's condition from its count (a loop whose count is
// zero does not run), and each k_loop_ctl counts its loop down and clears the condition after the
// last pass, so every loop ends after the stored number of passes.
__global__ void k_loop_set(int* left, int blocks, int singles) {
    left[0] = blocks;
    left[1] = singles;
}
__global__ void k_loop_arm(const int* left, cudaGraphConditionalHandle hb, cudaGraphConditionalHandle h1) {
    cudaGraphSetConditional(hb, left[0] > 0 ? 1u : 0u);
    cudaGraphSetConditional(h1, left[1] > 0 ? 1u : 0u);
}
__global__ void k_loop_ctl(int* left, cudaGraphConditionalHandle h) {
    const int r = *left - 1;
    *left = r;
    cudaGraphSetConditional(h, r > 0 ? 1u : 0u);
}

template <typename real>
__global__ void k_debug_wrap(int n, const double* uv_old, double* uv, double* th, double* vel, int* nw_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    real ex = (real)uv[2 * i], ey = (real)uv[2 * i + 1];
    real wx = (real)1, wy = (real)0;
    if (th) d_sincos((real)th[i], &wy, &wx);
    real vx = vel ? (real)vel[2 * i] : (real)0, vy = vel ? (real)vel[2 * i + 1] : (real)0;
    int nw = 0;
    seam_wrap((real)uv_old[2 * i], (real)uv_old[2 * i + 1], ex, ey, vx, vy, wx, wy, nw);
    uv[2 * i] = ex, uv[2 * i + 1] = ey;
    if (th) th[i] = d_atan2(wy, wx);
    if (vel) vel[2 * i] = vx, vel[2 * i + 1] = vy;
    if (nw_out) nw_out[i] = nw;
}

}  // namespace tdsk
