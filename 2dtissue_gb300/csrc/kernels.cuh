// sm_103a kernels of the per-step particle update (model form; see the design doc for the contract).
//
// One step is four launches on the handle's stream (captured in a CUDA graph by the host):
//   k_scan     single-pass exclusive scan of the cell-list counts (decoupled look-back)
//   k_scatter  counting-sort scatter: perm[start[key] + rank] = slot
//   k_step     fused pair sums + tangent projection + polarity update + UV advance + seam wrap
//              + face location + UV->3D map + next-step cell key/count + order-parameter partials
//   k_finalize order parameter per replica for this step
// Replaces (reference): Locomotion::simulate_flight + ForceHelper + OrientationHelper
// (Locomotion.cpp:57-162, ForceHelper.cpp:34-104, OrientationHelper.cpp:29-116),
// EuclideanTiling::diagonal_seam_edges_square_border (EuclideanTiling.cpp:31-208),
// CellHelper::get_r3d (CellHelper.cpp:71-160), Validation (Validation.cpp:40-72),
// count_particle_neighbors (2DTissue.cpp:254-268), calculate_order_parameter (LinearAlgebra.cpp:90-105).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "philox.cuh"

namespace tdsk {

enum : int {
    ST_NONFINITE = 1,
    ST_WRAP = 2,
    ST_LOCATE = 4,
    ST_NBR = 8,
    ST_CELL = 16,
    ST_SCAN_TIMEOUT = 32,
};

constexpr int kRec = 32;          // reals per face record
constexpr int kMaxWraps = 8;      // seam wraps per particle per step
constexpr int kNbrMax = 1024;     // neighbours covered by the fixed-point range
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kStepThreads = 256;
constexpr int kPhiCopies = 16;    // spread the order-parameter atomics over copies
constexpr double kPolScale = 1125899906842624.0;  // 2^50: fixed point of neighbour polarity sums

template <typename real>
struct alignas(4 * sizeof(real)) R4 {
    real x, y, z, w;
};
template <typename real>
struct alignas(2 * sizeof(real)) R2 {
    real x, y;
};

// Per-replica parameters (device copy).
template <typename real>
struct RepParams {
    real twoR, inv_twoR, k, adh_scale;  // adh_scale = k_adh / (r_max - 2R)
    real r_max2, v0, mu, inv_tau;
    real align, eta, dt, inv_h;
    real fscale, inv_fscale, pad0, pad1;  // force fixed point 2^S, 2^-S
    double phiscale;                      // order-parameter fixed point
    double inv_n;                         // 1 / particles in this replica
    int force_mode, base, lx, ly;
    int lz, n, off, pad3;  // off: global index of the replica's first particle
};

template <typename real>
struct StepArgs {
    const R4<real>* pos;  // (x, y, z, theta) in physical order
    const R2<real>* uv;
    const int* face;
    const int* ids;
    R4<real>* pos_o;      // outputs in this step's sorted order
    R2<real>* uv_o;
    int* face_o;
    int* ids_o;
    R2<real>* vel_o;
    int* cnt_o;
    int* key_o;
    int* rank_o;
    const int* perm;
    const int* start;
    int* count;
    const real* rec;
    int G;
    const int* bin_start;
    const int* bin_faces;
    const RepParams<real>* reps;
    int local_bits;
    real ox, oy, oz;
    real cx, cy, cz;
    const real* noise;  // nullable: angle increments by particle id
    unsigned long long* phi_acc;
    const long long* d_step;
    unsigned long long seed;
    int* status;
    int N;
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
__device__ __forceinline__ long long to_fix(float x, float s) { return __float2ll_rn(x * s); }
__device__ __forceinline__ long long to_fix(double x, double s) { return __double2ll_rn(x * s); }
__device__ __forceinline__ float from_fix(long long v, float inv) { return __ll2float_rn(v) * inv; }
__device__ __forceinline__ double from_fix(long long v, double inv) { return __ll2double_rn(v) * inv; }
__device__ __forceinline__ bool is_finite(float x) { return isfinite(x); }
__device__ __forceinline__ bool is_finite(double x) { return isfinite(x); }

template <typename real>
__device__ __forceinline__ real kPi() {
    return (real)3.14159265358979323846;
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
    const int bits = (int)r[28];
    const real P[3][2] = {{r[16], r[17]}, {r[18], r[19]}, {r[20], r[21]}};
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
    return fmin(e[0] * r[25], fmin(e[1] * r[26], e[2] * r[27]));
}
template <typename real>
__device__ __forceinline__ int bin_coord(real x, int G) {
    int b = (int)d_floor(x * (real)G);
    return b < 0 ? 0 : (b >= G ? G - 1 : b);
}
// 1. keep f_old if strictly inside; 2. lowest-index closed-containing face; 3. best score.
template <typename real>
__device__ int locate(const real* rec, int G, const int* bs, const int* bf, real px, real py, int f_old,
                      int& mode) {
    if (min_edge(rec + (size_t)f_old * kRec, px, py) > (real)0) {
        mode = 0;
        return f_old;
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
template <typename real>
__device__ int seam_wrap(real sx, real sy, real& ex, real& ey, real& th, real& vx, real& vy, int& nw) {
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
        if (best <= 1) {
            vnx = vy, vny = -vx;
            th = th - kPi<real>() * (real)0.5;
        } else {
            vnx = -vy, vny = vx;
            th = th + kPi<real>() * (real)0.5;
        }
        vx = vnx, vy = vny;
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

template <typename real>
__device__ __forceinline__ real norm_angle(real th) {
    const real pi = kPi<real>(), twopi = (real)2 * kPi<real>();
    if (th > pi || th <= -pi) th = th - twopi * d_floor((th + pi) / twopi);
    if (th <= -pi) th += twopi;
    return th;
}

// folded cell-grid bucket of a position
template <typename real>
__device__ __forceinline__ int bucket_of(const RepParams<real>& rp, real x, real y, real z, real ox, real oy,
                                         real oz) {
    const int ix = (int)d_floor((x - ox) * rp.inv_h), iy = (int)d_floor((y - oy) * rp.inv_h),
              iz = (int)d_floor((z - oz) * rp.inv_h);
    const unsigned mx = (1u << rp.lx) - 1u, my = (1u << rp.ly) - 1u, mz = (1u << rp.lz) - 1u;
    return rp.base + (int)(((unsigned)ix & mx) | (((unsigned)iy & my) << rp.lx) |
                           (((unsigned)iz & mz) << (rp.lx + rp.ly)));
}

// ---------------------------------------------------------------------------------------------
// k_step
// ---------------------------------------------------------------------------------------------
template <typename real>
__global__ void __launch_bounds__(kStepThreads) k_step(const StepArgs<real> a) {
    typedef R4<real> r4;
    const int q = blockIdx.x * kStepThreads + threadIdx.x;
    const bool active = q < a.N;
    int rep = -1;
    long long ph[6] = {0, 0, 0, 0, 0, 0};
    int st = 0;
    if (active) {
        const int s = a.perm[q];
        const r4 P = a.pos[s];
        const R2<real> U = a.uv[s];
        const int f = a.face[s];
        const int id = a.ids[s];
        rep = (int)((unsigned)id >> a.local_bits);
        const unsigned local = (unsigned)id & ((1u << a.local_bits) - 1u);
        const RepParams<real> rp = a.reps[rep];
        const real* g = a.rec + (size_t)f * kRec;
        const real J0 = g[0], J1 = g[1], J2 = g[2], J3 = g[3], J4 = g[4], J5 = g[5];
        const real nx = g[12], ny = g[13], nz = g[14];
        // own polarity: p = normalize(J (cos th, sin th))
        real sn, cs;
        d_sincos(P.w, &sn, &cs);
        real qx = J0 * cs + J3 * sn, qy = J1 * cs + J4 * sn, qz = J2 * cs + J5 * sn;
        real qn = d_sqrt(qx * qx + qy * qy + qz * qz);
        const real px = qx / qn, py = qy / qn, pz = qz / qn;

        // pair sums over the 27 cells around the particle (9 runs of 3 consecutive buckets)
        long long Fx = 0, Fy = 0, Fz = 0, Mx = 0, My = 0, Mz = 0;
        int cnt = 0;
        const real pscale = (real)kPolScale;
        auto pair = [&](int j) {
            if (j == s) return;
            const r4 Q = a.pos[j];
            const real dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
            const real d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 < rp.r_max2)) return;
            const real d = d_sqrt(d2);
            const real fm = d < rp.twoR ? rp.k * (rp.twoR - d) * rp.inv_twoR : -(rp.adh_scale * (d - rp.twoR));
            if (d > (real)0) {
                const real c = fm / d;
                Fx += to_fix(c * dx, rp.fscale);
                Fy += to_fix(c * dy, rp.fscale);
                Fz += to_fix(c * dz, rp.fscale);
            }
            const int fj = a.face[j];
            const real* gj = a.rec + (size_t)fj * kRec;
            real sj, cj;
            d_sincos(Q.w, &sj, &cj);
            const real ux = gj[0] * cj + gj[3] * sj, uy = gj[1] * cj + gj[4] * sj, uz = gj[2] * cj + gj[5] * sj;
            const real un = d_sqrt(ux * ux + uy * uy + uz * uz);
            Mx += to_fix(ux / un, pscale);
            My += to_fix(uy / un, pscale);
            Mz += to_fix(uz / un, pscale);
            ++cnt;
        };
        {
            const int ix = (int)d_floor((P.x - a.ox) * rp.inv_h), iy = (int)d_floor((P.y - a.oy) * rp.inv_h),
                      iz = (int)d_floor((P.z - a.oz) * rp.inv_h);
            const unsigned mxk = (1u << rp.lx) - 1u, myk = (1u << rp.ly) - 1u, mzk = (1u << rp.lz) - 1u;
            const unsigned Px = mxk + 1u;
            const unsigned x0 = (unsigned)(ix - 1) & mxk;
            for (int dz = -1; dz <= 1; ++dz) {
                const unsigned rz = ((unsigned)(iz + dz) & mzk) << (rp.lx + rp.ly);
                for (int dy = -1; dy <= 1; ++dy) {
                    const int row = rp.base + (int)(rz | (((unsigned)(iy + dy) & myk) << rp.lx));
                    if (x0 + 3u <= Px) {
                        const int e = a.start[row + x0 + 3];
                        for (int t = a.start[row + x0]; t < e; ++t) pair(a.perm[t]);
                    } else {
                        const int e0 = a.start[row + Px];
                        for (int t = a.start[row + x0]; t < e0; ++t) pair(a.perm[t]);
                        const int e1 = a.start[row + x0 + 3 - Px];
                        for (int t = a.start[row]; t < e1; ++t) pair(a.perm[t]);
                    }
                }
            }
        }
        if (cnt >= kNbrMax) st |= ST_NBR;
        const real Fxr = from_fix(Fx, rp.inv_fscale), Fyr = from_fix(Fy, rp.inv_fscale),
                   Fzr = from_fix(Fz, rp.inv_fscale);
        const real ips = (real)(1.0 / kPolScale);
        const real mxr = from_fix(Mx, ips), myr = from_fix(My, ips), mzr = from_fix(Mz, ips);

        // tangent projection and velocity
        const real Fn = Fxr * nx + Fyr * ny + Fzr * nz;
        const real Tx = Fxr - Fn * nx, Ty = Fyr - Fn * ny, Tz = Fzr - Fn * nz;
        real vx, vy, vz;
        if (rp.force_mode == 0) {
            vx = rp.v0 * px + rp.mu * Tx, vy = rp.v0 * py + rp.mu * Ty, vz = rp.v0 * pz + rp.mu * Tz;
        } else {
            const real sp = rp.v0 + d_sqrt(Tx * Tx + Ty * Ty + Tz * Tz);
            vx = sp * px, vy = sp * py, vz = sp * pz;
        }
        // polarity rotation about n: relaxation to v, alignment to neighbours, noise
        const real vn = d_sqrt(vx * vx + vy * vy + vz * vz);
        const real mn = d_sqrt(mxr * mxr + myr * myr + mzr * mzr);
        real omega = (real)0;
        if (vn > (real)0) {
            const real cx = py * vz - pz * vy, cy = pz * vx - px * vz, cz = px * vy - py * vx;
            omega += (cx * nx + cy * ny + cz * nz) / vn * rp.inv_tau;
        }
        if (mn > (real)0) {
            const real cx = py * mzr - pz * myr, cy = pz * mxr - px * mzr, cz = px * myr - py * mxr;
            omega += rp.align * (cx * nx + cy * ny + cz * nz) / mn;
        }
        const long long step = *a.d_step;
        real xi;
        if (a.noise) {
            xi = a.noise[rp.off + (int)local];
        } else {
            const unsigned bits = tdsr::noise_bits24(a.seed, step, local, (unsigned)rep);
            xi = rp.eta * ((real)bits * (real)(1.0 / 16777216.0) - (real)0.5);
        }
        const real delta = rp.dt * omega + xi;
        real sd, cd;
        d_sincos(delta, &sd, &cd);
        const real npx = ny * pz - nz * py, npy = nz * px - nx * pz, npz = nx * py - ny * px;
        const real p2x = cd * px + sd * npx, p2y = cd * py + sd * npy, p2z = cd * pz + sd * npz;
        const real w0 = g[6] * p2x + g[7] * p2y + g[8] * p2z;
        const real w1 = g[9] * p2x + g[10] * p2y + g[11] * p2z;
        real th = d_atan2(w1, w0);
        // chart advance with the face's affine map, then seam wrap
        real vu = g[6] * vx + g[7] * vy + g[8] * vz;
        real vv = g[9] * vx + g[10] * vy + g[11] * vz;
        real u2 = U.x + rp.dt * vu, v2 = U.y + rp.dt * vv;
        int nw = 0;
        const int wr = seam_wrap(U.x, U.y, u2, v2, th, vu, vv, nw);
        if (wr) st |= ST_WRAP;
        th = norm_angle(th);
        int mode = 0;
        const int f2 = locate(a.rec, a.G, a.bin_start, a.bin_faces, u2, v2, f, mode);
        if (mode == 2) st |= ST_LOCATE;
        const real* h = a.rec + (size_t)f2 * kRec;
        const real du = u2 - h[16], dv = v2 - h[17];
        const real rx = h[22] + h[0] * du + h[3] * dv;
        const real ry = h[23] + h[1] * du + h[4] * dv;
        const real rz = h[24] + h[2] * du + h[5] * dv;
        if (!(is_finite(rx) && is_finite(ry) && is_finite(rz) && is_finite(u2) && is_finite(v2) && is_finite(th)))
            st |= ST_NONFINITE;

        r4 o;
        o.x = rx, o.y = ry, o.z = rz, o.w = th;
        a.pos_o[q] = o;
        R2<real> uo;
        uo.x = u2, uo.y = v2;
        a.uv_o[q] = uo;
        a.face_o[q] = f2;
        a.ids_o[q] = id;
        R2<real> vo;
        vo.x = vu, vo.y = vv;
        a.vel_o[q] = vo;
        a.cnt_o[q] = cnt;
        // next step's cell key and rank (counting sort)
        const int key = bucket_of(rp, rx, ry, rz, a.ox, a.oy, a.oz);
        const int rank = atomicAdd(&a.count[key], 1);
        a.key_o[q] = key;
        a.rank_o[q] = rank;

        // order-parameter partials: normalize((r' - c) x v), v / |v|
        const real ax = rx - a.cx, ay = ry - a.cy, az = rz - a.cz;
        const real Lx = ay * vz - az * vy, Ly = az * vx - ax * vz, Lz = ax * vy - ay * vx;
        const real Ln = d_sqrt(Lx * Lx + Ly * Ly + Lz * Lz);
        const real ps = (real)rp.phiscale;
        if (Ln > (real)0) {
            ph[0] = to_fix(Lx / Ln, ps), ph[1] = to_fix(Ly / Ln, ps), ph[2] = to_fix(Lz / Ln, ps);
        }
        if (vn > (real)0) {
            ph[3] = to_fix(vx / vn, ps), ph[4] = to_fix(vy / vn, ps), ph[5] = to_fix(vz / vn, ps);
        }
    }
    if (st) atomicOr(a.status, st);

    // order-parameter reduction: warp (same replica) -> block -> atomics on one of kPhiCopies
    __shared__ long long s_ph[kStepThreads / 32][6];
    __shared__ int s_rep[kStepThreads / 32];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned amask = __ballot_sync(FULL, active);
    int rep0 = -1;
    if (amask) rep0 = __shfl_sync(FULL, rep, __ffs(amask) - 1);
    const bool same = __all_sync(FULL, !active || rep == rep0);
    const int copy = blockIdx.x % kPhiCopies;
    if (same) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            long long v = ph[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            ph[k] = v;
        }
        if (lane == 0) {
            s_rep[warp] = rep0;
#pragma unroll
            for (int k = 0; k < 6; ++k) s_ph[warp][k] = ph[k];
        }
    } else {
        if (active)
            for (int k = 0; k < 6; ++k)
                atomicAdd(&a.phi_acc[((size_t)rep * kPhiCopies + copy) * 6 + k], (unsigned long long)ph[k]);
        if (lane == 0) s_rep[warp] = -1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int cur = -1;
        long long acc[6] = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w <= kStepThreads / 32; ++w) {
            const int r = (w < kStepThreads / 32) ? s_rep[w] : -2;
            if (r != cur) {
                if (cur >= 0)
                    for (int k = 0; k < 6; ++k)
                        atomicAdd(&a.phi_acc[((size_t)cur * kPhiCopies + copy) * 6 + k], (unsigned long long)acc[k]);
                cur = r;
                for (int k = 0; k < 6; ++k) acc[k] = 0;
            }
            if (r >= 0)
                for (int k = 0; k < 6; ++k) acc[k] += s_ph[w][k];
        }
    }
}

// ---------------------------------------------------------------------------------------------
// cell-list kernels
// ---------------------------------------------------------------------------------------------
// Single-pass exclusive scan of count[0..M) into start[0..M), zeroing count. Tiles take a
// ticket (so every tile waits only on tiles already running) and publish
// (epoch, flag, value) words; flag 1 = aggregate, 2 = inclusive prefix.
__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long* p) {
    return *(volatile const unsigned long long*)p;
}

__global__ void __launch_bounds__(kScanThreads) k_scan(int* __restrict__ count, int* __restrict__ start, long long M,
                                                       unsigned long long* tile_state, unsigned* tickets,
                                                       const long long* d_step, int* status) {
    __shared__ int s_tile;
    __shared__ int s_warp[kScanThreads / 32];
    __shared__ int s_excl;
    const unsigned epoch = (unsigned)((*d_step + 2) & 0x3fffffff);
    const int slot = (int)(epoch & 1u);
    if (threadIdx.x == 0) {
        s_tile = (int)atomicAdd(&tickets[slot], 1u);
        if (s_tile == 0) tickets[slot ^ 1] = 0u;
    }
    __syncthreads();
    const int tile = s_tile;
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long long idx = base + i;
        v[i] = idx < M ? count[idx] : 0;
        sum += v[i];
    }
    // block exclusive scan of per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
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
    const int tile_total = s_warp[kScanThreads / 32 - 1];
    const int thread_excl = incl - sum + (warp ? s_warp[warp - 1] : 0);
    // decoupled look-back (warp 0)
    if (warp == 0) {
        const unsigned long long tag = (unsigned long long)epoch << 34;
        if (lane == 0) {
            const unsigned long long w =
                tag | ((unsigned long long)(tile == 0 ? 2u : 1u) << 32) | (unsigned)tile_total;
            atomicExch(&tile_state[tile], w);
        }
        int excl = 0;
        if (tile > 0) {
            int idx = tile - 1 - lane;
            bool done = false;
            long long spins = 0;
            while (!done) {
                unsigned long long w = 0;
                unsigned flag = 2;
                unsigned val = 0;
                if (idx >= 0) {
                    for (;;) {
                        w = ld_volatile_u64(&tile_state[idx]);
                        flag = ((w >> 34) == epoch) ? (unsigned)((w >> 32) & 3u) : 0u;
                        if (flag != 0) break;
                        if (++spins > (1ll << 22)) {
                            atomicOr(status, ST_SCAN_TIMEOUT);
                            flag = 2;
                            break;
                        }
                        __nanosleep(64);
                    }
                    val = (unsigned)w;
                }
                const unsigned pmask = __ballot_sync(0xffffffffu, flag == 2);
                int contrib;
                if (pmask) {
                    const int first = __ffs(pmask) - 1;  // nearest predecessor with a prefix
                    contrib = lane <= first ? (int)val : 0;
                    done = true;
                } else {
                    contrib = (int)val;
                    idx -= 32;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
                excl += contrib;
            }
            if (lane == 0)
                atomicExch(&tile_state[tile], tag | (2ull << 32) | (unsigned)(excl + tile_total));
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    int run = s_excl + thread_excl;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long long idx = base + i;
        if (idx < M) {
            start[idx] = run;
            count[idx] = 0;
        }
        run += v[i];
    }
}

__global__ void k_scatter(const int* __restrict__ key, const int* __restrict__ rank, const int* __restrict__ start,
                          int* __restrict__ perm, int N, long long* d_step) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) *d_step += 1;
    if (s < N) perm[start[key[s]] + rank[s]] = s;
}

// Cell keys and ranks of the current state (after start / set_state), counts must be zero.
template <typename real>
__global__ void k_prime(const R4<real>* pos, const int* ids, const RepParams<real>* reps, int local_bits, real ox,
                        real oy, real oz, int* count, int* key, int* rank, int N) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const R4<real> P = pos[s];
    const RepParams<real> rp = reps[(unsigned)ids[s] >> local_bits];
    const int k = bucket_of(rp, P.x, P.y, P.z, ox, oy, oz);
    key[s] = k;
    rank[s] = atomicAdd(&count[k], 1);
}

// Order parameter of the step just taken, per replica; zeroes the accumulators.
template <typename real>
__global__ void k_finalize(unsigned long long* phi_acc, const RepParams<real>* reps, int R, double* series,
                           long long series_base, long long cap_steps, const long long* d_step) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double s[6];
    for (int k = 0; k < 6; ++k) s[k] = 0;
    for (int c = 0; c < kPhiCopies; ++c)
        for (int k = 0; k < 6; ++k) {
            unsigned long long* p = &phi_acc[((size_t)r * kPhiCopies + c) * 6 + k];
            s[k] += (double)(long long)(*p);
            *p = 0ull;
        }
    const RepParams<real>& rp = reps[r];
    const double inv = 1.0 / rp.phiscale;
    const double Lx = s[0] * inv, Ly = s[1] * inv, Lz = s[2] * inv;
    const double phi = sqrt(Lx * Lx + Ly * Ly + Lz * Lz) * rp.inv_n;
    const double psi = sqrt(s[3] * s[3] + s[4] * s[4] + s[5] * s[5]) * inv * rp.inv_n;
    const long long t = *d_step - series_base;
    if (t >= 0 && t < cap_steps) {
        series[(size_t)t * 2 * R + r] = phi;
        series[(size_t)t * 2 * R + R + r] = psi;
    }
}

// Scatter the state (physical order) into id order, in double.
template <typename real>
__global__ void k_gather_state(const R4<real>* pos, const R2<real>* uv, const int* face, const int* ids,
                               const R2<real>* vel, const int* cnt, const RepParams<real>* reps, int local_bits,
                               double* o_uv, double* o_th, int* o_face, double* o_r3d, double* o_vel, int* o_cnt,
                               int N) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const unsigned id = (unsigned)ids[s];
    const int i = reps[id >> local_bits].off + (int)(id & ((1u << local_bits) - 1u));
    const R4<real> P = pos[s];
    const R2<real> U = uv[s];
    o_uv[2 * i] = U.x, o_uv[2 * i + 1] = U.y;
    o_th[i] = P.w;
    o_face[i] = face[s];
    o_r3d[3 * i] = P.x, o_r3d[3 * i + 1] = P.y, o_r3d[3 * i + 2] = P.z;
    if (vel) {
        const R2<real> V = vel[s];
        o_vel[2 * i] = V.x, o_vel[2 * i + 1] = V.y;
        o_cnt[i] = cnt[s];
    }
}

// Load a state given in id order (double) into physical slots = ids; locate faces that are
// < 0 and map r3d when it is not given.
template <typename real>
__global__ void k_load_state(const double* i_uv, const double* i_th, const int* i_face, const double* i_r3d,
                             int has_face, int has_r3d, const real* rec, int G, const int* bs, const int* bf,
                             const int* packed_ids, R4<real>* pos, R2<real>* uv, int* face, int* ids, R2<real>* vel,
                             int* cnt, int N, int* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const real u = (real)i_uv[2 * i], v = (real)i_uv[2 * i + 1];
    int f = has_face ? i_face[i] : -1;
    if (f < 0) {
        int mode = 0;
        // no previous face: start the search from face 0's test (strict) then the bins
        f = locate(rec, G, bs, bf, u, v, 0, mode);
        if (mode == 2) atomicOr(status, ST_LOCATE);
    }
    R4<real> P;
    if (has_r3d) {
        P.x = (real)i_r3d[3 * i], P.y = (real)i_r3d[3 * i + 1], P.z = (real)i_r3d[3 * i + 2];
    } else {
        const real* h = rec + (size_t)f * kRec;
        const real du = u - h[16], dv = v - h[17];
        P.x = h[22] + h[0] * du + h[3] * dv;
        P.y = h[23] + h[1] * du + h[4] * dv;
        P.z = h[24] + h[2] * du + h[5] * dv;
    }
    P.w = (real)i_th[i];
    pos[i] = P;
    R2<real> U;
    U.x = u, U.y = v;
    uv[i] = U;
    face[i] = f;
    ids[i] = packed_ids[i];
    R2<real> Z;
    Z.x = 0, Z.y = 0;
    vel[i] = Z;
    cnt[i] = 0;
}

template <typename real>
__global__ void k_debug_wrap(int n, const double* uv_old, double* uv, double* th, double* vel, int* nw_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    real ex = (real)uv[2 * i], ey = (real)uv[2 * i + 1];
    real t = th ? (real)th[i] : (real)0;
    real vx = vel ? (real)vel[2 * i] : (real)0, vy = vel ? (real)vel[2 * i + 1] : (real)0;
    int nw = 0;
    seam_wrap((real)uv_old[2 * i], (real)uv_old[2 * i + 1], ex, ey, t, vx, vy, nw);
    uv[2 * i] = ex, uv[2 * i + 1] = ey;
    if (th) th[i] = t;
    if (vel) vel[2 * i] = vx, vel[2 * i + 1] = vy;
    if (nw_out) nw_out[i] = nw;
}

}  // namespace tdsk
