// Reference-semantics step on the device (FP64): 2DTissue's own per-step algorithm, for exact
// reference-semantics studies on small meshes (the model-form step in kernels.cuh is the fast
// path). With the reference's formulas and conventions it replaces:
//   Locomotion::simulate_flight (Locomotion.cpp:57-89): the pair distance is the distance between
//     the particles' nearest mesh vertices, read from a dense Vuv x Vuv matrix
//     (get_distances_between_particles, Locomotion.cpp:94-111), min-symmetrised with a zero
//     diagonal (transform_into_symmetric_matrix, Locomotion.cpp:127-138); the pair direction is
//     the chart difference r_i - r_j (get_dist_vect, Locomotion.cpp:143-162); the force is
//     ForceHelper.cpp:34-104 (pairs with d >= 2 sigma skipped, d == 0 -> d + 0.001); the speed is
//     v0 + |F| along the integer-degree polarity; Euler step in the chart.
//   OrientationHelper::calculate_average_n_within_distance (OrientationHelper.cpp:29-116): the
//     circular mean of the angles within 2 sigma (self included), truncated to int, zero noise.
//   EuclideanTiling::diagonal_seam_edges_square_border (EuclideanTiling.cpp:31-208) with the
//     unit-square borders: first side in list order (left, right, up, down), exit coordinates
//     snapped to 0 within 1e-3, entry = transposed exit, repeated until the point is inside.
//   CellHelper::get_r3d / calculate_barycentric_3D_coord (CellHelper.cpp:71-160): argmin of the
//     chart point-triangle distance over all faces (ties -> lowest index), distance weights,
//     nearest corner.
//   count_particle_neighbors (2DTissue.cpp:254-268): d != 0 && d <= 2.4 sigma.
//   The order parameter as the sign sum of the chart angular momentum u*v' - v*u' (the
//     reference's 2-column cross product reads out of bounds, LinearAlgebra.cpp:67-105).
//   CellHelper::init_particle_position (CellHelper.cpp:43-67): a uniform face index, its chart
//     centroid, a uniform integer angle 0..359 -- drawn from Philox instead of std::random_device.
// This file is compiled with --fmad=false: every +, -, *, /, sqrt rounds as written (as in the
// FP64 oracle, built with -ffp-contract=off); results differ from it only through cos, sin and
// atan2 (last-place differences of the libraries), which can flip the integer truncation of a
// mean angle that lies within ~1e-13 of an integer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <queue>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/tds.h"
#include "philox.cuh"

namespace {

constexpr double kPiD = 3.14159265358979323846;
constexpr double kDegToRad = kPiD / 180.0;
constexpr double kRadToDeg = 180.0 / kPiD;
constexpr int kRefMaxWraps = 64;     // the oracle's guard on the reference's unbounded loop
constexpr int kRefLocateThreads = 256;
constexpr int kRefThreads = 128;       // pair threads per particle
constexpr int kRefMaxVuv = 32768;    // the dense distance matrix is Vuv^2 doubles (8 GiB at the limit)
constexpr int kRefMaxParticles = 65536;  // O(N^2) pair loop, as in the reference

// chart bounding box of a face (FP32: it only rules faces out, with a margin)
struct alignas(16) FaceBox {
    float u0, u1, v0, v1;
};

struct RefP {
    double v0, k, sigma, r_adh, k_adh, dt;
};

// ---- seam wrap (EuclideanTiling.cpp:112-208 on the unit square) ----
__device__ __forceinline__ bool r_inside(double x, double y) { return x >= 0 && x <= 1 && y >= 0 && y <= 1; }
__device__ __forceinline__ double r_min(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double r_max(double a, double b) { return a < b ? b : a; }

// is_point_on_segment (EuclideanTiling.cpp:156-168)
__device__ bool r_on_segment(double px, double py, double ax, double ay, double bx, double by) {
    if (px < r_min(ax, bx) || px > r_max(ax, bx) || py < r_min(ay, by) || py > r_max(ay, by)) return false;
    const double cr = (px - ax) * (by - ay) - (py - ay) * (bx - ax);
    return fabs(cr) < 1e-9;
}
// intersection_point (EuclideanTiling.cpp:170-208) of segment A->B with side C->D
__device__ bool r_intersection(double Ax, double Ay, double Bx, double By, double Cx, double Cy, double Dx, double Dy,
                               double* ox, double* oy) {
    if (r_on_segment(Ax, Ay, Cx, Cy, Dx, Dy)) return false;
    const double det = (Bx - Ax) * (Dy - Cy) - (By - Ay) * (Dx - Cx);
    if (fabs(det) < 1e-9) return false;
    const double t = ((Cx - Ax) * (Dy - Cy) - (Cy - Ay) * (Dx - Cx)) / det;
    const double s = ((Cx - Ax) * (By - Ay) - (Cy - Ay) * (Bx - Ax)) / det;
    if (t >= 0 && t <= 1 && s >= 0 && s <= 1) {
        *ox = Ax + t * (Bx - Ax);
        *oy = Ay + t * (By - Ay);
        return true;
    }
    return false;
}
// processPoints (EuclideanTiling.cpp:112-154) for one point: sides left, right, up, down in that
// order; gluing maps left (x,y)->(y,-x), right ->(y,2-x) with n -= 90, up ->(2-y,x), down ->(-y,x)
// with n -= 270.
__device__ void r_process_point(const double* pa, double* po, double* n, double* entry) {
    if (r_inside(po[0], po[1])) return;
    const double S[4][4] = {{0, 0, 0, 1}, {1, 0, 1, 1}, {0, 1, 1, 1}, {0, 0, 1, 0}};
    int side = -1;
    double ex = pa[0], ey = pa[1];
    for (int s = 0; s < 4 && side < 0; ++s) {
        double qx, qy;
        if (r_intersection(pa[0], pa[1], po[0], po[1], S[s][0], S[s][1], S[s][2], S[s][3], &qx, &qy)) {
            side = s;
            ex = fabs(qx) < 1e-3 ? 0.0 : qx;
            ey = fabs(qy) < 1e-3 ? 0.0 : qy;
        }
    }
    entry[0] = ey, entry[1] = ex;
    const double x = po[0], y = po[1];
    if (side == 0) {
        po[0] = y, po[1] = -x, *n -= 90.0;
    } else if (side == 1) {
        po[0] = y, po[1] = 2 - x, *n -= 90.0;
    } else if (side == 2) {
        po[0] = 2 - y, po[1] = x, *n -= 270.0;
    } else {
        po[0] = -y, po[1] = x, *n -= 270.0;
    }
}

// ---- point-triangle distance in the chart (CellHelper.cpp:162-222) ----
__device__ double r_seg_dist(double px, double py, double ax, double ay, double bx, double by) {
    const double abx = bx - ax, aby = by - ay;
    double t = (abx * (px - ax) + aby * (py - ay)) / (abx * abx + aby * aby);
    t = r_min(1.0, r_max(0.0, t));
    const double dx = ax + abx * t - px, dy = ay + aby * t - py;
    return sqrt(dx * dx + dy * dy);
}
__device__ double r_tri_dist(double px, double py, double2 a, double2 b, double2 c) {
    const double abx = b.x - a.x, aby = b.y - a.y, acx = c.x - a.x, acy = c.y - a.y;
    const double apx = px - a.x, apy = py - a.y, bpx = px - b.x, bpy = py - b.y, cpx = px - c.x, cpy = py - c.y;
    const double d_ab_ap = abx * apx + aby * apy, d_ac_ap = acx * apx + acy * apy;
    const double d_ab_bp = abx * bpx + aby * bpy, d_ac_bp = acx * bpx + acy * bpy;
    const double d_ab_cp = abx * cpx + aby * cpy, d_ac_cp = acx * cpx + acy * cpy;
    if (d_ab_ap <= 0.0 && d_ac_ap <= 0.0) return sqrt(apx * apx + apy * apy);
    if (d_ab_bp >= 0.0 && d_ac_bp <= d_ab_bp) return sqrt(bpx * bpx + bpy * bpy);
    if (d_ac_cp >= 0.0 && d_ab_cp <= d_ac_cp) return sqrt(cpx * cpx + cpy * cpy);
    const double vc = d_ab_ap * d_ac_bp - d_ab_bp * d_ac_ap;
    if (vc <= 0.0 && d_ab_ap >= 0.0 && d_ab_bp <= 0.0) return r_seg_dist(px, py, a.x, a.y, b.x, b.y);
    const double vb = d_ab_cp * d_ac_ap - d_ab_ap * d_ac_cp;
    if (vb <= 0.0 && d_ac_ap >= 0.0 && d_ac_cp <= 0.0) return r_seg_dist(px, py, a.x, a.y, c.x, c.y);
    const double va = d_ab_bp * d_ac_cp - d_ab_cp * d_ac_bp;
    if (va <= 0.0 && (d_ac_bp - d_ab_bp) >= 0.0 && (d_ab_cp - d_ac_cp) >= 0.0)
        return r_seg_dist(px, py, b.x, b.y, c.x, c.y);
    const double denom = 1.0 / (va + vb + vc), vv = vb * denom, ww = vc * denom;
    const double dx = a.x + abx * vv + acx * ww - px, dy = a.y + aby * vv + acy * ww - py;
    return sqrt(dx * dx + dy * dy);
}

// ---- kernels ----
// (cos, sin) of each integer-degree polarity (LinearAlgebra::angles_to_unit_vectors,
// LinearAlgebra.cpp:25-46), read by every particle's alignment sum and its own velocity.
__global__ void k_ref_unit(int N, const int* __restrict__ n, double2* __restrict__ cs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double r = (double)n[i] * kDegToRad;
    cs[i] = make_double2(cos(r), sin(r));
}

// One block per particle i: the block's threads take the pairs j = t, t + kRefThreads, ... (in
// increasing j) and their partial sums are combined by a fixed tree, so every run gives the same
// bits; thread 0 then forms the velocity, the Euler step, the truncated mean angle and the seam
// wrap. (The oracle sums the pairs in j order: the two agree to rounding.)
__global__ void __launch_bounds__(kRefThreads) k_ref_flight(int N, RefP p, int Vuv, const double* __restrict__ D,
                                                             const double2* __restrict__ uv,
                                                             const int* __restrict__ near,
                                                             const double2* __restrict__ cs,
                                                             double2* __restrict__ uv_o, int* __restrict__ n_o,
                                                             double2* __restrict__ rdot_o, int* __restrict__ cnt_o,
                                                             int* __restrict__ status) {
    __shared__ double s_a[4][kRefThreads];
    __shared__ int s_c[kRefThreads];
    const int i = blockIdx.x, t = threadIdx.x;
    const double2 ui = uv[i];
    const int a = near[i];
    const double* Da = D + (size_t)a * Vuv;
    double Fx = 0, Fy = 0, mx = 0, my = 0;
    int cnt = 0;
    for (int j = t; j < N; j += kRefThreads) {
        double d = 0.0;
        if (j != i) {
            const int b = near[j];
            const double d_ab = Da[b], d_ba = D[(size_t)b * Vuv + a];
            d = d_ba < d_ab ? d_ba : d_ab;
        }
        if (j != i && !(d >= 2 * p.sigma)) {
            const double2 uj = uv[j];
            const double dvx = ui.x - uj.x, dvy = ui.y - uj.y;
            double dist = d;
            if (dist == 0) dist += 0.001;
            double rep = 0, adh = 0;
            if (dist < 2 * p.sigma) rep = (-p.k * (2 * p.sigma - dist)) / (2 * p.sigma);
            if (dist >= 2 * p.sigma && dist <= p.r_adh) adh = (p.k_adh * (2 * p.sigma - dist)) / (2 * p.sigma - p.r_adh);
            const double fij = rep + adh;
            Fx += fij * (dvx / dist);
            Fy += fij * (dvy / dist);
        }
        if (d < 2 * p.sigma) {
            const double2 c = cs[j];
            mx += c.x;
            my += c.y;
        }
        if (d != 0 && d <= 2.4 * p.sigma) ++cnt;
    }
    s_a[0][t] = Fx, s_a[1][t] = Fy, s_a[2][t] = mx, s_a[3][t] = my, s_c[t] = cnt;
    __syncthreads();
    for (int o = kRefThreads / 2; o > 0; o >>= 1) {
        if (t < o) {
            for (int k = 0; k < 4; ++k) s_a[k][t] += s_a[k][t + o];
            s_c[t] += s_c[t + o];
        }
        __syncthreads();
    }
    if (t != 0) return;
    Fx = s_a[0][0], Fy = s_a[1][0], mx = s_a[2][0], my = s_a[3][0];
    const double2 ci = cs[i];
    const double am = sqrt(Fx * Fx + Fy * Fy) + p.v0;
    const double rdx = ci.x * am, rdy = ci.y * am;
    double po[2] = {ui.x + rdx * p.dt, ui.y + rdy * p.dt};
    const double nn = sqrt(mx * mx + my * my);
    if (nn > 0) mx /= nn, my /= nn;
    double deg = atan2(my, mx) * kRadToDeg;
    if (deg < 0) deg += 360.0;
    double nd = (double)(int)deg;
    double old[2] = {ui.x, ui.y};
    int st = 0;
    for (int guard = 0; guard < kRefMaxWraps; ++guard) {
        if (r_inside(po[0], po[1])) break;
        double entry[2];
        r_process_point(old, po, &nd, entry);
        if (!r_inside(po[0], po[1])) old[0] = entry[0], old[1] = entry[1];
        if (guard == kRefMaxWraps - 1) st |= TDS_STATUS_WRAP_LIMIT;
    }
    if (!(isfinite(po[0]) && isfinite(po[1]) && isfinite(rdx) && isfinite(rdy))) st |= TDS_STATUS_NONFINITE;
    if (st) atomicOr(status, st);
    uv_o[i] = make_double2(po[0], po[1]);
    n_o[i] = (int)nd;
    rdot_o[i] = make_double2(rdx, rdy);
    cnt_o[i] = s_c[0];
}

// One block per particle: the argmin over all faces of the chart point-triangle distance (ties ->
// lowest face index), then the distance-weighted 3D point and the nearest corner. The argmin is
// exact, but most faces are ruled out without evaluating the FP64 distance: the distance from the
// point to the nearest face centroid bounds the minimum from above, and a face whose bounding box
// lies farther than that cannot be the argmin. Both are computed in FP32 (GB300's FP64 rate is a
// small fraction of its FP32 rate); chart coordinates lie in [0, 1], where FP32 rounding moves a
// distance by less than 3e-7, so a margin of 2e-6 keeps every face that could attain the minimum.
// The oracle's distance, in FP64, is evaluated for the rest.
__global__ void __launch_bounds__(kRefLocateThreads) k_ref_locate(int F, const double2* __restrict__ uvv,
                                                                   const int* __restrict__ fuv,
                                                                   const FaceBox* __restrict__ fbox,
                                                                   const float2* __restrict__ fcen,
                                                                   const double* __restrict__ v3uv,
                                                                   const double2* __restrict__ uv,
                                                                   double* __restrict__ r3d, int* __restrict__ near) {
    __shared__ double s_d[kRefLocateThreads];
    __shared__ int s_f[kRefLocateThreads];
    const int i = blockIdx.x, t = threadIdx.x;
    __shared__ float s_u[kRefLocateThreads];
    const double2 P = uv[i];
    const float pxf = (float)P.x, pyf = (float)P.y;
    float u2 = 1e30f;
    for (int f = t; f < F; f += kRefLocateThreads) {
        const float2 c = fcen[f];
        const float ex = pxf - c.x, ey = pyf - c.y;
        const float e2 = ex * ex + ey * ey;
        u2 = e2 < u2 ? e2 : u2;
    }
    s_u[t] = u2;
    __syncthreads();
    for (int o = kRefLocateThreads / 2; o > 0; o >>= 1) {
        if (t < o && s_u[t + o] < s_u[t]) s_u[t] = s_u[t + o];
        __syncthreads();
    }
    const float kr = sqrtf(s_u[0]) + 2e-6f;
    const float keep = kr * kr;
    const bool finite = isfinite(P.x) && isfinite(P.y) && fabs(P.x) < 4.0 && fabs(P.y) < 4.0;
    double best = 1e300;
    int bf = 0x7fffffff;
    for (int f = t; f < F; f += kRefLocateThreads) {
        if (finite) {
            const FaceBox b = fbox[f];
            const float bx = pxf < b.u0 ? b.u0 - pxf : (pxf > b.u1 ? pxf - b.u1 : 0.0f);
            const float by = pyf < b.v0 ? b.v0 - pyf : (pyf > b.v1 ? pyf - b.v1 : 0.0f);
            if (bx * bx + by * by > keep) continue;
        }
        const double d = r_tri_dist(P.x, P.y, uvv[fuv[3 * f]], uvv[fuv[3 * f + 1]], uvv[fuv[3 * f + 2]]);
        if (d < best) best = d, bf = f;
    }
    s_d[t] = best, s_f[t] = bf;
    __syncthreads();
    for (int o = kRefLocateThreads / 2; o > 0; o >>= 1) {
        if (t < o) {
            const double d2 = s_d[t + o];
            const int f2 = s_f[t + o];
            if (d2 < s_d[t] || (d2 == s_d[t] && f2 < s_f[t])) s_d[t] = d2, s_f[t] = f2;
        }
        __syncthreads();
    }
    if (t != 0) return;
    const int g = s_f[0] == 0x7fffffff ? 0 : s_f[0];  // no face compared below 1e300 (non-finite point)
    const int tv[3] = {fuv[3 * g], fuv[3 * g + 1], fuv[3 * g + 2]};
    double w[3];
    for (int c = 0; c < 3; ++c) {
        const double ex = P.x - uvv[tv[c]].x, ey = P.y - uvv[tv[c]].y;
        w[c] = sqrt(ex * ex + ey * ey);
    }
    const double sw = w[0] + w[1] + w[2];
    for (int c = 0; c < 3; ++c) w[c] /= sw;
    double X[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) X[k] += w[c] * v3uv[3 * tv[c] + k];
    double dist[3];
    for (int c = 0; c < 3; ++c) {
        double s = 0;
        for (int k = 0; k < 3; ++k) {
            const double e = X[k] - v3uv[3 * tv[c] + k];
            s += e * e;
        }
        dist[c] = sqrt(s);
    }
    const double m12 = dist[2] < dist[1] ? dist[2] : dist[1];
    const double mn = m12 < dist[0] ? m12 : dist[0];
    near[i] = (mn == dist[0]) ? tv[0] : (mn == dist[1]) ? tv[1] : tv[2];
    for (int k = 0; k < 3; ++k) r3d[3 * (size_t)i + k] = X[k];
}

// |sum_i sign(u_i v'_i - v_i u'_i)| / N for the step (exact: an integer sum).
__global__ void __launch_bounds__(256) k_ref_order(int N, const double2* __restrict__ uv,
                                                   const double2* __restrict__ rdot, double* out) {
    __shared__ int s[256];
    int acc = 0;
    for (int i = threadIdx.x; i < N; i += 256) {
        const double2 u = uv[i], r = rdot[i];
        const double z = u.x * r.y - u.y * r.x;
        acc += (z > 0) - (z < 0);
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = fabs((double)s[0]) / N;
}

// init_particle_position: face = floor(u0 * F), chart centroid ((0 + a) + b + c) / 3, angle =
// floor(u1 * 360), from Philox4x32-10(ctr = (i, 0, 0xFFFFFFFE, 0), key = seed) words 0 and 1.
__global__ void k_ref_init(int N, int F, unsigned long long seed, const int* __restrict__ fuv,
                           const double2* __restrict__ uvv, double2* __restrict__ uv_o, int* __restrict__ n_o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t ctr[4] = {(uint32_t)i, 0u, 0xFFFFFFFEu, 0u};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    tdsr::philox10(ctr, key, o);
    const int f = (int)(((uint64_t)o[0] * (uint64_t)F) >> 32);
    const int ang = (int)(((uint64_t)o[1] * 360ull) >> 32);
    const double2 a = uvv[fuv[3 * f]], b = uvv[fuv[3 * f + 1]], c = uvv[fuv[3 * f + 2]];
    uv_o[i] = make_double2((((0.0 + a.x) + b.x) + c.x) / 3.0, (((0.0 + a.y) + b.y) + c.y) / 3.0);
    n_o[i] = ang;
}

}  // namespace

struct tds_ref_sim {
    int N = 0, F = 0, Vuv = 0;
    RefP p{};
    uint64_t seed = 0;
    long long step = 0;
    int cur = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    double* D = nullptr;
    double2* uvv = nullptr;
    int* fuv = nullptr;
    FaceBox* fbox = nullptr;  // per face: chart bounding box
    float2* fcen = nullptr;   // per face: chart centroid
    double* v3uv = nullptr;
    double2* uv[2] = {nullptr, nullptr};
    int* n[2] = {nullptr, nullptr};
    int* near = nullptr;
    double* r3d = nullptr;
    double2* rdot = nullptr;
    int* cnt = nullptr;
    double2* cs = nullptr;
    int* status = nullptr;
    double* order = nullptr;
    long long order_cap = 0;
    std::vector<void*> allocs;
};

namespace {

int ref_fail(tds_ref_sim* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}
#define RCK(call)                                                                                                 \
    do {                                                                                                          \
        cudaError_t e_ = (call);                                                                                  \
        if (e_ != cudaSuccess) return ref_fail(s, TDS_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int ref_alloc(tds_ref_sim* s, T** p, size_t bytes) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ref_fail(s, e == cudaErrorMemoryAllocation ? TDS_ERR_NOMEM : TDS_ERR_CUDA,
                        std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    s->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return TDS_OK;
}

struct HostMesh {
    int V = 0, F = 0, Vuv = 0;
    std::vector<double> v3, uv;
    std::vector<int> f3, fuv, uv2v;
};

int read_mesh(const tds_mesh* mesh, HostMesh& h) {
    double area = 0;
    int rc = tds_mesh_info(mesh, &h.V, &h.F, &h.Vuv, &area);
    if (rc) return rc;
    h.v3.resize((size_t)3 * h.V);
    h.f3.resize((size_t)3 * h.F);
    h.uv.resize((size_t)2 * h.Vuv);
    h.fuv.resize((size_t)3 * h.F);
    h.uv2v.resize(h.Vuv);
    return tds_mesh_arrays(mesh, h.v3.data(), h.f3.data(), h.uv.data(), h.fuv.data(), h.uv2v.data());
}

// Shortest paths along the chart mesh's edges (3D edge lengths) from every chart vertex: the
// stand-in for the reference's geodesic distance matrix of the cut-open mesh
// (CachedGeodesicDistanceHelper::get_mesh_distance_matrix, 2DTissue.cpp:102-105; its library is
// absent). Twins on the seam are distinct chart vertices with no edge between them, so paths do
// not cross the cut, as on the open mesh.
void vertex_distances(const HostMesh& h, double* out) {
    const int n = h.Vuv;
    std::vector<std::vector<std::pair<int, double>>> adj(n);
    for (int f = 0; f < h.F; ++f)
        for (int k = 0; k < 3; ++k) {
            const int a = h.fuv[3 * f + k], b = h.fuv[3 * f + (k + 1) % 3];
            const int A = h.uv2v[a], B = h.uv2v[b];
            double s = 0;
            for (int c = 0; c < 3; ++c) {
                const double e = h.v3[3 * A + c] - h.v3[3 * B + c];
                s += e * e;
            }
            const double w = std::sqrt(s);
            adj[a].push_back({b, w});
            adj[b].push_back({a, w});
        }
    auto run = [&](int src) {
        double* d = out + (size_t)src * n;
        for (int v = 0; v < n; ++v) d[v] = HUGE_VAL;
        d[src] = 0;
        typedef std::pair<double, int> QE;
        std::priority_queue<QE, std::vector<QE>, std::greater<QE>> q;
        q.push({0.0, src});
        while (!q.empty()) {
            const QE top = q.top();
            q.pop();
            if (top.first > d[top.second]) continue;
            for (const auto& e : adj[top.second]) {
                const double nd = top.first + e.second;
                if (nd < d[e.first]) {
                    d[e.first] = nd;
                    q.push({nd, e.first});
                }
            }
        }
    };
    const int nt = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (int src = t; src < n; src += nt) run(src);
        });
    for (auto& x : th) x.join();
}

int ensure_order_cap(tds_ref_sim* s, long long need) {
    if (need <= s->order_cap) return TDS_OK;
    long long cap = std::max<long long>(need, std::max<long long>(1024, 2 * s->order_cap));
    double* q = nullptr;
    if (int rc = ref_alloc(s, &q, (size_t)cap * sizeof(double))) return rc;
    if (s->order && s->step > 0)
        RCK(cudaMemcpyAsync(q, s->order, (size_t)s->step * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    if (s->order) {
        RCK(cudaStreamSynchronize(s->stream));
        cudaFree(s->order);
        s->allocs.erase(std::find(s->allocs.begin(), s->allocs.end(), (void*)s->order));
    }
    s->order = q;
    s->order_cap = cap;
    return TDS_OK;
}

int launch_locate(tds_ref_sim* s) {
    k_ref_locate<<<s->N, kRefLocateThreads, 0, s->stream>>>(s->F, s->uvv, s->fuv, s->fbox, s->fcen, s->v3uv,
                                                           s->uv[s->cur], s->r3d, s->near);
    RCK(cudaGetLastError());
    return TDS_OK;
}

int check_status(tds_ref_sim* s) {
    int st = 0;
    RCK(cudaMemcpyAsync(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    RCK(cudaStreamSynchronize(s->stream));
    if (st) {
        std::string m = "device status 0x" + std::to_string(st) + ":";
        if (st & TDS_STATUS_NONFINITE) m += " non-finite position or velocity (Validation::error_invalid_values);";
        if (st & TDS_STATUS_WRAP_LIMIT) m += " seam wrap did not end within 64 passes;";
        return ref_fail(s, TDS_ERR_STATE, m);
    }
    return TDS_OK;
}

}  // namespace

extern "C" {

int tds_ref_vertex_distances(const tds_mesh* mesh, double* out) {
    if (!mesh || !out) return TDS_ERR_ARG;
    HostMesh h;
    if (int rc = read_mesh(mesh, h)) return rc;
    vertex_distances(h, out);
    return TDS_OK;
}

int tds_ref_create(const tds_mesh* mesh, const double* vertex_dist, const tds_ref_params* params, int n_particles,
                   uint64_t seed, tds_ref_sim** out) {
    if (!mesh || !params || !out || n_particles < 1) return TDS_ERR_ARG;
    *out = nullptr;
    const RefP p{params->v0, params->k, params->sigma, params->r_adh, params->k_adh, params->step_size};
    const double chk[6] = {p.v0, p.k, p.sigma, p.r_adh, p.k_adh, p.dt};
    for (double x : chk)
        if (!std::isfinite(x)) return TDS_ERR_ARG;
    if (!(p.sigma > 0)) return TDS_ERR_ARG;  // the reference throws on an empty neighbourhood
    if (n_particles > kRefMaxParticles) return TDS_ERR_LIMIT;
    HostMesh h;
    if (int rc = read_mesh(mesh, h)) return rc;
    if (h.Vuv > kRefMaxVuv) return TDS_ERR_LIMIT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return TDS_ERR_CUDA;
    }
    auto* s = new tds_ref_sim();
    s->N = n_particles, s->F = h.F, s->Vuv = h.Vuv, s->p = p, s->seed = seed;
    const int N = n_particles;
    int rc = TDS_OK;
    std::vector<double> Dh;
    const double* D = vertex_dist;
    if (!D) {
        Dh.resize((size_t)h.Vuv * h.Vuv);
        vertex_distances(h, Dh.data());
        D = Dh.data();
    }
    std::vector<double> v3uv((size_t)3 * h.Vuv);
    for (int t = 0; t < h.Vuv; ++t)
        for (int c = 0; c < 3; ++c) v3uv[3 * t + c] = h.v3[3 * h.uv2v[t] + c];
    std::vector<float> box((size_t)4 * h.F), cen((size_t)2 * h.F);
    for (int f = 0; f < h.F; ++f) {
        const double* A = &h.uv[2 * (size_t)h.fuv[3 * f]];
        const double* B = &h.uv[2 * (size_t)h.fuv[3 * f + 1]];
        const double* Cc = &h.uv[2 * (size_t)h.fuv[3 * f + 2]];
        box[4 * f] = (float)std::min(A[0], std::min(B[0], Cc[0]));
        box[4 * f + 1] = (float)std::max(A[0], std::max(B[0], Cc[0]));
        box[4 * f + 2] = (float)std::min(A[1], std::min(B[1], Cc[1]));
        box[4 * f + 3] = (float)std::max(A[1], std::max(B[1], Cc[1]));
        cen[2 * f] = (float)((A[0] + B[0] + Cc[0]) / 3.0);
        cen[2 * f + 1] = (float)((A[1] + B[1] + Cc[1]) / 3.0);
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) rc = TDS_ERR_CUDA;
    if (!rc) rc = ref_alloc(s, &s->D, (size_t)h.Vuv * h.Vuv * sizeof(double));
    if (!rc) rc = ref_alloc(s, &s->uvv, (size_t)h.Vuv * sizeof(double2));
    if (!rc) rc = ref_alloc(s, &s->fuv, (size_t)3 * h.F * sizeof(int));
    if (!rc) rc = ref_alloc(s, &s->v3uv, v3uv.size() * sizeof(double));
    if (!rc) rc = ref_alloc(s, &s->fbox, box.size() * sizeof(float));
    if (!rc) rc = ref_alloc(s, &s->fcen, cen.size() * sizeof(float));
    for (int b = 0; b < 2 && !rc; ++b) {
        rc = ref_alloc(s, &s->uv[b], (size_t)N * sizeof(double2));
        if (!rc) rc = ref_alloc(s, &s->n[b], (size_t)N * sizeof(int));
    }
    if (!rc) rc = ref_alloc(s, &s->near, (size_t)N * sizeof(int));
    if (!rc) rc = ref_alloc(s, &s->r3d, (size_t)3 * N * sizeof(double));
    if (!rc) rc = ref_alloc(s, &s->rdot, (size_t)N * sizeof(double2));
    if (!rc) rc = ref_alloc(s, &s->cnt, (size_t)N * sizeof(int));
    if (!rc) rc = ref_alloc(s, &s->cs, (size_t)N * sizeof(double2));
    if (!rc) rc = ref_alloc(s, &s->status, sizeof(int));
    if (!rc) rc = ensure_order_cap(s, 1024);
    if (!rc) {
        const cudaError_t e[] = {
            cudaMemcpy(s->D, D, (size_t)h.Vuv * h.Vuv * sizeof(double), cudaMemcpyHostToDevice),
            cudaMemcpy(s->uvv, h.uv.data(), (size_t)h.Vuv * sizeof(double2), cudaMemcpyHostToDevice),
            cudaMemcpy(s->fuv, h.fuv.data(), (size_t)3 * h.F * sizeof(int), cudaMemcpyHostToDevice),
            cudaMemcpy(s->v3uv, v3uv.data(), v3uv.size() * sizeof(double), cudaMemcpyHostToDevice),
            cudaMemcpy(s->fbox, box.data(), box.size() * sizeof(float), cudaMemcpyHostToDevice),
            cudaMemcpy(s->fcen, cen.data(), cen.size() * sizeof(float), cudaMemcpyHostToDevice),
            cudaMemset(s->rdot, 0, (size_t)N * sizeof(double2)),
            cudaMemset(s->cnt, 0, (size_t)N * sizeof(int)),
            cudaMemset(s->status, 0, sizeof(int))};
        for (cudaError_t x : e)
            if (x != cudaSuccess) rc = TDS_ERR_CUDA;
    }
    if (rc) {
        tds_ref_destroy(s);
        return rc;
    }
    *out = s;
    return TDS_OK;
}

int tds_ref_start(tds_ref_sim* s) {
    if (!s) return TDS_ERR_ARG;
    s->cur = 0;
    s->step = 0;
    k_ref_init<<<(s->N + 127) / 128, 128, 0, s->stream>>>(s->N, s->F, s->seed, s->fuv, s->uvv, s->uv[0], s->n[0]);
    RCK(cudaGetLastError());
    if (int rc = launch_locate(s)) return rc;
    RCK(cudaMemsetAsync(s->rdot, 0, (size_t)s->N * sizeof(double2), s->stream));
    RCK(cudaMemsetAsync(s->cnt, 0, (size_t)s->N * sizeof(int), s->stream));
    return check_status(s);
}

int tds_ref_set_state(tds_ref_sim* s, const double* r_uv, const int* n_deg, const int* nearest_vertex) {
    if (!s) return TDS_ERR_ARG;
    if (!r_uv || !n_deg) return ref_fail(s, TDS_ERR_ARG, "r_uv and n_deg are required");
    const int N = s->N;
    if (nearest_vertex)
        for (int i = 0; i < N; ++i)
            if (nearest_vertex[i] < 0 || nearest_vertex[i] >= s->Vuv)
                return ref_fail(s, TDS_ERR_ARG, "nearest vertex out of range at particle " + std::to_string(i));
    for (int i = 0; i < 2 * N; ++i)
        if (!std::isfinite(r_uv[i])) return ref_fail(s, TDS_ERR_ARG, "non-finite r_uv");
    RCK(cudaMemcpyAsync(s->uv[s->cur], r_uv, (size_t)N * sizeof(double2), cudaMemcpyHostToDevice, s->stream));
    RCK(cudaMemcpyAsync(s->n[s->cur], n_deg, (size_t)N * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    if (int rc = launch_locate(s)) return rc;  // get_r3d: 3D position and nearest vertex
    if (nearest_vertex)
        RCK(cudaMemcpyAsync(s->near, nearest_vertex, (size_t)N * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    RCK(cudaStreamSynchronize(s->stream));
    return TDS_OK;
}

int tds_ref_step(tds_ref_sim* s, int n_steps) {
    if (!s || n_steps < 0) return TDS_ERR_ARG;
    if (int rc = ensure_order_cap(s, s->step + n_steps)) return rc;
    const int N = s->N, nb = (N + 127) / 128;
    for (int k = 0; k < n_steps; ++k) {
        const int c = s->cur, o = c ^ 1;
        k_ref_unit<<<nb, 128, 0, s->stream>>>(N, s->n[c], s->cs);
        k_ref_flight<<<N, kRefThreads, 0, s->stream>>>(N, s->p, s->Vuv, s->D, s->uv[c], s->near, s->cs, s->uv[o],
                                                        s->n[o], s->rdot, s->cnt, s->status);
        s->cur = o;
        if (int rc = launch_locate(s)) return rc;
        k_ref_order<<<1, 256, 0, s->stream>>>(N, s->uv[o], s->rdot, s->order + s->step);
        RCK(cudaGetLastError());
        ++s->step;
    }
    return check_status(s);
}

int tds_ref_get_state(tds_ref_sim* s, double* r_uv, int* n_deg, int* nearest_vertex, double* r3d, double* r_dot,
                      int* nbr_count) {
    if (!s) return TDS_ERR_ARG;
    const size_t N = (size_t)s->N;
    if (r_uv) RCK(cudaMemcpyAsync(r_uv, s->uv[s->cur], N * sizeof(double2), cudaMemcpyDeviceToHost, s->stream));
    if (n_deg) RCK(cudaMemcpyAsync(n_deg, s->n[s->cur], N * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    if (nearest_vertex) RCK(cudaMemcpyAsync(nearest_vertex, s->near, N * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    if (r3d) RCK(cudaMemcpyAsync(r3d, s->r3d, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (r_dot) RCK(cudaMemcpyAsync(r_dot, s->rdot, N * sizeof(double2), cudaMemcpyDeviceToHost, s->stream));
    if (nbr_count) RCK(cudaMemcpyAsync(nbr_count, s->cnt, N * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    RCK(cudaStreamSynchronize(s->stream));
    return TDS_OK;
}

int tds_ref_get_order_parameter(tds_ref_sim* s, double* out, int cap, int* n_steps) {
    if (!s || (!out && cap > 0) || cap < 0) return TDS_ERR_ARG;
    const long long n = std::min<long long>(cap, s->step);
    if (n > 0) RCK(cudaMemcpyAsync(out, s->order, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    RCK(cudaStreamSynchronize(s->stream));
    if (n_steps) *n_steps = (int)s->step;
    return TDS_OK;
}

int tds_ref_stream(tds_ref_sim* s, void** stream) {
    if (!s || !stream) return TDS_ERR_ARG;
    *stream = (void*)s->stream;
    return TDS_OK;
}

const char* tds_ref_last_error(const tds_ref_sim* s) { return s ? s->err.c_str() : "null handle"; }

void tds_ref_destroy(tds_ref_sim* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void* q : s->allocs) cudaFree(q);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

}  // extern "C"
