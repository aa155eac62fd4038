/*
 * ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h). Never linked into the product.
 *
 * FP64 CPU restatement of 2DTissue's per-step update. Every ref-form function cites the
 * reference file:line it restates; the model-form step follows the contract the GPU path
 * implements (reference divergences are documented beside each block).
 * Compiled with -ffp-contract=off so that results are identical on x86-64 and aarch64.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------------------------------
// Philox4x32-10, from the published description (Salmon et al., "Parallel random numbers:
// as easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with key bumps.
// ------------------------------------------------------------------------------------------
inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t o0 = hi1 ^ c[1] ^ k[0], o1 = lo1, o2 = hi0 ^ c[3] ^ k[1], o3 = lo0;
    c[0] = o0, c[1] = o1, c[2] = o2, c[3] = o3;
}
inline void philox10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k[2] = {key[0], key[1]};
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
        philox_round(c, k);
    }
    std::memcpy(out, c, sizeof c);
}
// Per-particle per-step uniform in [0,1) with 24 random bits (exact in float and double).
inline double noise_u01(uint64_t seed, int64_t step, uint32_t local, uint32_t rep) {
    const uint32_t ctr[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), local, rep};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    philox10(ctr, key, o);
    return (double)(o[0] >> 8) * (1.0 / 16777216.0);
}

// ------------------------------------------------------------------------------------------
// Forward-mode dual numbers (value + one tangent) for the derivative oracle.
// ------------------------------------------------------------------------------------------
struct Dual {
    double v, d;
    Dual(double x = 0, double t = 0) : v(x), d(t) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
inline Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
inline Dual sqrt(Dual a) {
    double s = std::sqrt(a.v);
    return {s, s > 0 ? a.d / (2 * s) : 0.0};
}
inline Dual sin(Dual a) { return {std::sin(a.v), std::cos(a.v) * a.d}; }
inline Dual cos(Dual a) { return {std::cos(a.v), -std::sin(a.v) * a.d}; }
inline Dual atan2(Dual y, Dual x) {
    double r2 = x.v * x.v + y.v * y.v;
    return {std::atan2(y.v, x.v), (x.v * y.d - y.v * x.d) / r2};
}
inline double val(double x) { return x; }
inline double val(const Dual& x) { return x.v; }
using std::atan2;
using std::cos;
using std::sin;
using std::sqrt;

template <class T>
struct Vec3 {
    T x, y, z;
};
template <class T>
inline T dot3(const Vec3<T>& a, const Vec3<T>& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class T>
inline Vec3<T> cross3(const Vec3<T>& a, const Vec3<T>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// ------------------------------------------------------------------------------------------
// Model-form mesh data (per-face affine chart maps) and point location.
// ------------------------------------------------------------------------------------------
struct Face {
    double a[2], b[2], c[2];  // UV corners (CCW)
    int iu[3];                // UV vertex ids (canonical edge orientation)
    double A[3];              // 3D corner of a
    double J[6];              // dX/d(uv): column u = J[0..2], column v = J[3..5]
    double Jp[6];             // pseudo-inverse rows: (J^T J)^-1 J^T
    double n[3];              // unit normal of the 3D triangle
    double elen[3];           // UV edge lengths
};

}  // namespace

struct orc_mesh {
    std::vector<Face> faces;
    std::vector<int> adj;  // 3 per face: chart face across edge k (corner k -> k+1), -1 on the border
    int G = 1;
    std::vector<int> bin_start, bin_faces;
};

namespace {

inline double orient(const double* P, const double* Q, double px, double py) {
    return std::fma(Q[0] - P[0], py - P[1], -((Q[1] - P[1]) * (px - P[0])));
}
// Edge value of edge k (corner k -> k+1) for point p: > 0 inside. The same value (up to an
// exact sign flip) is computed for both faces sharing the edge: canonical vertex order.
inline double edge_value(const Face& f, int k, double px, double py) {
    const double* C[3] = {f.a, f.b, f.c};
    const double *P = C[k], *Q = C[(k + 1) % 3];
    return f.iu[k] < f.iu[(k + 1) % 3] ? orient(P, Q, px, py) : -orient(Q, P, px, py);
}
inline double min_edge(const Face& f, double px, double py) {
    double e0 = edge_value(f, 0, px, py), e1 = edge_value(f, 1, px, py), e2 = edge_value(f, 2, px, py);
    return std::min(e0, std::min(e1, e2));
}
inline double face_score(const Face& f, double px, double py) {
    double s = edge_value(f, 0, px, py) / f.elen[0];
    s = std::min(s, edge_value(f, 1, px, py) / f.elen[1]);
    return std::min(s, edge_value(f, 2, px, py) / f.elen[2]);
}
inline int bin_coord(double x, int G) {
    int b = (int)std::floor(x * G);
    return b < 0 ? 0 : (b >= G ? G - 1 : b);
}

// Model point location rule (the reference takes the argmin of the point-triangle distance over
// all faces, lowest index on ties, CellHelper.cpp:104-117; for a point inside the chart that is
// the containing face):
//  1. keep f_old if p is strictly inside it;
//  2. else an edge-neighbour of f_old that strictly contains p (edges in order 0, 1, 2);
//  3. else the lowest-index face that contains p (closed triangle);
//  4. else the face with the largest minimum signed edge distance (ties -> lowest index).
int locate(const orc_mesh& M, double px, double py, int f_old, int* mode) {
    if (mode) *mode = 0;
    if (f_old >= 0 && f_old < (int)M.faces.size()) {
        if (min_edge(M.faces[f_old], px, py) > 0) return f_old;
        for (int k = 0; k < 3; ++k) {
            const int g = M.adj[3 * f_old + k];
            if (g >= 0 && min_edge(M.faces[g], px, py) > 0) return g;
        }
    }
    const int G = M.G;
    int bx = bin_coord(px, G), by = bin_coord(py, G);
    int b = by * G + bx;
    for (int e = M.bin_start[b]; e < M.bin_start[b + 1]; ++e) {
        int g = M.bin_faces[e];
        if (min_edge(M.faces[g], px, py) >= 0) {
            if (mode) *mode = 1;
            return g;
        }
    }
    int best = -1;
    double bs = -1e300;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            int x = bx + dx, y = by + dy;
            if (x < 0 || y < 0 || x >= G || y >= G) continue;
            int bb = y * G + x;
            for (int e = M.bin_start[bb]; e < M.bin_start[bb + 1]; ++e) {
                int g = M.bin_faces[e];
                double s = face_score(M.faces[g], px, py);
                if (s > bs || (s == bs && g < best)) bs = s, best = g;
            }
        }
    if (mode) *mode = 2;
    return best;
}

// ------------------------------------------------------------------------------------------
// Model-form seam wrap on the unit-square chart. Gluing maps as in
// EuclideanTiling::processPoints (EuclideanTiling.cpp:112-154):
//   left  (x,y) -> (y, -x),   angle -= 90 deg      right (x,y) -> (y, 2-x), angle -= 90 deg
//   up    (x,y) -> (2-y, x),  angle += 90 deg      down  (x,y) -> (-y, x),  angle += 90 deg
// Divergence (documented): the side crossed FIRST along the segment is taken (the reference
// takes the first side in list order that the segment meets), the exit coordinate is snapped
// exactly onto the side (the reference snaps |coord| < 1e-3 to 0), and the loop is bounded.
// ------------------------------------------------------------------------------------------
enum { SIDE_NONE = -1, SIDE_L = 0, SIDE_R = 1, SIDE_U = 2, SIDE_D = 3 };
const int kTwin[4] = {SIDE_D, SIDE_U, SIDE_R, SIDE_L};
const double kHalfPi = 1.57079632679489661923;

template <class T>
inline void apply_side(int side, T& x, T& y) {
    T nx, ny;
    switch (side) {
        case SIDE_L: nx = y, ny = -x; break;
        case SIDE_R: nx = y, ny = T(2.0) - x; break;
        case SIDE_U: nx = T(2.0) - y, ny = x; break;
        default: nx = -y, ny = x; break;
    }
    x = nx, y = ny;
}
template <class T>
inline void rotate_side(int side, T& vx, T& vy) {  // linear part of the gluing map
    T nx, ny;
    if (side == SIDE_L || side == SIDE_R) nx = vy, ny = -vx;
    else nx = -vy, ny = vx;
    vx = nx, vy = ny;
}

template <class T>
int wrap_model(T& sx, T& sy, T& ex, T& ey, T& th, T& vx, T& vy, int max_wraps, int* n_wraps) {
    int excl = SIDE_NONE, w = 0;
    for (; w < max_wraps; ++w) {
        const double Ex = val(ex), Ey = val(ey), Sx = val(sx), Sy = val(sy);
        if (Ex >= 0 && Ex <= 1 && Ey >= 0 && Ey <= 1) break;
        int best = SIDE_NONE;
        double tb = 1e300;
        if (excl != SIDE_L && Ex < 0) {
            double t = Sx / (Sx - Ex), y = Sy + t * (Ey - Sy);
            if (y >= 0 && y <= 1 && t < tb) tb = t, best = SIDE_L;
        }
        if (excl != SIDE_R && Ex > 1) {
            double t = (1 - Sx) / (Ex - Sx), y = Sy + t * (Ey - Sy);
            if (y >= 0 && y <= 1 && t < tb) tb = t, best = SIDE_R;
        }
        if (excl != SIDE_U && Ey > 1) {
            double t = (1 - Sy) / (Ey - Sy), x = Sx + t * (Ex - Sx);
            if (x >= 0 && x <= 1 && t < tb) tb = t, best = SIDE_U;
        }
        if (excl != SIDE_D && Ey < 0) {
            double t = Sy / (Sy - Ey), x = Sx + t * (Ex - Sx);
            if (x >= 0 && x <= 1 && t < tb) tb = t, best = SIDE_D;
        }
        if (best == SIDE_NONE) {
            if (n_wraps) *n_wraps = w;
            return 2;  // degenerate segment: no side found
        }
        // exit point on the side, snapped exactly onto it
        double qx = Sx + tb * (Ex - Sx), qy = Sy + tb * (Ey - Sy);
        if (best == SIDE_L) qx = 0;
        if (best == SIDE_R) qx = 1;
        if (best == SIDE_U) qy = 1;
        if (best == SIDE_D) qy = 0;
        qx = std::min(1.0, std::max(0.0, qx));
        qy = std::min(1.0, std::max(0.0, qy));
        T nsx(qx), nsy(qy);
        apply_side(best, nsx, nsy);
        sx = nsx, sy = nsy;
        apply_side(best, ex, ey);
        rotate_side(best, vx, vy);
        th = th + T((best == SIDE_L || best == SIDE_R) ? -kHalfPi : kHalfPi);
        excl = kTwin[best];
    }
    if (n_wraps) *n_wraps = w;
    const double Ex = val(ex), Ey = val(ey);
    if (!(Ex >= 0 && Ex <= 1 && Ey >= 0 && Ey <= 1)) {
        if (Ex < 0) ex = T(0.0);
        if (Ex > 1) ex = T(1.0);
        if (Ey < 0) ey = T(0.0);
        if (Ey > 1) ey = T(1.0);
        return 1;  // wrap limit hit
    }
    return 0;
}

// Angle normalised to (-pi, pi].
template <class T>
inline T norm_angle(T th) {
    const double twopi = 6.28318530717958647692;
    double v = val(th);
    if (v > M_PI || v <= -M_PI) th = th - T(twopi * std::floor((v + M_PI) / twopi));
    if (val(th) <= -M_PI) th = th + T(twopi);
    return th;
}

// ------------------------------------------------------------------------------------------
// Neighbour search: uniform 3D cell list with cell size r_max, sorted by cell key.
// ------------------------------------------------------------------------------------------
struct CellList {
    double lo[3], inv_h;
    int64_t nx, ny;
    std::vector<int64_t> keys;
    std::vector<int> order;
    std::unordered_map<int64_t, std::pair<int, int>> range;
    int64_t key_of(double x, double y, double z) const {
        int64_t ix = (int64_t)std::floor((x - lo[0]) * inv_h), iy = (int64_t)std::floor((y - lo[1]) * inv_h),
                iz = (int64_t)std::floor((z - lo[2]) * inv_h);
        return ix + nx * (iy + ny * iz);
    }
    void build(int N, const double* r, double h) {
        double hi[3] = {-1e300, -1e300, -1e300};
        lo[0] = lo[1] = lo[2] = 1e300;
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < 3; ++k) lo[k] = std::min(lo[k], r[3 * i + k]), hi[k] = std::max(hi[k], r[3 * i + k]);
        for (int k = 0; k < 3; ++k) lo[k] -= 2 * h, hi[k] += 2 * h;
        inv_h = 1.0 / h;
        nx = (int64_t)((hi[0] - lo[0]) * inv_h) + 3;
        ny = (int64_t)((hi[1] - lo[1]) * inv_h) + 3;
        keys.resize(N);
        for (int i = 0; i < N; ++i) keys[i] = key_of(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
        order.resize(N);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
        range.clear();
        range.reserve(N);
        for (int s = 0; s < N;) {
            int e = s;
            while (e < N && keys[order[e]] == keys[order[s]]) ++e;
            range[keys[order[s]]] = {s, e};
            s = e;
        }
    }
    template <class F>
    void for_candidates(double x, double y, double z, F&& fn) const {
        int64_t ix = (int64_t)std::floor((x - lo[0]) * inv_h), iy = (int64_t)std::floor((y - lo[1]) * inv_h),
                iz = (int64_t)std::floor((z - lo[2]) * inv_h);
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    auto it = range.find((ix + dx) + nx * ((iy + dy) + ny * (iz + dz)));
                    if (it == range.end()) continue;
                    for (int s = it->second.first; s < it->second.second; ++s) fn(order[s]);
                }
    }
};

template <class T>
struct Params {
    T R, k, k_adh, r_max, v0, mu, tau, align, eta, dt;
};

// One particle's model-form update. Returns status bits (1 = non-finite, 2 = wrap limit,
// 4 = location fallback used).
template <class T, class Nbr>
int model_particle(const orc_mesh& M, const Params<T>& P, int force_mode, double xi_in, bool use_xi,
                   double u01, const double* centroid, T u, T v, T th, int f, const T r[3], Nbr&& for_neighbours,
                   T& u2, T& v2, T& th2, int& f2, T r2[3], T vel[2], int& cnt, int& nwr, T phi[6]) {
    const Face& g = M.faces[f];
    const T c = cos(th), s = sin(th);
    Vec3<T> q{T(g.J[0]) * c + T(g.J[3]) * s, T(g.J[1]) * c + T(g.J[4]) * s, T(g.J[2]) * c + T(g.J[5]) * s};
    const T qn = sqrt(dot3(q, q));
    const Vec3<T> p{q.x / qn, q.y / qn, q.z / qn};
    const Vec3<T> n{T(g.n[0]), T(g.n[1]), T(g.n[2])};

    // Pair sums over neighbours j != i with |r_i - r_j| < r_max (3D chord distance).
    // Szabo piecewise-linear force, sign as physically intended (= minus ForceHelper.cpp:84-104):
    //   f(d) = k (2R - d)/(2R) for d < 2R (repulsive); -k_adh (d - 2R)/(r_max - 2R) up to r_max.
    Vec3<T> F{T(0.0), T(0.0), T(0.0)}, m{T(0.0), T(0.0), T(0.0)};
    cnt = 0;
    const T twoR = T(2.0) * P.R;
    for_neighbours([&](const T rj[3], T thj, int fj) {
        const T dx = r[0] - rj[0], dy = r[1] - rj[1], dz = r[2] - rj[2];
        const T d = sqrt(dx * dx + dy * dy + dz * dz);
        const T fm = val(d) < val(twoR) ? P.k * (twoR - d) / twoR : -(P.k_adh * (d - twoR) / (P.r_max - twoR));
        if (val(d) > 0) {
            F.x += fm * dx / d;
            F.y += fm * dy / d;
            F.z += fm * dz / d;
        }
        const Face& gj = M.faces[fj];
        const T cj = cos(thj), sj = sin(thj);
        Vec3<T> qj{T(gj.J[0]) * cj + T(gj.J[3]) * sj, T(gj.J[1]) * cj + T(gj.J[4]) * sj,
                   T(gj.J[2]) * cj + T(gj.J[5]) * sj};
        const T qjn = sqrt(dot3(qj, qj));
        m.x += qj.x / qjn;
        m.y += qj.y / qjn;
        m.z += qj.z / qjn;
        ++cnt;
    });
    // Projection onto the tangent plane of the particle's face.
    const T Fn = dot3(F, n);
    const Vec3<T> FT{F.x - Fn * n.x, F.y - Fn * n.y, F.z - Fn * n.z};
    Vec3<T> vv;
    if (force_mode == 0) {
        vv = {P.v0 * p.x + P.mu * FT.x, P.v0 * p.y + P.mu * FT.y, P.v0 * p.z + P.mu * FT.z};
    } else {  // reference speed-only form (Locomotion.cpp:71-81): |v| = v0 + |F|, along p
        const T sp = P.v0 + sqrt(dot3(FT, FT));
        vv = {sp * p.x, sp * p.y, sp * p.z};
    }
    // Polarity: relaxation towards v (time tau) + alignment towards the neighbour mean + noise,
    // as a rotation about the face normal.
    const T vn = sqrt(dot3(vv, vv));
    const T mn = sqrt(dot3(m, m));
    T omega(0.0);
    if (val(vn) > 0) omega = omega + dot3(cross3(p, vv), n) / (vn * P.tau);
    if (val(mn) > 0) omega = omega + P.align * dot3(cross3(p, m), n) / mn;
    const T xi = use_xi ? T(xi_in) : P.eta * T(u01 - 0.5);
    const T delta = P.dt * omega + xi;
    const T cd = cos(delta), sd = sin(delta);
    const Vec3<T> np = cross3(n, p);
    const Vec3<T> p2{cd * p.x + sd * np.x, cd * p.y + sd * np.y, cd * p.z + sd * np.z};
    const T w0 = T(g.Jp[0]) * p2.x + T(g.Jp[1]) * p2.y + T(g.Jp[2]) * p2.z;
    const T w1 = T(g.Jp[3]) * p2.x + T(g.Jp[4]) * p2.y + T(g.Jp[5]) * p2.z;
    th2 = atan2(w1, w0);
    // UV advance with the face's affine chart map, then seam wrap.
    vel[0] = T(g.Jp[0]) * vv.x + T(g.Jp[1]) * vv.y + T(g.Jp[2]) * vv.z;
    vel[1] = T(g.Jp[3]) * vv.x + T(g.Jp[4]) * vv.y + T(g.Jp[5]) * vv.z;
    u2 = u + P.dt * vel[0];
    v2 = v + P.dt * vel[1];
    T su = u, sv = v;
    int status = 0;
    int wr = wrap_model(su, sv, u2, v2, th2, vel[0], vel[1], 8, &nwr);
    if (wr) status |= 2;
    th2 = norm_angle(th2);
    int mode = 0;
    f2 = locate(M, val(u2), val(v2), f, &mode);
    if (mode == 2) status |= 4;
    const Face& h = M.faces[f2];
    const T du = u2 - T(h.a[0]), dv = v2 - T(h.a[1]);
    for (int k = 0; k < 3; ++k) r2[k] = T(h.A[k]) + T(h.J[k]) * du + T(h.J[3 + k]) * dv;
    // Order-parameter contributions: normalize((r' - c) x v) and v/|v|.
    const Vec3<T> rc{r2[0] - T(centroid[0]), r2[1] - T(centroid[1]), r2[2] - T(centroid[2])};
    const Vec3<T> L = cross3(rc, vv);
    const T Ln = sqrt(dot3(L, L));
    for (int k = 0; k < 6; ++k) phi[k] = T(0.0);
    if (val(Ln) > 0) phi[0] = L.x / Ln, phi[1] = L.y / Ln, phi[2] = L.z / Ln;
    if (val(vn) > 0) phi[3] = vv.x / vn, phi[4] = vv.y / vn, phi[5] = vv.z / vn;
    const double chk[6] = {val(u2), val(v2), val(th2), val(r2[0]), val(r2[1]), val(r2[2])};
    for (double x : chk)
        if (!std::isfinite(x)) status |= 1;
    return status;
}

// ------------------------------------------------------------------------------------------
// Ref-form helpers
// ------------------------------------------------------------------------------------------
const double DEG_TO_RAD = M_PI / 180.0, RAD_TO_DEG = 180.0 / M_PI;

// 2D point-segment / point-triangle distance (CellHelper.cpp:162-222, restated in the UV plane).
double seg_dist(double px, double py, double ax, double ay, double bx, double by) {
    double abx = bx - ax, aby = by - ay;
    double t = (abx * (px - ax) + aby * (py - ay)) / (abx * abx + aby * aby);
    t = std::min(1.0, std::max(0.0, t));
    double dx = ax + abx * t - px, dy = ay + aby * t - py;
    return std::sqrt(dx * dx + dy * dy);
}
double tri_dist(double px, double py, const double* a, const double* b, const double* c) {
    double abx = b[0] - a[0], aby = b[1] - a[1], acx = c[0] - a[0], acy = c[1] - a[1];
    double apx = px - a[0], apy = py - a[1], bpx = px - b[0], bpy = py - b[1], cpx = px - c[0], cpy = py - c[1];
    double d_ab_ap = abx * apx + aby * apy, d_ac_ap = acx * apx + acy * apy;
    double d_ab_bp = abx * bpx + aby * bpy, d_ac_bp = acx * bpx + acy * bpy;
    double d_ab_cp = abx * cpx + aby * cpy, d_ac_cp = acx * cpx + acy * cpy;
    if (d_ab_ap <= 0.0 && d_ac_ap <= 0.0) return std::sqrt(apx * apx + apy * apy);
    if (d_ab_bp >= 0.0 && d_ac_bp <= d_ab_bp) return std::sqrt(bpx * bpx + bpy * bpy);
    if (d_ac_cp >= 0.0 && d_ab_cp <= d_ac_cp) return std::sqrt(cpx * cpx + cpy * cpy);
    double vc = d_ab_ap * d_ac_bp - d_ab_bp * d_ac_ap;
    if (vc <= 0.0 && d_ab_ap >= 0.0 && d_ab_bp <= 0.0) return seg_dist(px, py, a[0], a[1], b[0], b[1]);
    double vb = d_ab_cp * d_ac_ap - d_ab_ap * d_ac_cp;
    if (vb <= 0.0 && d_ac_ap >= 0.0 && d_ac_cp <= 0.0) return seg_dist(px, py, a[0], a[1], c[0], c[1]);
    double va = d_ab_bp * d_ac_cp - d_ab_cp * d_ac_bp;
    if (va <= 0.0 && (d_ac_bp - d_ab_bp) >= 0.0 && (d_ab_cp - d_ac_cp) >= 0.0)
        return seg_dist(px, py, b[0], b[1], c[0], c[1]);
    double denom = 1.0 / (va + vb + vc), vv = vb * denom, ww = vc * denom;
    double dx = a[0] + abx * vv + acx * ww - px, dy = a[1] + aby * vv + acy * ww - py;
    return std::sqrt(dx * dx + dy * dy);
}

// Segment/border-polyline intersection (EuclideanTiling.cpp:156-208) on one straight side.
bool ref_on_segment(double px, double py, double ax, double ay, double bx, double by) {
    if (px < std::min(ax, bx) || px > std::max(ax, bx) || py < std::min(ay, by) || py > std::max(ay, by))
        return false;
    double cr = (px - ax) * (by - ay) - (py - ay) * (bx - ax);
    return std::fabs(cr) < 1e-9;
}
bool ref_intersection(double Ax, double Ay, double Bx, double By, const double* C, const double* D, double* out) {
    if (ref_on_segment(Ax, Ay, C[0], C[1], D[0], D[1])) return false;
    double det = (Bx - Ax) * (D[1] - C[1]) - (By - Ay) * (D[0] - C[0]);
    if (std::fabs(det) < 1e-9) return false;
    double t = ((C[0] - Ax) * (D[1] - C[1]) - (C[1] - Ay) * (D[0] - C[0])) / det;
    double s = ((C[0] - Ax) * (By - Ay) - (C[1] - Ay) * (Bx - Ax)) / det;
    if (t >= 0 && t <= 1 && s >= 0 && s <= 1) {
        out[0] = Ax + t * (Bx - Ax);
        out[1] = Ay + t * (By - Ay);
        return true;
    }
    return false;
}
bool ref_inside(double x, double y) { return x >= 0 && x <= 1 && y >= 0 && y <= 1; }

// processPoints (EuclideanTiling.cpp:112-154) with unit-square borders
// (left x=0, right x=1, up y=1, down y=0; checked in that list order).
void ref_process_point(const double* pa, double* po, double* n, double* entry) {
    if (ref_inside(po[0], po[1])) return;
    static const double S[4][2][2] = {{{0, 0}, {0, 1}}, {{1, 0}, {1, 1}}, {{0, 1}, {1, 1}}, {{0, 0}, {1, 0}}};
    int side = -1;
    double ex[2] = {pa[0], pa[1]};
    for (int s = 0; s < 4 && side < 0; ++s) {
        double q[2];
        if (ref_intersection(pa[0], pa[1], po[0], po[1], S[s][0], S[s][1], q)) {
            side = s;
            ex[0] = std::fabs(q[0]) < 1e-3 ? 0.0 : q[0];
            ex[1] = std::fabs(q[1]) < 1e-3 ? 0.0 : q[1];
        }
    }
    entry[0] = ex[1], entry[1] = ex[0];
    double x = po[0], y = po[1];
    if (side == 0) po[0] = y, po[1] = -x, *n -= 90.0;
    else if (side == 1) po[0] = y, po[1] = 2 - x, *n -= 90.0;
    else if (side == 2) po[0] = 2 - y, po[1] = x, *n -= 270.0;
    else po[0] = -y, po[1] = x, *n -= 270.0;
}

}  // namespace

extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox10(ctr, key, out); }

// LinearAlgebra::angles_to_unit_vectors (LinearAlgebra.cpp:25-46)
int orc_ref_angles_to_unit_vectors(const int* deg, int n, double* out) {
    for (int i = 0; i < n; ++i) {
        double r = deg[i] * DEG_TO_RAD;
        out[2 * i] = std::cos(r);
        out[2 * i + 1] = std::sin(r);
    }
    return 0;
}

// ForceHelper::repulsive_adhesion_motion (ForceHelper.cpp:84-104), reference sign convention.
void orc_ref_repulsive_adhesion(double k, double sigma, double dist, double r_adh, double k_adh, double dvx,
                                double dvy, double* out2) {
    double rep = 0, adh = 0;
    if (dist < 2 * sigma) rep = (-k * (2 * sigma - dist)) / (2 * sigma);
    if (dist >= 2 * sigma && dist <= r_adh) adh = (k_adh * (2 * sigma - dist)) / (2 * sigma - r_adh);
    double fij = rep + adh;
    out2[0] = fij * (dvx / dist);
    out2[1] = fij * (dvy / dist);
}

// OrientationHelper::mean_unit_circle_vector_angle_degrees (OrientationHelper.cpp:84-116).
// The reference throws std::invalid_argument on an empty input; here that is return -1.
int orc_ref_mean_angle_deg(const double* a, int n, double* out) {
    if (n <= 0) return -1;
    double mx = 0, my = 0;
    for (int i = 0; i < n; ++i) {
        double r = a[i] * DEG_TO_RAD;
        mx += std::cos(r);
        my += std::sin(r);
    }
    double nn = std::sqrt(mx * mx + my * my);
    if (nn > 0) mx /= nn, my /= nn;
    double deg = std::atan2(my, mx) * RAD_TO_DEG;
    if (deg < 0) deg += 360.0;
    *out = deg;
    return 0;
}

// Locomotion::transform_into_symmetric_matrix (Locomotion.cpp:127-138), row-major n x n.
void orc_ref_symmetrize_min(double* A, int n) {
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) A[i * n + j] = A[j * n + i] = std::min(A[i * n + j], A[j * n + i]);
}

// Locomotion::get_dist_vect (Locomotion.cpp:143-162): dx(i,j) = r_i.x - r_j.x, row-major.
void orc_ref_dist_vect(const double* r, int n, double* dx, double* dy) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            dx[i * n + j] = r[2 * i] - r[2 * j];
            dy[i * n + j] = r[2 * i + 1] - r[2 * j + 1];
        }
}

// OrientationHelper::calculate_average_n_within_distance (OrientationHelper.cpp:29-74):
// circular mean of the angles within 2*sigma (self included, d_ii = 0), truncated to int,
// zero noise (OrientationHelper.cpp:41).
int orc_ref_average_n(const double* dl, const int* n_in, int num, double sigma, int* n_out) {
    std::vector<double> ang;
    for (int i = 0; i < num; ++i) {
        ang.clear();
        for (int j = 0; j < num; ++j)
            if (dl[i * num + j] < 2 * sigma) ang.push_back((double)n_in[j]);
        double m;
        if (orc_ref_mean_angle_deg(ang.data(), (int)ang.size(), &m)) return -1;
        n_out[i] = (int)m;
    }
    return 0;
}

// EuclideanTiling::diagonal_seam_edges_square_border (EuclideanTiling.cpp:31-69) with the
// unit-square borders. The reference restarts from particle 0 after every re-wrap; particles
// already inside are unchanged by processPoints, so a per-particle loop gives the same result.
int orc_ref_seam_wrap(double* uv_old, double* uv, int* n_deg, int num) {
    for (int i = 0; i < num; ++i) {
        double nd = n_deg[i];
        for (int guard = 0; guard < 64; ++guard) {
            if (ref_inside(uv[2 * i], uv[2 * i + 1])) break;
            double entry[2];
            ref_process_point(&uv_old[2 * i], &uv[2 * i], &nd, entry);
            if (!ref_inside(uv[2 * i], uv[2 * i + 1])) uv_old[2 * i] = entry[0], uv_old[2 * i + 1] = entry[1];
            if (guard == 63) return -1;
        }
        n_deg[i] = (int)nd;
    }
    return 0;
}

// Full ref-form step: 2DTissue::update -> perform_particle_simulation (2DTissue.cpp:136-252)
// with Locomotion::simulate_flight (Locomotion.cpp:57-89), the seam wrap, get_r3d
// (CellHelper.cpp:71-160), count_particle_neighbors (2DTissue.cpp:254-268) and the order
// parameter. Face search in UV is the brute force argmin over all faces (ties -> lowest id).
// The order parameter is evaluated on zero-padded UV vectors (the reference's 2-column
// cross product is out of bounds, LinearAlgebra.cpp:67-105).
int orc_ref_step(int V, const double* v3, int F, const int* f3, int Vuv, const double* uvv, const int* fuv,
                 const int* uv2v, const double* dist_vv, double v0, double k, double sigma, double r_adh,
                 double k_adh, double step_size, int N, double* r_uv, int* n_deg, int* nearest, double* r3d,
                 double* r_dot, int* nbr_count, double* order_out) {
    (void)V, (void)f3;
    std::vector<double> dx((size_t)N * N), dy((size_t)N * N), dl((size_t)N * N);
    orc_ref_dist_vect(r_uv, N, dx.data(), dy.data());
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) dl[(size_t)i * N + j] = dist_vv[(size_t)nearest[i] * Vuv + nearest[j]];
    for (int i = 0; i < N; ++i) dl[(size_t)i * N + i] = 0.0;
    orc_ref_symmetrize_min(dl.data(), N);
    std::vector<double> Fx(N, 0.0), Fy(N, 0.0), old((size_t)2 * N);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            if (i == j) continue;
            double d = dl[(size_t)i * N + j];
            if (d >= 2 * sigma) continue;
            if (d == 0) d += 0.001;
            double f[2];
            orc_ref_repulsive_adhesion(k, sigma, d, r_adh, k_adh, dx[(size_t)i * N + j], dy[(size_t)i * N + j], f);
            Fx[i] += f[0], Fy[i] += f[1];
        }
    std::memcpy(old.data(), r_uv, sizeof(double) * 2 * N);
    for (int i = 0; i < N; ++i) {
        double a = std::sqrt(Fx[i] * Fx[i] + Fy[i] * Fy[i]) + v0;
        double r = n_deg[i] * DEG_TO_RAD;
        r_dot[2 * i] = std::cos(r) * a;
        r_dot[2 * i + 1] = std::sin(r) * a;
        r_uv[2 * i] += r_dot[2 * i] * step_size;
        r_uv[2 * i + 1] += r_dot[2 * i + 1] * step_size;
    }
    std::vector<int> n_new(N);
    if (orc_ref_average_n(dl.data(), n_deg, N, sigma, n_new.data())) return -1;
    std::memcpy(n_deg, n_new.data(), sizeof(int) * N);
    if (orc_ref_seam_wrap(old.data(), r_uv, n_deg, N)) return -2;
    for (int i = 0; i < N; ++i) {
        double px = r_uv[2 * i], py = r_uv[2 * i + 1];
        double best = 1e300;
        int bf = 0;
        for (int f = 0; f < F; ++f) {
            const int* t = &fuv[3 * f];
            double d = tri_dist(px, py, &uvv[2 * t[0]], &uvv[2 * t[1]], &uvv[2 * t[2]]);
            if (d < best) best = d, bf = f;
        }
        const int* t = &fuv[3 * bf];
        double w[3];
        for (int c = 0; c < 3; ++c) {
            double ex = px - uvv[2 * t[c]], ey = py - uvv[2 * t[c] + 1];
            w[c] = std::sqrt(ex * ex + ey * ey);
        }
        double sw = w[0] + w[1] + w[2];
        for (int c = 0; c < 3; ++c) w[c] /= sw;
        double P[3] = {0, 0, 0};
        for (int c = 0; c < 3; ++c)
            for (int d = 0; d < 3; ++d) P[d] += w[c] * v3[3 * uv2v[t[c]] + d];
        double dist[3];
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int d = 0; d < 3; ++d) {
                double e = P[d] - v3[3 * uv2v[t[c]] + d];
                s += e * e;
            }
            dist[c] = std::sqrt(s);
        }
        double mn = std::min(dist[0], std::min(dist[1], dist[2]));
        nearest[i] = (mn == dist[0]) ? t[0] : (mn == dist[1]) ? t[1] : t[2];
        for (int d = 0; d < 3; ++d) r3d[3 * i + d] = P[d];
    }
    for (int i = 0; i < N; ++i) {
        int c = 0;
        for (int j = 0; j < N; ++j) {
            double d = dl[(size_t)i * N + j];
            if (d != 0 && d <= 2.4 * sigma) ++c;
        }
        nbr_count[i] = c;
    }
    double sz = 0;
    for (int i = 0; i < N; ++i) {
        double z = r_uv[2 * i] * r_dot[2 * i + 1] - r_uv[2 * i + 1] * r_dot[2 * i];
        sz += (z > 0) - (z < 0);
    }
    *order_out = std::fabs(sz) / N;
    return 0;
}

// ---------------------------------------------------------------------------------------
// model-form entry points
// ---------------------------------------------------------------------------------------
orc_mesh* orc_mesh_create(int V, const double* v3, int F, const int* f3, int Vuv, const double* uvv,
                          const int* fuv) {
    (void)V, (void)Vuv;
    orc_mesh* M = new orc_mesh();
    M->faces.resize(F);
    for (int f = 0; f < F; ++f) {
        Face& g = M->faces[f];
        const int* t = &fuv[3 * f];
        const int* s = &f3[3 * f];
        for (int c = 0; c < 2; ++c) g.a[c] = uvv[2 * t[0] + c], g.b[c] = uvv[2 * t[1] + c], g.c[c] = uvv[2 * t[2] + c];
        for (int c = 0; c < 3; ++c) g.iu[c] = t[c];
        double A[3], B[3], C[3];
        for (int c = 0; c < 3; ++c) A[c] = v3[3 * s[0] + c], B[c] = v3[3 * s[1] + c], C[c] = v3[3 * s[2] + c];
        for (int c = 0; c < 3; ++c) g.A[c] = A[c];
        // M = [b-a, c-a] (2x2), E = [B-A, C-A] (3x2), J = E M^-1, Jp = (J^T J)^-1 J^T
        double m00 = g.b[0] - g.a[0], m01 = g.c[0] - g.a[0], m10 = g.b[1] - g.a[1], m11 = g.c[1] - g.a[1];
        double det = m00 * m11 - m01 * m10;
        double i00 = m11 / det, i01 = -m01 / det, i10 = -m10 / det, i11 = m00 / det;
        double E0[3], E1[3];
        for (int c = 0; c < 3; ++c) E0[c] = B[c] - A[c], E1[c] = C[c] - A[c];
        for (int c = 0; c < 3; ++c) {
            g.J[c] = E0[c] * i00 + E1[c] * i10;
            g.J[3 + c] = E0[c] * i01 + E1[c] * i11;
        }
        double a11 = g.J[0] * g.J[0] + g.J[1] * g.J[1] + g.J[2] * g.J[2];
        double a12 = g.J[0] * g.J[3] + g.J[1] * g.J[4] + g.J[2] * g.J[5];
        double a22 = g.J[3] * g.J[3] + g.J[4] * g.J[4] + g.J[5] * g.J[5];
        double dd = a11 * a22 - a12 * a12;
        double b11 = a22 / dd, b12 = -a12 / dd, b22 = a11 / dd;
        for (int c = 0; c < 3; ++c) {
            g.Jp[c] = b11 * g.J[c] + b12 * g.J[3 + c];
            g.Jp[3 + c] = b12 * g.J[c] + b22 * g.J[3 + c];
        }
        double nx = E0[1] * E1[2] - E0[2] * E1[1], ny = E0[2] * E1[0] - E0[0] * E1[2],
               nz = E0[0] * E1[1] - E0[1] * E1[0];
        double nn = std::sqrt(nx * nx + ny * ny + nz * nz);
        g.n[0] = nx / nn, g.n[1] = ny / nn, g.n[2] = nz / nn;
        const double* Cc[3] = {g.a, g.b, g.c};
        for (int k2 = 0; k2 < 3; ++k2) {
            double ex = Cc[(k2 + 1) % 3][0] - Cc[k2][0], ey = Cc[(k2 + 1) % 3][1] - Cc[k2][1];
            g.elen[k2] = std::sqrt(ex * ex + ey * ey);
        }
    }
    // chart edge adjacency from the UV triangles
    M->adj.assign((size_t)3 * F, -1);
    {
        std::unordered_map<uint64_t, int> dir;
        dir.reserve((size_t)3 * F);
        for (int f = 0; f < F; ++f)
            for (int k = 0; k < 3; ++k)
                dir[((uint64_t)(uint32_t)fuv[3 * f + k] << 32) | (uint32_t)fuv[3 * f + (k + 1) % 3]] = f;
        for (int f = 0; f < F; ++f)
            for (int k = 0; k < 3; ++k) {
                auto it = dir.find(((uint64_t)(uint32_t)fuv[3 * f + (k + 1) % 3] << 32) | (uint32_t)fuv[3 * f + k]);
                if (it != dir.end()) M->adj[3 * f + k] = it->second;
            }
    }
    // UV bin grid (closed bounding boxes), faces in ascending id per bin.
    int G = (int)std::ceil(std::sqrt((double)F));
    G = std::max(1, std::min(G, 2048));
    M->G = G;
    std::vector<int> cnt((size_t)G * G + 1, 0);
    auto bbox = [&](const Face& g, int& x0, int& x1, int& y0, int& y1) {
        double xmn = std::min(g.a[0], std::min(g.b[0], g.c[0])), xmx = std::max(g.a[0], std::max(g.b[0], g.c[0]));
        double ymn = std::min(g.a[1], std::min(g.b[1], g.c[1])), ymx = std::max(g.a[1], std::max(g.b[1], g.c[1]));
        x0 = bin_coord(xmn, G), x1 = bin_coord(xmx, G), y0 = bin_coord(ymn, G), y1 = bin_coord(ymx, G);
    };
    for (int f = 0; f < F; ++f) {
        int x0, x1, y0, y1;
        bbox(M->faces[f], x0, x1, y0, y1);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) cnt[y * G + x + 1]++;
    }
    for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
    M->bin_start = cnt;
    M->bin_faces.assign(cnt.back(), 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < F; ++f) {
        int x0, x1, y0, y1;
        bbox(M->faces[f], x0, x1, y0, y1);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) M->bin_faces[fill[y * G + x]++] = f;
    }
    return M;
}

void orc_mesh_free(orc_mesh* m) { delete m; }

void orc_mesh_face_data(const orc_mesh* m, int f, double* J6, double* Jp6, double* n3) {
    const Face& g = m->faces[f];
    std::memcpy(J6, g.J, sizeof g.J);
    std::memcpy(Jp6, g.Jp, sizeof g.Jp);
    std::memcpy(n3, g.n, sizeof g.n);
}

int orc_mesh_locate(const orc_mesh* m, double u, double v, int f_old, int* mode) {
    return locate(*m, u, v, f_old, mode);
}

void orc_mesh_map(const orc_mesh* m, int f, double u, double v, double* r3) {
    const Face& h = m->faces[f];
    double du = u - h.a[0], dv = v - h.a[1];
    for (int k = 0; k < 3; ++k) r3[k] = h.A[k] + h.J[k] * du + h.J[3 + k] * dv;
}

int orc_model_wrap(double* s_uv, double* e_uv, double* theta, double* vuv, int max_wraps, int* n_wraps) {
    return wrap_model<double>(s_uv[0], s_uv[1], e_uv[0], e_uv[1], *theta, vuv[0], vuv[1], max_wraps, n_wraps);
}

int orc_model_step(const orc_mesh* m, const double* prm, int force_mode, uint64_t seed, int64_t step,
                   int local_bits, const double* centroid, int N, const double* uv, const double* theta,
                   const int* face, const double* r3d, const int* ids, const double* noise, int n_sub,
                   const int* sub, double* uv_out, double* theta_out, int* face_out, double* r3d_out,
                   double* vel_uv_out, int* cnt_out, int* wraps_out, double* phi_sums, int* status_out,
                   int n_threads) {
    const orc_mesh& M = *m;
    Params<double> P{prm[0], prm[1], prm[2], prm[3], prm[4], prm[5], prm[6], prm[7], prm[8], prm[9]};
    CellList cl;
    cl.build(N, r3d, P.r_max);
    const int n = sub ? n_sub : N;
    const double r2max = P.r_max * P.r_max;
    int status_all = 0;
    double phi_all[6] = {0, 0, 0, 0, 0, 0};
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
#pragma omp parallel
    {
        double phi_loc[6] = {0, 0, 0, 0, 0, 0};
        int st_loc = 0;
#pragma omp for schedule(static)
        for (int q = 0; q < n; ++q) {
            const int i = sub ? sub[q] : q;
            const uint32_t id = (uint32_t)ids[i];
            const uint32_t rep = local_bits >= 32 ? 0u : (id >> local_bits);
            const uint32_t loc = local_bits >= 32 ? id : (id & ((1u << local_bits) - 1u));
            const double u01 = noise ? 0.0 : noise_u01(seed, step, loc, rep);
            const double* ri = &r3d[3 * i];
            auto nbrs = [&](auto&& fn) {
                cl.for_candidates(ri[0], ri[1], ri[2], [&](int j) {
                    if (j == i) return;
                    const double* rj = &r3d[3 * j];
                    double dx = ri[0] - rj[0], dy = ri[1] - rj[1], dz = ri[2] - rj[2];
                    if (dx * dx + dy * dy + dz * dz < r2max) fn(rj, theta[j], face[j]);
                });
            };
            double u2, v2, th2, r2[3], vel[2], ph[6];
            int f2, cnt, nwr;
            int st = model_particle<double>(M, P, force_mode, noise ? noise[i] : 0.0, noise != nullptr, u01,
                                            centroid, uv[2 * i], uv[2 * i + 1], theta[i], face[i], ri, nbrs, u2,
                                            v2, th2, f2, r2, vel, cnt, nwr, ph);
            uv_out[2 * q] = u2, uv_out[2 * q + 1] = v2;
            theta_out[q] = th2;
            face_out[q] = f2;
            for (int k = 0; k < 3; ++k) r3d_out[3 * q + k] = r2[k];
            if (vel_uv_out) vel_uv_out[2 * q] = vel[0], vel_uv_out[2 * q + 1] = vel[1];
            if (cnt_out) cnt_out[q] = cnt;
            if (wraps_out) wraps_out[q] = nwr;
            for (int k = 0; k < 6; ++k) phi_loc[k] += ph[k];
            st_loc |= st;
        }
#pragma omp critical
        {
            for (int k = 0; k < 6; ++k) phi_all[k] += phi_loc[k];
            status_all |= st_loc;
        }
    }
    if (phi_sums)
        for (int k = 0; k < 6; ++k) phi_sums[k] = phi_all[k];
    if (status_out) *status_out = status_all;
    return 0;
}

int orc_model_step_dual(const orc_mesh* m, const double* prm, const double* dprm, int force_mode, uint64_t seed,
                        int64_t step, int local_bits, const double* centroid, int N, const double* uv,
                        const double* duv, const double* theta, const double* dtheta, const int* face,
                        const double* r3d, const double* dr3d, const int* ids, const double* noise,
                        double* uv_out, double* duv_out, double* theta_out, double* dtheta_out, int* face_out,
                        double* r3d_out, double* dr3d_out, double* phi_sums, double* dphi_sums) {
    const orc_mesh& M = *m;
    Params<Dual> P{Dual(prm[0], dprm[0]), Dual(prm[1], dprm[1]), Dual(prm[2], dprm[2]), Dual(prm[3], dprm[3]),
                   Dual(prm[4], dprm[4]), Dual(prm[5], dprm[5]), Dual(prm[6], dprm[6]), Dual(prm[7], dprm[7]),
                   Dual(prm[8], dprm[8]), Dual(prm[9], dprm[9])};
    CellList cl;
    cl.build(N, r3d, prm[3]);
    const double r2max = prm[3] * prm[3];
    Dual phi_all[6];
    int status = 0;
    for (int i = 0; i < N; ++i) {
        const uint32_t id = (uint32_t)ids[i];
        const uint32_t rep = local_bits >= 32 ? 0u : (id >> local_bits);
        const uint32_t loc = local_bits >= 32 ? id : (id & ((1u << local_bits) - 1u));
        const double u01 = noise ? 0.0 : noise_u01(seed, step, loc, rep);
        const double* ri = &r3d[3 * i];
        Dual rid[3] = {Dual(ri[0], dr3d[3 * i]), Dual(ri[1], dr3d[3 * i + 1]), Dual(ri[2], dr3d[3 * i + 2])};
        auto nbrs = [&](auto&& fn) {
            cl.for_candidates(ri[0], ri[1], ri[2], [&](int j) {
                if (j == i) return;
                const double* rj = &r3d[3 * j];
                double dx = ri[0] - rj[0], dy = ri[1] - rj[1], dz = ri[2] - rj[2];
                if (dx * dx + dy * dy + dz * dz < r2max) {
                    Dual rjd[3] = {Dual(rj[0], dr3d[3 * j]), Dual(rj[1], dr3d[3 * j + 1]),
                                   Dual(rj[2], dr3d[3 * j + 2])};
                    fn(rjd, Dual(theta[j], dtheta[j]), face[j]);
                }
            });
        };
        Dual u2, v2, th2, r2[3], vel[2], ph[6];
        int f2, cnt, nwr;
        status |= model_particle<Dual>(M, P, force_mode, noise ? noise[i] : 0.0, noise != nullptr, u01, centroid,
                                       Dual(uv[2 * i], duv[2 * i]), Dual(uv[2 * i + 1], duv[2 * i + 1]),
                                       Dual(theta[i], dtheta[i]), face[i], rid, nbrs, u2, v2, th2, f2, r2, vel, cnt,
                                       nwr, ph);
        uv_out[2 * i] = u2.v, uv_out[2 * i + 1] = v2.v, duv_out[2 * i] = u2.d, duv_out[2 * i + 1] = v2.d;
        theta_out[i] = th2.v, dtheta_out[i] = th2.d;
        face_out[i] = f2;
        for (int k = 0; k < 3; ++k) r3d_out[3 * i + k] = r2[k].v, dr3d_out[3 * i + k] = r2[k].d;
        for (int k = 0; k < 6; ++k) phi_all[k] += ph[k];
    }
    for (int k = 0; k < 6; ++k) phi_sums[k] = phi_all[k].v, dphi_sums[k] = phi_all[k].d;
    return status;
}

}  // extern "C"
