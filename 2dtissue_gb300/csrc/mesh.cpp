// Closed-surface mesh generation, OFF IO and the unit-square UV chart (see mesh.hpp).
#include "mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <queue>
#include <sstream>
#include <unordered_map>

namespace tds {

namespace {

inline uint64_t ekey(int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

struct V3 {
    double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 vget(const Mesh& m, int i) { return {m.v3[3 * i], m.v3[3 * i + 1], m.v3[3 * i + 2]}; }

}  // namespace

void make_icosphere(int level, Mesh& m) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    const double base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                                {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    const int faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                              {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                              {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                              {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
    m = Mesh();
    for (auto& b : base) {
        double n = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        m.v3.push_back(b[0] / n);
        m.v3.push_back(b[1] / n);
        m.v3.push_back(b[2] / n);
    }
    for (auto& f : faces) m.f3.insert(m.f3.end(), {f[0], f[1], f[2]});
    for (int l = 0; l < level; ++l) {
        std::unordered_map<uint64_t, int> mid;
        mid.reserve(m.f3.size());
        auto midpoint = [&](int a, int b) {
            uint64_t k = ekey(std::min(a, b), std::max(a, b));
            auto it = mid.find(k);
            if (it != mid.end()) return it->second;
            V3 pa = vget(m, a), pb = vget(m, b);
            V3 c = {(pa.x + pb.x) * 0.5, (pa.y + pb.y) * 0.5, (pa.z + pb.z) * 0.5};
            double n = norm(c);
            int id = m.V();
            m.v3.insert(m.v3.end(), {c.x / n, c.y / n, c.z / n});
            mid.emplace(k, id);
            return id;
        };
        std::vector<int32_t> nf;
        nf.reserve(m.f3.size() * 4);
        for (int f = 0; f < m.F(); ++f) {
            int a = m.f3[3 * f], b = m.f3[3 * f + 1], c = m.f3[3 * f + 2];
            int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            nf.insert(nf.end(), {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca});
        }
        m.f3.swap(nf);
    }
    orient_outward(m);
}

void scale_axes(Mesh& m, double ax, double ay, double az) {
    for (int i = 0; i < m.V(); ++i) {
        m.v3[3 * i] *= ax;
        m.v3[3 * i + 1] *= ay;
        m.v3[3 * i + 2] *= az;
    }
}

void bumpy_sphere(Mesh& m, double amp, double scale) {
    const double c = 3.0 / 8.0 * std::sqrt(5.0 / (2.0 * M_PI));
    for (int i = 0; i < m.V(); ++i) {
        V3 p = vget(m, i);
        double r = norm(p);
        double ct = p.z / r, st2 = 1.0 - ct * ct;
        double phi = std::atan2(p.y, p.x);
        double y42 = c * st2 * (7.0 * ct * ct - 1.0) * std::cos(2.0 * phi);
        double s = (1.0 + amp * y42) * scale / r;
        m.v3[3 * i] = p.x * s;
        m.v3[3 * i + 1] = p.y * s;
        m.v3[3 * i + 2] = p.z * s;
    }
}

void orient_outward(Mesh& m) {
    V3 c = {0, 0, 0};
    for (int i = 0; i < m.V(); ++i) {
        V3 p = vget(m, i);
        c.x += p.x, c.y += p.y, c.z += p.z;
    }
    c.x /= m.V(), c.y /= m.V(), c.z /= m.V();
    for (int f = 0; f < m.F(); ++f) {
        int* t = &m.f3[3 * f];
        V3 a = vget(m, t[0]), b = vget(m, t[1]), cc = vget(m, t[2]);
        V3 n = cross(sub(b, a), sub(cc, a));
        V3 g = {(a.x + b.x + cc.x) / 3 - c.x, (a.y + b.y + cc.y) / 3 - c.y, (a.z + b.z + cc.z) / 3 - c.z};
        if (dot(n, g) < 0) std::swap(t[1], t[2]);
    }
}

namespace {

// Shortest edge path (3D Euclidean edge lengths) from src to dst avoiding `blocked` vertices.
// Ties are broken towards lower vertex ids so that the seam is deterministic.
std::vector<int> dijkstra_path(const std::vector<std::vector<std::pair<int, double>>>& adj, int src, int dst,
                               const std::vector<char>& blocked) {
    const int n = (int)adj.size();
    std::vector<double> dist(n, std::numeric_limits<double>::infinity());
    std::vector<int> prev(n, -1);
    using Item = std::pair<double, int>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
    dist[src] = 0;
    pq.push({0.0, src});
    while (!pq.empty()) {
        auto [d, u] = pq.top();
        pq.pop();
        if (d > dist[u]) continue;
        if (u == dst) break;
        for (auto [v, w] : adj[u]) {
            if (blocked[v]) continue;
            double nd = d + w;
            if (nd < dist[v] || (nd == dist[v] && u < prev[v])) {
                dist[v] = nd;
                prev[v] = u;
                pq.push({nd, v});
            }
        }
    }
    std::vector<int> path;
    if (prev[dst] < 0 && dst != src) return path;
    for (int v = dst; v != -1; v = prev[v]) path.push_back(v);
    std::reverse(path.begin(), path.end());
    return path;
}

// Jacobi-preconditioned conjugate gradients on the interior graph Laplacian (uniform weights):
// deg(i) u_i - sum_{j interior} u_j = sum_{j boundary} u_j. Serial, fixed operation order, so
// the chart is bit-identical on every host that compiles with -ffp-contract=off.
int solve_tutte(const std::vector<std::vector<int>>& nbr, const std::vector<char>& fixed, std::vector<double>& uv,
                std::string& err) {
    const int n = (int)nbr.size();
    std::vector<int> idx(n, -1), inv;
    for (int i = 0; i < n; ++i)
        if (!fixed[i]) {
            idx[i] = (int)inv.size();
            inv.push_back(i);
        }
    const int m = (int)inv.size();
    if (m == 0) return 0;
    std::vector<int> rs(m + 1, 0), cols;
    std::vector<double> diag(m);
    for (int k = 0; k < m; ++k) {
        int i = inv[k];
        diag[k] = (double)nbr[i].size();
        for (int j : nbr[i])
            if (!fixed[j]) cols.push_back(idx[j]);
        rs[k + 1] = (int)cols.size();
    }
    auto apply = [&](const std::vector<double>& in, std::vector<double>& out) {
        for (int k = 0; k < m; ++k) {
            double acc = diag[k] * in[k];
            for (int e = rs[k]; e < rs[k + 1]; ++e) acc -= in[cols[e]];
            out[k] = acc;
        }
    };
    for (int c = 0; c < 2; ++c) {
        std::vector<double> b(m, 0.0), x(m, 0.5), r(m), z(m), p(m), Ap(m);
        for (int k = 0; k < m; ++k)
            for (int j : nbr[inv[k]])
                if (fixed[j]) b[k] += uv[2 * j + c];
        apply(x, Ap);
        double bnorm = 0, rz = 0;
        for (int k = 0; k < m; ++k) {
            r[k] = b[k] - Ap[k];
            z[k] = r[k] / diag[k];
            p[k] = z[k];
            rz += r[k] * z[k];
            bnorm += b[k] * b[k];
        }
        bnorm = std::sqrt(std::max(bnorm, 1e-300));
        int it = 0;
        const int max_it = 100000;
        for (; it < max_it; ++it) {
            double rn = 0;
            for (int k = 0; k < m; ++k) rn += r[k] * r[k];
            if (std::sqrt(rn) <= 1e-13 * bnorm) break;
            apply(p, Ap);
            double pAp = 0;
            for (int k = 0; k < m; ++k) pAp += p[k] * Ap[k];
            const double alpha = rz / pAp;
            double rz_new = 0;
            for (int k = 0; k < m; ++k) {
                x[k] += alpha * p[k];
                r[k] -= alpha * Ap[k];
                z[k] = r[k] / diag[k];
                rz_new += r[k] * z[k];
            }
            const double beta = rz_new / rz;
            rz = rz_new;
            for (int k = 0; k < m; ++k) p[k] = z[k] + beta * p[k];
        }
        if (it == max_it) {
            err = "Tutte solve did not converge";
            return 1;
        }
        for (int k = 0; k < m; ++k) uv[2 * inv[k] + c] = x[k];
    }
    return 0;
}

}  // namespace

int build_chart(Mesh& m, std::string& err) {
    const int V = m.V(), F = m.F();
    if (V < 4 || F < 4) {
        err = "mesh too small";
        return 1;
    }
    if (2 * V - 4 != F) {
        err = "mesh is not a closed genus-0 triangulation (need F = 2V - 4)";
        return 1;
    }
    // Directed edge -> face, and vertex adjacency with 3D edge lengths.
    std::unordered_map<uint64_t, int> dface;
    dface.reserve((size_t)F * 3 * 2);
    std::vector<std::vector<std::pair<int, double>>> adj(V);
    for (int f = 0; f < F; ++f)
        for (int k = 0; k < 3; ++k) {
            int a = m.f3[3 * f + k], b = m.f3[3 * f + (k + 1) % 3];
            if (!dface.emplace(ekey(a, b), f).second) {
                err = "non-manifold or inconsistently oriented mesh";
                return 1;
            }
        }
    for (auto& kv : dface) {
        int a = (int)(kv.first >> 32), b = (int)(uint32_t)kv.first;
        if (!dface.count(ekey(b, a))) {
            err = "mesh has a boundary edge (not closed)";
            return 1;
        }
        adj[a].push_back({b, norm(sub(vget(m, a), vget(m, b)))});
    }
    for (auto& a : adj) std::sort(a.begin(), a.end());

    // Seam end points: P0 = min x, P2 = max x, P1 = max y (ties -> lowest id).
    int p0 = 0, p1 = 0, p2 = 0;
    for (int i = 1; i < V; ++i) {
        if (m.v3[3 * i] < m.v3[3 * p0]) p0 = i;
        if (m.v3[3 * i] > m.v3[3 * p2]) p2 = i;
        if (m.v3[3 * i + 1] > m.v3[3 * p1 + 1]) p1 = i;
    }
    std::vector<char> blocked(V, 0);
    blocked[p2] = 1;
    std::vector<int> path1 = dijkstra_path(adj, p0, p1, blocked);
    if (path1.size() < 2) {
        err = "no seam path P0->P1";
        return 1;
    }
    std::fill(blocked.begin(), blocked.end(), 0);
    for (size_t k = 0; k + 1 < path1.size(); ++k) blocked[path1[k]] = 1;
    std::vector<int> path2 = dijkstra_path(adj, p1, p2, blocked);
    if (path2.size() < 2) {
        err = "no seam path P1->P2";
        return 1;
    }
    std::vector<int> seam = path1;
    seam.insert(seam.end(), path2.begin() + 1, path2.end());
    const int nS = (int)seam.size(), mP1 = (int)path1.size() - 1;
    m.seam = seam;
    m.seam_p1 = mP1;

    // For every interior seam vertex, the faces on the left of the directed seam P0->P2.
    std::vector<int> seam_pos(V, -1);
    for (int k = 0; k < nS; ++k) seam_pos[seam[k]] = k;
    std::unordered_map<uint64_t, char> left_of;  // (face, vertex) -> 1 if face is on the left side
    for (int k = 1; k + 1 < nS; ++k) {
        int v = seam[k], nxt = seam[k + 1], prv = seam[k - 1];
        auto it = dface.find(ekey(v, nxt));
        if (it == dface.end()) {
            err = "seam edge missing";
            return 1;
        }
        int f = it->second;
        for (int guard = 0; guard < 4096; ++guard) {
            left_of[ekey(f, v)] = 1;
            int* t = &m.f3[3 * f];
            int c = (t[0] == v) ? 0 : (t[1] == v) ? 1 : 2;
            int b = t[(c + 2) % 3];  // face = (v, a, b) in CCW order
            if (b == prv) break;
            auto jt = dface.find(ekey(v, b));
            if (jt == dface.end()) {
                err = "fan walk failed";
                return 1;
            }
            f = jt->second;
            if (guard == 4095) {
                err = "fan walk did not terminate";
                return 1;
            }
        }
    }

    // Chart vertices: one per 3D vertex, plus a second copy (side B) for interior seam vertices.
    std::vector<int> uvA(V), uvB(V, -1);
    m.uv2v.clear();
    for (int i = 0; i < V; ++i) {
        uvA[i] = (int)m.uv2v.size();
        m.uv2v.push_back(i);
    }
    for (int k = 1; k + 1 < nS; ++k) {
        uvB[seam[k]] = (int)m.uv2v.size();
        m.uv2v.push_back(seam[k]);
    }
    const int Vuv = (int)m.uv2v.size();
    m.fuv.assign(m.f3.begin(), m.f3.end());
    for (int f = 0; f < F; ++f)
        for (int c = 0; c < 3; ++c) {
            int v = m.f3[3 * f + c];
            int k = seam_pos[v];
            if (k > 0 && k + 1 < nS && !left_of.count(ekey(f, v))) m.fuv[3 * f + c] = uvB[v];
            else m.fuv[3 * f + c] = uvA[v];
        }

    // Boundary: arc-length parameters along each seam segment.
    m.uv.assign((size_t)Vuv * 2, 0.5);
    std::vector<char> fixed(Vuv, 0);
    std::vector<double> s(nS, 0.0);
    for (int k = 1; k <= mP1; ++k) s[k] = s[k - 1] + norm(sub(vget(m, seam[k]), vget(m, seam[k - 1])));
    for (int k = 1; k < mP1; ++k) s[k] /= s[mP1];
    s[mP1] = 1.0;
    std::vector<double> u(nS, 0.0);
    for (int k = mP1 + 1; k < nS; ++k) u[k] = u[k - 1] + norm(sub(vget(m, seam[k]), vget(m, seam[k - 1])));
    for (int k = mP1 + 1; k < nS - 1; ++k) u[k] /= u[nS - 1];
    u[nS - 1] = 1.0;
    auto setuv = [&](int id, double x, double y) {
        m.uv[2 * id] = x;
        m.uv[2 * id + 1] = y;
        fixed[id] = 1;
    };
    setuv(uvA[seam[0]], 0.0, 0.0);
    for (int k = 1; k < mP1; ++k) {
        setuv(uvA[seam[k]], s[k], 0.0);
        setuv(uvB[seam[k]], 0.0, s[k]);
    }
    setuv(uvA[seam[mP1]], 1.0, 0.0);
    setuv(uvB[seam[mP1]], 0.0, 1.0);
    for (int k = mP1 + 1; k < nS - 1; ++k) {
        setuv(uvA[seam[k]], 1.0, u[k]);
        setuv(uvB[seam[k]], u[k], 1.0);
    }
    setuv(uvA[seam[nS - 1]], 1.0, 1.0);

    // Interior: uniform-weight Tutte embedding (a convex boundary gives a valid embedding).
    std::vector<std::vector<int>> nbr(Vuv);
    for (int f = 0; f < F; ++f)
        for (int c = 0; c < 3; ++c) {
            int a = m.fuv[3 * f + c], b = m.fuv[3 * f + (c + 1) % 3];
            nbr[a].push_back(b);
            nbr[b].push_back(a);
        }
    for (auto& n : nbr) {
        std::sort(n.begin(), n.end());
        n.erase(std::unique(n.begin(), n.end()), n.end());
    }
    if (solve_tutte(nbr, fixed, m.uv, err)) return 1;

    // Orientation: transpose the chart if it came out clockwise (the gluing is symmetric).
    int pos = 0, neg = 0;
    for (int f = 0; f < F; ++f) {
        const int* t = &m.fuv[3 * f];
        double ax = m.uv[2 * t[0]], ay = m.uv[2 * t[0] + 1];
        double bx = m.uv[2 * t[1]], by = m.uv[2 * t[1] + 1];
        double cx = m.uv[2 * t[2]], cy = m.uv[2 * t[2] + 1];
        double a2 = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
        (a2 > 0 ? pos : neg)++;
    }
    if (neg > pos)
        for (int i = 0; i < Vuv; ++i) std::swap(m.uv[2 * i], m.uv[2 * i + 1]);
    return check_chart(m, err);
}

int check_chart(const Mesh& m, std::string& err) {
    const int F = m.F(), Vuv = m.Vuv();
    double area = 0;
    for (int f = 0; f < F; ++f) {
        const int* t = &m.fuv[3 * f];
        double ax = m.uv[2 * t[0]], ay = m.uv[2 * t[0] + 1];
        double bx = m.uv[2 * t[1]], by = m.uv[2 * t[1] + 1];
        double cx = m.uv[2 * t[2]], cy = m.uv[2 * t[2] + 1];
        double a2 = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
        if (!(a2 > 0)) {
            char buf[128];
            std::snprintf(buf, sizeof buf, "chart face %d is flipped or degenerate (2A=%g)", f, a2);
            err = buf;
            return 1;
        }
        area += 0.5 * a2;
    }
    if (std::fabs(area - 1.0) > 1e-9) {
        err = "chart does not cover the unit square";
        return 1;
    }
    // Glued twins: (s,0) <-> (0,s) and (1,s) <-> (s,1) must be the same 3D vertex.
    std::unordered_map<uint64_t, int> at;
    auto q = [](double x) { return (uint64_t)std::llround(x * 1e12); };
    for (int i = 0; i < Vuv; ++i) {
        double x = m.uv[2 * i], y = m.uv[2 * i + 1];
        if (x < 0 || x > 1 || y < 0 || y > 1) {
            err = "chart vertex outside the unit square";
            return 1;
        }
        if (x == 0 || x == 1 || y == 0 || y == 1) at[(q(x) << 20) ^ q(y) * 1000003ull] = m.uv2v[i];
    }
    for (int i = 0; i < Vuv; ++i) {
        double x = m.uv[2 * i], y = m.uv[2 * i + 1];
        bool on_b = (y == 0 || x == 1), on_l = (x == 0 || y == 1);
        if (!(on_b || on_l)) continue;
        auto it = at.find((q(y) << 20) ^ q(x) * 1000003ull);  // transposed twin
        if (it == at.end() || it->second != m.uv2v[i]) {
            err = "seam twin mismatch";
            return 1;
        }
    }
    return 0;
}

int read_off(const std::string& path, Mesh& m, std::string& err) {
    std::ifstream in(path);
    if (!in) {
        err = "cannot open " + path;
        return 1;
    }
    std::string tok;
    auto next = [&](std::string& t) {
        while (in >> t) {
            if (t[0] == '#') {
                std::getline(in, t);
                continue;
            }
            return true;
        }
        return false;
    };
    if (!next(tok) || tok != "OFF") {
        err = "not an OFF file";
        return 1;
    }
    long nv, nf, ne;
    std::string a, b, c;
    if (!next(a) || !next(b) || !next(c)) {
        err = "truncated OFF header";
        return 1;
    }
    nv = std::stol(a), nf = std::stol(b), ne = std::stol(c);
    (void)ne;
    m = Mesh();
    m.v3.resize(nv * 3);
    for (long i = 0; i < nv * 3; ++i) {
        if (!next(tok)) {
            err = "truncated OFF vertices";
            return 1;
        }
        m.v3[i] = std::stod(tok);
    }
    for (long f = 0; f < nf; ++f) {
        if (!next(tok) || std::stol(tok) != 3) {
            err = "OFF face is not a triangle";
            return 1;
        }
        for (int k = 0; k < 3; ++k) {
            if (!next(tok)) {
                err = "truncated OFF faces";
                return 1;
            }
            long id = std::stol(tok);
            if (id < 0 || id >= nv) {
                err = "OFF face index out of range";
                return 1;
            }
            m.f3.push_back((int32_t)id);
        }
    }
    return 0;
}

int write_off(const std::string& path, const Mesh& m, std::string& err) {
    std::FILE* fp = std::fopen(path.c_str(), "w");
    if (!fp) {
        err = "cannot write " + path;
        return 1;
    }
    std::fprintf(fp, "OFF\n%d %d 0\n", m.V(), m.F());
    for (int i = 0; i < m.V(); ++i)
        std::fprintf(fp, "%.17g %.17g %.17g\n", m.v3[3 * i], m.v3[3 * i + 1], m.v3[3 * i + 2]);
    for (int f = 0; f < m.F(); ++f) std::fprintf(fp, "3 %d %d %d\n", m.f3[3 * f], m.f3[3 * f + 1], m.f3[3 * f + 2]);
    std::fclose(fp);
    return 0;
}

}  // namespace tds
