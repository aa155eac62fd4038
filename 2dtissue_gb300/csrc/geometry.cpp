#include "geometry.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include "philox.cuh"

namespace tds {

void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    tdsr::philox10(ctr, key, out);
}

void build_face_tables(const Mesh& m, FaceTables& t) {
    const int F = m.F();
    t.F = F;
    t.rec.assign((size_t)F * kFaceRec, 0.0);
    t.area_cdf.assign(F, 0.0);
    double acc = 0;
    for (int f = 0; f < F; ++f) {
        double* r = &t.rec[(size_t)f * kFaceRec];
        const int* tu = &m.fuv[3 * f];
        const int* t3 = &m.f3[3 * f];
        double a[2], b[2], c[2], A[3], B[3], C[3];
        for (int k = 0; k < 2; ++k) a[k] = m.uv[2 * tu[0] + k], b[k] = m.uv[2 * tu[1] + k], c[k] = m.uv[2 * tu[2] + k];
        for (int k = 0; k < 3; ++k) A[k] = m.v3[3 * t3[0] + k], B[k] = m.v3[3 * t3[1] + k], C[k] = m.v3[3 * t3[2] + k];
        const double m00 = b[0] - a[0], m01 = c[0] - a[0], m10 = b[1] - a[1], m11 = c[1] - a[1];
        const double det = m00 * m11 - m01 * m10;
        const double i00 = m11 / det, i01 = -m01 / det, i10 = -m10 / det, i11 = m00 / det;
        double E0[3], E1[3];
        for (int k = 0; k < 3; ++k) E0[k] = B[k] - A[k], E1[k] = C[k] - A[k];
        double J[6];
        for (int k = 0; k < 3; ++k) {
            J[k] = E0[k] * i00 + E1[k] * i10;
            J[3 + k] = E0[k] * i01 + E1[k] * i11;
        }
        const double a11 = J[0] * J[0] + J[1] * J[1] + J[2] * J[2];
        const double a12 = J[0] * J[3] + J[1] * J[4] + J[2] * J[5];
        const double a22 = J[3] * J[3] + J[4] * J[4] + J[5] * J[5];
        const double dd = a11 * a22 - a12 * a12;
        const double b11 = a22 / dd, b12 = -a12 / dd, b22 = a11 / dd;
        for (int k = 0; k < 6; ++k) r[k] = J[k];
        for (int k = 0; k < 3; ++k) {
            r[6 + k] = b11 * J[k] + b12 * J[3 + k];
            r[9 + k] = b12 * J[k] + b22 * J[3 + k];
        }
        const double nx = E0[1] * E1[2] - E0[2] * E1[1], ny = E0[2] * E1[0] - E0[0] * E1[2],
                     nz = E0[0] * E1[1] - E0[1] * E1[0];
        const double nn = std::sqrt(nx * nx + ny * ny + nz * nz);
        r[12] = nx / nn, r[13] = ny / nn, r[14] = nz / nn;
        r[16] = a[0], r[17] = a[1], r[18] = b[0], r[19] = b[1], r[20] = c[0], r[21] = c[1];
        r[24] = A[0], r[25] = A[1], r[26] = A[2];
        const double* P[3] = {a, b, c};
        int bits = 0;
        for (int k = 0; k < 3; ++k) {
            const double ex = P[(k + 1) % 3][0] - P[k][0], ey = P[(k + 1) % 3][1] - P[k][1];
            r[28 + k] = 1.0 / std::sqrt(ex * ex + ey * ey);
            if (tu[k] > tu[(k + 1) % 3]) bits |= 1 << k;
        }
        r[22] = (double)bits;
        acc += 0.5 * nn;
        t.area_cdf[f] = acc;
    }
    t.area = acc;
    for (int f = 0; f < F; ++f) t.area_cdf[f] /= acc;
    t.area_cdf[F - 1] = 1.0;

    // UV bins: closed bounding boxes widened by 1e-6 so that an FP32 bin assignment of a point
    // on a bin border still finds every face that contains it.
    int G = (int)std::ceil(std::sqrt((double)F));
    G = std::max(1, std::min(G, 4096));
    t.G = G;
    auto bc = [G](double x) {
        int v = (int)std::floor(x * G);
        return v < 0 ? 0 : (v >= G ? G - 1 : v);
    };
    const double eps = 1e-6;
    std::vector<int> cnt((size_t)G * G + 1, 0);
    auto box = [&](int f, int& x0, int& x1, int& y0, int& y1) {
        const double* r = &t.rec[(size_t)f * kFaceRec];
        double xmn = std::min(r[16], std::min(r[18], r[20])), xmx = std::max(r[16], std::max(r[18], r[20]));
        double ymn = std::min(r[17], std::min(r[19], r[21])), ymx = std::max(r[17], std::max(r[19], r[21]));
        x0 = bc(xmn - eps), x1 = bc(xmx + eps), y0 = bc(ymn - eps), y1 = bc(ymx + eps);
    };
    for (int f = 0; f < F; ++f) {
        int x0, x1, y0, y1;
        box(f, x0, x1, y0, y1);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) cnt[(size_t)y * G + x + 1]++;
    }
    for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
    t.bin_start = cnt;
    t.bin_faces.assign(cnt.back(), 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < F; ++f) {
        int x0, x1, y0, y1;
        box(f, x0, x1, y0, y1);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) t.bin_faces[fill[(size_t)y * G + x]++] = f;
    }

    for (int k = 0; k < 3; ++k) t.lo[k] = 1e300, t.hi[k] = -1e300, t.centroid[k] = 0;
    for (int i = 0; i < m.V(); ++i)
        for (int k = 0; k < 3; ++k) {
            t.lo[k] = std::min(t.lo[k], m.v3[3 * i + k]);
            t.hi[k] = std::max(t.hi[k], m.v3[3 * i + k]);
            t.centroid[k] += m.v3[3 * i + k];
        }
    for (int k = 0; k < 3; ++k) t.centroid[k] /= m.V();
}

void build_face_adjacency(const Mesh& m, std::vector<int>& adj) {
    const int F = m.F();
    adj.assign((size_t)3 * F, -1);
    std::unordered_map<uint64_t, int> dir;
    dir.reserve((size_t)3 * F);
    for (int f = 0; f < F; ++f)
        for (int k = 0; k < 3; ++k) {
            const uint32_t a = (uint32_t)m.fuv[3 * f + k], b = (uint32_t)m.fuv[3 * f + (k + 1) % 3];
            dir[((uint64_t)a << 32) | b] = 3 * f + k;
        }
    for (int f = 0; f < F; ++f)
        for (int k = 0; k < 3; ++k) {
            const uint32_t a = (uint32_t)m.fuv[3 * f + k], b = (uint32_t)m.fuv[3 * f + (k + 1) % 3];
            auto it = dir.find(((uint64_t)b << 32) | a);
            if (it != dir.end()) adj[3 * f + k] = it->second / 3;
        }
}

namespace {

// Triangle / axis-aligned box overlap by the separating-axis theorem: the box normals, the
// triangle normal and the nine cross products of box axes with triangle edges.
bool tri_box_overlap(const double c[3], const double hw[3], const double* v0, const double* v1, const double* v2) {
    double a[3], b[3], d[3];
    for (int k = 0; k < 3; ++k) a[k] = v0[k] - c[k], b[k] = v1[k] - c[k], d[k] = v2[k] - c[k];
    const double* v[3] = {a, b, d};
    for (int k = 0; k < 3; ++k) {
        double mn = std::min(a[k], std::min(b[k], d[k])), mx = std::max(a[k], std::max(b[k], d[k]));
        if (mn > hw[k] || mx < -hw[k]) return false;
    }
    double e[3][3];
    for (int k = 0; k < 3; ++k) e[0][k] = b[k] - a[k], e[1][k] = d[k] - b[k], e[2][k] = a[k] - d[k];
    const double nrm[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                           e[0][0] * e[1][1] - e[0][1] * e[1][0]};
    {
        const double p = nrm[0] * a[0] + nrm[1] * a[1] + nrm[2] * a[2];
        const double r = hw[0] * std::fabs(nrm[0]) + hw[1] * std::fabs(nrm[1]) + hw[2] * std::fabs(nrm[2]);
        if (std::fabs(p) > r) return false;
    }
    for (int i = 0; i < 3; ++i)      // box axis
        for (int j = 0; j < 3; ++j) {  // triangle edge
            double ax[3] = {0, 0, 0};
            // axis = unit_i x e_j
            const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            ax[i1] = -e[j][i2];
            ax[i2] = e[j][i1];
            double mn = 1e300, mx = -1e300;
            for (int t = 0; t < 3; ++t) {
                const double p = ax[0] * v[t][0] + ax[1] * v[t][1] + ax[2] * v[t][2];
                mn = std::min(mn, p), mx = std::max(mx, p);
            }
            const double r = hw[0] * std::fabs(ax[0]) + hw[1] * std::fabs(ax[1]) + hw[2] * std::fabs(ax[2]);
            if (mn > r || mx < -r) return false;
        }
    return true;
}

}  // namespace

void build_cell_level(const Mesh& m, double h, const double origin[3], CellLevel& L) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, amax = 0;
    for (int i = 0; i < m.V(); ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], m.v3[3 * i + k]), hi[k] = std::max(hi[k], m.v3[3 * i + k]);
            amax = std::max(amax, std::fabs(m.v3[3 * i + k]));
        }
    L.h = h;
    L.gx = (int)std::ceil((hi[0] - origin[0]) / h) + 3;
    L.gy = (int)std::ceil((hi[1] - origin[1]) / h) + 3;
    L.gz = (int)std::ceil((hi[2] - origin[2]) / h) + 3;
    // Cells are widened by eps so that a position rounded to FP32 (error ~ 2^-23 |r|) always
    // falls into a listed cell.
    const double eps = 1e-5 * (amax + h);
    const double hw[3] = {0.5 * h + eps, 0.5 * h + eps, 0.5 * h + eps};
    std::vector<int64_t> keys;
    for (int f = 0; f < m.F(); ++f) {
        const double* p[3] = {&m.v3[3 * m.f3[3 * f]], &m.v3[3 * m.f3[3 * f + 1]], &m.v3[3 * m.f3[3 * f + 2]]};
        int c0[3], c1[3];
        for (int k = 0; k < 3; ++k) {
            double mn = std::min(p[0][k], std::min(p[1][k], p[2][k])), mx = std::max(p[0][k], std::max(p[1][k], p[2][k]));
            c0[k] = (int)std::floor((mn - eps - origin[k]) / h);
            c1[k] = (int)std::floor((mx + eps - origin[k]) / h);
        }
        for (int iz = c0[2]; iz <= c1[2]; ++iz)
            for (int iy = c0[1]; iy <= c1[1]; ++iy)
                for (int ix = c0[0]; ix <= c1[0]; ++ix) {
                    const double cc[3] = {origin[0] + (ix + 0.5) * h, origin[1] + (iy + 0.5) * h,
                                          origin[2] + (iz + 0.5) * h};
                    if (tri_box_overlap(cc, hw, p[0], p[1], p[2]))
                        keys.push_back(((int64_t)iz * L.gy + iy) * L.gx + ix);
                }
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    L.C = (int)keys.size();
    L.rows.assign((size_t)2 * L.gy * L.gz, 0);
    L.ivals.clear();
    for (size_t i = 0; i < keys.size();) {
        const int64_t row = keys[i] / L.gx;
        const int x0 = (int)(keys[i] % L.gx);
        size_t j = i + 1;
        while (j < keys.size() && keys[j] == keys[j - 1] + 1 && keys[j] / L.gx == row) ++j;
        const int x1 = x0 + (int)(j - i) - 1;
        if (L.rows[2 * row + 1] == 0) L.rows[2 * row] = (int)(L.ivals.size() / 4);
        L.rows[2 * row + 1] += 1;
        L.ivals.insert(L.ivals.end(), {x0, x1, (int)i, 0});
        i = j;
    }
}

void build_cell_descriptors(const CellLevel& L, std::vector<uint32_t>& desc) {
    desc.assign((size_t)L.C * 8, 0u);
    for (int r = 0; r < L.gy * L.gz; ++r) {
        const int iy = r % L.gy, iz = r / L.gy;
        for (int k = 0; k < L.rows[2 * r + 1]; ++k) {
            const int* I = &L.ivals[4 * (L.rows[2 * r] + k)];
            for (int ix = I[0]; ix <= I[1]; ++ix) {
                const int id = I[2] + ix - I[0];
                int w = 0;
                for (int e = 0; e < 9; ++e) {
                    const int dy = e % 3 - 1, dz = e / 3 - 1;
                    int first = -1, len = 0;
                    if (iy + dy >= 0 && iy + dy < L.gy && iz + dz >= 0 && iz + dz < L.gz) {
                        const int rr = (iz + dz) * L.gy + (iy + dy);
                        for (int q = 0; q < L.rows[2 * rr + 1]; ++q) {
                            const int* J = &L.ivals[4 * (L.rows[2 * rr] + q)];
                            const int lo = std::max(J[0], ix - 1), hi = std::min(J[1], ix + 1);
                            if (lo > hi) continue;
                            // ids are consecutive along the row; runs from two intervals are merged
                            if (first < 0) first = J[2] + lo - J[0];
                            len = (J[2] + hi - J[0]) - first + 1;
                        }
                    }
                    if (e == 4) {
                        // the cell's own row: first = id - L, len = 1 + L + R, with L, R whether
                        // x-1 and x+1 are surface cells; kept as two bits of word 0
                        const int Lb = id - first, Rb = len - 1 - Lb;
                        desc[(size_t)id * 8] |= ((uint32_t)Lb << 2) | ((uint32_t)Rb << 3);
                        continue;
                    }
                    if (first >= 0) desc[(size_t)id * 8 + w] |= ((uint32_t)first << 4) | (uint32_t)len;
                    ++w;
                }
            }
        }
    }
}


}  // namespace tds
