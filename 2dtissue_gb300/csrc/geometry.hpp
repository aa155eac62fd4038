// Host-side tables derived from a charted mesh: per-face chart maps, the UV bin grid for point
// location, the folded 3D cell-grid layout, and seeded initial particle placement.
#pragma once
#include <cstdint>
#include <vector>

#include "mesh.hpp"

namespace tds {

// Per-face record, 32 reals (one 128-byte line in FP32):
//   [0..5]   J   = dX/d(uv), column u = [0..2], column v = [3..5]
//   [6..11]  Jp  = (J^T J)^-1 J^T, row 0 = [6..8], row 1 = [9..11]
//   [12..14] n   = unit normal of the 3D triangle (outward)
//   [16..21] UV corners a, b, c (CCW)
//   [22..24] 3D corner A (image of a)
//   [25..27] 1 / UV edge length of edges a->b, b->c, c->a
//   [28]     canonical-orientation bits: bit k set when edge k runs from the higher to the
//            lower chart-vertex id (its orientation value is evaluated reversed and negated)
constexpr int kFaceRec = 32;

struct FaceTables {
    int F = 0;
    std::vector<double> rec;  // F * kFaceRec
    int G = 1;                // UV bin grid G x G over [0,1]^2
    std::vector<int> bin_start, bin_faces;
    double lo[3], hi[3];      // 3D bounding box
    double centroid[3];       // mean of the 3D vertices
    std::vector<double> area_cdf;  // cumulative 3D face areas (normalised to 1)
    double area = 0;               // total 3D surface area
};

void build_face_tables(const Mesh& m, FaceTables& t);

// Folded cell grid for one replica: bucket = base + (ix & (2^lx-1)) | (iy & (2^ly-1)) << lx
//                                              | (iz & (2^lz-1)) << (lx+ly)
struct Fold {
    int lx = 2, ly = 2, lz = 2;
    int64_t M = 64;
};
Fold choose_fold(int n_particles, const FaceTables& t, double h);

// Seeded placement: face picked with probability proportional to its 3D area, uniform
// barycentric position, polarity angle uniform in [0, 2pi) in the face frame
// (e1 = normalize(B - A), e2 = n x e1), expressed as a chart angle.
void init_particles(const Mesh& m, const FaceTables& t, int n, uint64_t seed, uint32_t rep, double* uv,
                    double* theta, int* face, double* r3d);

// Host Philox4x32-10 (same generator as the device), for placement draws.
void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

}  // namespace tds
