// Host-side tables derived from a charted mesh: per-face chart maps, the UV bin grid for point
// location, the folded 3D cell-grid layout, and seeded initial particle placement.
#pragma once
#include <cstdint>
#include <vector>

#include "mesh.hpp"

namespace tds {

// Per-face record, 32 reals (one 128-byte line in FP32), grouped by use in the step kernel:
//   [0..5]   J   = dX/d(uv), column u = [0..2], column v = [3..5]
//   [6..11]  Jp  = (J^T J)^-1 J^T, row 0 = [6..8], row 1 = [9..11]
//   [12..14] n   = unit normal of the 3D triangle (outward)
//   [16..21] UV corners a, b, c (CCW)
//   [22]     canonical-orientation bits: bit k set when edge k runs from the higher to the
//            lower chart-vertex id (its orientation value is evaluated reversed and negated)
//   [24..26] 3D corner A (image of a)
//   [28..30] 1 / UV edge length of edges a->b, b->c, c->a
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

// Chart edge adjacency: for face f, edge k (corner k -> k+1) borders face adj[3f+k]
// (-1 on the square's boundary).
void build_face_adjacency(const Mesh& m, std::vector<int>& adj);

// Compact surface-cell list of one cell size h. Particles always lie on the mesh, so the only
// cells that can hold particles are those the triangles pass through; they are numbered in
// (iz, iy, ix) order, so the cells of one x-row that are consecutive in x have consecutive ids.
// A row (iy, iz) lists its x-intervals; rows[r] = (first interval, count), intervals are
// (x_lo, x_hi, id of x_lo, 0). Cells are found exactly: no hashing, no collisions.
struct CellLevel {
    double h = 0;
    int gx = 0, gy = 0, gz = 0;
    int C = 0;  // number of surface cells
    std::vector<int> rows;   // 2 per row: first interval, count
    std::vector<int> ivals;  // 4 per interval
};
// origin: grid corner (mesh bounding box minus a margin of >= 2 cells).
void build_cell_level(const Mesh& m, double h, const double origin[3], CellLevel& L);

// Per surface cell, the ids of its 27 neighbour cells as 9 x-runs (rows dy, dz in -1..1, in the
// order r = (dz + 1) * 3 + (dy + 1)), in 8 words (32 bytes, one sector): the 8 runs other than the
// cell's own row, entry = id of the run's first cell << 4 | number of cells in the run (0..3);
// the own row's run is the cell itself and its x-neighbours when they are surface cells (first =
// id - L, length 1 + L + R, consecutive ids), with L and R in bits 2 and 3 of word 0.
void build_cell_descriptors(const CellLevel& L, std::vector<uint32_t>& desc);


// Host Philox4x32-10 (same generator as the device), for placement draws.
void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

}  // namespace tds
