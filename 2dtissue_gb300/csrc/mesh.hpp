// Host-side closed-surface mesh and its unit-square UV chart.
//
// The reference gets these from MeshCartographyLib (an empty, unpinned submodule):
// loadMeshFaces / create_uv_surface / get_borders (2DTissue.cpp:85-107,
// EuclideanTiling.cpp:34). This module builds the same kind of input from scratch:
//   * icosphere / ellipsoid / bumpy-sphere meshes and an OFF reader/writer;
//   * a seam cut P0 -> P1 -> P2 along shortest edge paths;
//   * a Tutte (uniform-weight) embedding of the cut disk into [0,1]^2 whose boundary
//     obeys the gluing that EuclideanTiling::processPoints encodes
//     (EuclideanTiling.cpp:112-154): bottom (s,0) == left (0,s), right (1,s) == top (s,1).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace tds {

struct Mesh {
    std::vector<double> v3;     // V x 3, 3D vertex positions
    std::vector<int32_t> f3;    // F x 3, outward (CCW seen from outside) triangles
    std::vector<double> uv;     // Vuv x 2, chart coordinates in [0,1]^2
    std::vector<int32_t> fuv;   // F x 3, chart triangles (CCW in UV); row f matches f3 row f
    std::vector<int32_t> uv2v;  // Vuv, chart vertex -> 3D vertex
    std::vector<int32_t> seam;  // 3D vertex ids of the seam path P0 .. P1 .. P2
    int seam_p1 = 0;            // position of P1 in `seam`

    int V() const { return (int)(v3.size() / 3); }
    int F() const { return (int)(f3.size() / 3); }
    int Vuv() const { return (int)(uv.size() / 2); }
};

// Unit icosphere after `level` midpoint subdivisions: V = 10*4^L + 2, F = 20*4^L.
void make_icosphere(int level, Mesh& m);
// Per-axis scaling (ellipsoid semi-axes when applied to the unit sphere).
void scale_axes(Mesh& m, double ax, double ay, double az);
// Radial bump r(theta,phi) = 1 + amp * Re Y_4^2(theta,phi) (complex orthonormal convention:
// Re Y_4^2 = (3/8) sqrt(5/(2 pi)) sin^2(theta) (7 cos^2(theta) - 1) cos(2 phi)), then uniform scale.
void bumpy_sphere(Mesh& m, double amp, double scale);
// Re-orients faces so that every triangle is CCW seen from outside (normal away from centroid).
void orient_outward(Mesh& m);

// Cuts the closed mesh along a seam and maps it onto the unit square (see header comment).
// Returns 0 on success, else fills `err`.
int build_chart(Mesh& m, std::string& err);

// Checks the chart: every UV triangle has positive area, boundary vertices lie on the square,
// the glued twin of each boundary vertex maps to the same 3D vertex, UV areas sum to 1.
int check_chart(const Mesh& m, std::string& err);

int read_off(const std::string& path, Mesh& m, std::string& err);
int write_off(const std::string& path, const Mesh& m, std::string& err);

}  // namespace tds
