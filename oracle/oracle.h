/*
 * ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * A CPU (FP64) restatement of 2DTissue's per-step particle update, used by tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm as the checker.
 * The product (2dtissue_gb300) never links or calls this library.
 *
 * Two layers:
 *   ref-form   exact restatements of the reference's formulas, pinned by the reference's own
 *              known-answer tests (tests/simulation/test_*.cpp):
 *                orc_ref_angles_to_unit_vectors     LinearAlgebra.cpp:25-46
 *                orc_ref_repulsive_adhesion         ForceHelper.cpp:84-104
 *                orc_ref_mean_angle_deg             OrientationHelper.cpp:84-116
 *                orc_ref_symmetrize_min             Locomotion.cpp:127-138
 *                orc_ref_dist_vect                  Locomotion.cpp:143-162
 *                orc_ref_average_n                  OrientationHelper.cpp:29-74
 *                orc_ref_seam_wrap                  EuclideanTiling.cpp:31-208 (unit-square borders)
 *                orc_ref_step                       2DTissue.cpp:136-268 + Locomotion.cpp:57-89
 *   model-form the step the GPU implements (vector Szabo force in 3D, tangent projection,
 *              polarity relaxation + Philox noise, UV advance with seam wrap, face location,
 *              barycentric UV->3D map, order parameter).
 *
 * Parity of the chart itself is unpinned: the reference's MeshCartographyLib is absent.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- ref-form ---- */
int orc_ref_angles_to_unit_vectors(const int* deg, int n, double* out_xy);
void orc_ref_repulsive_adhesion(double k, double sigma, double dist, double r_adh, double k_adh, double dvx,
                                double dvy, double* out2);
int orc_ref_mean_angle_deg(const double* angles_deg, int n, double* out); /* -1 on empty input */
void orc_ref_symmetrize_min(double* A, int n);
void orc_ref_dist_vect(const double* r_xy, int n, double* dx, double* dy);
int orc_ref_average_n(const double* dist_length, const int* n_in, int num, double sigma, int* n_out);
int orc_ref_seam_wrap(double* uv_old, double* uv, int* n_deg, int num);

/* Full ref-form step on a mesh (O(N^2) pair matrices, O(N*F) face search, vertex-distance
 * matrix gathered per step). dist_vv is V x V (a stand-in for the geodesic matrix). */
int orc_ref_step(int V, const double* v3, int F, const int* f3, int Vuv, const double* uvv, const int* fuv,
                 const int* uv2v, const double* dist_vv, double v0, double k, double sigma, double r_adh,
                 double k_adh, double step_size, int N, double* r_uv, int* n_deg, int* nearest_vtx, double* r3d,
                 double* r_dot, int* nbr_count, double* order_out);

/* ---- model-form ---- */
typedef struct orc_mesh orc_mesh;
orc_mesh* orc_mesh_create(int V, const double* v3, int F, const int* f3, int Vuv, const double* uvv,
                          const int* fuv);
void orc_mesh_free(orc_mesh* m);
/* face data: J (6, column major 3x2), Jp (6, row major 2x3), n (3) per face */
void orc_mesh_face_data(const orc_mesh* m, int f, double* J6, double* Jp6, double* n3);
int orc_mesh_locate(const orc_mesh* m, double u, double v, int f_old, int* mode);
void orc_mesh_map(const orc_mesh* m, int f, double u, double v, double* r3);

/* prm: [R, k, k_adh, r_max, v0, mu, tau, align, eta, dt] */
int orc_model_wrap(double* s_uv, double* e_uv, double* theta, double* vuv, int max_wraps, int* n_wraps);

int orc_model_step(const orc_mesh* m, const double* prm, int force_mode, uint64_t seed, int64_t step,
                   int local_bits, const double* centroid, int N, const double* uv, const double* theta,
                   const int* face, const double* r3d, const int* ids, const double* noise, int n_sub,
                   const int* sub, double* uv_out, double* theta_out, int* face_out, double* r3d_out,
                   double* vel_uv_out, int* cnt_out, int* wraps_out, double* phi_sums, int* status_out,
                   int n_threads);

/* Directional derivative (forward-mode dual numbers) of one model step: tangents of the inputs
 * (uv, theta; parameter tangents dprm[10]) propagate to tangents of uv_out/theta_out/r3d_out and
 * the order-parameter sums. Neighbour sets, faces and wraps follow the primal. */
int orc_model_step_dual(const orc_mesh* m, const double* prm, const double* dprm, int force_mode, uint64_t seed,
                        int64_t step, int local_bits, const double* centroid, int N, const double* uv,
                        const double* duv, const double* theta, const double* dtheta, const int* face,
                        const double* r3d, const double* dr3d, const int* ids, const double* noise,
                        double* uv_out, double* duv_out, double* theta_out, double* dtheta_out, int* face_out,
                        double* r3d_out, double* dr3d_out, double* phi_sums, double* dphi_sums);

#ifdef __cplusplus
}
#endif
