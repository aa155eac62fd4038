/*
 * tds.h — C-ABI of 2dtissue_gb300: the per-step active-particle update of 2DTissue on a
 * triangulated closed surface, run on one GB300 (sm_103a).
 *
 * The reference has no FFI; the boundary it sits behind is the C++ class _2DTissue
 * (src/simulation/2DTissue.h:35-60) and the operator seam LocomotionHelperInterface
 * (src/simulation/LocomotionHelperInterface.h:3-13). Each entry point below names the
 * reference member it replaces. Conventions:
 *   - every call returns an int status: TDS_OK (0) or a TDS_ERR_* code; no exception crosses
 *     the boundary; tds_last_error() / tds_mesh_last_error() give the message;
 *   - handles own their device memory; caller buffers are borrowed for the call only;
 *   - one handle is used by one host thread at a time; handles are independent and each has
 *     its own CUDA stream;
 *   - particle arrays passed across the boundary are in particle-id order, structure of arrays.
 */
#ifndef TDS_H
#define TDS_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDS_OK 0
#define TDS_ERR_ARG 1     /* invalid argument (reference: std::invalid_argument) */
#define TDS_ERR_CUDA 2    /* CUDA runtime error, or no CUDA device */
#define TDS_ERR_MESH 3    /* mesh could not be read / charted */
#define TDS_ERR_STATE 4   /* the device status word is non-zero after a step (see TDS_STATUS_*) */
#define TDS_ERR_NOMEM 5
#define TDS_ERR_LIMIT 6   /* a size is above a stated maximum */

/* Device status bits (reference: Validation::error_invalid_values -> exit(1),
 * Validation::error_lost_particles -> throw, Validation.cpp:40-72). */
#define TDS_STATUS_NONFINITE 1      /* NaN/Inf in a new position or polarity */
#define TDS_STATUS_WRAP_LIMIT 2     /* more than 8 seam wraps in one step (position clamped) */
#define TDS_STATUS_LOCATE_FALLBACK 4 /* no chart face contained the point (nearest face used) */
#define TDS_STATUS_RESERVED 8
#define TDS_STATUS_CELL_OVERFLOW 16 /* a position fell outside the surface-cell list (lost particle) */

typedef struct tds_mesh tds_mesh;
typedef struct tds_sim tds_sim;

/* Model parameters (reference ctor arguments, 2DTissue.h:37-54: sigma -> radius,
 * k -> k_rep, r_adh -> r_max, k_adh, v0, mu, step_size -> dt). */
typedef struct tds_params {
    double radius;  /* particle radius R; contact distance 2R */
    double k_rep;   /* repulsion stiffness for d < 2R */
    double k_adh;   /* adhesion stiffness for 2R <= d < r_max */
    double r_max;   /* interaction cut-off (reference r_adh = 2.4 sigma) */
    double v0;      /* self-propulsion speed */
    double mu;      /* mobility */
    double tau;     /* polarity relaxation time towards the velocity */
    double align;   /* strength of alignment with the neighbours' polarity */
    double eta;     /* angular noise amplitude: U[-eta/2, eta/2] per step */
    double dt;      /* time step */
    int force_mode; /* 0: v = v0 p + mu F_t;  1: reference speed-only |v| = v0 + |F_t| along p */
    int reserved;
} tds_params;

/* Particle state in id order. Any pointer may be NULL where noted. */
typedef struct tds_state_view {
    double* uv;        /* 2N chart coordinates */
    double* theta;     /* N polarity angle in the chart (radians) */
    int* face;         /* N containing chart face (set: NULL or -1 entries -> located) */
    double* r3d;       /* 3N 3D positions (set: NULL -> mapped from uv/face) */
    double* vel_uv;    /* 2N chart velocity of the last step (get only, may be NULL) */
    int* nbr_count;    /* N neighbours within r_max in the last step (get only, may be NULL) */
} tds_state_view;

/* ---- mesh + chart (reference: loadMeshFaces / SurfaceParametrization::create_uv_surface,
 *      2DTissue.cpp:85-107; MeshCartographyLib is absent, this builds its own chart) ---- */
int tds_mesh_ellipsoid(int level, double ax, double ay, double az, tds_mesh** out);
int tds_mesh_bumpy_sphere(int level, double amp, double scale, tds_mesh** out);
int tds_mesh_from_arrays(const double* v3, int V, const int* f3, int F, tds_mesh** out);
int tds_mesh_load_off(const char* path, tds_mesh** out);
int tds_mesh_save_off(const tds_mesh* m, const char* path);
int tds_mesh_info(const tds_mesh* m, int* V, int* F, int* Vuv, double* area);
/* v3: 3V, f3: 3F, uv: 2Vuv, fuv: 3F, uv2v: Vuv; any may be NULL */
int tds_mesh_arrays(const tds_mesh* m, double* v3, int* f3, double* uv, int* fuv, int* uv2v);
void tds_mesh_destroy(tds_mesh* m);
const char* tds_mesh_last_error(void);

/* ---- simulation (reference: _2DTissue ctor / start() / update() / is_finished() /
 *      get_order_parameter(), 2DTissue.cpp:20-134,136-206,208-215) ---- */
/* precision: 32 (FP32 state, the fast path) or 64 (FP64 build, the correctness path). */
int tds_create(const tds_mesh* mesh, const tds_params* params, int n_particles, uint64_t seed, int precision,
               tds_sim** out);
/* Ragged ensemble of independent replicas in one set of launches; params has n_replicas entries. */
int tds_ensemble_create(const tds_mesh* mesh, int n_replicas, const int* n_particles, const tds_params* params,
                        uint64_t seed, int precision, tds_sim** out);
/* ---- tuning (no counterpart in the reference) ----
 * cells_per_particle: a replica's cell size is r_max * 2^k for the smallest k whose surface-cell
 *   count is <= max(64, cells_per_particle * N_r) (small replicas on a large surface take
 *   coarser cells); default 4.
 * step_block: threads per block of the step kernel, 128 or 256 (default 128).
 * graph_steps: 0 (default): a run of n >= 2 steps is one launch of the handle's loop graph
 *   (conditional WHILE nodes around blocks of 16 steps and single steps; the counts are set on the
 *   device before the launch);
 *   2..256 (even): runs are launched as captured graphs of this many steps, the rest directly.
 * lanes_per_particle: lanes of the step kernel per particle, 1 (default; 32 particles per warp),
 *   2 or 4 (16 or 8 particles per warp: the lanes split the particle's candidates and add their
 *   partial sums in a fixed order; needs step_block 128); 0 means 1. */
typedef struct tds_tuning {
    double cells_per_particle;
    int step_block;
    int graph_steps;
    int lanes_per_particle;
} tds_tuning;
/* tds_ensemble_create with a tuning (NULL = defaults); n_replicas = 1 for a plain system. */
int tds_create_ex(const tds_mesh* mesh, int n_replicas, const int* n_particles, const tds_params* params,
                  uint64_t seed, int precision, const tds_tuning* tuning, tds_sim** out);
int tds_get_tuning(const tds_sim* sim, tds_tuning* out);
/* Autotuner: creates the workload with each candidate tuning, places it, and times trial_steps
 * graph-launched steps on the device (best of two timings): cells_per_particle 1, 4, 16 x
 * step_block 128, 256 (one lane per particle, the loop graph), then on the fastest of those
 * lanes_per_particle 2 and 4 and graph_steps 16; returns the fastest tuning and its
 * particle-steps/s. */
int tds_autotune(const tds_mesh* mesh, int n_replicas, const int* n_particles, const tds_params* params,
                 uint64_t seed, int precision, int trial_steps, tds_tuning* best, double* best_rate);

/* Area-weighted random placement, polarity uniform in the face tangent frame (Philox, seeded). */
int tds_start(tds_sim* sim);
/* n_steps of the update. noise: NULL (Philox noise) or n_steps x N angle increments in id order. */
int tds_step(tds_sim* sim, int n_steps, const double* noise);
/* update() semantics: one step, then the state is copied into `out` (host buffers). */
int tds_update(tds_sim* sim, tds_state_view* out);
int tds_set_state(tds_sim* sim, const tds_state_view* in);
int tds_get_state(tds_sim* sim, tds_state_view* out);
/* Same result as tds_get_state, without any device allocation: no counterpart in the reference
 * (its state lives in host memory). For callers that cannot allocate device memory where they
 * read the state back -- a host framework that owns all device memory through its own allocator,
 * a device-memory budget fixed after start-up, or a loop that must not call cudaMalloc/cudaFree
 * because they synchronise the device. The state is staged in one fixed 16 MiB array that the
 * library holds on every GPU that loads it, so at most 233,016 particles (72 bytes each); larger
 * handles get TDS_ERR_LIMIT. The handle's device must be current. The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress), so make that first call before any stream
 * capture. All calls share the array: calls that overlap on the GPU (other threads or streams)
 * race and must be serialised by the caller; nothing in it needs clearing between calls. */
int tds_get_state_noalloc(tds_sim* sim, tds_state_view* out);
/* The reference's per-particle output record (Particle, src/simulation/Struct.h:9-29), same fields,
 * order and layout (88 bytes): chart position and velocity, the polarity angle in degrees (the
 * reference stores int degrees), the two compass fields the reference never sets (0), the 3D
 * position and the neighbour count. */
typedef struct tds_particle {
    double x_UV, y_UV;
    double x_velocity_UV, y_velocity_UV;
    double alignment_UV;
    double compass_north_pole_UV, compass_south_pole_UV;
    double x_3D, y_3D, z_3D;
    int neighbor_count;
} tds_particle;
/* update()'s System.particles (2DTissue.cpp:148-162): the records are packed on the device, in id
 * order, and copied to out (N records) in one transfer. */
int tds_get_particles(tds_sim* sim, tds_particle* out);
/* phi = |sum normalize((r - c) x v)| / N, psi = |sum v/|v|| / N per step and replica:
 * arrays of cap entries, step-major ([step][replica]); *n_steps gets the number of steps stored. */
int tds_get_order_parameter(tds_sim* sim, double* phi, double* psi, int cap, int* n_steps);
int tds_get_step(const tds_sim* sim, int64_t* step);
int tds_get_status(tds_sim* sim, int* status);
int tds_clear_status(tds_sim* sim);
int tds_num_particles(const tds_sim* sim, int* n_total, int* n_replicas);
/* Launches n_steps on the handle's stream and returns without waiting; the status word is
 * checked by the next tds_step / tds_get_status. For pipelined callers and device-timed loops. */
int tds_step_async(tds_sim* sim, int n_steps);
/* Pipelined state transfer (no counterpart in the reference, whose state never leaves host
 * memory). Same results as tds_set_state / tds_get_state, but they only enqueue and return:
 * uploads run on the handle's upload stream, downloads on its download stream, the load, the
 * gather and the steps on its compute stream, ordered by events. The host link carries both
 * directions at once, so in a loop set(k) -> step -> get(k) the upload of step k+1 overlaps the
 * download of step k. Host arrays passed in must stay untouched (inputs) or unread (outputs)
 * until tds_sync returns; pinned host memory makes the copies asynchronous. Face indices are
 * checked on the device: a load with an index >= F is refused as a whole (the state, the cell
 * lists and everything after it stay as they were) and tds_sync reports it as TDS_ERR_ARG;
 * tds_set_state reports it itself. Negative indices mean "locate". */
int tds_set_state_async(tds_sim* sim, const tds_state_view* in);
int tds_get_state_async(tds_sim* sim, tds_state_view* out);
/* The state of an FP32 handle in its own precision (no counterpart in the reference, which is
 * FP64 throughout): the fields and meaning of tds_state_view with float arrays. The values are the
 * device state exactly -- tds_get_state returns the same values widened to double -- so a caller
 * that reads an FP32 simulation moves 40 instead of 72 bytes per particle over the host link (16
 * instead of 28 for an upload of uv, theta and face). FP64 handles get TDS_ERR_ARG. The _async
 * forms behave as tds_set_state_async / tds_get_state_async. */
typedef struct tds_state_view_f32 {
    float* uv;      /* 2N */
    float* theta;   /* N */
    int* face;      /* N */
    float* r3d;     /* 3N */
    float* vel_uv;  /* 2N (get only, may be NULL) */
    int* nbr_count; /* N (get only, may be NULL) */
} tds_state_view_f32;
int tds_set_state_f32(tds_sim* sim, const tds_state_view_f32* in);
int tds_get_state_f32(tds_sim* sim, tds_state_view_f32* out);
int tds_set_state_f32_async(tds_sim* sim, const tds_state_view_f32* in);
int tds_get_state_f32_async(tds_sim* sim, tds_state_view_f32* out);
/* Waits for all work of the handle (transfers and steps); TDS_ERR_STATE if the device status
 * word is non-zero. */
int tds_sync(tds_sim* sim);

/* Replaces the model parameters (params has one entry per replica). radius and r_max fix the
 * cell lists and must stay as created (TDS_ERR_ARG otherwise); the state is kept. The reference
 * fixes its parameters in the _2DTissue constructor (2DTissue.h:37-54). */
int tds_set_params(tds_sim* sim, const tds_params* params);

/* ---- adjoint (no counterpart in the reference, which has no derivatives) ----
 * Loss over a run of n_steps from the current state:
 *   L = w_pos * sum_r (1/N_r) sum_{i in r} |r_T,i - r*_i|^2  +  w_phi * sum_t sum_r (phi_t,r - phi*_t,r)^2
 * with r_T the 3D positions after the last step and phi_t the order parameter of step t. The
 * gradients are those of the step with neighbour sets, faces and seam-wrap sequences held at the
 * forward run's (reverse mode, hand-written), with Philox noise fixed by the seed. The initial
 * 3D positions are taken as the chart map of the initial uv (r = A_f + J_f (uv - a_f)). */
typedef struct tds_adjoint_spec {
    int n_steps;
    int checkpoint_stride;     /* steps between checkpoints; 0 = the largest that fits in memory */
    const double* r3d_target;  /* 3N in id order, or NULL (no position term) */
    double w_pos;
    const double* phi_target;  /* n_steps x n_replicas, step-major, or NULL (no order-parameter term) */
    double w_phi;
    /* 0 (or >= n_steps): the exact gradient of the whole run. 0 < window < n_steps: a truncated
     * gradient -- the first n_steps - window steps run forward only and the reverse sweep covers
     * the last `window` steps: d_params sums the parameter sensitivities of those steps (the
     * order-parameter terms of the earlier steps enter the loss value but not the gradient), and
     * d_uv0 / d_theta0 are with respect to the state at the window's first step. Over long horizons
     * the exact gradient of a contact-dominated run grows geometrically with the step count (each
     * explicit-Euler contact step can multiply a separation error by |1 - 2 dt mu k / 2R|) and
     * overflows; the window bounds that growth. */
    int window;
    /* lanes per particle of the reverse step's neighbour gather: 0 = by system size (4 below
     * 131,072 particles, where one particle's chain of candidate loads sets the time, else 1), or
     * 1 or 4. The gradients agree to rounding (the lanes' partial sums are added in a fixed order,
     * so each choice is deterministic). */
    int gather_lanes;
} tds_adjoint_spec;
typedef struct tds_adjoint_result {
    double loss;
    /* n_replicas x 8: dL/d(k_rep, k_adh, v0, mu, tau, align, eta), 0 (may be NULL) */
    double* d_params;
    double* d_uv0;     /* 2N, dL/d(initial uv) in id order (may be NULL) */
    double* d_theta0;  /* N, dL/d(initial polarity angle) (may be NULL) */
    int checkpoint_stride; /* out: the stride used */
} tds_adjoint_result;
/* Runs n_steps forward (the handle advances exactly as tds_step would), storing a checkpoint every
 * checkpoint_stride steps, evaluates L, then the reverse sweep: segment by segment from the last,
 * recomputing each segment from its checkpoint with every step's sorted state kept, and two
 * kernels per step. */
int tds_adjoint_run(tds_sim* sim, const tds_adjoint_spec* spec, tds_adjoint_result* out);
/* tds_adjoint_run keeps its work memory (checkpoints, the per-step store: up to 80% of the free
 * device memory) in the handle between calls, so that repeated runs (parameter inference) do not map
 * and unmap it each time; this frees it now (tds_destroy frees it too). */
int tds_adjoint_release(tds_sim* sim);
/* Per-kernel CUDA-event timing of directly launched steps (graphs are not used while enabled).
 * tds_kernel_times returns, per kernel (0 scan + order-parameter finalize, 1 scatter, 2 order, 3 step,
 * 4 standalone finalize before a series read), the summed device time in ms and the launch count
 * since timing was enabled (arrays of 5). */
int tds_kernel_timing(tds_sim* sim, int enable);
int tds_kernel_times(tds_sim* sim, double* total_ms, long long* launches);
/* The CUDA stream every kernel of this handle runs on (cudaStream_t). */
int tds_stream(tds_sim* sim, void** stream);
/* Kernels launched per step (for launch accounting). */
int tds_kernels_per_step(const tds_sim* sim, int* n);
const char* tds_last_error(const tds_sim* sim);
void tds_destroy(tds_sim* sim);

/* ---- reference-semantics step (FP64, small meshes) ----
 * The reference's own per-step algorithm on the device, for exact reference-semantics studies
 * (the model-form calls above are the fast path). It keeps the reference's state and rules:
 * integer-degree polarity n, the pair distance between the particles' nearest chart vertices read
 * from a dense Vuv x Vuv matrix (Locomotion.cpp:94-138), chart-difference force directions with
 * only |F| used (Locomotion.cpp:57-89, ForceHelper.cpp:34-104), the circular mean of the angles
 * within 2 sigma truncated to int (OrientationHelper.cpp:29-116), the list-order seam wrap
 * (EuclideanTiling.cpp:31-208), the brute-force chart face search with distance weights and the
 * nearest corner (CellHelper.cpp:71-160), the neighbour count d != 0 && d <= 2.4 sigma
 * (2DTissue.cpp:254-268) and, per step, |sum sign(u v' - v u')| / N as the order parameter (the
 * reference's own evaluation reads out of bounds, LinearAlgebra.cpp:67-105). Cost is O(N^2 + N F)
 * per step, as in the reference: N <= 65,536, Vuv <= 32,768. */
typedef struct tds_ref_params { /* _2DTissue ctor arguments (2DTissue.h:37-54) */
    double v0;        /* default 0.1 */
    double k;         /* default 1 */
    double sigma;     /* default 0.41667 */
    double r_adh;     /* default 1 */
    double k_adh;     /* default 0.75 */
    double step_size; /* default 0.001 */
} tds_ref_params;
typedef struct tds_ref_sim tds_ref_sim;
/* Shortest paths along the chart mesh's edges (3D edge lengths), Vuv x Vuv row-major into out:
 * the stand-in for CachedGeodesicDistanceHelper::get_mesh_distance_matrix (2DTissue.cpp:102-105),
 * whose library is absent. Paths do not cross the seam (the reference measures on the open mesh). */
int tds_ref_vertex_distances(const tds_mesh* mesh, double* out);
/* _2DTissue ctor (2DTissue.cpp:20-111): vertex_dist = Vuv x Vuv matrix, or NULL to compute
 * tds_ref_vertex_distances. */
int tds_ref_create(const tds_mesh* mesh, const double* vertex_dist, const tds_ref_params* params, int n_particles,
                   uint64_t seed, tds_ref_sim** out);
/* start() (2DTissue.cpp:117-134): init_particle_position (uniform face index, its chart centroid,
 * uniform integer angle; Philox-seeded) and get_r3d. */
int tds_ref_start(tds_ref_sim* sim);
/* State in particle order: r_uv 2N, n_deg N; nearest_vertex N chart vertex ids or NULL (then
 * taken from the face search, as get_r3d does). */
int tds_ref_set_state(tds_ref_sim* sim, const double* r_uv, const int* n_deg, const int* nearest_vertex);
/* update() physics (2DTissue.cpp:136-165, 222-252) n_steps times; TDS_ERR_STATE on a non-finite
 * position (Validation::error_invalid_values) or a seam wrap that does not end. */
int tds_ref_step(tds_ref_sim* sim, int n_steps);
/* Any pointer may be NULL: r_uv 2N, n_deg N, nearest_vertex N, r3d 3N, r_dot 2N, nbr_count N. */
int tds_ref_get_state(tds_ref_sim* sim, double* r_uv, int* n_deg, int* nearest_vertex, double* r3d, double* r_dot,
                      int* nbr_count);
/* get_order_parameter() (2DTissue.cpp:213-216): one value per step taken. */
int tds_ref_get_order_parameter(tds_ref_sim* sim, double* out, int cap, int* n_steps);
int tds_ref_stream(tds_ref_sim* sim, void** stream);
const char* tds_ref_last_error(const tds_ref_sim* sim);
void tds_ref_destroy(tds_ref_sim* sim);

/* ---- test hooks ---- */
/* One step (as tds_step(sim, 1, NULL)) that also returns the neighbours the step used: lists is
 * N x cap, row i (particle i, id order) holds the indices of its neighbours (j != i, chord distance
 * below r_max, as the step's pair loop decided) in the step's visiting order, -1 past the last;
 * a particle with more than cap neighbours keeps the first cap (its count is in nbr_count). The
 * neighbour sets of the reference's step are its distance matrix rows (Locomotion.cpp:94-138). */
int tds_step_neighbors(tds_sim* sim, int cap, int* lists);
/* Runs the device seam wrap (the model form of EuclideanTiling::diagonal_seam_edges_square_border,
 * EuclideanTiling.cpp:31-69) on n points: uv holds the advanced points on entry and the wrapped
 * points on return; theta and vel_uv (2n, may be NULL) are rotated with them. */
int tds_debug_seam_wrap(int n, const double* uv_old, double* uv, double* theta, double* vel_uv, int* n_wraps,
                        int precision);

#ifdef __cplusplus
}
#endif
#endif /* TDS_H */
