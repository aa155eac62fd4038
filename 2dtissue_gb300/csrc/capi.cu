// C-ABI implementation (include/tds.h): mesh/chart handles, simulation handles, step launch
// sequencing, CUDA-graph capture of the step loop, state transfer and the device status word.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/tds.h"
#include "adjoint.cuh"
#include "geometry.hpp"
#include "kernels.cuh"
#include "mesh.hpp"

using tdsk::R2;
using tdsk::R4;
using tdsk::RepParams;

struct tds_mesh {
    tds::Mesh m;
    tds::FaceTables t;
};

namespace {

thread_local std::string g_mesh_err;

// NVTX range over a library phase (header-only NVTX v3: a no-op unless a profiler is attached), so
// that profiles of a caller's program show the steps, state transfers and adjoint passes by name.
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

int mesh_fail(const std::string& msg) {
    g_mesh_err = msg;
    return TDS_ERR_MESH;
}

int finish_mesh(tds::Mesh& m, tds_mesh** out) {
    std::string err;
    if (tds::build_chart(m, err)) return mesh_fail(err);
    auto* h = new tds_mesh();
    h->m = std::move(m);
    tds::build_face_tables(h->m, h->t);
    *out = h;
    return TDS_OK;
}

int ceil_log2(long long x) {
    int l = 0;
    while ((1ll << l) < x) ++l;
    return l;
}

}  // namespace

struct tds_sim {
    int precision = 32;
    int R = 1, N = 0, local_bits = 31;
    std::vector<int> n_rep, off;
    std::vector<tds_params> prm;
    std::vector<int> level_of;  // replica -> cell level
    int4* rows = nullptr;       // all levels' row records (two int4 per grid row)
    int4* ivals = nullptr;      // all levels' x-intervals
    int4* adj = nullptr;        // chart edge adjacency per face
    uint4* desc = nullptr;      // per-cell neighbour-run descriptors (3 uint4 per cell)
    int* tile_sum = nullptr;    // [2][n_tiles] per-tile counts (step parity)
    uint64_t seed = 0;
    long long step = 0;  // completed steps
    const tds_mesh* mesh = nullptr;
    std::string err;
    cudaStream_t stream = nullptr;
    size_t rsz = 4;  // sizeof(real)
    // device
    void* rec = nullptr;
    int* bin_start = nullptr;
    int* bin_faces = nullptr;
    int G = 1;
    void* reps = nullptr;
    std::vector<unsigned char> reps_host;  // host copy of the replica table
    // every replica has replica 0's pair constants: the step kernel takes them from its parameters
    // (the constant bank) instead of the replica table (the 4,096-replica ensemble's step kernel
    // 564 -> 559 us)
    bool uniform_pair = true;
    long long M = 0;
    int n_tiles = 0;
    void* pos[2] = {nullptr, nullptr};
    void* pol[2] = {nullptr, nullptr};
    void* uv[2] = {nullptr, nullptr};
    int* ids[2] = {nullptr, nullptr};
    void* vel[2] = {nullptr, nullptr};
    int* cnt[2] = {nullptr, nullptr};
    int* key[2] = {nullptr, nullptr};
    int* perm = nullptr;
    int* tmp = nullptr;  // scatter output before the per-cell id order
    int* start = nullptr;
    int* count = nullptr;
    unsigned long long* phi_acc = nullptr;
    int* phi_pending = nullptr;  // a step's order parameter awaits finalizing (next k_scan or a flush)
    double* series = nullptr;
    long long series_cap = 0;  // steps
    int* status = nullptr;
    int* load_flag = nullptr;  // [b] the load from input staging b was refused, [2] a refused load not yet reported
    long long* d_step = nullptr;
    int* packed_ids = nullptr;
    void* noise = nullptr;
    size_t noise_cap = 0;
    // transfer staging, two of each so that a transfer of call k+1 can run while call k's
    // buffer is still in use on the other side (the gather of step k+1 during the download of
    // step k; the upload of step k+1 before the load of step k has run)
    double* st_d[2] = {nullptr, nullptr};  // output staging (double) 8N
    int* st_i[2] = {nullptr, nullptr};     // output staging (int) 2N
    double* in_d[2] = {nullptr, nullptr};  // input staging (double) 6N
    int* in_i[2] = {nullptr, nullptr};     // input staging (int) N
    int in_next = 0, out_next = 0;         // staging buffer of the next upload / download
    // state transfers: uploads and downloads on their own streams, so that the two directions of
    // the host link run at the same time; events order them against the compute stream
    cudaStream_t up = nullptr, down = nullptr;
    // the adjoint's reverse sweep (created on first use), beside the recompute on the compute stream
    cudaStream_t rev = nullptr;
    cudaEvent_t ev_in_ready[2] = {nullptr, nullptr}, ev_in_free[2] = {nullptr, nullptr};
    cudaEvent_t ev_out_ready[2] = {nullptr, nullptr}, ev_out_free[2] = {nullptr, nullptr};
    int cur = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    // the whole run as one graph launch: conditional WHILE nodes around the steps (graph_steps 0)
    cudaGraphExec_t loop_graph = nullptr;
    // a single step (tds_step / tds_step_async of one step) as one graph launch
    cudaGraphExec_t step_graph = nullptr;
    int* loop_left = nullptr;  // device: [0] step blocks, [1] single steps left in the running loop graph
    int graph_steps = 0;         // 0: loop graph; 2..256 (even): steps per captured chunk (tuning)
    int step_block = 128;        // threads per k_step block (tuning: 128 or 256)
    int lanes = 1;               // lanes per particle in k_step (tuning: 1, 2 or 4; > 1 with 128-thread blocks)
    double cells_per_particle = 4.0;  // cell-level rule (tuning): finest level with C <= max(64, this * N_r)
    double origin[3] = {0, 0, 0};
    std::vector<void*> allocs;
    // adjoint work memory (checkpoints, the per-step store, adjoint buffers): one device block kept
    // between tds_adjoint_run calls and grown when a call needs more (tds_adjoint_release frees it)
    void* adj_ws = nullptr;
    size_t adj_ws_bytes = 0;
    tds_particle* pk = nullptr;  // Particle records staged for tds_get_particles (allocated on first use)
    // per-kernel event timing
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    double k_ms[5] = {0, 0, 0, 0, 0};
    long long k_n[5] = {0, 0, 0, 0, 0};
};

namespace {

int fail(tds_sim* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}
#define CK(call)                                                                                            \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return fail(s, TDS_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int dalloc(tds_sim* s, T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return fail(s, TDS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    s->allocs.push_back(q);
    *p = (T*)q;
    return TDS_OK;
}

void free_graphs(tds_sim* s) {
    for (auto& g : s->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    if (s->loop_graph) {
        cudaGraphExecDestroy(s->loop_graph);
        s->loop_graph = nullptr;
    }
    if (s->step_graph) {
        cudaGraphExecDestroy(s->step_graph);
        s->step_graph = nullptr;
    }
}

template <typename real>
void set_uniform_pair(tds_sim* s) {
    const RepParams<real>* h = (const RepParams<real>*)s->reps_host.data();
    bool same = true;
    for (int r = 1; r < s->R && same; ++r)
        same = h[r].r_max2 == h[0].r_max2 && h[r].twoR == h[0].twoR && h[r].inv_twoR == h[0].inv_twoR &&
               h[r].k == h[0].k && h[r].adh_scale == h[0].adh_scale;
    s->uniform_pair = same;
}

// Model parameters of one replica into its device record (the cell-level fields stay).
template <typename real>
void fill_params(RepParams<real>& q, const tds_params& p) {
    q.twoR = (real)(2 * p.radius);
    q.inv_twoR = (real)(1.0 / (2 * p.radius));
    q.k = (real)p.k_rep;
    q.adh_scale = (real)(p.k_adh / (p.r_max - 2 * p.radius));
    q.inv_adh_w = (real)(1.0 / (p.r_max - 2 * p.radius));
    q.r_max2 = (real)(p.r_max * p.r_max);
    q.v0 = (real)p.v0;
    q.mu = (real)p.mu;
    q.inv_tau = (real)(1.0 / p.tau);
    q.align = (real)p.align;
    q.eta = (real)p.eta;
    q.dt = (real)p.dt;
    q.force_mode = p.force_mode;
}

template <typename real>
int upload_tables(tds_sim* s) {
    const tds::FaceTables& t = s->mesh->t;
    // device face record (16 reals): chart corners, edge bits, A, J (see kernels.cuh)
    std::vector<real> rec((size_t)t.F * tdsk::kRec);
    for (int f = 0; f < t.F; ++f) {
        const double* h = &t.rec[(size_t)f * tds::kFaceRec];
        real* d = &rec[(size_t)f * tdsk::kRec];
        for (int k = 0; k < 6; ++k) d[k] = (real)h[16 + k];
        d[6] = (real)h[22];
        d[7] = (real)h[24];
        for (int k = 0; k < 6; ++k) d[8 + k] = (real)h[k];
        d[14] = (real)h[25];
        d[15] = (real)h[26];
    }
    int rc;
    if ((rc = dalloc(s, (real**)&s->rec, rec.size() * sizeof(real)))) return rc;
    CK(cudaMemcpy(s->rec, rec.data(), rec.size() * sizeof(real), cudaMemcpyHostToDevice));
    s->G = t.G;
    if ((rc = dalloc(s, &s->bin_start, t.bin_start.size() * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->bin_faces, t.bin_faces.size() * sizeof(int)))) return rc;
    CK(cudaMemcpy(s->bin_start, t.bin_start.data(), t.bin_start.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->bin_faces, t.bin_faces.data(), t.bin_faces.size() * sizeof(int), cudaMemcpyHostToDevice));

    // chart edge adjacency (int4 per face: the three edge neighbours, -1 on the border)
    {
        std::vector<int> adj;
        tds::build_face_adjacency(s->mesh->m, adj);
        std::vector<int4> a4(t.F);
        for (int f = 0; f < t.F; ++f) a4[f] = make_int4(adj[3 * f], adj[3 * f + 1], adj[3 * f + 2], -1);
        if ((rc = dalloc(s, &s->adj, a4.size() * sizeof(int4)))) return rc;
        CK(cudaMemcpy(s->adj, a4.data(), a4.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }

    // cell levels: cell size r_max * 2^k; a replica takes the finest level whose surface-cell
    // count is at most max(64, 4 N_r), so that small replicas do not scan many empty cells
    struct Level {
        double rmax;
        int k;
        double origin[3];
        tds::CellLevel L;
    };
    std::vector<Level> levels;
    auto get_level = [&](double rmax, int k) -> int {
        for (size_t i = 0; i < levels.size(); ++i)
            if (levels[i].rmax == rmax && levels[i].k == k) return (int)i;
        Level lv;
        lv.rmax = rmax, lv.k = k;
        const double h = std::ldexp(rmax, k);
        for (int d = 0; d < 3; ++d) lv.origin[d] = t.lo[d] - 2.0 * h;
        tds::build_cell_level(s->mesh->m, h, lv.origin, lv.L);
        levels.push_back(std::move(lv));
        return (int)levels.size() - 1;
    };
    s->level_of.assign(s->R, 0);
    for (int r = 0; r < s->R; ++r) {
        int li = 0;
        for (int k = 0; k <= 6; ++k) {
            li = get_level(s->prm[r].r_max, k);
            if ((double)levels[li].L.C <= std::max(64.0, s->cells_per_particle * s->n_rep[r])) break;
        }
        s->level_of[r] = li;
    }
    std::vector<int> row_off(levels.size()), desc_off(levels.size());
    std::vector<int4> rows;
    std::vector<int4> ivals;
    std::vector<uint32_t> desc;
    for (size_t i = 0; i < levels.size(); ++i) {
        const tds::CellLevel& L = levels[i].L;
        if (L.C >= (1 << 28)) return fail(s, TDS_ERR_LIMIT, "more than 2^28 surface cells in one level");
        desc_off[i] = (int)(desc.size() / 4);
        std::vector<uint32_t> d;
        tds::build_cell_descriptors(L, d);
        desc.insert(desc.end(), d.begin(), d.end());
        row_off[i] = (int)(rows.size() / 2);
        const int ib = (int)ivals.size();
        for (size_t r = 0; r < L.rows.size() / 2; ++r) {
            // the row's first two intervals inline, the rest (if any) in ivals from index first + 2
            const int first = L.rows[2 * r], n = L.rows[2 * r + 1];
            int4 a = make_int4(0, -1, 0, n), b = make_int4(0, -1, 0, ib + first);
            if (n > 0) a = make_int4(L.ivals[4 * first], L.ivals[4 * first + 1], L.ivals[4 * first + 2], n);
            if (n > 1)
                b = make_int4(L.ivals[4 * (first + 1)], L.ivals[4 * (first + 1) + 1], L.ivals[4 * (first + 1) + 2],
                              ib + first);
            rows.push_back(a);
            rows.push_back(b);
        }
        for (size_t v = 0; v < L.ivals.size() / 4; ++v)
            ivals.push_back(make_int4(L.ivals[4 * v], L.ivals[4 * v + 1], L.ivals[4 * v + 2], 0));
    }
    if (ivals.empty()) ivals.push_back(make_int4(0, -1, 0, 0));
    if ((rc = dalloc(s, &s->rows, rows.size() * sizeof(int4)))) return rc;
    if ((rc = dalloc(s, &s->ivals, ivals.size() * sizeof(int4)))) return rc;
    CK(cudaMemcpy(s->rows, rows.data(), rows.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->ivals, ivals.data(), ivals.size() * sizeof(int4), cudaMemcpyHostToDevice));
    if (desc.empty()) desc.assign(4, 0u);
    if ((rc = dalloc(s, &s->desc, desc.size() * sizeof(uint32_t)))) return rc;
    CK(cudaMemcpy(s->desc, desc.data(), desc.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));

    // replica table: parameters, fixed-point scales, cell level and bucket range
    std::vector<RepParams<real>> rp(s->R);
    long long base = 0;
    for (int r = 0; r < s->R; ++r) {
        const tds_params& p = s->prm[r];
        RepParams<real>& q = rp[r];
        std::memset(&q, 0, sizeof q);
        const Level& lv = levels[s->level_of[r]];
        const double h = lv.L.h;
        fill_params(q, p);
        q.inv_h = (real)(1.0 / h);
        // order parameter: warp sums (|.| <= 32) in 64-bit fixed point, N_r terms per replica
        q.phiscale = std::ldexp(1.0, 62 - ceil_log2((long long)s->n_rep[r] + 1));
        q.inv_n = 1.0 / std::max(1, s->n_rep[r]);
        q.ox = (real)lv.origin[0], q.oy = (real)lv.origin[1], q.oz = (real)lv.origin[2];
        q.base = (int)base;
        q.C = lv.L.C;
        q.gx = lv.L.gx, q.gy = lv.L.gy, q.gz = lv.L.gz;
        q.row_off = row_off[s->level_of[r]];
        q.desc_off = desc_off[s->level_of[r]];
        q.n = s->n_rep[r];
        q.off = s->off[r];
        base += (long long)lv.L.C + 1;  // + the bucket of particles off the surface cells
    }
    if (base > (1ll << 30)) return fail(s, TDS_ERR_LIMIT, "cell-list buckets exceed 2^30");
    s->M = base;
    if ((rc = dalloc(s, (RepParams<real>**)&s->reps, rp.size() * sizeof(RepParams<real>)))) return rc;
    CK(cudaMemcpy(s->reps, rp.data(), rp.size() * sizeof(RepParams<real>), cudaMemcpyHostToDevice));
    s->reps_host.assign((const unsigned char*)rp.data(), (const unsigned char*)(rp.data() + rp.size()));
    set_uniform_pair<real>(s);
    return TDS_OK;
}

template <typename real>
int alloc_state(tds_sim* s) {
    const size_t N = (size_t)s->N;
    int rc;
    for (int b = 0; b < 2; ++b) {
        if ((rc = dalloc(s, (R4<real>**)&s->pos[b], N * sizeof(R4<real>)))) return rc;
        if ((rc = dalloc(s, (R4<real>**)&s->pol[b], N * sizeof(R4<real>)))) return rc;
        if ((rc = dalloc(s, (R2<real>**)&s->uv[b], N * sizeof(R2<real>)))) return rc;
        if ((rc = dalloc(s, &s->ids[b], N * sizeof(int)))) return rc;
        if ((rc = dalloc(s, (R2<real>**)&s->vel[b], N * sizeof(R2<real>)))) return rc;
        if ((rc = dalloc(s, &s->cnt[b], N * sizeof(int)))) return rc;
        if ((rc = dalloc(s, &s->key[b], N * sizeof(int)))) return rc;
    }
    if ((rc = dalloc(s, &s->perm, N * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->tmp, N * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->start, (size_t)(s->M + 1) * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->count, (size_t)s->M * sizeof(int)))) return rc;
    s->n_tiles = (int)((s->M + tdsk::kScanTile - 1) / tdsk::kScanTile);
    if ((rc = dalloc(s, &s->tile_sum, (size_t)2 * s->n_tiles * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->phi_acc, (size_t)s->R * tdsk::kPhiCopies * 6 * sizeof(unsigned long long)))) return rc;
    if ((rc = dalloc(s, &s->status, sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->load_flag, 4 * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->phi_pending, sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->d_step, sizeof(long long)))) return rc;
    if ((rc = dalloc(s, &s->loop_left, 2 * sizeof(int)))) return rc;
    if ((rc = dalloc(s, &s->packed_ids, N * sizeof(int)))) return rc;
    for (int b = 0; b < 2; ++b) {
        if ((rc = dalloc(s, &s->st_d[b], 8 * N * sizeof(double)))) return rc;
        if ((rc = dalloc(s, &s->st_i[b], 2 * N * sizeof(int)))) return rc;
        if ((rc = dalloc(s, &s->in_d[b], 6 * N * sizeof(double)))) return rc;
        if ((rc = dalloc(s, &s->in_i[b], N * sizeof(int)))) return rc;
    }
    CK(cudaMemset(s->count, 0, (size_t)s->M * sizeof(int)));
    CK(cudaMemset(s->tile_sum, 0, (size_t)2 * s->n_tiles * sizeof(int)));
    CK(cudaMemset(s->phi_acc, 0, (size_t)s->R * tdsk::kPhiCopies * 6 * sizeof(unsigned long long)));
    CK(cudaMemset(s->status, 0, sizeof(int)));
    CK(cudaMemset(s->load_flag, 0, 4 * sizeof(int)));
    CK(cudaMemset(s->phi_pending, 0, sizeof(int)));
    const int nN = s->N;
    CK(cudaMemcpy(s->start + s->M, &nN, sizeof(int), cudaMemcpyHostToDevice));
    const long long m1 = -1;
    CK(cudaMemcpy(s->d_step, &m1, sizeof m1, cudaMemcpyHostToDevice));
    std::vector<int> pid(N);
    for (int r = 0; r < s->R; ++r)
        for (int i = 0; i < s->n_rep[r]; ++i) pid[s->off[r] + i] = (int)(((unsigned)r << s->local_bits) | (unsigned)i);
    CK(cudaMemcpy(s->packed_ids, pid.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    // the current order's ids by slot start as the identity order (state loads fill each slot with
    // the particle it holds, so the array is a permutation of the packed ids from here on)
    CK(cudaMemcpy(s->ids[0], pid.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    return TDS_OK;
}

int ensure_series(tds_sim* s, long long steps_needed) {
    if (steps_needed <= s->series_cap) return TDS_OK;
    long long cap = std::max<long long>(1024, s->series_cap);
    while (cap < steps_needed) cap *= 2;
    double* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (size_t)cap * 2 * s->R * sizeof(double));
    if (e != cudaSuccess) return fail(s, TDS_ERR_NOMEM, "order-parameter series allocation failed");
    CK(cudaMemsetAsync(p, 0, (size_t)cap * 2 * s->R * sizeof(double), s->stream));
    if (s->series) {
        CK(cudaMemcpyAsync(p, s->series, (size_t)s->series_cap * 2 * s->R * sizeof(double), cudaMemcpyDeviceToDevice,
                           s->stream));
        CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->series);
    }
    s->series = p;
    s->series_cap = cap;
    free_graphs(s);
    return TDS_OK;
}

cudaEvent_t take_event(tds_sim* s) {
    if (s->ev_pool.empty()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;  // the launch goes untimed
        }
        return e;
    }
    cudaEvent_t e = s->ev_pool.back();
    s->ev_pool.pop_back();
    return e;
}

// Records an event pair around kernel `k` when timing is enabled.
struct KernelTimer {
    tds_sim* s;
    int k;
    cudaEvent_t a = nullptr;
    KernelTimer(tds_sim* s_, int k_) : s(s_), k(k_) {
        if (s->timing && (a = take_event(s))) cudaEventRecord(a, s->stream);
    }
    ~KernelTimer() {
        if (!a) return;
        cudaEvent_t b = take_event(s);
        if (!b) {
            s->ev_pool.push_back(a);
            return;
        }
        cudaEventRecord(b, s->stream);
        s->ev_pending.push_back({k, {a, b}});
    }
};

void collect_times(tds_sim* s) {
    if (s->ev_pending.empty()) return;
    cudaStreamSynchronize(s->stream);
    for (auto& p : s->ev_pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        s->k_ms[p.first] += ms;
        s->k_n[p.first] += 1;
        s->ev_pool.push_back(p.second.first);
        s->ev_pool.push_back(p.second.second);
    }
    s->ev_pending.clear();
}

// What a step can leave behind for the adjoint: its sorted state and cell starts (copied right
// after k_order) and its order-parameter sums.
struct StepStore {
    void* pos = nullptr;
    void* pol = nullptr;
    void* uv = nullptr;
    int* ids = nullptr;
    int* key = nullptr;
    int* start = nullptr;
    void* sum_f = nullptr;  // the step's pair sums by slot (null: the reverse step recomputes them)
    void* sum_m = nullptr;
};
struct StepHooks {
    const StepStore* store = nullptr;
    double* phisum = nullptr;
    long long phisum_base = 0, phisum_cap = 0;
};

template <typename real>
tdsk::FinArgs<real> fin_args(tds_sim* s, const StepHooks* hk) {
    tdsk::FinArgs<real> f;
    f.phi_acc = s->phi_acc;
    f.reps = (const RepParams<real>*)s->reps;
    f.R = s->R;
    f.series = s->series;
    f.cap_steps = s->series_cap;
    f.phisum = hk ? hk->phisum : nullptr;
    f.phisum_base = hk ? hk->phisum_base : 0;
    f.phisum_cap = hk ? hk->phisum_cap : 0;
    f.pending = s->phi_pending;
    return f;
}

// Finalizes the order parameter of the last step if no k_scan has done it yet (before the series
// is read).
template <typename real>
void flush_finalize(tds_sim* s, const StepHooks* hk = nullptr) {
    {
        KernelTimer kt(s, 4);
        tdsk::k_finalize<real><<<(s->R + tdsk::kFinWarps - 1) / tdsk::kFinWarps, 32 * tdsk::kFinWarps, 0, s->stream>>>(
            fin_args<real>(s, hk), s->d_step);
    }
    cudaMemsetAsync(s->phi_pending, 0, sizeof(int), s->stream);
}

// k_scatter and k_order take two particles per thread from this many particles on: with one, the
// GPU holds every particle's load chain at once up to ~0.3M particles; with two, a system needs
// ~0.6M to fill it
constexpr int kOrderPairN = 1 << 19;

// Buffer roles: index 0 = step output (and set_state target), index 1 = sorted copy.
template <typename real>
void launch_one_step(tds_sim* s, const real* noise, const StepHooks* hk = nullptr, int* nbr_list = nullptr,
                     int nbr_cap = 0) {
    const int c = 1, o = 0;
    cudaStream_t st = s->stream;
    // the sorted copy and the cell starts of this step go to the handle's buffer 1, or straight
    // into an adjoint store slot
    const StepStore* x = hk ? hk->store : nullptr;
    R4<real>* cpos = (R4<real>*)(x ? x->pos : s->pos[c]);
    R4<real>* cpol = (R4<real>*)(x ? x->pol : s->pol[c]);
    R2<real>* cuv = (R2<real>*)(x ? x->uv : s->uv[c]);
    int* cids = x ? x->ids : s->ids[c];
    int* ckey = x ? x->key : s->key[c];
    int* start = x ? x->start : s->start;
    {
        KernelTimer kt(s, 0);
        tdsk::k_scan<real><<<s->n_tiles + (s->R + tdsk::kFinWarps - 1) / tdsk::kFinWarps, tdsk::kScanThreads, 0, st>>>(
            s->count, start, s->M, s->tile_sum, s->n_tiles, s->d_step, fin_args<real>(s, hk));
    }
    const int nb = (s->N + 255) / 256;
    {
        KernelTimer kt(s, 1);
        if (s->N >= kOrderPairN)  // two slots per thread: 4,096-replica ensemble 49.1 -> 45.4 us
            tdsk::k_scatter<2><<<(s->N + 511) / 512, 256, 0, st>>>(s->key[o], s->count, start, s->tmp, s->N,
                                                                    s->d_step, s->phi_pending);
        else
            tdsk::k_scatter<1><<<nb, 256, 0, st>>>(s->key[o], s->count, start, s->tmp, s->N, s->d_step,
                                                    s->phi_pending);
    }
    {
        KernelTimer kt(s, 2);
        // two particles per thread on a large system (their load chains in flight together: the
        // 4,096-replica ensemble's k_order 121 -> 110 us); one on a small one, which needs the blocks
        if (s->N >= kOrderPairN)
            tdsk::k_order<real, 2><<<(s->N + 511) / 512, 256, 0, st>>>(
                s->tmp, s->key[o], s->ids[o], start, (const R4<real>*)s->pos[o], (const R4<real>*)s->pol[o],
                (const R2<real>*)s->uv[o], cpos, cpol, cuv, cids, ckey, s->N);
        else
            tdsk::k_order<real, 1><<<nb, 256, 0, st>>>(s->tmp, s->key[o], s->ids[o], start,
                                                        (const R4<real>*)s->pos[o], (const R4<real>*)s->pol[o],
                                                        (const R2<real>*)s->uv[o], cpos, cpol, cuv, cids, ckey, s->N);
    }
    tdsk::StepArgs<real> a;
    a.pos = cpos;
    a.pol = cpol;
    a.uv = cuv;
    a.ids = cids;
    a.pos_o = (R4<real>*)s->pos[o];
    a.pol_o = (R4<real>*)s->pol[o];
    a.uv_o = (R2<real>*)s->uv[o];
    a.ids_o = s->ids[o];
    a.vel_o = (R2<real>*)s->vel[o];
    a.cnt_o = s->cnt[o];
    a.key_o = s->key[o];
    a.key_in = ckey;
    a.desc = s->desc;
    a.start = start;
    a.count = s->count;
    a.tile_sum = s->tile_sum;
    a.n_tiles = s->n_tiles;
    a.rec = (const real*)s->rec;
    a.adj = s->adj;
    a.G = s->G;
    a.bin_start = s->bin_start;
    a.bin_faces = s->bin_faces;
    a.rows = s->rows;
    a.ivals = s->ivals;
    a.reps = (const RepParams<real>*)s->reps;
    a.local_bits = s->local_bits;
    a.cx = (real)s->mesh->t.centroid[0], a.cy = (real)s->mesh->t.centroid[1], a.cz = (real)s->mesh->t.centroid[2];
    a.noise = noise;
    a.phi_acc = s->phi_acc;
    a.phi_pending = s->phi_pending;
    a.d_step = s->d_step;
    a.seed = s->seed;
    a.status = s->status;
    a.N = s->N;
    a.single = s->uniform_pair;
    a.nbr_list = nbr_list;
    a.nbr_cap = nbr_cap;
    a.sum_f = x ? (R4<real>*)x->sum_f : nullptr;
    a.sum_m = x ? (R2<real>*)x->sum_m : nullptr;
    {
        const RepParams<real>& r0 = *(const RepParams<real>*)s->reps_host.data();
        a.pc0.r_max2 = r0.r_max2, a.pc0.twoR = r0.twoR, a.pc0.inv_twoR = r0.inv_twoR, a.pc0.k = r0.k;
        a.pc0.adh_scale = r0.adh_scale;
        a.rp0 = r0;
    }
    {
        KernelTimer kt(s, 3);
        const long long lanes = (long long)s->N * s->lanes;
        // a stored step of the adjoint: the same sums as the plain step of the same tuning, bit for bit
        if (a.sum_f && s->lanes == 2)
            tdsk::k_step<real, 128, false, 2, false, true><<<(unsigned)((lanes + 127) / 128), 128, 0, st>>>(a);
        else if (a.sum_f && s->lanes == 4)
            tdsk::k_step<real, 128, false, 4, false, true><<<(unsigned)((lanes + 127) / 128), 128, 0, st>>>(a);
        else if (a.sum_f && s->R == 1)
            tdsk::k_step<real, 128, false, 1, true, true><<<(s->N + 127) / 128, 128, 0, st>>>(a);
        else if (a.sum_f)
            tdsk::k_step<real, 128, false, 1, false, true><<<(s->N + 127) / 128, 128, 0, st>>>(a);
        else if (nbr_list)
            tdsk::k_step<real, 128, true><<<(s->N + 127) / 128, 128, 0, st>>>(a);
        else if (s->lanes == 2)
            tdsk::k_step<real, 128, false, 2><<<(unsigned)((lanes + 127) / 128), 128, 0, st>>>(a);
        else if (s->lanes == 4)
            tdsk::k_step<real, 128, false, 4><<<(unsigned)((lanes + 127) / 128), 128, 0, st>>>(a);
        else if (s->step_block == 128 && s->R == 1)
            tdsk::k_step<real, 128, false, 1, true><<<(s->N + 127) / 128, 128, 0, st>>>(a);
        else if (s->step_block == 128)
            tdsk::k_step<real, 128><<<(s->N + 127) / 128, 128, 0, st>>>(a);
        else
            tdsk::k_step<real, 256><<<(s->N + 255) / 256, 256, 0, st>>>(a);
    }
}

// The loop graph: k_loop_arm, then a conditional WHILE node whose body (captured from the stream)
// is kLoopBlock steps and k_loop_ctl, then one whose body is a single step and k_loop_ctl. A run of n
// steps stores n / kLoopBlock and n % kLoopBlock on the device (k_loop_set) and launches the graph
// once; the step kernels' arguments are the same every step (the step counter, the order-parameter
// index and the cell lists live on the device). The block body keeps the per-pass cost of the loop
// (a conditional re-launch of the body) off every step of a small system.
constexpr int kLoopBlock = 16;

template <typename real>
int build_loop_graph(tds_sim* s) {
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle hb = 0, h1 = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&hb, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h1, g, 0, cudaGraphCondAssignDefault);
    cudaGraphNode_t arm = nullptr, nb = nullptr, n1 = nullptr;
    if (e == cudaSuccess) {
        int* left = s->loop_left;
        void* args[] = {&left, &hb, &h1};
        cudaKernelNodeParams kp = {};
        kp.func = (void*)tdsk::k_loop_arm;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(1);
        kp.kernelParams = args;
        e = cudaGraphAddKernelNode(&arm, g, nullptr, 0, &kp);
    }
    // one WHILE node after `dep` whose body is `steps` steps and the count-down of left[which]
    auto add_loop = [&](cudaGraphNode_t dep, cudaGraphConditionalHandle h, int steps, int which,
                        cudaGraphNode_t* out) -> cudaError_t {
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaError_t r = cudaGraphAddNode(out, g, &dep, nullptr, 1, &np);
        if (r != cudaSuccess) return r;
        cudaGraph_t body = np.conditional.phGraph_out[0];
        r = cudaStreamBeginCaptureToGraph(s->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (r != cudaSuccess) return r;
        for (int k = 0; k < steps; ++k) launch_one_step<real>(s, nullptr);
        tdsk::k_loop_ctl<<<1, 1, 0, s->stream>>>(s->loop_left + which, h);
        return cudaStreamEndCapture(s->stream, &body);
    };
    if (e == cudaSuccess) e = add_loop(arm, hb, kLoopBlock, 0, &nb);
    if (e == cudaSuccess) e = add_loop(nb, h1, 1, 1, &n1);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&s->loop_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        s->loop_graph = nullptr;
        return fail(s, TDS_ERR_CUDA, std::string("loop graph: ") + cudaGetErrorString(e));
    }
    return TDS_OK;
}

template <typename real>
int run_steps(tds_sim* s, int n, const double* noise_host, bool sync = true) {
    Range range("tds_step");
    int rc;
    if ((rc = ensure_series(s, s->step + n))) return rc;
    if (noise_host) {
        const size_t N = (size_t)s->N;
        if (s->noise_cap < N) {
            if (s->noise) cudaFree(s->noise);
            s->noise = nullptr;
            CK(cudaMalloc(&s->noise, N * sizeof(real)));
            s->noise_cap = N;
        }
        std::vector<real> tmp(N);
        for (int k = 0; k < n; ++k) {
            for (size_t i = 0; i < N; ++i) tmp[i] = (real)noise_host[(size_t)k * N + i];
            CK(cudaMemcpyAsync(s->noise, tmp.data(), N * sizeof(real), cudaMemcpyHostToDevice, s->stream));
            launch_one_step<real>(s, (const real*)s->noise);
            CK(cudaStreamSynchronize(s->stream));
        }
    } else {
        int left = n;
        if (!s->timing && s->graph_steps == 0 && left >= 2) {
            if (!s->loop_graph) {
                int rc2;
                if ((rc2 = build_loop_graph<real>(s))) return rc2;
            }
            tdsk::k_loop_set<<<1, 1, 0, s->stream>>>(s->loop_left, left / kLoopBlock, left % kLoopBlock);
            CK(cudaGraphLaunch(s->loop_graph, s->stream));
            left = 0;
        }
        while (!s->timing && s->graph_steps > 0 && left >= s->graph_steps) {
            const int c = s->cur;
            if (!s->graph[c]) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
                for (int k = 0; k < s->graph_steps; ++k) launch_one_step<real>(s, nullptr);
                CK(cudaStreamEndCapture(s->stream, &g));
                s->cur = c;  // capture recorded the launches; the state did not advance
                CK(cudaGraphInstantiate(&s->graph[c], g, 0));
                cudaGraphDestroy(g);
            }
            CK(cudaGraphLaunch(s->graph[c], s->stream));
            // graph_steps is even: the current buffer is the same after the chunk
            left -= s->graph_steps;
        }
        if (!s->timing && left == 1) {
            // one step: the four kernels as one graph launch (fewer gaps between them than four
            // stream launches)
            if (!s->step_graph) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
                launch_one_step<real>(s, nullptr);
                CK(cudaStreamEndCapture(s->stream, &g));
                CK(cudaGraphInstantiate(&s->step_graph, g, 0));
                cudaGraphDestroy(g);
            }
            CK(cudaGraphLaunch(s->step_graph, s->stream));
            left = 0;
        }
        for (int k = 0; k < left; ++k) launch_one_step<real>(s, nullptr);
        CK(cudaGetLastError());
    }
    s->step += n;
    if (!sync) return TDS_OK;
    int st = 0;
    CK(cudaMemcpyAsync(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (st) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "device status 0x%x after step %lld (1 non-finite, 2 wrap limit, 4 locate fallback, "
                      "16 particle outside the surface cells)", st, s->step);
        return fail(s, TDS_ERR_STATE, buf);
    }
    return TDS_OK;
}

// Device memory of one call (placement tables, adjoint buffers), released when it returns.
struct Arena {
    std::vector<void*> p;
    ~Arena() {
        for (void* q : p) cudaFree(q);
    }
    template <typename T>
    T* get(size_t n) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(n * sizeof(T), 16)) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (T*)q;
    }
};

// Sub-buffers carved from one block (256-byte aligned). In measuring mode it only adds up the
// bytes and hands out non-null placeholders.
struct Carve {
    char* base = nullptr;
    size_t cap = 0, used = 0;
    bool measure = true;
    template <typename T>
    T* get(size_t n) {
        const size_t bytes = (std::max<size_t>(n * sizeof(T), 16) + 255) & ~(size_t)255;
        const size_t off = used;
        used += bytes;
        if (measure) return reinterpret_cast<T*>((size_t)256 + off);
        return used <= cap ? reinterpret_cast<T*>(base + off) : nullptr;
    }
};

// Loads the state waiting in the input staging (k_load_state computes polarity, cell keys and
// counts) on the compute stream; per-tile counts for the next scan. I: the staged element type
// (uv 2N, theta N, r3d 3N values of I at the start of the staging).
// A load refused on the device (k_check_faces: a face index >= F) is reported once, by the
// caller's next synchronising call: tds_set_state itself, or tds_sync after tds_set_state_async.
int take_refused_load(tds_sim* s, const char* who) {
    // on the handle's (non-blocking) stream, so that the clear is ordered before any later load
    int refused = 0;
    CK(cudaMemcpyAsync(&refused, s->load_flag + 2, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (!refused) return TDS_OK;
    CK(cudaMemsetAsync(s->load_flag + 2, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return fail(s, TDS_ERR_ARG, std::string(who) + ": face index out of range; the load was refused and the "
                                                   "state is the one before it");
}

// The face indices are checked on the device (k_check_faces) rather than by a host loop over the
// caller's array (the host loop took ~0.23 ms of host time per call at 1M particles, about as long
// as the whole pipelined step): on the upload stream, right after the upload, so that the check
// is off the compute stream's chain (load_state); its outcome for staging b is load_flag[b]. A
// refused load changes nothing.
template <typename real, typename I = double>
int load_from_staging(tds_sim* s, int b, bool has_face, bool has_r3d, bool sync, bool checked) {
    const size_t N = (size_t)s->N;
    s->cur = 0;
    const int nb = (s->N + 255) / 256;
    const I* in = reinterpret_cast<const I*>(s->in_d[b]);
    int* flag = s->load_flag + b;
    if (!checked) CK(cudaMemsetAsync(flag, 0, sizeof(int), s->stream));
    const int nc = (int)std::min<long long>((s->M + 255) / 256, 8 * 152);
    tdsk::k_clear_counts<<<nc, 256, 0, s->stream>>>(s->count, s->M, s->tile_sum, 2 * s->n_tiles, flag);
    tdsk::k_load_state<real, I><<<nb, 256, 0, s->stream>>>(
        in, in + 2 * N, s->in_i[b], in + 3 * N, has_face, has_r3d, (const real*)s->rec, s->adj, s->G,
        s->bin_start, s->bin_faces, (const RepParams<real>*)s->reps, s->local_bits, s->rows, s->ivals, s->ids[0],
        (R4<real>*)s->pos[0], (R4<real>*)s->pol[0], (R2<real>*)s->uv[0], s->ids[0], (R2<real>*)s->vel[0], s->cnt[0],
        s->key[0], s->count, s->N, s->status, flag);
    tdsk::k_tile_sums<<<s->n_tiles, tdsk::kScanThreads, 0, s->stream>>>(s->count, s->M, s->tile_sum, s->n_tiles,
                                                                         s->d_step, flag);
    CK(cudaGetLastError());
    CK(cudaEventRecord(s->ev_in_free[b], s->stream));
    if (!sync) return TDS_OK;
    CK(cudaStreamSynchronize(s->stream));
    return take_refused_load(s, "set_state");
}

// Input: host -> input staging on the upload stream, then the load on the compute stream. The
// upload waits until the previous load has consumed the staging. View: tds_state_view (double)
// or tds_state_view_f32 (float; the staging holds 6N doubles, room for 6N floats).
template <typename real, typename View>
int load_state(tds_sim* s, const View* in, bool sync) {
    Range range("tds_set_state");
    typedef typename std::remove_pointer<decltype(View::uv)>::type I;
    const size_t N = (size_t)s->N;
    if (!in || !in->uv || !in->theta) return fail(s, TDS_ERR_ARG, "set_state needs uv and theta");
    const int b = s->in_next;
    s->in_next ^= 1;
    I* d_uv = reinterpret_cast<I*>(s->in_d[b]);
    I* d_th = d_uv + 2 * N;
    I* d_r3 = d_uv + 3 * N;
    int* d_face = s->in_i[b];
    CK(cudaStreamWaitEvent(s->up, s->ev_in_free[b], 0));
    CK(cudaMemcpyAsync(d_uv, in->uv, 2 * N * sizeof(I), cudaMemcpyHostToDevice, s->up));
    CK(cudaMemcpyAsync(d_th, in->theta, N * sizeof(I), cudaMemcpyHostToDevice, s->up));
    if (in->face) CK(cudaMemcpyAsync(d_face, in->face, N * sizeof(int), cudaMemcpyHostToDevice, s->up));
    if (in->r3d) CK(cudaMemcpyAsync(d_r3, in->r3d, 3 * N * sizeof(I), cudaMemcpyHostToDevice, s->up));
    CK(cudaMemsetAsync(s->load_flag + b, 0, sizeof(int), s->up));
    if (in->face)
        tdsk::k_check_faces<<<(s->N + 255) / 256, 256, 0, s->up>>>(d_face, s->N, s->mesh->t.F, s->load_flag + b,
                                                                   s->load_flag + 2);
    CK(cudaEventRecord(s->ev_in_ready[b], s->up));
    CK(cudaStreamWaitEvent(s->stream, s->ev_in_ready[b], 0));
    return load_from_staging<real, I>(s, b, in->face != nullptr, in->r3d != nullptr, sync, true);
}

// Places particles on the device (k_place) into the input staging and loads them.
template <typename real>
int start_device(tds_sim* s) {
    const tds::FaceTables& t = s->mesh->t;
    const tds::Mesh& m = s->mesh->m;
    const int F = t.F;
    std::vector<double> pr((size_t)F * tdsk::kPlaceRec);
    for (int f = 0; f < F; ++f) {
        const double* r = &t.rec[(size_t)f * tds::kFaceRec];
        double* d = &pr[(size_t)f * tdsk::kPlaceRec];
        for (int k = 0; k < 6; ++k) d[k] = r[16 + k];     // uv corners
        for (int k = 0; k < 3; ++k) d[6 + k] = r[24 + k];  // A
        for (int k = 0; k < 6; ++k) d[9 + k] = r[k];       // J: column u, column v
        for (int k = 0; k < 3; ++k) d[15 + k] = r[12 + k]; // normal
        const int* t3 = &m.f3[3 * (size_t)f];
        double e1[3], nrm = 0;
        for (int k = 0; k < 3; ++k) e1[k] = m.v3[3 * (size_t)t3[1] + k] - m.v3[3 * (size_t)t3[0] + k], nrm += e1[k] * e1[k];
        nrm = std::sqrt(nrm);
        for (int k = 0; k < 3; ++k) d[18 + k] = e1[k] / nrm;
    }
    Arena A;
    double* dpr = A.get<double>(pr.size());
    double* dcdf = A.get<double>((size_t)F);
    if (!dpr || !dcdf) return fail(s, TDS_ERR_NOMEM, "start: placement tables");
    CK(cudaMemcpy(dpr, pr.data(), pr.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dcdf, t.area_cdf.data(), (size_t)F * sizeof(double), cudaMemcpyHostToDevice));
    const size_t N = (size_t)s->N;
    const int b = s->in_next;
    s->in_next ^= 1;
    CK(cudaStreamWaitEvent(s->stream, s->ev_in_free[b], 0));
    tdsk::k_place<<<(s->N + 255) / 256, 256, 0, s->stream>>>(dpr, dcdf, F, s->packed_ids, s->local_bits, s->seed,
                                                              s->in_d[b], s->in_d[b] + 2 * N, s->in_i[b],
                                                              s->in_d[b] + 3 * N, s->N);
    CK(cudaGetLastError());
    // synchronises before the tables are freed; the placed faces are in range by construction
    return load_from_staging<real>(s, b, true, true, true, false);
}

// The current state in global index order into o_* (device arrays) on the compute stream; the
// slot table goes through the handle's perm array.
template <typename real, typename O>
void gather_state(tds_sim* s, O* o_uv, O* o_th, int* o_face, O* o_r3d, O* o_vel, int* o_cnt) {
    const int c = s->cur;
    const int nb = (s->N + 255) / 256;
    tdsk::k_slot_of<real><<<nb, 256, 0, s->stream>>>(s->ids[c], (const RepParams<real>*)s->reps, s->local_bits,
                                                     s->perm, s->N);
    tdsk::k_gather_state<real, O><<<nb, 256, 0, s->stream>>>(
        (const R4<real>*)s->pos[c], (const R4<real>*)s->pol[c], (const R2<real>*)s->uv[c], (const R2<real>*)s->vel[c],
        s->cnt[c], s->perm, o_uv, o_th, o_face, o_r3d, o_vel, o_cnt, s->N);
}

// Output: gather into the output staging on the compute stream, then device -> host on the
// download stream. The gather waits until the previous download has left the staging. View:
// tds_state_view (double) or tds_state_view_f32 (float; the staging holds 8N doubles, room for
// 8N floats).
template <typename real, typename View>
int save_state(tds_sim* s, View* out, bool sync) {
    Range range("tds_get_state");
    typedef typename std::remove_pointer<decltype(View::uv)>::type O;
    const size_t N = (size_t)s->N;
    const int b = s->out_next;
    s->out_next ^= 1;
    O* d_uv = reinterpret_cast<O*>(s->st_d[b]);
    O* d_th = d_uv + 2 * N;
    O* d_r3 = d_uv + 3 * N;
    O* d_vel = d_uv + 6 * N;
    int* d_face = s->st_i[b];
    int* d_cnt = s->st_i[b] + N;
    CK(cudaStreamWaitEvent(s->stream, s->ev_out_free[b], 0));
    gather_state<real, O>(s, d_uv, d_th, d_face, d_r3, d_vel, d_cnt);
    CK(cudaGetLastError());
    CK(cudaEventRecord(s->ev_out_ready[b], s->stream));
    CK(cudaStreamWaitEvent(s->down, s->ev_out_ready[b], 0));
    cudaStream_t d = s->down;
    if (out->uv) CK(cudaMemcpyAsync(out->uv, d_uv, 2 * N * sizeof(O), cudaMemcpyDeviceToHost, d));
    if (out->theta) CK(cudaMemcpyAsync(out->theta, d_th, N * sizeof(O), cudaMemcpyDeviceToHost, d));
    if (out->face) CK(cudaMemcpyAsync(out->face, d_face, N * sizeof(int), cudaMemcpyDeviceToHost, d));
    if (out->r3d) CK(cudaMemcpyAsync(out->r3d, d_r3, 3 * N * sizeof(O), cudaMemcpyDeviceToHost, d));
    if (out->vel_uv) CK(cudaMemcpyAsync(out->vel_uv, d_vel, 2 * N * sizeof(O), cudaMemcpyDeviceToHost, d));
    if (out->nbr_count) CK(cudaMemcpyAsync(out->nbr_count, d_cnt, N * sizeof(int), cudaMemcpyDeviceToHost, d));
    CK(cudaEventRecord(s->ev_out_free[b], d));
    if (sync) CK(cudaStreamSynchronize(d));
    return TDS_OK;
}

// update()'s Particle records, packed on the device (id order) and copied in one transfer.
template <typename real>
int get_particles(tds_sim* s, tds_particle* out) {
    Range range("tds_get_particles");
    const size_t N = (size_t)s->N;
    if (!s->pk) {
        void* q = nullptr;
        if (cudaMalloc(&q, N * sizeof(tds_particle)) != cudaSuccess) {
            cudaGetLastError();
            return fail(s, TDS_ERR_NOMEM, "get_particles: staging allocation");
        }
        s->pk = (tds_particle*)q;
    }
    const int c = s->cur;
    tdsk::k_pack_particles<real><<<(s->N + 255) / 256, 256, 0, s->stream>>>(
        (const R4<real>*)s->pos[c], (const R2<real>*)s->uv[c], s->ids[c], (const R2<real>*)s->vel[c], s->cnt[c],
        (const RepParams<real>*)s->reps, s->local_bits, s->pk, s->N);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, s->pk, N * sizeof(tds_particle), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TDS_OK;
}

// Waits for every stream of the handle; a non-zero device status word is an error.
int sync_all(tds_sim* s) {
    CK(cudaStreamSynchronize(s->up));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaStreamSynchronize(s->down));
    if (s->rev) CK(cudaStreamSynchronize(s->rev));  // an adjoint that returned early leaves nothing in flight
    if (int rc = take_refused_load(s, "set_state_async")) return rc;
    int st = 0;
    CK(cudaMemcpy(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        char buf[224];
        std::snprintf(buf, sizeof buf, "device status 0x%x after step %lld (1 non-finite, 2 wrap limit, 4 locate fallback, "
                      "16 particle outside the surface cells)", st, s->step);
        return fail(s, TDS_ERR_STATE, buf);
    }
    return TDS_OK;
}

// One step that also exports every particle's neighbours (test hook).
template <typename real>
int step_neighbors(tds_sim* s, int cap, int* lists) {
    int rc;
    if ((rc = sync_all(s))) return rc;
    if ((rc = ensure_series(s, s->step + 1))) return rc;
    const long long total = (long long)s->N * cap;
    int* d = nullptr;
    if (cudaMalloc(&d, (size_t)total * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return fail(s, TDS_ERR_NOMEM, "step_neighbors: list allocation");
    }
    CK(cudaMemsetAsync(d, 0xFF, (size_t)total * sizeof(int), s->stream));
    launch_one_step<real>(s, nullptr, nullptr, d, cap);
    tdsk::k_nbr_ids<real><<<(unsigned)((total + 255) / 256), 256, 0, s->stream>>>(
        d, cap, s->ids[1], (const RepParams<real>*)s->reps, s->local_bits, total);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(lists, d, (size_t)total * sizeof(int), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(s, TDS_ERR_CUDA, std::string("step_neighbors: ") + cudaGetErrorString(e));
    s->step += 1;
    return sync_all(s);
}


// ---------------------------------------------------------------------------------------------
// Adjoint run (tds_adjoint_run): forward with checkpoints, loss, reverse sweep
// ---------------------------------------------------------------------------------------------
// The input state of a step: buffer 0, the cell counts, the per-tile counts and the step counter.
template <typename real>
struct Snapshot {
    R4<real>* pos = nullptr;
    R4<real>* pol = nullptr;
    R2<real>* uv = nullptr;
    int* ids = nullptr;
    int* key = nullptr;
    int* count = nullptr;
    int* tile_sum = nullptr;
    long long* d_step = nullptr;
    bool alloc(Carve& A, size_t N, size_t M, int n_tiles) {
        pos = A.get<R4<real>>(N), pol = A.get<R4<real>>(N), uv = A.get<R2<real>>(N);
        ids = A.get<int>(N), key = A.get<int>(N), count = A.get<int>(M), tile_sum = A.get<int>(2 * (size_t)n_tiles);
        d_step = A.get<long long>(1);
        return pos && pol && uv && ids && key && count && tile_sum && d_step;
    }
};

template <typename real>
void snapshot_copy(tds_sim* s, const Snapshot<real>& x, bool take) {
    const size_t N = (size_t)s->N;
    auto cp = [&](void* snap, void* live, size_t bytes) {
        if (take)
            cudaMemcpyAsync(snap, live, bytes, cudaMemcpyDeviceToDevice, s->stream);
        else
            cudaMemcpyAsync(live, snap, bytes, cudaMemcpyDeviceToDevice, s->stream);
    };
    cp(x.pos, s->pos[0], N * sizeof(R4<real>));
    cp(x.pol, s->pol[0], N * sizeof(R4<real>));
    cp(x.uv, s->uv[0], N * sizeof(R2<real>));
    cp(x.ids, s->ids[0], N * sizeof(int));
    cp(x.key, s->key[0], N * sizeof(int));
    cp(x.count, s->count, (size_t)s->M * sizeof(int));
    cp(x.tile_sum, s->tile_sum, 2 * (size_t)s->n_tiles * sizeof(int));
    cp(x.d_step, s->d_step, sizeof(long long));
}

// The two captured K-step segments of an adjoint run (without and with the per-step store).
template <typename real>
struct SegGraphs {
    tds_sim* s;
    int K;
    const StepHooks* hk;
    const StepStore* store;
    cudaGraphExec_t g[2] = {nullptr, nullptr};
    SegGraphs(tds_sim* s_, int K_, const StepHooks* hk_, const StepStore* store_) : s(s_), K(K_), hk(hk_), store(store_) {}
    ~SegGraphs() {
        for (cudaGraphExec_t x : g)
            if (x) cudaGraphExecDestroy(x);
    }
    int launch(bool stored) {
        cudaGraphExec_t& x = g[stored ? 1 : 0];
        if (!x) {
            cudaGraph_t graph = nullptr;
            CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            StepHooks h = *hk;
            for (int k = 0; k < K; ++k) {
                h.store = stored ? &store[k] : nullptr;
                launch_one_step<real>(s, nullptr, &h);
            }
            const cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
            if (e != cudaSuccess) return fail(s, TDS_ERR_CUDA, std::string("adjoint segment capture: ") + cudaGetErrorString(e));
            const cudaError_t e2 = cudaGraphInstantiate(&x, graph, 0);
            cudaGraphDestroy(graph);
            if (e2 != cudaSuccess) {
                x = nullptr;
                return fail(s, TDS_ERR_CUDA, std::string("adjoint segment graph: ") + cudaGetErrorString(e2));
            }
        }
        CK(cudaGraphLaunch(x, s->stream));
        return TDS_OK;
    }
};

template <typename real>
int adjoint_run(tds_sim* s, const tds_adjoint_spec* sp_in, tds_adjoint_result* res) {
    Range range("tds_adjoint_run");
    if (sp_in->n_steps < 1) return fail(s, TDS_ERR_ARG, "adjoint: n_steps must be >= 1");
    if (!(sp_in->w_pos >= 0 && sp_in->w_phi >= 0)) return fail(s, TDS_ERR_ARG, "adjoint: weights must be >= 0");
    if (sp_in->window < 0) return fail(s, TDS_ERR_ARG, "adjoint: window must be >= 0");
    if (sp_in->gather_lanes != 0 && sp_in->gather_lanes != 1 && sp_in->gather_lanes != 4)
        return fail(s, TDS_ERR_ARG, "adjoint: gather_lanes must be 0, 1 or 4");
    int rc;
    if ((rc = sync_all(s))) return rc;
    // A window shorter than the run: the steps before it run forward only (their order-parameter
    // terms are added to the loss value), and the reverse sweep covers the window.
    tds_adjoint_spec spw = *sp_in;
    double pre_loss = 0.0;
    if (sp_in->window > 0 && sp_in->window < sp_in->n_steps) {
        const int pre = sp_in->n_steps - sp_in->window;
        const long long t_pre = s->step;
        if ((rc = run_steps<real>(s, pre, nullptr, true))) return rc;
        if (sp_in->phi_target && sp_in->w_phi > 0) {
            flush_finalize<real>(s);
            const size_t R = (size_t)s->R;
            std::vector<double> ser((size_t)pre * 2 * R);
            CK(cudaMemcpyAsync(ser.data(), s->series + (size_t)t_pre * 2 * R, ser.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            for (int t = 0; t < pre; ++t)
                for (size_t r = 0; r < R; ++r) {
                    const double d = ser[(size_t)t * 2 * R + r] - sp_in->phi_target[(size_t)t * R + r];
                    pre_loss += sp_in->w_phi * d * d;
                }
        }
        spw.n_steps = sp_in->window;
        spw.phi_target = sp_in->phi_target ? sp_in->phi_target + (size_t)pre * s->R : nullptr;
    }
    const tds_adjoint_spec* sp = &spw;
    const int T = sp->n_steps;
    const size_t N = (size_t)s->N, M = (size_t)s->M, R = (size_t)s->R;
    const size_t b_state = N * (2 * sizeof(R4<real>) + sizeof(R2<real>) + 2 * sizeof(int));
    // a stored step keeps its pair sums (24 B per particle in FP32), as the step kernel computed them
    const size_t b_store = b_state + (M + 1) * sizeof(int) + N * (sizeof(R4<real>) + sizeof(R2<real>));
    const size_t b_snap = b_state + M * sizeof(int) + 2 * (size_t)s->n_tiles * sizeof(int) + 64;
    const size_t b_fixed = 2 * 4 * N * sizeof(real) + 3 * N * sizeof(R4<real>) + N * tdsk::kGPar * sizeof(real) +
                           (size_t)T * R * (7 * sizeof(double) + sizeof(R4<real>)) + 3 * N * sizeof(double) + b_snap;
    // checkpoint stride: the largest that fits (one stored segment + the checkpoints)
    int K = sp->checkpoint_stride;
    if (K <= 0) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        fr += s->adj_ws_bytes;  // the cached work block is reused (or freed and replaced)
        const double budget = fr > b_fixed ? 0.8 * (double)(fr - b_fixed) : 0.0;
        for (int k = T; k >= 1; --k) {
            const double need = (double)((T + k - 1) / k) * (double)b_snap + (double)k * (double)b_store;
            if (need <= budget) {
                K = k;
                break;
            }
        }
        if (K <= 0) return fail(s, TDS_ERR_NOMEM, "adjoint: not enough device memory for one stored step");
    }
    K = std::min(K, T);
    const int nseg = (T + K - 1) / K;
    // Two sets of store slots when the memory allows: the reverse sweep of a segment (on the
    // handle's reverse stream) then runs beside the recompute of the segment before it (on the
    // compute stream), which writes the other set. On a small system both are latency-bound and
    // fill a fraction of the GPU, so they overlap almost fully.
    bool two_sets = false;
    if (nseg > 1) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        fr += s->adj_ws_bytes;
        const double budget = fr > b_fixed ? 0.8 * (double)(fr - b_fixed) : 0.0;
        two_sets = (double)nseg * (double)b_snap + 2.0 * (double)K * (double)b_store <= budget;
    }

    std::vector<Snapshot<real>> snaps(nseg);
    Snapshot<real> fin;
    std::vector<StepStore> store((size_t)(two_sets ? 2 : 1) * K);
    real* lam[2] = {nullptr, nullptr};
    R4<real>*aF = nullptr, *aM = nullptr, *aP = nullptr;
    real* gpar = nullptr;
    R4<real>* dSb = nullptr;  // dL/dS per stored step and replica (k_adj_phib)
    double *phisum = nullptr, *phibar = nullptr, *rtgt = nullptr, *d_gp = nullptr, *d_ploss = nullptr;
    int *d_off = nullptr, *d_cnt = nullptr, *d_t0 = nullptr;
    // all work buffers come from one block: measured first, then carved
    auto carve = [&](Carve& A) -> bool {
        bool ok = true;
        for (auto& x : snaps) ok = x.alloc(A, N, M, s->n_tiles) && ok;
        ok = fin.alloc(A, N, M, s->n_tiles) && ok;
        for (auto& x : store) {
            x.pos = A.get<R4<real>>(N), x.pol = A.get<R4<real>>(N), x.uv = A.get<R2<real>>(N);
            x.ids = A.get<int>(N), x.key = A.get<int>(N), x.start = A.get<int>(M + 1);
            x.sum_f = A.get<R4<real>>(N), x.sum_m = A.get<R2<real>>(N);
            ok = ok && x.pos && x.pol && x.uv && x.ids && x.key && x.start && x.sum_f && x.sum_m;
        }
        lam[0] = A.get<real>(4 * N), lam[1] = A.get<real>(4 * N);
        aF = A.get<R4<real>>(N), aM = A.get<R4<real>>(N), aP = A.get<R4<real>>(N);
        gpar = A.get<real>(N * tdsk::kGPar);
        phisum = A.get<double>((size_t)T * R * 6);
        phibar = A.get<double>((size_t)T * R);
        dSb = A.get<R4<real>>((size_t)T * R);
        rtgt = sp->r3d_target ? A.get<double>(3 * N) : nullptr;
        d_ploss = A.get<double>(R);
        d_off = A.get<int>(R), d_cnt = A.get<int>(R), d_t0 = A.get<int>(1);
        d_gp = A.get<double>(R * tdsk::kGPar);
        return ok && lam[0] && lam[1] && aF && aM && aP && gpar && phisum && phibar && dSb && d_off && d_cnt && d_t0 &&
               d_gp && d_ploss &&
               (!sp->r3d_target || rtgt);
    };
    {
        Carve m;
        carve(m);
        if (m.used > s->adj_ws_bytes) {
            if (s->adj_ws) cudaFree(s->adj_ws);
            s->adj_ws = nullptr, s->adj_ws_bytes = 0;
            void* q = nullptr;
            if (cudaMalloc(&q, m.used) != cudaSuccess) {
                cudaGetLastError();
                return fail(s, TDS_ERR_NOMEM, "adjoint: work memory allocation");
            }
            s->adj_ws = q, s->adj_ws_bytes = m.used;
        }
        Carve c;
        c.base = (char*)s->adj_ws, c.cap = s->adj_ws_bytes, c.measure = false;
        if (!carve(c)) return fail(s, TDS_ERR_NOMEM, "adjoint: work memory carving");
    }
    {
        const int nN = s->N;  // the scan writes start[0..M); start[M] = N stays
        for (auto& x : store) CK(cudaMemcpyAsync(x.start + M, &nN, sizeof(int), cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if ((rc = ensure_series(s, s->step + T))) return rc;
    free_graphs(s);
    {
        // replica slot ranges (the per-replica sums) and the position target, uploaded before the run
        std::vector<int> off(s->off.begin(), s->off.end()), cnt(s->n_rep.begin(), s->n_rep.end());
        CK(cudaMemcpyAsync(d_off, off.data(), R * sizeof(int), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(d_cnt, cnt.data(), R * sizeof(int), cudaMemcpyHostToDevice, s->stream));
        if (rtgt)
            CK(cudaMemcpyAsync(rtgt, sp->r3d_target, 3 * N * sizeof(double), cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }

    // ---- forward: checkpoints every K steps, the last segment stored step by step ----
    const long long t_base = s->step;
    StepHooks hk;
    hk.phisum = phisum, hk.phisum_base = t_base, hk.phisum_cap = T;
    // A full segment's K steps are the same launches every time (the store slots are reused by
    // each segment, and the step counter and the order-parameter index live on the device), so
    // they are captured once as a CUDA graph without the store (the forward's earlier segments)
    // and once with it (the forward's last segment and every recomputed segment). On a small
    // system the step is launch-bound and the graphs remove the launch gaps.
    SegGraphs<real> sg(s, K, &hk, store.data());
    SegGraphs<real> sg1(s, K, &hk, store.data() + (two_sets ? K : 0));
    auto run_segment = [&](int t0, int t1, bool stored, int set) -> int {
        if (t1 - t0 == K && !s->timing) return (set ? sg1 : sg).launch(stored);
        for (int t = t0; t < t1; ++t) {
            hk.store = stored ? &store[(size_t)set * K + (t - t0)] : nullptr;
            launch_one_step<real>(s, nullptr, &hk);
        }
        return TDS_OK;
    };
    {
        Range fwd("adjoint forward");
        for (int seg = 0; seg < nseg; ++seg) {
            snapshot_copy<real>(s, snaps[seg], true);
            if ((rc = run_segment(seg * K, std::min(T, seg * K + K), seg == nseg - 1, 0))) return rc;
        }
        flush_finalize<real>(s, &hk);
    }
    CK(cudaGetLastError());
    s->step += T;
    snapshot_copy<real>(s, fin, true);
    if ((rc = sync_all(s))) return rc;

    // ---- loss (double): the position term per replica on the device, the order-parameter term here ----
    double loss = 0;
    std::vector<double> phib((size_t)T * R, 0.0);
    if (sp->r3d_target && sp->w_pos > 0) {
        tdsk::k_adj_pos_loss<real><<<(int)R, 256, 0, s->stream>>>((const R4<real>*)s->pos[s->cur], s->ids[s->cur],
                                                                  (const RepParams<real>*)s->reps, s->local_bits,
                                                                  rtgt, d_off, d_cnt, d_ploss);
        std::vector<double> pl(R);
        CK(cudaMemcpyAsync(pl.data(), d_ploss, R * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (size_t r = 0; r < R; ++r) loss += sp->w_pos * pl[r] / s->n_rep[r];
    }
    const bool phi_term = sp->phi_target && sp->w_phi > 0;
    if (phi_term) {
        std::vector<double> ser((size_t)T * 2 * R);
        CK(cudaMemcpy(ser.data(), s->series + (size_t)t_base * 2 * R, ser.size() * sizeof(double),
                      cudaMemcpyDeviceToHost));
        for (int t = 0; t < T; ++t)
            for (size_t r = 0; r < R; ++r) {
                const double d = ser[(size_t)t * 2 * R + r] - sp->phi_target[(size_t)t * R + r];
                loss += sp->w_phi * d * d;
                phib[(size_t)t * R + r] = 2 * sp->w_phi * d;
            }
        CK(cudaMemcpyAsync(phibar, phib.data(), phib.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    }
    // ---- reverse sweep ----
    Range rev("adjoint reverse");
    CK(cudaMemsetAsync(lam[0], 0, 4 * N * sizeof(real), s->stream));
    CK(cudaMemsetAsync(gpar, 0, N * tdsk::kGPar * sizeof(real), s->stream));
    if (phi_term)
        tdsk::k_adj_phib<real><<<(unsigned)(((long long)T * R + 255) / 256), 256, 0, s->stream>>>(
            phisum, phibar, (const RepParams<real>*)s->reps, (int)R, (long long)T * R, dSb);
    tdsk::AdjArgs<real> a;
    std::memset(&a, 0, sizeof a);
    a.desc = s->desc;
    a.rec = (const real*)s->rec;
    a.adj = s->adj;
    a.G = s->G;
    a.bin_start = s->bin_start;
    a.bin_faces = s->bin_faces;
    a.reps = (const RepParams<real>*)s->reps;
    a.local_bits = s->local_bits;
    a.cx = (real)s->mesh->t.centroid[0], a.cy = (real)s->mesh->t.centroid[1], a.cz = (real)s->mesh->t.centroid[2];
    a.seed = s->seed;
    a.w_pos = sp->w_pos;
    a.aF = aF, a.aM = aM, a.aP = aP;
    a.gpar = gpar;
    a.N = s->N;
    a.t0 = d_t0;
    a.T = T;
    a.R = (int)R;
    a.step0 = t_base;
    a.phib = phi_term ? dSb : nullptr;
    a.r_target = (rtgt && sp->w_pos > 0) ? rtgt : nullptr;
    a.lam[0] = lam[0], a.lam[1] = lam[1];
    const unsigned nbA = (unsigned)((s->N + tdsk::kAdjThreads - 1) / tdsk::kAdjThreads);
    // lanes per particle of the neighbour gather (k_adj_b): on a small system one particle's chain
    // of candidate loads sets the reverse step's time, and four lanes shorten it (10,000 particles:
    // forward+adjoint 48.0 -> 46.1 us per step); on a large one the GPU is full either way
    const int glanes = sp->gather_lanes ? sp->gather_lanes : (s->N < (1 << 17) ? 4 : 1);
    const unsigned nbB = (unsigned)((4ll * s->N + tdsk::kAdjThreads - 1) / tdsk::kAdjThreads);
    if (!s->rev && cudaStreamCreateWithFlags(&s->rev, cudaStreamNonBlocking) != cudaSuccess) {
        s->rev = nullptr;
        return fail(s, TDS_ERR_CUDA, "adjoint: reverse stream");
    }
    cudaStream_t rs = s->rev;
    // events: [0] the reverse may start / the reverse is done, [1..2] store set recomputed,
    // [3..4] store set read by its reverse sweep
    struct Events {
        cudaEvent_t e[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        ~Events() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } ev;
    for (cudaEvent_t& x : ev.e) CK(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    cudaEvent_t* ev_rec = ev.e + 1;
    cudaEvent_t* ev_read = ev.e + 3;
    CK(cudaEventRecord(ev.e[0], s->stream));
    CK(cudaStreamWaitEvent(rs, ev.e[0], 0));
    // the reverse launches of steps t0 + n - 1 .. t0 of a segment (slots n - 1 .. 0 of a store set);
    // t0 is read on the device, so a full segment's launches are the same for every segment
    auto reverse_launches = [&](int n, const StepStore* base) {
        for (int j = n - 1; j >= 0; --j) {
            const StepStore& x = base[j];
            a.pos = (const R4<real>*)x.pos, a.pol = (const R4<real>*)x.pol, a.uv = (const R2<real>*)x.uv;
            a.ids = x.ids, a.key = x.key, a.start = x.start;
            a.sum_f = (const R4<real>*)x.sum_f, a.sum_m = (const R2<real>*)x.sum_m;
            a.j = j;
            tdsk::k_adj_a<real><<<nbA, tdsk::kAdjThreads, 0, rs>>>(a);
            if (glanes == 4)
                tdsk::k_adj_b<real, 4><<<nbB, tdsk::kAdjThreads, 0, rs>>>(a);
            else
                tdsk::k_adj_b<real, 1><<<nbA, tdsk::kAdjThreads, 0, rs>>>(a);
        }
    };
    // A full segment's reverse launches as one CUDA graph per store set (captured once per call):
    // on a small system the reverse step is launch-bound
    struct Graphs {
        cudaGraphExec_t g[2] = {nullptr, nullptr};
        ~Graphs() {
            for (cudaGraphExec_t x : g)
                if (x) cudaGraphExecDestroy(x);
        }
    } rgraph;
    // the recompute of segment g into store set `set` (compute stream), after the reverse sweep that
    // last read that set
    auto recompute = [&](int g, int set) -> int {
        CK(cudaStreamWaitEvent(s->stream, ev_read[set], 0));
        snapshot_copy<real>(s, snaps[g], false);
        // (the order-parameter sums of these steps are written again, with the same values)
        int r = run_segment(g * K, std::min(T, g * K + K), true, set);
        if (r) return r;
        flush_finalize<real>(s);  // the next restore must not finalize this segment's last step
        CK(cudaEventRecord(ev_rec[set], s->stream));
        return TDS_OK;
    };
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int t0 = seg * K, t1 = std::min(T, t0 + K);
        const int set = two_sets ? (nseg - 1 - seg) & 1 : 0;
        // the last segment's store is the forward's; an earlier one is recomputed from its checkpoint:
        // with two sets, the segment before this one is recomputed now, beside this one's reverse
        if (!two_sets && seg != nseg - 1 && (rc = recompute(seg, 0))) return rc;
        if (two_sets && seg >= 1 && (rc = recompute(seg - 1, set ^ 1))) return rc;
        if (seg != nseg - 1) CK(cudaStreamWaitEvent(rs, ev_rec[set], 0));
        const StepStore* base = store.data() + (size_t)set * K;
        tdsk::k_adj_segment<<<1, 1, 0, rs>>>(d_t0, t0);
        if (t1 - t0 == K && K > 1 && !s->timing) {
            cudaGraphExec_t& g = rgraph.g[set];
            if (!g) {
                cudaGraph_t graph = nullptr;
                CK(cudaStreamBeginCapture(rs, cudaStreamCaptureModeThreadLocal));
                reverse_launches(K, base);
                const cudaError_t e = cudaStreamEndCapture(rs, &graph);
                if (e != cudaSuccess)
                    return fail(s, TDS_ERR_CUDA, std::string("adjoint reverse capture: ") + cudaGetErrorString(e));
                const cudaError_t e2 = cudaGraphInstantiate(&g, graph, 0);
                cudaGraphDestroy(graph);
                if (e2 != cudaSuccess) {
                    g = nullptr;
                    return fail(s, TDS_ERR_CUDA, std::string("adjoint reverse graph: ") + cudaGetErrorString(e2));
                }
            }
            CK(cudaGraphLaunch(g, rs));
        } else {
            reverse_launches(t1 - t0, base);
        }
        CK(cudaEventRecord(ev_read[set], rs));
    }
    CK(cudaEventRecord(ev.e[0], rs));
    CK(cudaStreamWaitEvent(s->stream, ev.e[0], 0));
    tdsk::k_adj_reduce<real><<<(int)R, 256, 0, s->stream>>>(gpar, (long long)N, d_off, d_cnt, d_gp);
    CK(cudaGetLastError());
    snapshot_copy<real>(s, fin, false);  // the handle ends where the forward ended
    std::vector<double> gh(R * tdsk::kGPar);
    CK(cudaMemcpyAsync(gh.data(), d_gp, gh.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (res->d_uv0 || res->d_theta0) {
        // the initial state's adjoint as the caller's doubles, converted on the device into the
        // output staging (8N doubles) and copied straight into the caller's arrays
        double* d_uv = s->st_d[0];
        double* d_th = d_uv + 2 * N;
        tdsk::k_adj_out<real><<<(unsigned)((N + 255) / 256), 256, 0, s->stream>>>(lam[T & 1], d_uv, d_th, (int)N);
        if (res->d_uv0)
            CK(cudaMemcpyAsync(res->d_uv0, d_uv, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        if (res->d_theta0)
            CK(cudaMemcpyAsync(res->d_theta0, d_th, N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    }
    if ((rc = sync_all(s))) return rc;
    res->loss = pre_loss + loss;
    res->checkpoint_stride = K;
    if (res->d_params)
        for (size_t i = 0; i < gh.size(); ++i) res->d_params[i] = gh[i];
    return TDS_OK;
}

int check_params(const tds_params& p, std::string& why);

template <typename real>
int set_params(tds_sim* s, const tds_params* prm) {
    std::vector<RepParams<real>> rp(s->R);
    std::memcpy(rp.data(), s->reps_host.data(), rp.size() * sizeof(RepParams<real>));
    for (int r = 0; r < s->R; ++r) {
        std::string why;
        if (check_params(prm[r], why)) return fail(s, TDS_ERR_ARG, "set_params: " + why);
        if (prm[r].radius != s->prm[r].radius || prm[r].r_max != s->prm[r].r_max)
            return fail(s, TDS_ERR_ARG, "set_params: radius and r_max fix the cell lists and cannot change");
        fill_params(rp[r], prm[r]);
    }
    int rc;
    if ((rc = sync_all(s))) return rc;
    CK(cudaMemcpy(s->reps, rp.data(), rp.size() * sizeof(RepParams<real>), cudaMemcpyHostToDevice));
    s->reps_host.assign((const unsigned char*)rp.data(), (const unsigned char*)(rp.data() + rp.size()));
    set_uniform_pair<real>(s);
    for (int r = 0; r < s->R; ++r) s->prm[r] = prm[r];
    free_graphs(s);  // captured launches carry the single-replica pair constants
    return TDS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// State read-back that allocates nothing (tds_get_state_noalloc)
// ---------------------------------------------------------------------------------------------
// Some callers cannot allocate device memory at the point where they read the state back: a host
// framework that owns all device memory through its own allocator, a memory budget that is fixed
// after start-up, or a loop that must not call cudaMalloc/cudaFree because those synchronise the
// device. For them the read-back stages the state in this fixed file-scope array instead of the
// handle's staging buffers: 16 MiB, i.e. at most 233,016 particles at 72 bytes each (uv, theta,
// r3d and chart velocity as double, face and neighbour count as int). Every GPU that loads the
// library holds the array until the process exits.
constexpr size_t kNoAllocStagingBytes = (size_t)16 << 20;
constexpr size_t kNoAllocBytesPerParticle = 8 * sizeof(double) + 2 * sizeof(int);
static __device__ __align__(256) unsigned char g_noalloc_staging[kNoAllocStagingBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {};  // device address of the staging array, per device ordinal

// Device address of the staging array on the current device. The symbol's name is only a
// host-side stand-in, so the address is looked up once per device (with that device current).
int noalloc_staging(tds_sim* s, void** addr) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return fail(s, TDS_ERR_LIMIT, "device ordinal above 255");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_staging);
        if (e != cudaSuccess) return fail(s, TDS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    *addr = g_noalloc_addr[dev];
    return TDS_OK;
}

template <typename real>
int save_state_noalloc(tds_sim* s, tds_state_view* out) {
    const size_t N = (size_t)s->N;
    if (N * kNoAllocBytesPerParticle > kNoAllocStagingBytes) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "tds_get_state_noalloc: %zu particles exceed the fixed staging of %zu bytes "
                      "(at most %zu particles)", N, kNoAllocStagingBytes, kNoAllocStagingBytes / kNoAllocBytesPerParticle);
        return fail(s, TDS_ERR_LIMIT, buf);
    }
    void* base = nullptr;
    int rc;
    if ((rc = noalloc_staging(s, &base))) return rc;
    // every staged value is written by the gather for all N particles: nothing needs clearing
    double* d_uv = (double*)base;
    double* d_th = d_uv + 2 * N;
    double* d_r3 = d_uv + 3 * N;
    double* d_vel = d_uv + 6 * N;
    int* d_face = (int*)(d_uv + 8 * N);
    int* d_cnt = d_face + N;
    gather_state<real, double>(s, d_uv, d_th, d_face, d_r3, d_vel, d_cnt);
    CK(cudaGetLastError());
    if (out->uv) CK(cudaMemcpyAsync(out->uv, d_uv, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (out->theta) CK(cudaMemcpyAsync(out->theta, d_th, N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (out->face) CK(cudaMemcpyAsync(out->face, d_face, N * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    if (out->r3d) CK(cudaMemcpyAsync(out->r3d, d_r3, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (out->vel_uv) CK(cudaMemcpyAsync(out->vel_uv, d_vel, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    if (out->nbr_count) CK(cudaMemcpyAsync(out->nbr_count, d_cnt, N * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TDS_OK;
}

int check_params(const tds_params& p, std::string& why) {
    if (!(p.radius > 0)) return why = "radius must be > 0", 1;
    if (!(p.r_max > 2 * p.radius)) return why = "r_max must exceed 2*radius", 1;
    if (!(p.tau > 0)) return why = "tau must be > 0", 1;
    if (!(p.dt > 0)) return why = "dt must be > 0", 1;
    if (!(p.k_rep >= 0 && p.k_adh >= 0)) return why = "stiffnesses must be >= 0", 1;
    if (p.force_mode != 0 && p.force_mode != 1) return why = "force_mode must be 0 or 1", 1;
    return 0;
}

int create_impl(const tds_mesh* mesh, int R, const int* n, const tds_params* prm, uint64_t seed, int precision,
                tds_sim** out, const tds_tuning* tune = nullptr) {
    if (!out) return TDS_ERR_ARG;
    *out = nullptr;
    auto s = std::make_unique<tds_sim>();
    if (!mesh) return fail(nullptr, TDS_ERR_ARG, "");
    if (precision != 32 && precision != 64) return TDS_ERR_ARG;
    if (R < 1) return TDS_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return TDS_ERR_CUDA;
    s->mesh = mesh;
    s->precision = precision;
    if (tune) {
        const int lanes = tune->lanes_per_particle ? tune->lanes_per_particle : 1;
        if (!(tune->cells_per_particle > 0) || (tune->step_block != 128 && tune->step_block != 256) ||
            (tune->graph_steps != 0 && (tune->graph_steps < 2 || tune->graph_steps % 2 || tune->graph_steps > 256)) ||
            (lanes != 1 && lanes != 2 && lanes != 4) || (lanes > 1 && tune->step_block != 128))
            return TDS_ERR_ARG;
        s->cells_per_particle = tune->cells_per_particle;
        s->step_block = tune->step_block;
        s->graph_steps = tune->graph_steps;
        s->lanes = lanes;
    }
    s->rsz = precision == 32 ? 4 : 8;
    s->R = R;
    s->seed = seed;
    long long total = 0;
    int nmax = 0;
    for (int r = 0; r < R; ++r) {
        std::string why;
        if (n[r] < 1 || check_params(prm[r], why)) return TDS_ERR_ARG;
        s->off.push_back((int)total);
        s->n_rep.push_back(n[r]);
        s->prm.push_back(prm[r]);
        total += n[r];
        nmax = std::max(nmax, n[r]);
    }
    if (total > (1ll << 30)) return TDS_ERR_LIMIT;
    s->N = (int)total;
    s->local_bits = R == 1 ? 31 : std::max(1, ceil_log2(nmax));
    if (R > 1 && ceil_log2(R) + s->local_bits > 31) return TDS_ERR_LIMIT;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->up, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->down, cudaStreamNonBlocking) != cudaSuccess) {
        tds_destroy(s.release());
        return TDS_ERR_CUDA;
    }
    for (cudaEvent_t* e : {&s->ev_in_ready[0], &s->ev_in_free[0], &s->ev_out_ready[0], &s->ev_out_free[0],
                           &s->ev_in_ready[1], &s->ev_in_free[1], &s->ev_out_ready[1], &s->ev_out_free[1]})
        if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
            tds_destroy(s.release());
            return TDS_ERR_CUDA;
        }
    tds_sim* sp = s.get();
    int rc = precision == 32 ? upload_tables<float>(sp) : upload_tables<double>(sp);
    if (!rc) rc = precision == 32 ? alloc_state<float>(sp) : alloc_state<double>(sp);
    if (!rc) rc = ensure_series(sp, 1024);
    if (rc) {
        tds_destroy(s.release());
        return rc;
    }
    *out = s.release();
    return TDS_OK;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------------------
// mesh
// ---------------------------------------------------------------------------------------------
int tds_mesh_ellipsoid(int level, double ax, double ay, double az, tds_mesh** out) {
    if (!out || level < 0 || level > 9 || !(ax > 0 && ay > 0 && az > 0)) return mesh_fail("bad arguments"), TDS_ERR_ARG;
    tds::Mesh m;
    tds::make_icosphere(level, m);
    tds::scale_axes(m, ax, ay, az);
    return finish_mesh(m, out);
}

int tds_mesh_bumpy_sphere(int level, double amp, double scale, tds_mesh** out) {
    if (!out || level < 0 || level > 9 || !(scale > 0) || !(std::fabs(amp) < 1))
        return mesh_fail("bad arguments"), TDS_ERR_ARG;
    tds::Mesh m;
    tds::make_icosphere(level, m);
    tds::bumpy_sphere(m, amp, scale);
    tds::orient_outward(m);
    return finish_mesh(m, out);
}

int tds_mesh_from_arrays(const double* v3, int V, const int* f3, int F, tds_mesh** out) {
    if (!out || !v3 || !f3 || V < 4 || F < 4) return mesh_fail("bad arguments"), TDS_ERR_ARG;
    tds::Mesh m;
    m.v3.assign(v3, v3 + 3 * (size_t)V);
    m.f3.assign(f3, f3 + 3 * (size_t)F);
    for (int i = 0; i < 3 * F; ++i)
        if (m.f3[i] < 0 || m.f3[i] >= V) return mesh_fail("face index out of range"), TDS_ERR_ARG;
    tds::orient_outward(m);
    return finish_mesh(m, out);
}

int tds_mesh_load_off(const char* path, tds_mesh** out) {
    if (!out || !path) return mesh_fail("bad arguments"), TDS_ERR_ARG;
    tds::Mesh m;
    std::string err;
    if (tds::read_off(path, m, err)) return mesh_fail(err);
    tds::orient_outward(m);
    return finish_mesh(m, out);
}

int tds_mesh_save_off(const tds_mesh* h, const char* path) {
    if (!h || !path) return TDS_ERR_ARG;
    std::string err;
    if (tds::write_off(path, h->m, err)) return mesh_fail(err);
    return TDS_OK;
}

int tds_mesh_info(const tds_mesh* h, int* V, int* F, int* Vuv, double* area) {
    if (!h) return TDS_ERR_ARG;
    if (V) *V = h->m.V();
    if (F) *F = h->m.F();
    if (Vuv) *Vuv = h->m.Vuv();
    if (area) *area = h->t.area;
    return TDS_OK;
}

int tds_mesh_arrays(const tds_mesh* h, double* v3, int* f3, double* uv, int* fuv, int* uv2v) {
    if (!h) return TDS_ERR_ARG;
    const tds::Mesh& m = h->m;
    if (v3) std::memcpy(v3, m.v3.data(), m.v3.size() * sizeof(double));
    if (f3) std::memcpy(f3, m.f3.data(), m.f3.size() * sizeof(int));
    if (uv) std::memcpy(uv, m.uv.data(), m.uv.size() * sizeof(double));
    if (fuv) std::memcpy(fuv, m.fuv.data(), m.fuv.size() * sizeof(int));
    if (uv2v) std::memcpy(uv2v, m.uv2v.data(), m.uv2v.size() * sizeof(int));
    return TDS_OK;
}

void tds_mesh_destroy(tds_mesh* h) { delete h; }

const char* tds_mesh_last_error(void) { return g_mesh_err.c_str(); }

// ---------------------------------------------------------------------------------------------
// simulation
// ---------------------------------------------------------------------------------------------
int tds_create(const tds_mesh* mesh, const tds_params* params, int n_particles, uint64_t seed, int precision,
               tds_sim** out) {
    if (!params) return TDS_ERR_ARG;
    return create_impl(mesh, 1, &n_particles, params, seed, precision, out);
}

int tds_ensemble_create(const tds_mesh* mesh, int n_replicas, const int* n_particles, const tds_params* params,
                        uint64_t seed, int precision, tds_sim** out) {
    if (!n_particles || !params) return TDS_ERR_ARG;
    return create_impl(mesh, n_replicas, n_particles, params, seed, precision, out);
}

int tds_create_ex(const tds_mesh* mesh, int n_replicas, const int* n_particles, const tds_params* params,
                  uint64_t seed, int precision, const tds_tuning* tuning, tds_sim** out) {
    if (!n_particles || !params) return TDS_ERR_ARG;
    return create_impl(mesh, n_replicas, n_particles, params, seed, precision, out, tuning);
}

int tds_get_tuning(const tds_sim* s, tds_tuning* out) {
    if (!s || !out) return TDS_ERR_ARG;
    out->cells_per_particle = s->cells_per_particle;
    out->step_block = s->step_block;
    out->graph_steps = s->graph_steps;
    out->lanes_per_particle = s->lanes;
    return TDS_OK;
}

int tds_autotune(const tds_mesh* mesh, int n_replicas, const int* n_particles, const tds_params* params,
                 uint64_t seed, int precision, int trial_steps, tds_tuning* best, double* best_rate) {
    if (!mesh || !n_particles || !params || !best || trial_steps < 1) return TDS_ERR_ARG;
    // candidates are timed on the caller's workload (created, placed, warmed up, then trial_steps
    // graph-launched steps, the best of two timings): first the cell-level rule x the step block
    // (one lane per particle, the loop graph), then, on the best of those, 2 and 4 lanes per
    // particle and graphs of 16 steps
    double best_r = -1;
    tds_tuning bt{4.0, 128, 0, 1};
    long long total = 0;
    for (int r = 0; r < n_replicas; ++r) total += n_particles[r];
    auto time_one = [&](const tds_tuning& t, double* rate) -> int {
        tds_sim* s = nullptr;
        int rc = create_impl(mesh, n_replicas, n_particles, params, seed, precision, &s, &t);
        if (rc) return rc;
        const int g = t.graph_steps;
        const int steps = g ? (trial_steps + g - 1) / g * g : trial_steps;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        rc = tds_start(s);
        if (!rc) rc = tds_step(s, g ? g : 16, nullptr);  // warm-up: graph capture
        double best_ms = 0;
        if (!rc && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
            for (int rep = 0; rep < 2 && !rc; ++rep) {
                float ms = 0;
                cudaEventRecord(e0, s->stream);
                rc = tds_step_async(s, steps);
                cudaEventRecord(e1, s->stream);
                if (!rc) rc = tds_sync(s);
                if (!rc) cudaEventElapsedTime(&ms, e0, e1);
                if (ms > 0 && (best_ms == 0 || ms < best_ms)) best_ms = ms;
            }
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        tds_destroy(s);
        *rate = best_ms > 0 ? (double)total * steps / (best_ms * 1e-3) : 0.0;
        return rc;
    };
    for (double c : {1.0, 4.0, 16.0})
        for (int b : {128, 256}) {
            const tds_tuning t{c, b, 0, 1};
            double rate = 0;
            if (int rc = time_one(t, &rate)) return rc;
            if (rate > best_r) best_r = rate, bt = t;
        }
    const tds_tuning base = bt;
    const tds_tuning more[] = {{base.cells_per_particle, 128, 0, 2}, {base.cells_per_particle, 128, 0, 4},
                               {base.cells_per_particle, base.step_block, 16, 1}};
    for (const tds_tuning& t : more) {
        double rate = 0;
        if (int rc = time_one(t, &rate)) return rc;
        if (rate > best_r) best_r = rate, bt = t;
    }
    *best = bt;
    if (best_rate) *best_rate = best_r;
    return TDS_OK;
}

int tds_start(tds_sim* s) {
    if (!s) return TDS_ERR_ARG;
    int rc;
    if ((rc = sync_all(s))) return rc;
    return s->precision == 32 ? start_device<float>(s) : start_device<double>(s);
}

int tds_step(tds_sim* s, int n_steps, const double* noise) {
    if (!s || n_steps < 0) return TDS_ERR_ARG;
    if (n_steps == 0) return TDS_OK;
    return s->precision == 32 ? run_steps<float>(s, n_steps, noise) : run_steps<double>(s, n_steps, noise);
}

int tds_step_async(tds_sim* s, int n_steps) {
    if (!s || n_steps < 0) return TDS_ERR_ARG;
    if (n_steps == 0) return TDS_OK;
    return s->precision == 32 ? run_steps<float>(s, n_steps, nullptr, false)
                              : run_steps<double>(s, n_steps, nullptr, false);
}

int tds_kernel_timing(tds_sim* s, int enable) {
    if (!s) return TDS_ERR_ARG;
    collect_times(s);
    s->timing = enable != 0;
    for (int k = 0; k < 5; ++k) s->k_ms[k] = 0, s->k_n[k] = 0;
    return TDS_OK;
}

int tds_kernel_times(tds_sim* s, double* total_ms, long long* launches) {
    if (!s) return TDS_ERR_ARG;
    collect_times(s);
    for (int k = 0; k < 5; ++k) {
        if (total_ms) total_ms[k] = s->k_ms[k];
        if (launches) launches[k] = s->k_n[k];
    }
    return TDS_OK;
}

int tds_update(tds_sim* s, tds_state_view* out) {
    int rc = tds_step(s, 1, nullptr);
    if (rc) return rc;
    return out ? tds_get_state(s, out) : TDS_OK;
}

int tds_set_state(tds_sim* s, const tds_state_view* in) {
    if (!s) return TDS_ERR_ARG;
    return s->precision == 32 ? load_state<float>(s, in, true) : load_state<double>(s, in, true);
}

int tds_get_state(tds_sim* s, tds_state_view* out) {
    if (!s || !out) return TDS_ERR_ARG;
    return s->precision == 32 ? save_state<float>(s, out, true) : save_state<double>(s, out, true);
}

int tds_set_state_async(tds_sim* s, const tds_state_view* in) {
    if (!s) return TDS_ERR_ARG;
    return s->precision == 32 ? load_state<float>(s, in, false) : load_state<double>(s, in, false);
}

int tds_get_state_async(tds_sim* s, tds_state_view* out) {
    if (!s || !out) return TDS_ERR_ARG;
    return s->precision == 32 ? save_state<float>(s, out, false) : save_state<double>(s, out, false);
}

// The FP32 views: FP32 handles only (an FP64 state would be rounded on the way out).
static int f32_only(tds_sim* s, const void* view) {
    if (!s || !view) return TDS_ERR_ARG;
    if (s->precision != 32) return fail(s, TDS_ERR_ARG, "the FP32 state views need an FP32 handle (precision 32)");
    return TDS_OK;
}

int tds_set_state_f32(tds_sim* s, const tds_state_view_f32* in) {
    if (int rc = f32_only(s, in)) return rc;
    return load_state<float>(s, in, true);
}

int tds_get_state_f32(tds_sim* s, tds_state_view_f32* out) {
    if (int rc = f32_only(s, out)) return rc;
    return save_state<float>(s, out, true);
}

int tds_set_state_f32_async(tds_sim* s, const tds_state_view_f32* in) {
    if (int rc = f32_only(s, in)) return rc;
    return load_state<float>(s, in, false);
}

int tds_get_state_f32_async(tds_sim* s, tds_state_view_f32* out) {
    if (int rc = f32_only(s, out)) return rc;
    return save_state<float>(s, out, false);
}

int tds_sync(tds_sim* s) {
    if (!s) return TDS_ERR_ARG;
    return sync_all(s);
}

int tds_set_params(tds_sim* s, const tds_params* params) {
    if (!s || !params) return TDS_ERR_ARG;
    return s->precision == 32 ? set_params<float>(s, params) : set_params<double>(s, params);
}

int tds_adjoint_release(tds_sim* s) {
    if (!s) return TDS_ERR_ARG;
    if (s->adj_ws) {
        if (int rc = sync_all(s)) return rc;
        cudaFree(s->adj_ws);
        s->adj_ws = nullptr, s->adj_ws_bytes = 0;
    }
    return TDS_OK;
}

int tds_adjoint_run(tds_sim* s, const tds_adjoint_spec* spec, tds_adjoint_result* out) {
    if (!s || !spec || !out) return TDS_ERR_ARG;
    return s->precision == 32 ? adjoint_run<float>(s, spec, out) : adjoint_run<double>(s, spec, out);
}

int tds_step_neighbors(tds_sim* s, int cap, int* lists) {
    if (!s || !lists || cap < 1) return TDS_ERR_ARG;
    return s->precision == 32 ? step_neighbors<float>(s, cap, lists) : step_neighbors<double>(s, cap, lists);
}

int tds_get_particles(tds_sim* s, tds_particle* out) {
    if (!s || !out) return TDS_ERR_ARG;
    return s->precision == 32 ? get_particles<float>(s, out) : get_particles<double>(s, out);
}

int tds_get_state_noalloc(tds_sim* s, tds_state_view* out) {
    if (!s || !out) return TDS_ERR_ARG;
    return s->precision == 32 ? save_state_noalloc<float>(s, out) : save_state_noalloc<double>(s, out);
}

int tds_get_order_parameter(tds_sim* s, double* phi, double* psi, int cap, int* n_steps) {
    if (!s) return TDS_ERR_ARG;
    const long long n = std::min<long long>(s->step, s->series_cap);
    if (n_steps) *n_steps = (int)n;
    if (n == 0 || cap <= 0) return TDS_OK;
    if (s->precision == 32)
        flush_finalize<float>(s);
    else
        flush_finalize<double>(s);
    std::vector<double> tmp((size_t)n * 2 * s->R);
    CK(cudaMemcpyAsync(tmp.data(), s->series, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const long long m = std::min<long long>((long long)cap, n * s->R);
    for (long long k = 0; k < m; ++k) {
        const long long t = k / s->R, r = k % s->R;
        if (phi) phi[k] = tmp[(size_t)t * 2 * s->R + r];
        if (psi) psi[k] = tmp[(size_t)t * 2 * s->R + s->R + r];
    }
    return TDS_OK;
}

int tds_get_step(const tds_sim* s, int64_t* step) {
    if (!s || !step) return TDS_ERR_ARG;
    *step = s->step;
    return TDS_OK;
}

int tds_get_status(tds_sim* s, int* status) {
    if (!s || !status) return TDS_ERR_ARG;
    CK(cudaMemcpyAsync(status, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TDS_OK;
}

int tds_clear_status(tds_sim* s) {
    if (!s) return TDS_ERR_ARG;
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TDS_OK;
}

int tds_num_particles(const tds_sim* s, int* n_total, int* n_replicas) {
    if (!s) return TDS_ERR_ARG;
    if (n_total) *n_total = s->N;
    if (n_replicas) *n_replicas = s->R;
    return TDS_OK;
}

int tds_stream(tds_sim* s, void** stream) {
    if (!s || !stream) return TDS_ERR_ARG;
    *stream = (void*)s->stream;
    return TDS_OK;
}

int tds_kernels_per_step(const tds_sim* s, int* n) {
    if (!s || !n) return TDS_ERR_ARG;
    *n = 4;
    return TDS_OK;
}

const char* tds_last_error(const tds_sim* s) { return s ? s->err.c_str() : "null handle"; }

void tds_destroy(tds_sim* s) {
    if (!s) return;
    if (s->up) cudaStreamSynchronize(s->up);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->down) cudaStreamSynchronize(s->down);
    if (s->rev) cudaStreamSynchronize(s->rev);
    collect_times(s);
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    free_graphs(s);
    for (void* p : s->allocs) cudaFree(p);
    if (s->adj_ws) cudaFree(s->adj_ws);
    if (s->pk) cudaFree(s->pk);
    if (s->series) cudaFree(s->series);
    if (s->noise) cudaFree(s->noise);
    for (cudaEvent_t e : {s->ev_in_ready[0], s->ev_in_free[0], s->ev_out_ready[0], s->ev_out_free[0],
                          s->ev_in_ready[1], s->ev_in_free[1], s->ev_out_ready[1], s->ev_out_free[1]})
        if (e) cudaEventDestroy(e);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->up) cudaStreamDestroy(s->up);
    if (s->down) cudaStreamDestroy(s->down);
    if (s->rev) cudaStreamDestroy(s->rev);
    delete s;
}

int tds_debug_seam_wrap(int n, const double* uv_old, double* uv, double* theta, double* vel_uv, int* n_wraps,
                        int precision) {
    tds_sim* s = nullptr;
    if (n <= 0 || !uv_old || !uv) return TDS_ERR_ARG;
    double *d_old = nullptr, *d_uv = nullptr, *d_th = nullptr, *d_vel = nullptr;
    int* d_nw = nullptr;
    CK(cudaMalloc(&d_old, 2 * n * sizeof(double)));
    CK(cudaMalloc(&d_uv, 2 * n * sizeof(double)));
    CK(cudaMalloc(&d_th, n * sizeof(double)));
    CK(cudaMalloc(&d_vel, 2 * n * sizeof(double)));
    CK(cudaMalloc(&d_nw, n * sizeof(int)));
    CK(cudaMemcpy(d_old, uv_old, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_uv, uv, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemset(d_th, 0, n * sizeof(double)));
    CK(cudaMemset(d_vel, 0, 2 * n * sizeof(double)));
    if (theta) CK(cudaMemcpy(d_th, theta, n * sizeof(double), cudaMemcpyHostToDevice));
    if (vel_uv) CK(cudaMemcpy(d_vel, vel_uv, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
    if (precision == 64)
        tdsk::k_debug_wrap<double><<<(n + 127) / 128, 128>>>(n, d_old, d_uv, d_th, d_vel, d_nw);
    else
        tdsk::k_debug_wrap<float><<<(n + 127) / 128, 128>>>(n, d_old, d_uv, d_th, d_vel, d_nw);
    CK(cudaGetLastError());
    CK(cudaMemcpy(uv, d_uv, 2 * n * sizeof(double), cudaMemcpyDeviceToHost));
    if (theta) CK(cudaMemcpy(theta, d_th, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (vel_uv) CK(cudaMemcpy(vel_uv, d_vel, 2 * n * sizeof(double), cudaMemcpyDeviceToHost));
    if (n_wraps) CK(cudaMemcpy(n_wraps, d_nw, n * sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(d_old), cudaFree(d_uv), cudaFree(d_th), cudaFree(d_vel), cudaFree(d_nw);
    return TDS_OK;
}

}  // extern "C"
