// Reverse mode (adjoint) of the model step, with the neighbour sets, the face locations and the
// seam-wrap sequences held at the values of the forward step.
//
// State per particle: chart position uv and polarity angle theta (the face is discrete). The 3D
// position is r = A_f + J_f (uv - a_f) and the 3D polarity p = normalize(J_f (cos th, sin th)),
// so the adjoint state is (ubar, vbar, thetabar) per particle, indexed by global particle index.
//
// One reverse step of step t is two launches over step t's sorted state:
//   k_adj_a  per particle: recomputes the forward update (pair sums -- read from the forward's
//            store, or recomputed with the step kernel's loop --, velocity, polarity rotation,
//            chart advance, seam wrap, location, map) and runs its reverse from the adjoint of the
//            state after the step (plus the loss terms on the new positions and the order
//            parameter) down to the adjoints of the pair sums F (force) and m (neighbour polarity)
//            and the particle's own direct terms; parameter terms of v0, mu, tau, align, eta.
//   k_adj_b  per particle k, over the same neighbours j (the relation is symmetric):
//            rbar_k = sum_j K(r_k - r_j) (Fbar_k - Fbar_j),  pbar_k += sum_j mbar_j,
//            K(x) = f'(d) e e^T + f(d)/d (I - e e^T) the Jacobian of one pair force, e = x/d;
//            terms of k_rep, k_adh; then the adjoint of (uv, theta) before the step.
// Gathering over neighbours instead of scattering keeps the sums free of atomics and in a fixed
// order, so the adjoint is deterministic like the forward step.
#pragma once
#include "kernels.cuh"

namespace tdsk {

enum : int { G_KREP = 0, G_KADH = 1, G_V0 = 2, G_MU = 3, G_TAU = 4, G_ALIGN = 5, G_ETA = 6, kGPar = 8 };
// Block of k_adj_a / k_adj_b. Their candidate-run tables are shared-memory columns (entry r of
// thread t at run[r * kAdjThreads]) rather than stack arrays, and the register limits trade a few
// spills for occupancy (FP32: k_adj_a at 6 blocks per SM when it reads stored pair sums, 4 when it
// runs the pair loop, k_adj_b at 5; k_adj_a at 4 rather than 3 blocks took forward+adjoint from
// 2.48e9 to 2.61e9 particle-steps/s on the 512-replica bumpy-sphere ensemble).
constexpr int kAdjThreads = 256;

template <typename real>
struct AdjArgs {
    // step t's sorted state (k_order output) and cell starts
    const R4<real>* pos;
    const R4<real>* pol;
    const R2<real>* uv;
    const int* ids;
    const int* key;
    const int* start;
    const R4<real>* sum_f;  // step t's pair sums by slot, as its step kernel stored them: (F, m.x), (m.y, m.z)
    const R2<real>* sum_m;
    const uint4* desc;
    const real* rec;
    const int4* adj;
    int G;
    const int* bin_start;
    const int* bin_faces;
    const RepParams<real>* reps;
    int local_bits;
    real cx, cy, cz;
    // Step t of the run (0 .. T - 1) is *t0 + j: t0, the first step of the current segment, is
    // read on the device, so that a segment's reverse launches (j = K - 1 .. 0) are the same for
    // every segment and are captured once as a CUDA graph.
    const int* t0;
    int j;
    int T;
    int R;
    long long step0;  // noise counter of step 0 of the run
    unsigned long long seed;
    const real* noise;  // injected noise of step t by global index, or null
    // loss terms
    const R4<real>* phib;    // [T][R] the order-parameter adjoint per step and replica: (dL/dS, S != 0),
                             // S the step's sum of normalize((r' - c) x v) (null: no order-parameter term)
    const double* r_target;  // [3N] by global index, the last step's term (null: none)
    double w_pos;
    // adjoint state: [N] x 4 by global index, (u, v, theta) padded to 16 bytes (one vector access);
    // the adjoint after step t is lam[(T - 1 - t) & 1], the one before it the other
    real* lam[2];
    R4<real>* aF;        // [N] by slot: (Fbar, ubar_direct.x)
    R4<real>* aM;        // [N] by slot: (mbar, ubar_direct.y)
    R4<real>* aP;        // [N] by slot: (pbar_direct, 0)
    real* gpar;          // [kGPar][N] by slot, in the working precision (a replica's slots are the
                         // same range in every step's sorted order)
    int N;
};

// The non-empty ones of the 9 candidate runs of a particle's cell (slot ranges in the sorted state),
// in order, as the step kernel builds them (so pair_sums_s walks them the same way).
template <typename real>
__device__ __forceinline__ int candidate_runs(const RepParams<real>& rp, const uint4* desc, const int* start, int key,
                                              int2* run) {
    int total = 0, nrun = 0;
    const int id0 = key - rp.base;
    run[0] = make_int2(0, 0);
    if (id0 < rp.C) {
        const uint4* dp = desc + (size_t)rp.desc_off + (size_t)id0 * 2;
        const uint4 d0 = dp[0], d1 = dp[1];
        const unsigned e[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
        const int Lb = (int)((d0.x >> 2) & 1u), Rb = (int)((d0.x >> 3) & 1u);
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const int first = r == 4 ? id0 - Lb : (int)(e[r < 4 ? r : r - 1] >> 4);
            const int len = r == 4 ? 1 + Lb + Rb : (int)(e[r < 4 ? r : r - 1] & 3u);
            const int b0 = rp.base + first;
            const int t0 = len ? start[b0] : 0;
            const int t1 = len ? start[b0 + len] : 0;
            if (t1 > t0) {
                run[nrun * kAdjThreads] = make_int2(t0, t1 - t0);
                ++nrun;
            }
            total += t1 - t0;
        }
    }
    return total;
}

template <typename real>
__device__ __forceinline__ void cross(const real a[3], const real b[3], real o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename real>
__device__ __forceinline__ real dot(const real a[3], const real b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// The pair sums are the ones the forward's step kernel stored for this step (a.sum_f, a.sum_m:
// its own values, whatever its lanes per particle), so the kernel has no pair loop. Two phases, so that few values are live at any point: the forward recompute runs through the
// step's discrete decisions (seam wraps, the new face) and the new position, whose adjoint terms
// are taken at once; the reverse of the polarity and velocity update then recomputes what it
// needs from the step's inputs, read again (L1/L2 hits), rather than keeping the forward's
// intermediates live (or spilled) across the wrap and the location: FP32 spills 180/356 -> 60/52
// bytes per thread at 6 blocks per SM, forward+adjoint +1.5% on the 512-replica bumpy-sphere
// ensemble, the results unchanged.
template <typename real>
__global__ void __launch_bounds__(kAdjThreads, (sizeof(real) == 4 ? 6 : 2)) k_adj_a(const AdjArgs<real> a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.N) return;
    const int t = *a.t0 + a.j;
    real cd, sd, u01 = (real)0.5, ub2x, ub2y, thb2, vb[3] = {0, 0, 0};
    {
        const R4<real> PL = a.pol[q];
        const R2<real> U = a.uv[q];
        const int id = a.ids[q];
        const int rep = (int)((unsigned)id >> a.local_bits);
        const unsigned local = (unsigned)id & ((1u << a.local_bits) - 1u);
        const RepParams<real>& rp = a.reps[rep];
        const int gid = rp.off + (int)local;
        const int f = real_to_face(PL.w);
        const real* g = a.rec + (size_t)f * kRec;

        // ---- forward recompute (the arithmetic of k_step), from the stored pair sums ----
        const R4<real> sf = a.sum_f[q];
        const R2<real> sm = a.sum_m[q];
        const real p[3] = {PL.x, PL.y, PL.z};
        const real F[3] = {sf.x, sf.y, sf.z};
        const real m[3] = {sf.w, sm.x, sm.y};
        real n[3], Jp[6];
        face_frame(g, n, Jp);
        const real Fn = dot(F, n);
        const real FT[3] = {F[0] - Fn * n[0], F[1] - Fn * n[1], F[2] - Fn * n[2]};
        real v[3];
        if (rp.force_mode == 0) {
            for (int k = 0; k < 3; ++k) v[k] = rp.v0 * p[k] + rp.mu * FT[k];
        } else {
            const real t2 = dot(FT, FT);
            const real FTn = t2 > (real)0 ? t2 * d_rsqrt(t2) : (real)0;
            const real sp = rp.v0 + FTn;
            for (int k = 0; k < 3; ++k) v[k] = sp * p[k];
        }
        const real vn2 = dot(v, v), mn2 = dot(m, m);
        const real ivn = vn2 > (real)0 ? d_rsqrt(vn2) : (real)0;
        const real imn = mn2 > (real)0 ? d_rsqrt(mn2) : (real)0;
        real pxv[3], pxm[3];
        cross(p, v, pxv);
        cross(p, m, pxm);
        const real A1 = dot(pxv, n), B1 = dot(pxm, n);
        const real omega = A1 * ivn * rp.inv_tau + rp.align * B1 * imn;
        real xi;
        if (a.noise) {
            xi = a.noise[gid];
        } else {
            const unsigned bits = tdsr::noise_bits24(a.seed, a.step0 + t, local, (unsigned)rep);
            u01 = (real)bits * (real)(1.0 / 16777216.0);
            xi = rp.eta * (u01 - (real)0.5);
        }
        const real delta = rp.dt * omega + xi;
        d_sincos(delta, &sd, &cd);
        real np[3];
        cross(n, p, np);
        const real p2[3] = {cd * p[0] + sd * np[0], cd * p[1] + sd * np[1], cd * p[2] + sd * np[2]};
        const real w0 = Jp[0] * p2[0] + Jp[1] * p2[1] + Jp[2] * p2[2];
        const real w1 = Jp[3] * p2[0] + Jp[4] * p2[1] + Jp[5] * p2[2];
        const real vu = Jp[0] * v[0] + Jp[1] * v[1] + Jp[2] * v[2];
        const real vv = Jp[3] * v[0] + Jp[4] * v[1] + Jp[5] * v[2];
        const real u2 = U.x + rp.dt * vu, v2 = U.y + rp.dt * vv;
        real ex = u2, ey = v2, tvu = vu, tvv = vv, tw0 = w0, tw1 = w1;
        int nw = 0;
        seam_wrap(U.x, U.y, ex, ey, tvu, tvv, tw0, tw1, nw);
        // linear part of the composed gluing maps: the same wrap applied to the unit vectors
        real R00 = 1, R10 = 0, R01 = 0, R11 = 1;
        if (nw > 0) {
            real ex2 = u2, ey2 = v2;
            int nw2 = 0;
            seam_wrap(U.x, U.y, ex2, ey2, R00, R10, R01, R11, nw2);
        }
        int mode = 0;
        const int f2 = locate(a.rec, a.adj, a.G, a.bin_start, a.bin_faces, ex, ey, f, mode);
        const real* h = a.rec + (size_t)f2 * kRec;
        real r2[3];
        face_map(h, ex, ey, r2[0], r2[1], r2[2]);

        // ---- reverse of the new position's terms ----
        const R4<real> lin = reinterpret_cast<const R4<real>*>(a.lam[(a.T - 1 - t) & 1])[gid];
        real ub3x = lin.x, ub3y = lin.y;
        thb2 = lin.z;
        real rb2[3] = {0, 0, 0};
        if (a.r_target && t == a.T - 1) {
            const real s = (real)(2.0 * a.w_pos) * (real)rp.inv_n;
            for (int k = 0; k < 3; ++k) rb2[k] += s * (r2[k] - (real)a.r_target[3 * (size_t)gid + k]);
        }
        if (a.phib) {
            // phi = |S| / N_r with S = sum_i normalize((r2_i - c) x v_i); dL/dS per replica (k_adj_phib)
            const R4<real> sb = a.phib[(size_t)t * a.R + rep];
            const real rc3[3] = {r2[0] - a.cx, r2[1] - a.cy, r2[2] - a.cz};
            real L[3];
            cross(rc3, v, L);
            const real Ln2 = dot(L, L);
            if (sb.w > (real)0 && Ln2 > (real)0) {
                const real Sb[3] = {sb.x, sb.y, sb.z};
                const real iL = d_rsqrt(Ln2);
                const real ell[3] = {L[0] * iL, L[1] * iL, L[2] * iL};
                const real se = dot(Sb, ell);
                const real Lb[3] = {(Sb[0] - se * ell[0]) * iL, (Sb[1] - se * ell[1]) * iL,
                                    (Sb[2] - se * ell[2]) * iL};
                real t1[3], t2[3];
                cross(v, Lb, t1);    // rc3bar = v x Lbar
                cross(Lb, rc3, t2);  // vbar  += Lbar x rc
                for (int k = 0; k < 3; ++k) rb2[k] += t1[k], vb[k] += t2[k];
            }
        }
        // r2 = A' + J' (uv3 - a')
        const R4<real> h2 = rq(h, 2), h3 = rq(h, 3);
        ub3x += h2.x * rb2[0] + h2.y * rb2[1] + h2.z * rb2[2];
        ub3y += h2.w * rb2[0] + h3.x * rb2[1] + h3.y * rb2[2];
        // uv3 = R uv2 + t
        ub2x = R00 * ub3x + R10 * ub3y, ub2y = R01 * ub3x + R11 * ub3y;
    }

    // ---- reverse of the polarity and velocity update, on values recomputed from the inputs ----
    const R4<real> PL = reload(a.pol, q);
    const int id = reload(a.ids, q);
    const RepParams<real>& rp = a.reps[(unsigned)id >> a.local_bits];
    const real* g = a.rec + (size_t)real_to_face(PL.w) * kRec;
    asm volatile("" : "+l"(g));
    const real p[3] = {PL.x, PL.y, PL.z};
    real n[3];
    real vbv[3], p2b[3];
    {
        real Jp[6];
        face_frame(g, n, Jp);
        real np[3];
        cross(n, p, np);
        const real p2[3] = {cd * p[0] + sd * np[0], cd * p[1] + sd * np[1], cd * p[2] + sd * np[2]};
        const real w0 = Jp[0] * p2[0] + Jp[1] * p2[1] + Jp[2] * p2[2];
        const real w1 = Jp[3] * p2[0] + Jp[4] * p2[1] + Jp[5] * p2[2];
        // uv2 = uv + dt (Jp v)
        const real velbx = rp.dt * ub2x, velby = rp.dt * ub2y;
        for (int k = 0; k < 3; ++k) vbv[k] = Jp[k] * velbx + Jp[3 + k] * velby;
        // theta2 = atan2(w1, w0) + const (the gluing rotations only add constants)
        const real iw2 = (real)1 / (w0 * w0 + w1 * w1);
        const real wb0 = -w1 * iw2 * thb2, wb1 = w0 * iw2 * thb2;
        // w = Jp p2
        for (int k = 0; k < 3; ++k) p2b[k] = Jp[k] * wb0 + Jp[3 + k] * wb1;
    }
    for (int k = 0; k < 3; ++k) vb[k] += vbv[k];
    // p2 = cos(delta) p + sin(delta) (n x p)
    real deltab, pb[3];
    {
        real np[3];
        cross(n, p, np);
        deltab = p2b[0] * (cd * np[0] - sd * p[0]) + p2b[1] * (cd * np[1] - sd * p[1]) +
                 p2b[2] * (cd * np[2] - sd * p[2]);
        real p2bxn[3];
        cross(p2b, n, p2bxn);
        for (int k = 0; k < 3; ++k) pb[k] = cd * p2b[k] + sd * p2bxn[k];
    }
    // delta = dt omega + eta (u - 1/2)
    const real omegab = rp.dt * deltab;
    // parameter terms in the working precision (GB300 runs FP64 at a small fraction of the FP32 rate)
    real gv0 = 0, gmu = 0, gtau = 0, galign = 0, geta = 0;
    if (!a.noise) geta = deltab * (u01 - (real)0.5);
    // the stored pair sums, read again
    const R4<real> sf = reload(a.sum_f, q);
    const R2<real> sm = reload(a.sum_m, q);
    const real F[3] = {sf.x, sf.y, sf.z}, m[3] = {sf.w, sm.x, sm.y};
    const real Fn = dot(F, n);
    const real FT[3] = {F[0] - Fn * n[0], F[1] - Fn * n[1], F[2] - Fn * n[2]};
    real v[3], sp = (real)0, FTn = (real)0;
    if (rp.force_mode == 0) {
        for (int k = 0; k < 3; ++k) v[k] = rp.v0 * p[k] + rp.mu * FT[k];
    } else {
        const real t2 = dot(FT, FT);
        FTn = t2 > (real)0 ? t2 * d_rsqrt(t2) : (real)0;
        sp = rp.v0 + FTn;
        for (int k = 0; k < 3; ++k) v[k] = sp * p[k];
    }
    real mb[3] = {0, 0, 0};
    real nxp[3];
    cross(n, p, nxp);
    const real vn2 = dot(v, v);
    if (vn2 > (real)0) {
        // omega_1 = A1 / (|v| tau), A1 = p . (v x n)
        const real ivn = d_rsqrt(vn2);
        real pxv[3];
        cross(p, v, pxv);
        const real A1 = dot(pxv, n);
        const real A1b = omegab * ivn * rp.inv_tau;
        const real vnb = -A1 * ivn * ivn * rp.inv_tau * omegab;
        gtau += -A1 * ivn * rp.inv_tau * rp.inv_tau * omegab;
        real vxn[3];
        cross(v, n, vxn);
        for (int k = 0; k < 3; ++k) pb[k] += A1b * vxn[k], vb[k] += A1b * nxp[k] + vnb * v[k] * ivn;
    }
    const real mn2 = dot(m, m);
    if (mn2 > (real)0) {
        // omega_2 = align B1 / |m|, B1 = p . (m x n)
        const real imn = d_rsqrt(mn2);
        real pxm[3];
        cross(p, m, pxm);
        const real B1 = dot(pxm, n);
        const real B1b = rp.align * omegab * imn;
        const real mnb = -rp.align * B1 * imn * imn * omegab;
        galign += B1 * imn * omegab;
        real mxn[3];
        cross(m, n, mxn);
        for (int k = 0; k < 3; ++k) pb[k] += B1b * mxn[k], mb[k] += B1b * nxp[k] + mnb * m[k] * imn;
    }
    real FTb[3];
    if (rp.force_mode == 0) {
        // v = v0 p + mu FT
        gv0 += dot(vb, p);
        gmu += dot(vb, FT);
        for (int k = 0; k < 3; ++k) pb[k] += rp.v0 * vb[k], FTb[k] = rp.mu * vb[k];
    } else {
        // v = (v0 + |FT|) p
        const real spb = dot(vb, p);
        gv0 += spb;
        const real s = FTn > (real)0 ? spb / FTn : (real)0;
        for (int k = 0; k < 3; ++k) pb[k] += sp * vb[k], FTb[k] = s * FT[k];
    }
    // FT = F - (F . n) n
    const real Fbn = dot(FTb, n);
    R4<real> oF, oM, oP;
    oF.x = FTb[0] - Fbn * n[0], oF.y = FTb[1] - Fbn * n[1], oF.z = FTb[2] - Fbn * n[2], oF.w = ub2x;
    oM.x = mb[0], oM.y = mb[1], oM.z = mb[2], oM.w = ub2y;
    oP.x = pb[0], oP.y = pb[1], oP.z = pb[2], oP.w = (real)0;
    a.aF[q] = oF;
    a.aM[q] = oM;
    a.aP[q] = oP;
    // by slot: the slots of a replica are the same range in every step's order, so the sums over
    // that range are the replica's (coalesced, where an index by particle was a random access:
    // forward+adjoint 2.99e9 -> 3.40e9 particle-steps/s on the 512-replica bumpy-sphere ensemble)
    real* gp = a.gpar + q;
    const size_t N = (size_t)a.N;
    gp[G_V0 * N] += gv0;
    gp[G_MU * N] += gmu;
    gp[G_TAU * N] += gtau;
    gp[G_ALIGN * N] += galign;
    gp[G_ETA * N] += geta;
}

template <typename real, int LPP>
__global__ void __launch_bounds__(kAdjThreads, (sizeof(real) == 4 ? 5 : 3)) k_adj_b(const AdjArgs<real> a) {
    const int q0 = (int)((blockIdx.x * blockDim.x + threadIdx.x) / LPP);
    const int sub = LPP > 1 ? (int)(threadIdx.x % LPP) : 0;
    if (LPP == 1 && q0 >= a.N) return;
    // with several lanes per particle, the lanes of a particle past the end stay for the group sums
    const bool active = q0 < a.N;
    const int q = active ? q0 : a.N - 1;
    const R4<real> P = a.pos[q];
    const R4<real> PL = a.pol[q];
    const int id = a.ids[q];
    const int rep = (int)((unsigned)id >> a.local_bits);
    const unsigned local = (unsigned)id & ((1u << a.local_bits) - 1u);
    const RepParams<real>& rp = a.reps[rep];
    const int gid = rp.off + (int)local;
    const int f = real_to_face(PL.w);
    const real* g = a.rec + (size_t)f * kRec;
    const R4<real> myF = a.aF[q], myM = a.aM[q], myP = a.aP[q];

    __shared__ int2 s_run[9 * kAdjThreads];
    int2* run = s_run + threadIdx.x;
    const int total = candidate_runs(rp, a.desc, a.start, a.key[q], run);
    real rb[3] = {0, 0, 0}, msum[3] = {0, 0, 0};
    real gk = 0, gkadh = 0;  // the particle's few pair terms, summed in the working precision
    const real inv_w = rp.inv_adh_w;
    // one neighbour's terms (candidate order, as the forward adds them)
    auto nbr_term = [&](int t, const R4<real>& Q) {
        const real dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
        const real d2 = pair_d2(P, Q);
        const R4<real> Fj = a.aF[t], Mj = a.aM[t];
        msum[0] += Mj.x, msum[1] += Mj.y, msum[2] += Mj.z;
        if (d2 > (real)0) {
            const real rd = d_rsqrt(d2);
            const real d = d2 * rd;
            const bool rep_branch = d < rp.twoR;
            const real fm = rep_branch ? rp.k * (rp.twoR - d) * rp.inv_twoR : -(rp.adh_scale * (d - rp.twoR));
            const real fp = rep_branch ? -rp.k * rp.inv_twoR : -rp.adh_scale;
            const real e[3] = {dx * rd, dy * rd, dz * rd};
            const real D[3] = {myF.x - Fj.x, myF.y - Fj.y, myF.z - Fj.z};
            const real eD = dot(e, D);
            const real fd = fm * rd;
            for (int k = 0; k < 3; ++k) rb[k] += fd * D[k] + (fp - fd) * eD * e[k];
            const real Fe = myF.x * e[0] + myF.y * e[1] + myF.z * e[2];
            if (rep_branch)
                gk += Fe * (rp.twoR - d) * rp.inv_twoR;
            else
                gkadh += -Fe * (d - rp.twoR) * inv_w;
        }
    };
    if (LPP > 1) {
        // lane `sub` takes the candidates sub, sub + LPP, ... of the visiting order; the group's
        // partial sums are added with a fixed butterfly below
        const int mine = total > sub ? (total - sub + LPP - 1) / LPP : 0;
        const int2* sp = run;
        int t = 0, left = 0;
        if (total > 0) {
            const int2 x0 = *sp;
            t = x0.x, left = x0.y;
        }
        int skip = sub;
        for (int i = 0; i < mine; ++i) {
            while (skip >= left) {
                skip -= left;
                sp += kAdjThreads;
                const int2 x = *sp;
                t = x.x, left = x.y;
            }
            t += skip, left -= skip;
            const int tj = t++;
            --left;
            skip = LPP - 1;
            const R4<real> Q = a.pos[tj];
            if (pair_d2(P, Q) < rp.r_max2 && tj != q) nbr_term(tj, Q);
        }
        const unsigned gm = ((1u << LPP) - 1u) << ((threadIdx.x & 31) & ~(unsigned)(LPP - 1));
#pragma unroll
        for (int o = 1; o < LPP; o <<= 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                rb[k] += __shfl_xor_sync(gm, rb[k], o);
                msum[k] += __shfl_xor_sync(gm, msum[k], o);
            }
            gk += __shfl_xor_sync(gm, gk, o);
            gkadh += __shfl_xor_sync(gm, gkadh, o);
        }
        if (sub != 0 || !active) return;
    } else if (total > 0) {
        // two candidates per iteration: both distance tests (the forward's neighbour test, rounded
        // the same way) before either neighbour's terms
        const int2* sp = run;
        int2 x0 = *sp;
        int t = x0.x, left = x0.y;
        for (int rem = total; rem > 0; rem -= 2) {
            if (left == 0) {
                sp += kAdjThreads;
                const int2 x = *sp;
                t = x.x, left = x.y;
            }
            const int ta = t++;
            --left;
            int tb = ta;
            if (rem > 1) {
                if (left == 0) {
                    sp += kAdjThreads;
                    const int2 x = *sp;
                    t = x.x, left = x.y;
                }
                tb = t++;
                --left;
            }
            const R4<real> Qa = a.pos[ta], Qb = a.pos[tb];
            const bool na = pair_d2(P, Qa) < rp.r_max2 && ta != q;
            const bool nb = rem > 1 && pair_d2(P, Qb) < rp.r_max2 && tb != q;
            if (na) nbr_term(ta, Qa);
            if (nb) nbr_term(tb, Qb);
        }
    }
    // r = A + J (uv - a)
    const R4<real> g2 = rq(g, 2), g3 = rq(g, 3);
    const real Ju[3] = {g2.x, g2.y, g2.z}, Jv[3] = {g2.w, g3.x, g3.y};
    const real ubx = myF.w + Ju[0] * rb[0] + Ju[1] * rb[1] + Ju[2] * rb[2];
    const real uby = myM.w + Jv[0] * rb[0] + Jv[1] * rb[1] + Jv[2] * rb[2];
    // p = normalize(J (cos th, sin th))
    const real pbt[3] = {myP.x + msum[0], myP.y + msum[1], myP.z + msum[2]};
    real sn, cs;
    d_sincos(P.w, &sn, &cs);
    const real qv[3] = {Ju[0] * cs + Jv[0] * sn, Ju[1] * cs + Jv[1] * sn, Ju[2] * cs + Jv[2] * sn};
    const real iq = d_rsqrt(dot(qv, qv));
    const real pp[3] = {qv[0] * iq, qv[1] * iq, qv[2] * iq};
    const real pq = dot(pbt, pp);
    const real qb[3] = {(pbt[0] - pq * pp[0]) * iq, (pbt[1] - pq * pp[1]) * iq, (pbt[2] - pq * pp[2]) * iq};
    const real cb0 = Ju[0] * qb[0] + Ju[1] * qb[1] + Ju[2] * qb[2];
    const real cb1 = Jv[0] * qb[0] + Jv[1] * qb[1] + Jv[2] * qb[2];
    R4<real> lo;
    lo.x = ubx, lo.y = uby, lo.z = -sn * cb0 + cs * cb1, lo.w = (real)0;
    reinterpret_cast<R4<real>*>(a.lam[(a.T - *a.t0 - a.j) & 1])[gid] = lo;
    real* gp = a.gpar + q;
    gp[G_KREP * (size_t)a.N] += gk;
    gp[G_KADH * (size_t)a.N] += gkadh;
}

// dL/dS of every stored step and replica, once per adjoint run: phi_t = |S_t| / N_r gives
// The first step of the segment whose reverse launches follow (read by k_adj_a / k_adj_b).
__global__ void k_adj_segment(int* t0, int v) { *t0 = v; }

// dL/dS = phibar_t / (N_r |S_t|) S_t (the FP64 square root and division once per replica and step,
// not once per particle); w = 1 when S_t != 0.
template <typename real>
__global__ void k_adj_phib(const double* phisum, const double* phibar, const RepParams<real>* reps, int R,
                           long long TR, R4<real>* out) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= TR) return;
    const int r = (int)(e % R);
    const double S0 = phisum[e * 6], S1 = phisum[e * 6 + 1], S2 = phisum[e * 6 + 2];
    const double Sn = sqrt(S0 * S0 + S1 * S1 + S2 * S2);
    R4<real> o;
    o.x = o.y = o.z = o.w = (real)0;
    if (Sn > 0) {
        const double c = phibar[e] * reps[r].inv_n / Sn;
        o.x = (real)(c * S0), o.y = (real)(c * S1), o.z = (real)(c * S2), o.w = (real)1;
    }
    out[e] = o;
}

// Position term of the loss per replica: sum over the replica's particles of |r_T - r*|^2 in FP64
// (the final state by slot: a replica's slots are off[r] .. off[r] + cnt[r] - 1; the target by
// particle index), in a fixed order (one block per replica, a fixed tree).
template <typename real>
__global__ void k_adj_pos_loss(const R4<real>* pos, const int* ids, const RepParams<real>* reps, int local_bits,
                               const double* tgt, const int* off, const int* cnt, double* out) {
    __shared__ double s[256];
    const int r = blockIdx.x;
    double acc = 0;
    for (int q = off[r] + threadIdx.x; q < off[r] + cnt[r]; q += 256) {
        const unsigned id = (unsigned)ids[q];
        const size_t gid = (size_t)(reps[id >> local_bits].off + (int)(id & ((1u << local_bits) - 1u)));
        const R4<real> P = pos[q];
        const double dx = (double)P.x - tgt[3 * gid], dy = (double)P.y - tgt[3 * gid + 1];
        const double dz = (double)P.z - tgt[3 * gid + 2];
        acc += dx * dx + dy * dy + dz * dz;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[r] = s[0];
}

// The adjoint of the initial state, (u, v, theta) padded to 4 reals by particle index, as the
// caller's double arrays: d_uv [2N], d_theta [N].
template <typename real>
__global__ void k_adj_out(const real* lam, double* d_uv, double* d_th, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const R4<real> l = reinterpret_cast<const R4<real>*>(lam)[i];
    d_uv[2 * (size_t)i] = (double)l.x, d_uv[2 * (size_t)i + 1] = (double)l.y;
    d_th[i] = (double)l.z;
}

// Per-replica sums of the per-slot parameter terms (replica r: slots off[r] .. off[r] + cnt[r] - 1),
// in a fixed order (one block per replica).
template <typename real>
__global__ void k_adj_reduce(const real* gpar, long long N, const int* off, const int* cnt, double* out) {
    __shared__ double s[256][kGPar];
    const int r = blockIdx.x;
    double acc[kGPar] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = off[r] + threadIdx.x; i < off[r] + cnt[r]; i += 256)
        for (int k = 0; k < kGPar; ++k) acc[k] += (double)gpar[(size_t)k * N + i];
    for (int k = 0; k < kGPar; ++k) s[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < kGPar; ++k) s[threadIdx.x][k] += s[threadIdx.x + w][k];
        __syncthreads();
    }
    if (threadIdx.x < kGPar) out[(size_t)r * kGPar + threadIdx.x] = s[0][threadIdx.x];
}

}  // namespace tdsk
