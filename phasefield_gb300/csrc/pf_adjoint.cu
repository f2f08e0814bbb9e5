// pf_adjoint.cu -- hand-written adjoint of the explicit time step (sm_103a).
//
// The calibration model is the compact four-slot step of the FP32 path
// (Phase_field_solver, solver.cpp:147-304, and the multiphase carbon diffusion
// with partitioning, solver.cpp:343-405), written here once for a real type R
// so that it runs in FP64 (the finite-difference reference) and in FP32 with
// FP64 reductions.  State per cell: 4 local grain ids, their phi, the 3 phase
// fractions, the total carbon.  (Mn does not enter the phase update or the
// carbon diffusion, so the gradients below do not depend on it.)
//
// Parameters: scale factors s = (mobility, interface energy, D_C, D_Mn) on
// m_ij, sigma_ij, D_C,p, D_Mn,p.  The time step and the sub-step count are
// those of s = 1 and are held fixed, so the step is a smooth function of s
// between discrete events.
//
// Objectives at the final time:  J0 = mean ferrite fraction (1/N) sum phi_1,
// J1 = mean austenite carbon  sum phi_2 c_2 / sum phi_2.
//
// Adjoint: the discrete decisions of every step (stencil list membership, the
// cutoff and unit clamps, the top-four choice) are recomputed from the stored
// pre-step state with the same code as the forward step and held fixed.  With
// lambda the adjoint of the state after a sweep:
// * diffusion sub-step (linear in C for fixed phase fractions):
//     lam_C(m) = lam(m) + sum_p D_p s_p(m)/t1_p(m) sum_nb s_p(nb) (lam(nb) - lam(m))
//   (the same stencil as the flux, with lambda in place of c), plus the
//   phase-fraction adjoint from s_p = sqrt(phi_p) and c_p(phi);
// * phase sweep: the normalisation and the pair terms are differentiated per
//   cell; the neighbour sums S_e = sum_nb phi_nb(e) are returned to the
//   neighbours' slots by a gather over the neighbours' published lists.
// Checkpoints every K steps; a segment is recomputed forward storing every
// step's pre-step state and the carbon after each diffusion sub-step, then
// swept backwards; the derived quantities (s_p, c_p, 1/t1_p) are recomputed
// from those where needed, which costs far less than storing and reloading
// them.  The reverse diffusion sub-steps of a step run as one cooperative
// launch with bounded grid barriers.  Full segments are replayed from one
// captured CUDA graph.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "pf_dev.cuh"
#include "pf_host.h"
#include "pf_kernels.h"

namespace {

constexpr int LMAX = PF_NSTENCIL;
constexpr int kCoopCells = 4;                              // cells per thread of the cooperative reverse diffusion
constexpr unsigned long long kCoopTimeoutNs = 2000000000ull;  // its barrier wait limit

template <typename R>
struct AP {
    int ix, iy, iz, nnb, n_sub, b1, b2;
    long long N;
    R cutoff;
    R A[9], B[9], G[9], E[9];  // dt*m*sigma*f1, dt*m*sigma*f2, dt*m*f3*entropy/dcdT, eq  (scaled)
    R D[3];                    // D_C,p * dt_sub/dx^2 (scaled)
    R k[9], c[9];              // carbon partition
    R s_m, s_s, s_c;           // the scales (for gradients of scaled terms)
};

__device__ __forceinline__ int lphase(int l, int b1, int b2) { return l == 0 ? 0 : (l <= b1 ? 1 : (l <= b2 ? 2 : 3)); }


// Sum of v over the block (blockDim.x == PF_CELL_THREADS), added to *dst by
// one atomic per block instead of one per warp (the gradient accumulators are
// a handful of doubles that every block of a launch hits).  Every thread of
// the block must call it.
__device__ __forceinline__ void block_add(double v, double *dst) {
    __shared__ double part[PF_CELL_THREADS / 32];
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    const int w = threadIdx.x >> 5;
    __syncthreads();  // part[] may still be read by a previous call
    if ((threadIdx.x & 31) == 0) part[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < PF_CELL_THREADS / 32; k++) t += part[k];
        if (t != 0) atomicAdd(dst, t);
    }
}

template <typename R>
__device__ __forceinline__ void partition(const AP<R> &P, R C, const R ph[3], R c[3], R t1[3]) {
    for (int i = 0; i < 3; i++) {
        R a = 0, b = 0;
        for (int j = 0; j < 3; j++) {
            a += ph[j] * P.k[i + 3 * j];
            b += ph[j] * P.c[i + 3 * j];
        }
        t1[i] = a;
        c[i] = (C - b) / a;
    }
}

// The per-cell stencil list of the phase sweep, with every decision.
template <typename R>
struct Lst {
    int num, bulk, kept;
    int id[LMAX], pe[LMAX], own[LMAX];
    R v1[LMAX], S[LMAX], draw[LMAX], d[LMAX];
    int perm[4];
    R sum;
    int oid[4];
    R ov[4];
    R ph_old[3], c[3], t1[3];
};

template <typename R>
__device__ void build_list(const AP<R> &P, int ci, int cj, int ck, long long n, const ushort4 *gid, const R *phi,
                           const R *C, Lst<R> &L) {
    long long nb[6];
    pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nb);
    const ushort4 g = gid[n];
    L.oid[0] = g.x; L.oid[1] = g.y; L.oid[2] = g.z; L.oid[3] = g.w;
    for (int a = 0; a < 4; a++) L.ov[a] = phi[4 * n + a];
    int num = 0;
    for (int a = 0; a < 4; a++)
        if (L.ov[a] > P.cutoff) {
            L.id[num] = L.oid[a]; L.v1[num] = L.ov[a]; L.S[num] = 0; L.own[num] = a;
            num++;
        }
    for (int b = 0; b < P.nnb; b++) {
        const long long m = nb[b];
        const ushort4 q = gid[m];
        const int qid[4] = {q.x, q.y, q.z, q.w};
        for (int a = 0; a < 4; a++) {
            const int t = qid[a];
            if (t == 0) break;
            const R v = phi[4 * m + a];
            int kk = 0;
            while (kk < num && L.id[kk] != t) kk++;
            if (kk < num) L.S[kk] += v;
            else if (num < LMAX) {
                L.id[num] = t; L.v1[num] = 0; L.S[num] = v; L.own[num] = -1;
                num++;
            }
        }
    }
    L.num = num;
    L.bulk = (num == 1);
    for (int e = 0; e < num; e++) L.pe[e] = lphase(L.id[e], P.b1, P.b2);
    for (int p = 0; p < 3; p++) L.ph_old[p] = 0;
    for (int a = 0; a < 4; a++) {
        const int p = lphase(L.oid[a], P.b1, P.b2);
        if (p > 0) L.ph_old[p - 1] += L.ov[a];
    }
    partition(P, C[n], L.ph_old, L.c, L.t1);
    if (L.bulk) return;
    for (int e = 0; e < num; e++) {
        R acc = 0;
        const int pe = L.pe[e];
        for (int f = 0; f < num; f++) {
            if (f == e) continue;
            const int x = (pe - 1) + 3 * (L.pe[f] - 1);
            const R X = L.S[e] * L.v1[f] - L.S[f] * L.v1[e];
            const R Y = L.v1[e] - L.v1[f];
            const R Z = sqrt(L.v1[e] * L.v1[f]);
            acc += P.A[x] * X + P.B[x] * Y + P.G[x] * Z * (L.c[pe - 1] - P.E[x]);
        }
        const R dr = L.v1[e] + acc;
        L.draw[e] = dr;
        L.d[e] = dr > (R)1 ? (R)1 : (dr < P.cutoff ? (R)0 : dr);
    }
    // Top four, first maximum wins (solver.cpp:426-432).
    int idx[LMAX];
    for (int e = 0; e < num; e++) idx[e] = e;
    L.kept = 0;
    L.sum = 0;
    for (int a = 0; a < 4; a++) {
        L.perm[a] = -1;
        if (a >= num) continue;
        int mx = a;
        for (int b = a + 1; b < num; b++)
            if (L.d[idx[b]] > L.d[idx[mx]]) mx = b;
        const int t = idx[a]; idx[a] = idx[mx]; idx[mx] = t;
        if (L.d[idx[a]] > P.cutoff) {
            L.perm[a] = idx[a];
            L.kept++;
            L.sum += L.d[idx[a]];
        }
    }
}

// ---------------------------------------------------------------- forward --
// Derived quantities of a step's diffusion.  With the phase fractions fixed
// over the step, s_p = sqrt(phi_p), 1/t1_p and t2_p (t1_p = sum_j phi_j k_pj,
// t2_p = sum_j phi_j c_pj) are computed once per step and kept as planes
// (DS: 9N values, planes s, 1/t1, t2 for p = 0..2); each sub-step then gets
// the partitioned carbon c_p = (C - t2_p) / t1_p as (C - t2_p) * (1/t1_p), a
// single multiply-add, forward and reverse alike.
template <typename R>
__device__ __forceinline__ void step_planes(const AP<R> &P, long long n, const R p[3], R *DS) {
    for (int i = 0; i < 3; i++) {
        R a = 0, b = 0;
        for (int j = 0; j < 3; j++) {
            a += p[j] * P.k[i + 3 * j];
            b += p[j] * P.c[i + 3 * j];
        }
        DS[i * P.N + n] = sqrt(p[i]);
        DS[(3 + i) * P.N + n] = (R)1 / a;
        DS[(6 + i) * P.N + n] = b;
    }
}
template <typename R>
__device__ __forceinline__ R cpart(const AP<R> &P, const R *DS, int p, long long n, R C) {
    return (C - DS[(6 + p) * P.N + n]) * DS[(3 + p) * P.N + n];
}

// Phase sweep; also writes the step's diffusion planes (step_planes) of the
// new phase fractions.
template <typename R>
__global__ void k_fwd_phase(const AP<R> P, int patch, const ushort4 *gid, const R *phi, const R *ph, const R *C,
                            ushort4 *gid2, R *phi2, R *ph2, R *DS) {
    int ci, cj, ck;
    long long n;
    if (!pf_cell_map(patch, P.ix, P.iy, P.iz, ci, cj, ck, n)) return;
    Lst<R> L;
    build_list(P, ci, cj, ck, n, gid, phi, C, L);
    if (L.bulk) {
        gid2[n] = gid[n];
        for (int a = 0; a < 4; a++) phi2[4 * n + a] = phi[4 * n + a];
        const R pp[3] = {ph[3 * n], ph[3 * n + 1], ph[3 * n + 2]};
        for (int p = 0; p < 3; p++) ph2[3 * n + p] = pp[p];
        step_planes(P, n, pp, DS);
        return;
    }
    const R inv = (R)1 / L.sum;
    int oid[4] = {0, 0, 0, 0};
    R q[3] = {0, 0, 0};
    for (int a = 0; a < 4; a++) {
        R v = 0;
        if (L.perm[a] >= 0) {
            const int e = L.perm[a];
            oid[a] = L.id[e];
            v = L.d[e] * inv;
            q[L.pe[e] - 1] += L.d[e];
        }
        phi2[4 * n + a] = v;
    }
    gid2[n] = make_ushort4((unsigned short)oid[0], (unsigned short)oid[1], (unsigned short)oid[2], (unsigned short)oid[3]);
    R pp[3];
    for (int p = 0; p < 3; p++) {
        pp[p] = q[p] * inv;
        ph2[3 * n + p] = pp[p];
    }
    step_planes(P, n, pp, DS);
}

// Forward sub-step (solver.cpp:343-372):
//   C' = C + sum_p s_p D_p sum_nb s_p^nb (c_p^nb - c_p),
// from the step's planes DS and C.  Cst, when given, receives a copy of C'
// (the reverse sweep's record of this sub-step).  Phases with D_p = 0
// contribute exactly zero and are skipped.
template <typename R>
__global__ void k_fwd_diffuse_d(const AP<R> P, const R *DS, const R *C, R *C2, R *Cst) {
    int ci, cj, ck;
    long long n;
    if (!pf_cell(P.ix, P.iy, ci, cj, ck, n)) return;
    long long nb[6];
    pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nb);
    const R C0 = C[n];
    R f = 0;
    for (int p = 0; p < 3; p++) {
        if (P.D[p] == (R)0) continue;
        const R c0 = cpart(P, DS, p, n, C0);
        R a = 0;
        // The diffusion sums carry no discrete decision: fused multiply-adds
        // are used explicitly (this file is otherwise built without contraction).
        for (int b = 0; b < P.nnb; b++) {
            const long long m = nb[b];
            a = fma(DS[p * P.N + m], cpart(P, DS, p, m, C[m]) - c0, a);
        }
        f = fma(DS[p * P.N + n] * P.D[p], a, f);
    }
    const R cn = C0 + f;
    C2[n] = cn;
    if (Cst) Cst[n] = cn;
}

// Reverse of one diffusion sub-step for cell n.  In: lam (adjoint of C after
// the sub-step; read through L2 when LCG, i.e. when other blocks of the same
// launch wrote it), the step's planes DS and the carbon Cin before the
// sub-step.  Returns the adjoint of C before the sub-step; adds the
// phase-fraction part (through s_p and c_p(phi)) to lph_add and s_C * dJ/ds_C
// to g (kept in the working precision per thread: FP64 arithmetic is scarce
// on GB300; the block sums are FP64).
template <typename R, bool LCG>
__device__ __forceinline__ R bwd_diffuse_cell(const AP<R> &P, long long n, const long long nb[6], const R *DS,
                                              const R *Cin, const R *lam, R lph_add[3], R &g) {
    auto ld = [&](const R *p) { return LCG ? __ldcg(p) : *p; };
    const R l0 = ld(lam + n);
    const R C0 = Cin[n];
    R out = l0, dL_ds[3], dL_dc[3], c0s[3], it0[3], s0s[3], flux = 0;
    for (int p = 0; p < 3; p++) {
        dL_ds[p] = dL_dc[p] = c0s[p] = it0[p] = s0s[p] = 0;
        if (P.D[p] == (R)0) continue;  // no flux, no derivative
        const R s0 = DS[p * P.N + n], c0 = cpart(P, DS, p, n, C0);
        R al = 0, ac = 0, ads = 0;
        for (int b = 0; b < P.nnb; b++) {
            const long long m = nb[b];
            const R sm = DS[p * P.N + m], dcm = cpart(P, DS, p, m, Cin[m]) - c0, lm = ld(lam + m);
            al = fma(sm, lm - l0, al);
            ac = fma(sm, dcm, ac);
            ads = fma(sm * dcm, l0 - lm, ads);
        }
        it0[p] = DS[(3 + p) * P.N + n];
        c0s[p] = c0;
        s0s[p] = s0;
        out = fma(P.D[p] * s0 * it0[p], al, out);
        dL_dc[p] = P.D[p] * s0 * al;
        dL_ds[p] = P.D[p] * ads;
        flux = fma(s0 * P.D[p], ac, flux);
    }
    for (int j = 0; j < 3; j++) {
        R v = 0;
        for (int p = 0; p < 3; p++)
            if (P.D[p] != (R)0) v += dL_dc[p] * (-(P.c[p + 3 * j] + c0s[p] * P.k[p + 3 * j]) * it0[p]);
        if (s0s[j] > (R)0) v += dL_ds[j] / ((R)2 * s0s[j]);
        lph_add[j] += v;
    }
    g = fma(l0, flux, g);
    return out;
}

// Reverse of one diffusion sub-step (one launch per sub-step).  Out: lam2,
// lph += the phase-fraction part, grad[2] += dJ/ds_C.
template <typename R>
__global__ void k_bwd_diffuse_d(const AP<R> P, const R *DS, const R *Cin, const R *lam, R *lam2, R *lph,
                                double *grad) {
    int ci, cj, ck;
    long long n;
    const bool in = pf_cell(P.ix, P.iy, ci, cj, ck, n);
    R g = 0;
    if (in) {
        long long nb[6];
        pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nb);
        R add[3] = {0, 0, 0};
        lam2[n] = bwd_diffuse_cell<R, false>(P, n, nb, DS, Cin, lam, add, g);
        for (int j = 0; j < 3; j++) lph[3 * n + j] += add[j];
    }
    block_add((double)g / (double)P.s_c, grad + 2);
}

__device__ __forceinline__ unsigned long long adj_globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier among all blocks of a cooperative launch (all resident).  The wait
// is bounded by a wall-clock limit: a block that waits longer sets *err, and
// every block leaves at its next barrier.  Returns false when leaving.
__device__ __forceinline__ bool adj_grid_barrier(unsigned long long *ctr, unsigned long long target, int *err,
                                                 unsigned long long timeout_ns) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1ull);
        const unsigned long long t0 = adj_globaltimer();
        int good = 1;
        while (true) {
            if (atomicAdd(ctr, 0ull) >= target) break;
            if (*(volatile int *)err) { good = 0; break; }
            if (adj_globaltimer() - t0 > timeout_ns) {
                atomicExch(err, 1);
                good = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// gather_cell (the neighbour part of the reverse phase sweep) is defined below.
template <typename R>
__device__ __forceinline__ void gather_cell(const AP<R> &P, long long m, const long long nb[6], const ushort4 *gid,
                                            const int *pub_id, const R *pub_l, R *lphi_pre);

// All n_sub reverse diffusion sub-steps of one step in one cooperative
// launch: each thread keeps up to CPT cells (grid-stride), their phase-fraction
// adjoints accumulate in registers across the sub-steps, and the sub-steps are
// separated by a grid barrier.  lam starts in lamA; the result lands in lamA
// for an even n_sub, lamB for an odd one (as with one launch per sub-step).
// The carbon before sub-step k is C0 (k = 0) or Csub + N (k - 1).
// With gat_gid != NULL the launch first completes the neighbour part of the
// previous reverse step's phase sweep (gather_cell into gat_lphi): it touches
// other data than the diffusion, so it needs no barrier.
template <typename R, int CPT>
__global__ void __launch_bounds__(PF_CELL_THREADS) k_bwd_diffuse_all(const AP<R> P, const R *DS, const R *C0,
                                                                     const R *Csub, R *lamA, R *lamB, R *lph,
                                                                     double *grad, unsigned long long *ctr, int *err,
                                                                     unsigned long long timeout_ns,
                                                                     const ushort4 *gat_gid, const int *pub_id,
                                                                     const R *pub_l, R *gat_lphi) {
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gat_gid)
        for (int c = 0; c < CPT; c++) {
            const long long n = t + c * T;
            if (n < P.N) {
                const int plane = P.ix * P.iy;
                const int ck = (int)(n / plane), rem = (int)(n - (long long)ck * plane);
                const int cj = rem / P.ix, ci = rem - cj * P.ix;
                long long nb[6];
                pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nb);
                gather_cell(P, n, nb, gat_gid, pub_id, pub_l, gat_lphi);
            }
        }
    R add[CPT][3];
    for (int c = 0; c < CPT; c++) add[c][0] = add[c][1] = add[c][2] = 0;
    R g = 0;
    R *lin = lamA, *lout = lamB;
    unsigned long long target = 0;
    bool alive = true;
    for (int k = P.n_sub - 1; k >= 0 && alive; k--) {
        const R *Cin = k == 0 ? C0 : Csub + (size_t)P.N * (k - 1);
        for (int c = 0; c < CPT; c++) {
            const long long n = t + c * T;
            if (n < P.N) {
                const int plane = P.ix * P.iy;
                const int ck = (int)(n / plane), rem = (int)(n - (long long)ck * plane);
                const int cj = rem / P.ix, ci = rem - cj * P.ix;
                long long nb[6];
                pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nb);
                lout[n] = bwd_diffuse_cell<R, true>(P, n, nb, DS, Cin, lin, add[c], g);
            }
        }
        R *tmp = lin; lin = lout; lout = tmp;
        if (k > 0) {
            target += gridDim.x;
            alive = adj_grid_barrier(ctr, target, err, timeout_ns);
        }
    }
    for (int c = 0; c < CPT; c++) {
        const long long n = t + c * T;
        if (n < P.N)
            for (int j = 0; j < 3; j++) lph[3 * n + j] += add[c][j];
    }
    block_add((double)g / (double)P.s_c, grad + 2);
}

// Objective sums in FP64: out[0] = sum phi_1, out[1] = sum phi_2, out[2] = sum phi_2 c_2.
template <typename R>
__global__ void k_objective_sums(const AP<R> P, const R *ph, const R *C, double *out) {
    double a = 0, b = 0, cc = 0;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < P.N; n += (long long)gridDim.x * blockDim.x) {
        const R p[3] = {ph[3 * n], ph[3 * n + 1], ph[3 * n + 2]};
        R c[3], t[3];
        partition(P, C[n], p, c, t);
        a += (double)p[0];
        b += (double)p[1];
        cc += (double)p[1] * (double)c[1];
    }
    for (int s = 16; s > 0; s >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, s);
        b += __shfl_down_sync(0xffffffffu, b, s);
        cc += __shfl_down_sync(0xffffffffu, cc, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, a);
        atomicAdd(out + 1, b);
        atomicAdd(out + 2, cc);
    }
}

// ---------------------------------------------------------------- adjoint --
// Seed at the final state.  obj 0: J = sum phi_1 / N.  obj 1: J = sum phi_2 c_2 / W.
template <typename R>
__global__ void k_seed(const AP<R> P, int obj, const R *ph, const R *C, double W, double J, R *lph, R *lC, R *lphi) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.N) return;
    for (int a = 0; a < 4; a++) lphi[4 * n + a] = 0;
    if (obj == 0) {
        lph[3 * n] = (R)(1.0 / (double)P.N);
        lph[3 * n + 1] = 0;
        lph[3 * n + 2] = 0;
        lC[n] = 0;
        return;
    }
    const R p[3] = {ph[3 * n], ph[3 * n + 1], ph[3 * n + 2]};
    R c[3], t[3];
    partition(P, C[n], p, c, t);
    const R iw = (R)(1.0 / W);
    lC[n] = p[1] / t[1] * iw;
    for (int j = 0; j < 3; j++) {
        const R dc = -(P.c[1 + 3 * j] + c[1] * P.k[1 + 3 * j]) / t[1];  // dc_2/dphi_j
        R v = p[1] * dc;
        if (j == 1) v += c[1] - (R)J;
        lph[3 * n + j] = v * iw;
    }
}

// Reverse of the phase sweep, own-cell part.  In: pre-step state, lam_phi /
// lam_ph of the post-sweep state, lam_C (adjoint of C after the sweep, which
// the sweep does not change).  Out: lam_phi_pre (own part), lam_ph_pre,
// lam_C += driving-force part, the published neighbour-sum adjoints (ids, lS),
// grad[0..1] += dJ/ds_m, dJ/ds_sigma.
template <typename R>
__global__ void k_bwd_phase_own(const AP<R> P, int patch, const ushort4 *gid, const R *phi, const R *ph_pre,
                                const R *C, const R *lphi_post, const R *lph_post, R *lC, R *lphi_pre, R *lph_pre,
                                int *pub_id, R *pub_l, double *grad) {
    int ci, cj, ck;
    long long n;
    const bool in = pf_cell_map(patch, P.ix, P.iy, P.iz, ci, cj, ck, n);
    R gm = 0, gs = 0;  // s_m dJ/ds_m and s_sigma dJ/ds_sigma of this cell
    if (in) {
        Lst<R> L;
        build_list(P, ci, cj, ck, n, gid, phi, C, L);
        pub_id[LMAX * n] = 0;  // empty published list unless the cell is an interface cell
        if (L.bulk) {
            for (int a = 0; a < 4; a++) lphi_pre[4 * n + a] = lphi_post[4 * n + a];
            for (int p = 0; p < 3; p++) lph_pre[3 * n + p] = lph_post[3 * n + p];
        } else {
            for (int p = 0; p < 3; p++) lph_pre[3 * n + p] = 0;
            // Normalisation: phi'_a = d_perm(a)/D, ph'_p = sum_{a in p} d/D.
            const R D = L.sum, inv = (R)1 / D;
            R mu = 0;
            for (int a = 0; a < 4; a++)
                if (L.perm[a] >= 0) {
                    const int e = L.perm[a];
                    mu += lphi_post[4 * n + a] * L.d[e] * inv;
                }
            R q[3] = {0, 0, 0};
            for (int a = 0; a < 4; a++)
                if (L.perm[a] >= 0) q[L.pe[L.perm[a]] - 1] += L.d[L.perm[a]];
            for (int p = 0; p < 3; p++) mu += lph_post[3 * n + p] * q[p] * inv;
            mu *= inv;
            R ld[LMAX];
            for (int e = 0; e < L.num; e++) ld[e] = 0;
            for (int a = 0; a < 4; a++)
                if (L.perm[a] >= 0) {
                    const int e = L.perm[a];
                    ld[e] = (lphi_post[4 * n + a] + lph_post[3 * n + L.pe[e] - 1]) * inv - mu;
                }
            // Clamps: only values strictly inside [cutoff, 1] carry a derivative.
            for (int e = 0; e < L.num; e++)
                if (L.draw[e] > (R)1 || L.draw[e] < P.cutoff) ld[e] = 0;
            // Pair terms.
            R lv1[LMAX], lS[LMAX], lc[3] = {0, 0, 0};
            for (int e = 0; e < L.num; e++) { lv1[e] = ld[e]; lS[e] = 0; }
            for (int e = 0; e < L.num; e++) {
                if (ld[e] == (R)0) continue;
                const int pe = L.pe[e];
                for (int f = 0; f < L.num; f++) {
                    if (f == e) continue;
                    const int x = (pe - 1) + 3 * (L.pe[f] - 1);
                    const R X = L.S[e] * L.v1[f] - L.S[f] * L.v1[e];
                    const R Y = L.v1[e] - L.v1[f];
                    const R Z = sqrt(L.v1[e] * L.v1[f]);
                    const R Q = L.c[pe - 1] - P.E[x];
                    const R le = ld[e];
                    lS[e] += le * P.A[x] * L.v1[f];
                    lS[f] -= le * P.A[x] * L.v1[e];
                    R dZe = 0, dZf = 0;
                    if (Z > (R)0) {
                        dZe = L.v1[f] / ((R)2 * Z);
                        dZf = L.v1[e] / ((R)2 * Z);
                    }
                    lv1[e] += le * (-P.A[x] * L.S[f] + P.B[x] + P.G[x] * Q * dZe);
                    lv1[f] += le * (P.A[x] * L.S[e] - P.B[x] + P.G[x] * Q * dZf);
                    lc[pe - 1] += le * P.G[x] * Z;
                    const R T = P.A[x] * X + P.B[x] * Y + P.G[x] * Z * Q;
                    gm = fma(le, T, gm);
                    gs = fma(le, P.A[x] * X + P.B[x] * Y, gs);
                }
            }
            // Carbon partition of the driving force: c_p(C, ph_old).
            R lpo[3] = {0, 0, 0};
            R addC = 0;
            for (int p = 0; p < 3; p++) {
                addC += lc[p] / L.t1[p];
                for (int j = 0; j < 3; j++) lpo[j] += lc[p] * (-(P.c[p + 3 * j] + L.c[p] * P.k[p + 3 * j]) / L.t1[p]);
            }
            lC[n] += addC;
            // Own slots: v1 (entries from own slots) and ph_old (all own slots).
            R lo[4] = {0, 0, 0, 0};
            for (int e = 0; e < L.num; e++)
                if (L.own[e] >= 0) lo[L.own[e]] += lv1[e];
            for (int a = 0; a < 4; a++) {
                const int p = lphase(L.oid[a], P.b1, P.b2);
                if (p > 0) lo[a] += lpo[p - 1];
                lphi_pre[4 * n + a] = lo[a];
            }
            for (int e = 0; e < L.num; e++) {
                pub_id[LMAX * n + e] = L.id[e];
                pub_l[LMAX * n + e] = lS[e];
            }
            if (L.num < LMAX) pub_id[LMAX * n + L.num] = 0;  // terminator (the gather stops at id 0)
        }
    }
    block_add((double)gm / (double)P.s_m, grad + 0);
    block_add((double)gs / (double)P.s_s, grad + 1);
}

// Reverse of the phase sweep, neighbour part: every slot of cell m that its
// neighbours scanned (up to the first empty slot) receives the neighbours'
// published adjoint of their stencil sum for that grain.
template <typename R>
__device__ __forceinline__ void gather_cell(const AP<R> &P, long long m, const long long nb[6], const ushort4 *gid,
                                            const int *pub_id, const R *pub_l, R *lphi_pre) {
    const ushort4 g = gid[m];
    const int id[4] = {g.x, g.y, g.z, g.w};
    R add[4] = {0, 0, 0, 0};
    for (int b = 0; b < P.nnb; b++) {
        const long long n = nb[b];
        for (int a = 0; a < 4; a++) {
            if (id[a] == 0) break;
            for (int e = 0; e < LMAX; e++) {
                const int t = pub_id[LMAX * n + e];
                if (t == 0) break;
                if (t == id[a]) { add[a] += pub_l[LMAX * n + e]; break; }
            }
        }
    }
    for (int a = 0; a < 4; a++) lphi_pre[4 * m + a] += add[a];
}

template <typename R>
__global__ void k_bwd_phase_gather(const AP<R> P, const ushort4 *gid, const int *pub_id, const R *pub_l, R *lphi_pre) {
    int ci, cj, ck;
    long long m;
    if (!pf_cell(P.ix, P.iy, ci, cj, ck, m)) return;
    long long nb[6];
    pf_neighbours3(ci, cj, ck, m, P.ix, P.iy, P.iz, nb);
    gather_cell(P, m, nb, gid, pub_id, pub_l, lphi_pre);
}

// Reference layout -> calibration layout (carbon only; at most 4 slots kept).
template <typename R>
__global__ void k_adj_pack(long long N, pf_f32_map map, const int *ids64, const double *phi64, const double *phase64,
                           const double *C64, ushort4 *gid, R *phi, R *ph, R *C) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    int l[4];
    for (int a = 0; a < 4; a++) {
        const int id = ids64[6 * n + a];
        int v = 0;
        if (id > 0) {
            const int c = id / PF_MAXGRAIN_PER_PHASE;
            v = map.off[c] + (id - c * PF_MAXGRAIN_PER_PHASE) + (c > 0 ? 1 : 0);
        }
        l[a] = v;
        phi[4 * n + a] = (R)phi64[6 * n + a];
    }
    gid[n] = make_ushort4((unsigned short)l[0], (unsigned short)l[1], (unsigned short)l[2], (unsigned short)l[3]);
    for (int p = 0; p < 3; p++) ph[3 * n + p] = (R)phase64[3 * n + p];
    C[n] = (R)C64[n];
}

inline unsigned blocks(long long N) { return (unsigned)((N + 255) / 256); }

}  // namespace

// ============================================================== host side ==
struct pf_adj_impl {
    virtual ~pf_adj_impl() {}
};

template <typename R>
struct AdjCtx : pf_adj_impl {
    pf_model model;
    long long N = 0;
    int K = 100;
    cudaStream_t s = nullptr;
    double scales[4] = {1, 1, 1, 1};
    double t0 = 0;
    int nsteps = 0, n_sub = 1;
    AP<R> P{};
    // state buffers
    ushort4 *gid0 = nullptr;
    R *phi0 = nullptr, *ph0 = nullptr, *C0 = nullptr;        // uploaded initial state
    std::vector<ushort4 *> ck_gid;                            // checkpoints
    std::vector<R *> ck_phi, ck_ph, ck_C;
    // segment storage: per step pre-step state and pre-sub-step carbon
    std::vector<ushort4 *> sg_gid;
    std::vector<R *> sg_phi, sg_ph, sg_C, sg_Csub;  // sg_Csub: each step's diffusion record
    // Record mode (checkpoint_every = 0): the forward keeps every step's
    // record, slices of one arena, and the gradient only sweeps backwards.
    bool record = false;
    char *arena = nullptr;
    int arena_steps = 0;
    std::vector<ushort4 *> rg_gid;
    std::vector<R *> rg_phi, rg_ph, rg_C, rg_Csub;
    cudaGraphExec_t rec_fwd = nullptr, rec_bwd = nullptr;
    int rec_fwd_steps = -1, rec_bwd_steps = -1;
    R *rb_C = nullptr, *rb_phi = nullptr, *rb_ph = nullptr;  // adjoint buffer roles at the reverse capture
    R *dscr = nullptr;  // the step planes of a forward run without records (9N)
    ushort4 *w_gid = nullptr, *v_gid = nullptr;  // w_*, v_*: the forward's two state sets
    R *w_phi = nullptr, *w_ph = nullptr, *w_C = nullptr, *w_C2 = nullptr;
    R *v_phi = nullptr, *v_ph = nullptr, *v_C = nullptr;
    // adjoint buffers
    R *l_phi = nullptr, *l_ph = nullptr, *l_C = nullptr, *l_phi2 = nullptr, *l_ph2 = nullptr, *l_C2 = nullptr;
    int *pub_id = nullptr;
    R *pub_l = nullptr;
    double *d_acc = nullptr;  // 3 objective sums + 4 gradient components
    // Cooperative reverse diffusion (all sub-steps of a step in one launch):
    // barrier counter, error flag, resident-block capacity.
    unsigned long long *d_ctr = nullptr;
    int *d_err = nullptr;
    int coop_blocks = 0;
    double J[2] = {0, 0}, W = 0;
    double ms_fwd = 0, ms_bwd = 0;
    pf_f32_map map{};
    bool have_state = false, have_fwd = false;
    // Graphs of one full checkpoint segment: forward (per starting buffer set)
    // and recompute + reverse sweep.  Rebuilt whenever the parameters change.
    cudaGraphExec_t fwd_graph[2] = {nullptr, nullptr};
    cudaGraphExec_t seg_graph = nullptr;
    AP<R> gP{};  // parameters the graphs were captured with
    R *g_C = nullptr, *g_phi = nullptr, *g_ph = nullptr;  // adjoint buffer roles at capture
    const R *fin_ph = nullptr, *fin_C = nullptr;            // final state of the last forward run

    void drop_graphs() {
        for (auto &g : fwd_graph)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        if (seg_graph) { cudaGraphExecDestroy(seg_graph); seg_graph = nullptr; }
        if (rec_fwd) { cudaGraphExecDestroy(rec_fwd); rec_fwd = nullptr; }
        if (rec_bwd) { cudaGraphExecDestroy(rec_bwd); rec_bwd = nullptr; }
        rec_fwd_steps = rec_bwd_steps = -1;
    }

    // Bytes of one step's record: pre-step state and diffusion record, each
    // slice on a 256-byte boundary (vector loads).
    static size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }
    size_t record_step_bytes() const {
        const size_t n = (size_t)N;
        return up256(n * sizeof(ushort4)) + up256(4 * n * sizeof(R)) + up256(3 * n * sizeof(R)) +
               up256(n * sizeof(R)) + up256(record_size(n_sub, n) * sizeof(R));
    }
    // The arena for nsteps recorded steps (grown when needed; the graphs hold
    // its addresses, so growing drops them).
    bool ensure_arena(int nsteps) {
        if (arena && arena_steps >= nsteps) return true;
        drop_graphs();
        if (arena) cudaFree(arena);
        arena = nullptr;
        arena_steps = 0;
        rg_gid.clear(); rg_phi.clear(); rg_ph.clear(); rg_C.clear(); rg_Csub.clear();
        const size_t per = record_step_bytes();
        if (cudaMalloc((void **)&arena, per * (size_t)nsteps) != cudaSuccess) {
            cudaGetLastError();
            arena = nullptr;
            return false;
        }
        const size_t n = (size_t)N;
        for (int t = 0; t < nsteps; t++) {
            char *b = arena + per * (size_t)t;
            rg_gid.push_back((ushort4 *)b);
            b += up256(n * sizeof(ushort4));
            rg_phi.push_back((R *)b);
            b += up256(4 * n * sizeof(R));
            rg_ph.push_back((R *)b);
            b += up256(3 * n * sizeof(R));
            rg_C.push_back((R *)b);
            b += up256(n * sizeof(R));
            rg_Csub.push_back((R *)b);
        }
        arena_steps = nsteps;
        return true;
    }

    ~AdjCtx() override {
        cudaStreamSynchronize(s);
        drop_graphs();
        auto f = [](void *p) { if (p) cudaFree(p); };
        f(gid0); f(phi0); f(ph0); f(C0);
        for (size_t i = 0; i < ck_gid.size(); i++) { f(ck_gid[i]); f(ck_phi[i]); f(ck_ph[i]); f(ck_C[i]); }
        for (size_t i = 0; i < sg_gid.size(); i++) { f(sg_gid[i]); f(sg_phi[i]); f(sg_ph[i]); f(sg_C[i]); f(sg_Csub[i]); }
        f(arena);
        f(w_gid); f(w_phi); f(w_ph); f(w_C); f(w_C2); f(dscr);
        f(v_gid); f(v_phi); f(v_ph); f(v_C);
        f(l_phi); f(l_ph); f(l_C); f(l_phi2); f(l_ph2); f(l_C2); f(pub_id); f(pub_l); f(d_acc);
        f(d_ctr); f(d_err);
        if (s) cudaStreamDestroy(s);
    }

    template <class T>
    bool alloc(T **p, size_t count) { return cudaMalloc((void **)p, count * sizeof(T)) == cudaSuccess; }

    void params() {
        pf_step_params p;
        pf_compute_params(model, t0, p);  // dt and n_sub of the unscaled model, held fixed
        std::memset(&P, 0, sizeof(P));
        P.ix = p.ix; P.iy = p.iy; P.iz = p.iz; P.nnb = p.nnb; P.n_sub = p.n_sub; P.N = p.N;
        P.b1 = map.off[2]; P.b2 = map.off[3];
        P.cutoff = (R)p.cutoff;
        const double sm = scales[0], ss = scales[1], sc = scales[2];
        for (int i = 1; i <= 3; i++)
            for (int j = 1; j <= 3; j++) {
                const int e = (i - 1) + 3 * (j - 1);
                const bool inter = std::abs(i - j) != 2;
                const double dm = p.pfm_dt * p.m[e] * sm;
                P.A[e] = inter ? (R)(dm * p.sigma[e] * ss * p.factor1) : (R)0;
                P.B[e] = inter ? (R)(dm * p.sigma[e] * ss * p.factor2) : (R)0;
                P.G[e] = (inter && i != j) ? (R)(dm * p.factor3 * p.entropy[e] / p.dcdT[e]) : (R)0;
                P.E[e] = (R)p.eq[e];
                P.k[e] = (R)p.k[0][e];
                P.c[e] = (R)p.c[0][e];
            }
        for (int q = 0; q < 3; q++) P.D[q] = (R)(p.D[0][q] * sc * p.coef_diff);
        P.s_m = (R)sm; P.s_s = (R)ss; P.s_c = (R)sc;
        n_sub = p.n_sub;
    }

    // The reverse sweep's record of one step's diffusion: the step's planes
    // (9N, step_planes) and the carbon after sub-steps 0 .. n_sub-2 (the
    // carbon before sub-step 0 is the stored pre-step state, the last
    // sub-step's result is the next step's).
    static size_t record_size(int nsub, size_t n) { return (size_t)(9 + (nsub > 1 ? nsub - 1 : 0)) * n; }

    // One forward step; with Drec (record_size values) the step's diffusion
    // record is kept there for the reverse sweep, else the planes go to the
    // scratch.
    int step(const ushort4 *g, const R *phi, const R *ph, const R *C, ushort4 *g2, R *phi2, R *ph2, R *C2,
             R *Drec) {
        const dim3 g3 = pf_cell_grid(P.ix, P.iy, P.iz);
        R *DS = Drec ? Drec : dscr;
        R *Csub = Drec ? Drec + 9 * N : nullptr;
        const int pt = pf_use_patch(P.iy, P.iz);  // warps on compact cell patches
        k_fwd_phase<R><<<pf_map_grid(pt, P.ix, P.iy, P.iz), PF_CELL_THREADS, 0, s>>>(P, pt, g, phi, ph, C, g2, phi2,
                                                                                   ph2, DS);
        // Sub-step k writes buf[(n_sub-1-k) % 2] with buf = {C2, w_C2}: the last
        // one lands in C2 and no sub-step reads the buffer it writes.
        R *buf[2] = {C2, w_C2};
        const R *cin = C;
        for (int k = 0; k < n_sub; k++) {
            R *cout = buf[(n_sub - 1 - k) % 2];
            k_fwd_diffuse_d<R><<<g3, PF_CELL_THREADS, 0, s>>>(P, DS, cin, cout,
                                                              Csub && k + 1 < n_sub ? Csub + (size_t)k * N : nullptr);
            cin = cout;
        }
        return cudaGetLastError() == cudaSuccess ? PF_OK : pf_fail(PF_ERR_CUDA, "adjoint forward launch");
    }
};

struct pf_adj {
    int prec;
    pf_adj_impl *impl;
};

template <typename R>
static AdjCtx<R> *as(pf_adj *a) { return static_cast<AdjCtx<R> *>(a->impl); }

// The reverse diffusion sub-steps of one step: one cooperative launch when
// every cell fits kCoopCells per resident thread, else one launch per
// sub-step.  The adjoint of C ends in the same buffer either way.
template <typename R>
static void bwd_diffusion(AdjCtx<R> *c, const AP<R> &P, const R *Drec, const R *C0, const ushort4 *gat_gid,
                          R *gat_lphi) {
    const size_t N = (size_t)c->N;
    const R *DS = Drec, *Csub = Drec + 9 * N;
    const long long need = (c->N + PF_CELL_THREADS - 1) / PF_CELL_THREADS;
    const long long blocks = need < c->coop_blocks ? need : c->coop_blocks;
    if (blocks > 0 && blocks * PF_CELL_THREADS * kCoopCells >= c->N) {
        cudaMemsetAsync(c->d_ctr, 0, sizeof(unsigned long long), c->s);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)blocks);
        cfg.blockDim = dim3(PF_CELL_THREADS);
        cfg.stream = c->s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_bwd_diffuse_all<R, kCoopCells>, P, DS, C0, Csub, c->l_C, c->l_C2,
                           c->l_ph, c->d_acc + 3, c->d_ctr, c->d_err, kCoopTimeoutNs, gat_gid, (const int *)c->pub_id,
                           (const R *)c->pub_l, gat_lphi);
        if (c->n_sub & 1) std::swap(c->l_C, c->l_C2);
        return;
    }
    const dim3 g3 = pf_cell_grid(P.ix, P.iy, P.iz);
    if (gat_gid) k_bwd_phase_gather<R><<<g3, PF_CELL_THREADS, 0, c->s>>>(P, gat_gid, c->pub_id, c->pub_l, gat_lphi);
    for (int k = c->n_sub - 1; k >= 0; k--) {
        const R *cin = k == 0 ? C0 : Csub + (size_t)(k - 1) * N;
        k_bwd_diffuse_d<R><<<g3, PF_CELL_THREADS, 0, c->s>>>(P, DS, cin, c->l_C, c->l_C2, c->l_ph, c->d_acc + 3);
        std::swap(c->l_C, c->l_C2);
    }
}

template <typename R>
static int adj_create(const pf_model *m, int K, pf_adj_impl **out) {
    auto *c = new AdjCtx<R>();
    c->model = *m;
    c->N = (long long)m->ix * m->iy * m->iz;
    c->record = K == 0;
    c->K = K == 0 ? 1 : K;
    const size_t N = (size_t)c->N;
    bool ok = cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && c->alloc(&c->gid0, N) && c->alloc(&c->phi0, 4 * N) && c->alloc(&c->ph0, 3 * N) && c->alloc(&c->C0, N);
    ok = ok && c->alloc(&c->dscr, 9 * N);
    ok = ok && c->alloc(&c->v_gid, N) && c->alloc(&c->v_phi, 4 * N) && c->alloc(&c->v_ph, 3 * N) && c->alloc(&c->v_C, N);
    ok = ok && c->alloc(&c->w_gid, N) && c->alloc(&c->w_phi, 4 * N) && c->alloc(&c->w_ph, 3 * N) &&
         c->alloc(&c->w_C, N) && c->alloc(&c->w_C2, N);
    ok = ok && c->alloc(&c->l_phi, 4 * N) && c->alloc(&c->l_ph, 3 * N) && c->alloc(&c->l_C, N) &&
         c->alloc(&c->l_phi2, 4 * N) && c->alloc(&c->l_ph2, 3 * N) && c->alloc(&c->l_C2, N);
    ok = ok && c->alloc(&c->pub_id, LMAX * N) && c->alloc(&c->pub_l, LMAX * N) && c->alloc(&c->d_acc, 8);
    ok = ok && c->alloc(&c->d_ctr, 1) && c->alloc(&c->d_err, 1);
    if (ok) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bwd_diffuse_all<R, kCoopCells>, PF_CELL_THREADS,
                                                          0) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 0;
        }
        c->coop_blocks = per_sm * sms;
        cudaMemsetAsync(c->d_err, 0, sizeof(int), c->s);
    }
    if (!ok) {
        cudaGetLastError();
        delete c;
        return pf_fail(PF_ERR_NOMEM, "pf_adj_create: allocation failed");
    }
    *out = c;
    return PF_OK;
}

extern "C" int pf_adj_create(const pf_model *model, int precision, int checkpoint_every, pf_adj **out) {
    if (!model || !out || checkpoint_every < 0) return pf_fail(PF_ERR_ARG, "pf_adj_create: bad arguments");
    if (precision != PF_PREC_FP64 && precision != PF_PREC_FP32C) return pf_fail(PF_ERR_ARG, "pf_adj_create: bad precision");
    if (model->thermo_model != 0)
        return pf_fail(PF_ERR_ARG, "pf_adj_create: the adjoint differentiates the linear-line thermodynamics only");
    *out = nullptr;
    pf_adj *a = new pf_adj();
    a->prec = precision;
    int st = precision == PF_PREC_FP64 ? adj_create<double>(model, checkpoint_every, &a->impl)
                                       : adj_create<float>(model, checkpoint_every, &a->impl);
    if (st != PF_OK) {
        delete a;
        return st;
    }
    *out = a;
    return PF_OK;
}

extern "C" int pf_adj_destroy(pf_adj *a) {
    if (!a) return PF_OK;
    delete a->impl;
    delete a;
    return PF_OK;
}

template <typename R>
static int adj_upload(AdjCtx<R> *c, const int32_t *ids, const double *phi, const double *phase, const double *C,
                      double time) {
    const size_t N = (size_t)c->N;
    int *d_ids = nullptr;
    double *d_phi = nullptr, *d_phase = nullptr, *d_C = nullptr;
    int *d_span = nullptr;
    bool ok = cudaMalloc(&d_ids, 6 * N * sizeof(int)) == cudaSuccess && cudaMalloc(&d_phi, 6 * N * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&d_phase, 3 * N * sizeof(double)) == cudaSuccess && cudaMalloc(&d_C, N * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&d_span, 8 * sizeof(int)) == cudaSuccess;
    int st = PF_OK;
    if (!ok) {
        cudaGetLastError();
        st = pf_fail(PF_ERR_NOMEM, "pf_adj_upload: staging allocation failed");
    } else {
        cudaMemcpyAsync(d_ids, ids, 6 * N * sizeof(int), cudaMemcpyHostToDevice, c->s);
        cudaMemcpyAsync(d_phi, phi, 6 * N * sizeof(double), cudaMemcpyHostToDevice, c->s);
        cudaMemcpyAsync(d_phase, phase, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->s);
        cudaMemcpyAsync(d_C, C, N * sizeof(double), cudaMemcpyHostToDevice, c->s);
        cudaMemsetAsync(d_span, 0, 8 * sizeof(int), c->s);
        pf_launch_id_span(d_ids, c->N, d_span, c->s);
        int span[8];
        cudaMemcpyAsync(span, d_span, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->s);
        cudaError_t e = cudaStreamSynchronize(c->s);
        if (e != cudaSuccess) st = pf_fail(PF_ERR_CUDA, cudaGetErrorString(e));
        else if (span[4]) st = pf_fail(PF_ERR_RANGE, "pf_adj_upload: grain id outside 0..399999");
        else {
            c->map.off[0] = 0; c->map.off[1] = span[0]; c->map.off[2] = span[0] + span[1];
            c->map.off[3] = span[0] + span[1] + span[2]; c->map.total = c->map.off[3] + span[3];
            if (c->map.total > 65535) st = pf_fail(PF_ERR_RANGE, "pf_adj_upload: more than 65535 grains");
        }
        if (st == PF_OK) {
            k_adj_pack<R><<<blocks(c->N), 256, 0, c->s>>>(c->N, c->map, d_ids, d_phi, d_phase, d_C, c->gid0, c->phi0,
                                                        c->ph0, c->C0);
            if (cudaStreamSynchronize(c->s) != cudaSuccess) st = pf_fail(PF_ERR_CUDA, "pf_adj_upload: pack failed");
        }
    }
    cudaFree(d_ids); cudaFree(d_phi); cudaFree(d_phase); cudaFree(d_C); cudaFree(d_span);
    if (st == PF_OK) {
        c->t0 = time;
        c->have_state = true;
        c->have_fwd = false;
    }
    return st;
}

extern "C" int pf_adj_upload(pf_adj *a, const int32_t *ids, const double *phi, const double *phase, const double *C,
                             double time) {
    if (!a || !ids || !phi || !phase || !C) return pf_fail(PF_ERR_ARG, "pf_adj_upload: null argument");
    return a->prec == PF_PREC_FP64 ? adj_upload(as<double>(a), ids, phi, phase, C, time)
                                   : adj_upload(as<float>(a), ids, phi, phase, C, time);
}

extern "C" int pf_adj_set_scales(pf_adj *a, const double scales[4]) {
    if (!a || !scales) return pf_fail(PF_ERR_ARG, "pf_adj_set_scales: null argument");
    double *dst = a->prec == PF_PREC_FP64 ? as<double>(a)->scales : as<float>(a)->scales;
    for (int i = 0; i < 4; i++) dst[i] = scales[i];
    if (a->prec == PF_PREC_FP64) as<double>(a)->have_fwd = false;
    else as<float>(a)->have_fwd = false;
    return PF_OK;
}

template <typename R>
static int ensure_ck(AdjCtx<R> *c, size_t nck, size_t nseg) {
    const size_t N = (size_t)c->N;
    while (c->ck_gid.size() < nck) {
        ushort4 *g; R *p, *h, *C;
        if (!c->alloc(&g, N) || !c->alloc(&p, 4 * N) || !c->alloc(&h, 3 * N) || !c->alloc(&C, N)) {
            cudaGetLastError();
            return pf_fail(PF_ERR_NOMEM, "adjoint checkpoint allocation failed");
        }
        c->ck_gid.push_back(g); c->ck_phi.push_back(p); c->ck_ph.push_back(h); c->ck_C.push_back(C);
    }
    while (c->sg_gid.size() < nseg) {
        ushort4 *g; R *p, *h, *C, *Cs;
        if (!c->alloc(&g, N) || !c->alloc(&p, 4 * N) || !c->alloc(&h, 3 * N) || !c->alloc(&C, N) ||
            !c->alloc(&Cs, AdjCtx<R>::record_size(c->n_sub, N))) {
            cudaGetLastError();
            return pf_fail(PF_ERR_NOMEM, "adjoint segment allocation failed");
        }
        c->sg_gid.push_back(g); c->sg_phi.push_back(p); c->sg_ph.push_back(h); c->sg_C.push_back(C); c->sg_Csub.push_back(Cs);
    }
    return PF_OK;
}

template <typename R>
static void copy_state(AdjCtx<R> *c, const ushort4 *g, const R *p, const R *h, const R *C, ushort4 *g2, R *p2, R *h2,
                       R *C2) {
    const size_t N = (size_t)c->N;
    cudaMemcpyAsync(g2, g, N * sizeof(ushort4), cudaMemcpyDeviceToDevice, c->s);
    cudaMemcpyAsync(p2, p, 4 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
    cudaMemcpyAsync(h2, h, 3 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
    cudaMemcpyAsync(C2, C, N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
}

// The objective sums of the final state (ph, C) into J, with the forward's timing.
template <typename R>
static int adj_finish_forward(AdjCtx<R> *c, R *ph, R *C, cudaEvent_t e0, cudaEvent_t e1, double J[2]) {
    cudaMemsetAsync(c->d_acc, 0, 8 * sizeof(double), c->s);
    AP<R> P = c->P;
    c->fin_ph = ph;
    c->fin_C = C;
    k_objective_sums<R><<<256, 256, 0, c->s>>>(P, ph, C, c->d_acc);
    double h[8];
    cudaMemcpyAsync(h, c->d_acc, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s);
    cudaEventRecord(e1, c->s);
    if (cudaStreamSynchronize(c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "pf_adj_forward failed");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    c->ms_fwd = ms;
    c->J[0] = h[0] / (double)c->N;
    c->W = h[1];
    c->J[1] = h[1] > 0 ? h[2] / h[1] : 0.0;
    J[0] = c->J[0];
    J[1] = c->J[1];
    c->have_fwd = true;
    return PF_OK;
}

// Record mode: the forward writes every step's pre-step state and diffusion
// record into the arena (the work a checkpointed gradient spends recomputing
// segments), as one captured graph per step count.
template <typename R>
static int adj_forward_record(AdjCtx<R> *c, int nsteps, double J[2]) {
    c->params();
    c->nsteps = nsteps;
    if (std::memcmp(&c->gP, &c->P, sizeof(c->P)) != 0) {
        c->drop_graphs();
        c->gP = c->P;
    }
    if (!c->ensure_arena(nsteps))
        return pf_fail(PF_ERR_NOMEM, "pf_adj_forward: the record of every step does not fit on the device "
                                     "(use a checkpoint interval)");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0, c->s);
    auto run = [&]() -> int {
        copy_state(c, c->gid0, c->phi0, c->ph0, c->C0, c->rg_gid[0], c->rg_phi[0], c->rg_ph[0], c->rg_C[0]);
        for (int t = 0; t < nsteps; t++) {
            const bool last = t + 1 == nsteps;
            const int s2 = c->step(c->rg_gid[t], c->rg_phi[t], c->rg_ph[t], c->rg_C[t],
                                   last ? c->w_gid : c->rg_gid[t + 1], last ? c->w_phi : c->rg_phi[t + 1],
                                   last ? c->w_ph : c->rg_ph[t + 1], last ? c->w_C : c->rg_C[t + 1], c->rg_Csub[t]);
            if (s2 != PF_OK) return s2;
        }
        return PF_OK;
    };
    if (!c->rec_fwd || c->rec_fwd_steps != nsteps) {
        if (c->rec_fwd) { cudaGraphExecDestroy(c->rec_fwd); c->rec_fwd = nullptr; }
        cudaGraph_t g;
        if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
        const int st = run();
        if (cudaStreamEndCapture(c->s, &g) != cudaSuccess || st != PF_OK)
            return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
        const bool okg = cudaGraphInstantiate(&c->rec_fwd, g, 0) == cudaSuccess;
        cudaGraphDestroy(g);
        if (!okg) return pf_fail(PF_ERR_CUDA, "adjoint: graph instantiation failed");
        c->rec_fwd_steps = nsteps;
    }
    if (cudaGraphLaunch(c->rec_fwd, c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "adjoint: graph launch failed");
    return adj_finish_forward(c, c->w_ph, c->w_C, e0, e1, J);
}

template <typename R>
static int adj_forward(AdjCtx<R> *c, int nsteps, double J[2]) {
    if (!c->have_state) return pf_fail(PF_ERR_ARG, "pf_adj_forward: no state uploaded");
    if (c->record) return adj_forward_record(c, nsteps, J);
    c->params();
    c->nsteps = nsteps;
    const int nck = (nsteps + c->K - 1) / c->K + 1;
    int st = ensure_ck(c, (size_t)nck, 0);
    if (st != PF_OK) return st;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0, c->s);
    // Two state sets alternate: the work buffers and the spare checkpoint slot
    // (slot nck-1 is never a checkpoint).  Checkpoints are copies taken every K steps.
    ushort4 *ga = c->w_gid, *gb = c->v_gid;
    R *pa = c->w_phi, *pb = c->v_phi, *ha = c->w_ph, *hb = c->v_ph;
    R *Ca = c->w_C, *Cb = c->v_C;
    copy_state(c, c->gid0, c->phi0, c->ph0, c->C0, ga, pa, ha, Ca);
    // Captured graphs bake the parameters in: keep them while they are unchanged.
    if (std::memcmp(&c->gP, &c->P, sizeof(c->P)) != 0) {
        c->drop_graphs();
        c->gP = c->P;
    }
    // A full segment of K steps is one CUDA graph (per starting buffer set);
    // the checkpoint copy in front of it depends on the segment and stays outside.
    auto run_steps = [&](int n) -> int {
        for (int t = 0; t < n; t++) {
            int s2 = c->step(ga, pa, ha, Ca, gb, pb, hb, Cb, nullptr);
            if (s2 != PF_OK) return s2;
            std::swap(ga, gb); std::swap(pa, pb); std::swap(ha, hb); std::swap(Ca, Cb);
        }
        return PF_OK;
    };
    for (int t = 0; t < nsteps; t += c->K) {
        const int n = std::min(c->K, nsteps - t);
        copy_state(c, ga, pa, ha, Ca, c->ck_gid[t / c->K], c->ck_phi[t / c->K], c->ck_ph[t / c->K], c->ck_C[t / c->K]);
        if (n < c->K) {
            st = run_steps(n);
        } else {
            const int set = (ga == c->w_gid) ? 0 : 1;
            if (!c->fwd_graph[set]) {
                cudaGraph_t g;
                if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                    return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
                st = run_steps(n);
                if (cudaStreamEndCapture(c->s, &g) != cudaSuccess || st != PF_OK)
                    return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
                const bool okg = cudaGraphInstantiate(&c->fwd_graph[set], g, 0) == cudaSuccess;
                cudaGraphDestroy(g);
                if (!okg) return pf_fail(PF_ERR_CUDA, "adjoint: graph instantiation failed");
            } else {
                // Replay: the host-side buffer roles advance as during capture.
                for (int q = 0; q < n; q++) {
                    std::swap(ga, gb); std::swap(pa, pb); std::swap(ha, hb); std::swap(Ca, Cb);
                }
            }
            if (cudaGraphLaunch(c->fwd_graph[set], c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "adjoint: graph launch failed");
        }
        if (st != PF_OK) return st;
    }
    return adj_finish_forward(c, ha, Ca, e0, e1, J);
}

extern "C" int pf_adj_forward(pf_adj *a, int nsteps, double J[2]) {
    if (!a || !J || nsteps < 1) return pf_fail(PF_ERR_ARG, "pf_adj_forward: bad arguments");
    return a->prec == PF_PREC_FP64 ? adj_forward(as<double>(a), nsteps, J) : adj_forward(as<float>(a), nsteps, J);
}

// The gradient sums, the barrier-timeout flag and the gradient's timing.
template <typename R>
static int adj_finish_gradient(AdjCtx<R> *c, cudaEvent_t e0, cudaEvent_t e1, double grad[4]) {
    double h[8];
    int herr = 0;
    cudaMemcpyAsync(h, c->d_acc, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s);
    cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->s);
    cudaEventRecord(e1, c->s);
    if (cudaStreamSynchronize(c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "pf_adj_gradient failed");
    if (herr) {
        cudaMemsetAsync(c->d_err, 0, sizeof(int), c->s);
        cudaStreamSynchronize(c->s);
        return pf_fail(PF_ERR_TIMEOUT, "pf_adj_gradient: a grid barrier of the reverse diffusion timed out");
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    c->ms_bwd = ms;
    grad[0] = h[3];
    grad[1] = h[4];
    grad[2] = h[5];
    grad[3] = 0.0;  // Mn does not enter the phase update or the carbon field
    return PF_OK;
}

// Record mode: seed from the final state and sweep every recorded step
// backwards, as one captured graph per step count that ends with the adjoint
// buffers back in the roles it was captured with.
template <typename R>
static int adj_gradient_record(AdjCtx<R> *c, int obj, double grad[4]) {
    const int T = c->nsteps;
    const size_t N = (size_t)c->N;
    AP<R> P = c->P;
    const dim3 g3 = pf_cell_grid(P.ix, P.iy, P.iz);
    const int pt = pf_use_patch(P.iy, P.iz);  // reverse phase sweep: warps on compact cell patches
    const dim3 gp = pf_map_grid(pt, P.ix, P.iy, P.iz);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0, c->s);
    cudaMemsetAsync(c->d_acc, 0, 8 * sizeof(double), c->s);
    k_seed<R><<<blocks(c->N), 256, 0, c->s>>>(P, obj, c->w_ph, c->w_C, c->W, c->J[1], c->l_ph, c->l_C, c->l_phi);
    auto reverse = [&]() {
        const ushort4 *pend_gid = nullptr;
        R *pend_lphi = nullptr;
        for (int t = T - 1; t >= 0; t--) {
            bwd_diffusion(c, P, c->rg_Csub[t], c->rg_C[t], pend_gid, pend_lphi);
            k_bwd_phase_own<R><<<gp, PF_CELL_THREADS, 0, c->s>>>(P, pt, c->rg_gid[t], c->rg_phi[t], c->rg_ph[t],
                                                                 c->rg_C[t], c->l_phi, c->l_ph, c->l_C, c->l_phi2,
                                                                 c->l_ph2, c->pub_id, c->pub_l, c->d_acc + 3);
            pend_gid = c->rg_gid[t];
            pend_lphi = c->l_phi2;
            std::swap(c->l_phi, c->l_phi2);
            std::swap(c->l_ph, c->l_ph2);
        }
        if (pend_gid)
            k_bwd_phase_gather<R><<<g3, PF_CELL_THREADS, 0, c->s>>>(P, pend_gid, c->pub_id, c->pub_l, pend_lphi);
    };
    // Move the seeded adjoint into the buffers the graph starts from.
    auto to_roles = [&](R *gC, R *gphi, R *gph) {
        if (c->l_C != gC) {
            cudaMemcpyAsync(gC, c->l_C, N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
            std::swap(c->l_C, c->l_C2);
        }
        if (c->l_phi != gphi) {
            cudaMemcpyAsync(gphi, c->l_phi, 4 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
            std::swap(c->l_phi, c->l_phi2);
        }
        if (c->l_ph != gph) {
            cudaMemcpyAsync(gph, c->l_ph, 3 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
            std::swap(c->l_ph, c->l_ph2);
        }
    };
    if (!c->rec_bwd || c->rec_bwd_steps != T) {
        if (c->rec_bwd) { cudaGraphExecDestroy(c->rec_bwd); c->rec_bwd = nullptr; }
        R *cC = c->l_C, *cphi = c->l_phi, *cph = c->l_ph;
        c->rb_C = cC; c->rb_phi = cphi; c->rb_ph = cph;
        cudaGraph_t g;
        if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
        reverse();
        to_roles(cC, cphi, cph);
        if (cudaStreamEndCapture(c->s, &g) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
        const bool okg = cudaGraphInstantiate(&c->rec_bwd, g, 0) == cudaSuccess;
        cudaGraphDestroy(g);
        if (!okg) return pf_fail(PF_ERR_CUDA, "adjoint: graph instantiation failed");
        c->rec_bwd_steps = T;
    } else {
        to_roles(c->rb_C, c->rb_phi, c->rb_ph);
    }
    if (cudaGraphLaunch(c->rec_bwd, c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "adjoint: graph launch failed");
    return adj_finish_gradient(c, e0, e1, grad);
}

template <typename R>
static int adj_gradient(AdjCtx<R> *c, int obj, double grad[4]) {
    if (!c->have_fwd) return pf_fail(PF_ERR_ARG, "pf_adj_gradient: run pf_adj_forward first");
    if (c->record) return adj_gradient_record(c, obj, grad);
    const int nck = (c->nsteps + c->K - 1) / c->K + 1;
    int st = ensure_ck(c, (size_t)nck, (size_t)c->K);
    if (st != PF_OK) return st;
    const size_t N = (size_t)c->N;
    const unsigned nb = blocks(c->N);
    AP<R> P = c->P;
    const dim3 g3 = pf_cell_grid(P.ix, P.iy, P.iz);
    const int pt = pf_use_patch(P.iy, P.iz);  // reverse phase sweep: warps on compact cell patches
    const dim3 gp = pf_map_grid(pt, P.ix, P.iy, P.iz);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0, c->s);
    // Final state: recompute the last segment, then seed from its end state.
    cudaMemsetAsync(c->d_acc, 0, 8 * sizeof(double), c->s);
    bool seeded = false;
    const int nseg = (c->nsteps + c->K - 1) / c->K;
    auto recompute = [&](int t0, int t1) -> int {
        for (int t = t0; t < t1; t++) {
            const int i = t - t0;
            ushort4 *g2 = (i + 1 < c->K) ? c->sg_gid[i + 1] : c->w_gid;
            R *p2 = (i + 1 < c->K) ? c->sg_phi[i + 1] : c->w_phi;
            R *h2 = (i + 1 < c->K) ? c->sg_ph[i + 1] : c->w_ph;
            R *C2 = (i + 1 < c->K) ? c->sg_C[i + 1] : c->w_C;
            if (t == t1 - 1) { g2 = c->w_gid; p2 = c->w_phi; h2 = c->w_ph; C2 = c->w_C; }
            int s2 = c->step(c->sg_gid[i], c->sg_phi[i], c->sg_ph[i], c->sg_C[i], g2, p2, h2, C2, c->sg_Csub[i]);
            if (s2 != PF_OK) return s2;
        }
        return PF_OK;
    };
    auto reverse = [&](int t0, int t1) {
        // The neighbour part of each reverse phase sweep runs inside the next
        // reverse diffusion launch (pending), the segment's last one alone.
        const ushort4 *pend_gid = nullptr;
        R *pend_lphi = nullptr;
        for (int t = t1 - 1; t >= t0; t--) {
            const int i = t - t0;
            // Reverse the diffusion sub-steps (the step's record holds what
            // they need of the post-sweep phase fractions).
            bwd_diffusion(c, P, c->sg_Csub[i], c->sg_C[i], pend_gid, pend_lphi);
            // Reverse the phase sweep, own part.
            k_bwd_phase_own<R><<<gp, PF_CELL_THREADS, 0, c->s>>>(P, pt, c->sg_gid[i], c->sg_phi[i], c->sg_ph[i], c->sg_C[i], c->l_phi,
                                                    c->l_ph, c->l_C, c->l_phi2, c->l_ph2, c->pub_id, c->pub_l, c->d_acc + 3);
            pend_gid = c->sg_gid[i];
            pend_lphi = c->l_phi2;
            std::swap(c->l_phi, c->l_phi2);
            std::swap(c->l_ph, c->l_ph2);
        }
        if (pend_gid)
            k_bwd_phase_gather<R><<<g3, PF_CELL_THREADS, 0, c->s>>>(P, pend_gid, c->pub_id, c->pub_l, pend_lphi);
    };
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int t0 = sg * c->K, t1 = std::min(c->nsteps, t0 + c->K);
        // Recompute the segment from its checkpoint, storing every pre-step
        // state and every sub-step's carbon, then sweep it backwards.
        copy_state(c, c->ck_gid[sg], c->ck_phi[sg], c->ck_ph[sg], c->ck_C[sg], c->sg_gid[0], c->sg_phi[0], c->sg_ph[0],
                   c->sg_C[0]);
        if (!seeded || t1 - t0 != c->K) {
            st = recompute(t0, t1);
            if (st != PF_OK) return st;
            if (!seeded) {
                k_seed<R><<<nb, 256, 0, c->s>>>(P, obj, c->w_ph, c->w_C, c->W, c->J[1], c->l_ph, c->l_C, c->l_phi);
                seeded = true;
            }
            reverse(t0, t1);
            continue;
        }
        // Every other segment is identical launch for launch: one graph,
        // captured once, ending with the adjoint buffers back in their roles.
        if (c->seg_graph) {
            // Replays start from the buffer roles of the capture.
            if (c->l_C != c->g_C) {
                cudaMemcpyAsync(c->g_C, c->l_C, N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
                std::swap(c->l_C, c->l_C2);
            }
            if (c->l_phi != c->g_phi) {
                cudaMemcpyAsync(c->g_phi, c->l_phi, 4 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
                std::swap(c->l_phi, c->l_phi2);
            }
            if (c->l_ph != c->g_ph) {
                cudaMemcpyAsync(c->g_ph, c->l_ph, 3 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
                std::swap(c->l_ph, c->l_ph2);
            }
        } else {
            R *cC = c->l_C, *cphi = c->l_phi, *cph = c->l_ph;
            c->g_C = cC; c->g_phi = cphi; c->g_ph = cph;
            cudaGraph_t g;
            if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
            st = recompute(t0, t1);
            reverse(t0, t1);
            if (c->l_C != cC) {
                cudaMemcpyAsync(cC, c->l_C, N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
                std::swap(c->l_C, c->l_C2);
            }
            if (c->l_phi != cphi) {
                cudaMemcpyAsync(cphi, c->l_phi, 4 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
                std::swap(c->l_phi, c->l_phi2);
            }
            if (c->l_ph != cph) {
                cudaMemcpyAsync(cph, c->l_ph, 3 * N * sizeof(R), cudaMemcpyDeviceToDevice, c->s);
                std::swap(c->l_ph, c->l_ph2);
            }
            if (cudaStreamEndCapture(c->s, &g) != cudaSuccess || st != PF_OK)
                return pf_fail(PF_ERR_CUDA, "adjoint: capture failed");
            const bool okg = cudaGraphInstantiate(&c->seg_graph, g, 0) == cudaSuccess;
            cudaGraphDestroy(g);
            if (!okg) return pf_fail(PF_ERR_CUDA, "adjoint: graph instantiation failed");
        }
        if (cudaGraphLaunch(c->seg_graph, c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "adjoint: graph launch failed");
    }
    return adj_finish_gradient(c, e0, e1, grad);
}

extern "C" int pf_adj_gradient(pf_adj *a, int objective, double grad[4]) {
    if (!a || !grad || objective < 0 || objective > 1) return pf_fail(PF_ERR_ARG, "pf_adj_gradient: bad arguments");
    return a->prec == PF_PREC_FP64 ? adj_gradient(as<double>(a), objective, grad)
                                   : adj_gradient(as<float>(a), objective, grad);
}

template <typename R>
static int adj_final(AdjCtx<R> *c, double *phase, double *C) {
    if (!c->have_fwd || !c->fin_ph) return pf_fail(PF_ERR_ARG, "pf_adj_final_state: run pf_adj_forward first");
    const size_t N = (size_t)c->N;
    std::vector<R> h(3 * N), hc(N);
    cudaMemcpyAsync(h.data(), c->fin_ph, 3 * N * sizeof(R), cudaMemcpyDeviceToHost, c->s);
    cudaMemcpyAsync(hc.data(), c->fin_C, N * sizeof(R), cudaMemcpyDeviceToHost, c->s);
    if (cudaStreamSynchronize(c->s) != cudaSuccess) return pf_fail(PF_ERR_CUDA, "pf_adj_final_state failed");
    for (size_t i = 0; i < 3 * N; i++) phase[i] = (double)h[i];
    for (size_t i = 0; i < N; i++) C[i] = (double)hc[i];
    return PF_OK;
}

extern "C" int pf_adj_final_state(pf_adj *a, double *phase, double *C) {
    if (!a || !phase || !C) return pf_fail(PF_ERR_ARG, "pf_adj_final_state: null argument");
    return a->prec == PF_PREC_FP64 ? adj_final(as<double>(a), phase, C) : adj_final(as<float>(a), phase, C);
}

extern "C" int pf_adj_timings(pf_adj *a, double ms[2]) {
    if (!a || !ms) return pf_fail(PF_ERR_ARG, "pf_adj_timings: null argument");
    if (a->prec == PF_PREC_FP64) { ms[0] = as<double>(a)->ms_fwd; ms[1] = as<double>(a)->ms_bwd; }
    else { ms[0] = as<float>(a)->ms_fwd; ms[1] = as<float>(a)->ms_bwd; }
    return PF_OK;
}
