// pf_f32.cu -- compact FP32 step kernels with compensated solute updates (sm_103a).
//
// Model: the Steinbach pairwise phase update and multiphase diffusion of
// zhubq/PhaseField (C++-openmp-cuda/src/solver.cpp:147-372), stored compactly:
//   gid   ushort4 / cell   up to 4 local grain ids (0 = empty)
//   phi   float4  / cell   their phase-field values
//   phase float[3][N]      phase fractions, one plane per phase
//   sol   float2[N][nsol]  solute total concentration and its Kahan
//                          compensation (true value = x - y)
// Phase concentrations are not stored: every kernel re-partitions C with the
// linear partition of solver.cpp:389-405 where it needs them.  The local grain
// id encodes the phase by range: id <= b1 -> ferrite(1), <= b2 -> austenite(2),
// else cementite(3).
//
// Built with -prec-div=false -prec-sqrt=false: divisions and square roots are
// the approximate (<= 2 ulp) forms; the solute increment itself is summed with
// Kahan compensation so total carbon and Mn stay conserved to FP32 round-off
// of the increments rather than of the concentrations.
#include "pf_dev.cuh"
#include "pf_kernels.h"

namespace {

__device__ __forceinline__ int pf_lphase(int l, int b1, int b2) {
    return l == 0 ? 0 : (l <= b1 ? 1 : (l <= b2 ? 2 : 3));
}

__device__ __forceinline__ float pf_sel3(int p, float a, float b, float c) {
    return p == 1 ? a : (p == 2 ? b : c);
}

// solver.cpp:389-405 in FP32.
__device__ __forceinline__ void pf_partition_f32(float C, const float ph[3], const float *k9,
                                                 const float *c9, float out[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float t1 = ph[0] * k9[i] + ph[1] * k9[i + 3] + ph[2] * k9[i + 6];
        float t2 = ph[0] * c9[i] + ph[1] * c9[i + 3] + ph[2] * c9[i + 6];
        out[i] = (C - t2) / t1;
    }
}

// Phase sweep (solver.cpp:147-304) on the compact layout, one thread per cell.
template <int NSOL>
__global__ void __launch_bounds__(256) k_phase_f32(const __grid_constant__ pf_f32_params P,
                                                   const ushort4 *__restrict__ gid1,
                                                   const float4 *__restrict__ phi1,
                                                   ushort4 *__restrict__ gid2,
                                                   float4 *__restrict__ phi2,
                                                   float *__restrict__ phase,
                                                   const float2 *__restrict__ sol) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.N) return;
    long long nbr[6];
    pf_neighbours(n, P.ix, P.iy, P.iz, nbr);
    const float cutoff = P.cutoff;
    const int b1 = P.b1, b2 = P.b2;

    const ushort4 g = __ldg(gid1 + n);
    const float4 v = __ldg(phi1 + n);
    const int oid[4] = {g.x, g.y, g.z, g.w};
    const float ov[4] = {v.x, v.y, v.z, v.w};
    int sid[PF_NSTENCIL], sph[PF_NSTENCIL];
    float s1[PF_NSTENCIL], s2[PF_NSTENCIL];
#pragma unroll
    for (int a = 0; a < PF_NSTENCIL; a++) {
        sid[a] = 0; sph[a] = 0; s1[a] = 0.f; s2[a] = 0.f;
    }
    int num = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        if (ov[a] > cutoff) {
            num += 1;
            sid[a] = oid[a];
            sph[a] = pf_lphase(oid[a], b1, b2);
            s1[a] = ov[a];
        }
    }
#pragma unroll
    for (int b = 0; b < 6; b++) {
        if (b < P.nnb) {
            const ushort4 ng = __ldg(gid1 + nbr[b]);
            const float4 nv4 = __ldg(phi1 + nbr[b]);
            const int nid[4] = {ng.x, ng.y, ng.z, ng.w};
            const float nv[4] = {nv4.x, nv4.y, nv4.z, nv4.w};
            bool live = true;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int tid = nid[a];
                live = live && (tid != 0);
                if (live) {
                    bool found = false;
#pragma unroll
                    for (int kk = 0; kk < PF_NSTENCIL; kk++) {
                        if (!found && tid == sid[kk]) {
                            s2[kk] += nv[a];
                            found = true;
                        }
                    }
                    if (!found && num < PF_NSTENCIL) {
#pragma unroll
                        for (int kk = 0; kk < PF_NSTENCIL; kk++) {
                            if (kk == num) {
                                sid[kk] = tid;
                                sph[kk] = pf_lphase(tid, b1, b2);
                                s2[kk] += nv[a];
                            }
                        }
                        num += 1;
                    }
                }
            }
        }
    }
    if (num == 1) {  // bulk: copy and leave the phase fractions untouched
        gid2[n] = g;
        phi2[n] = v;
        return;
    }
    // Carbon concentration of each phase in this cell, partitioned with the
    // phase fractions implied by the current slots.
    float ph_old[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int p = pf_lphase(oid[a], b1, b2);
        if (p == 1) ph_old[0] += ov[a];
        else if (p == 2) ph_old[1] += ov[a];
        else if (p == 3) ph_old[2] += ov[a];
    }
    float lc[3];
    pf_partition_f32(__ldg(sol + n * NSOL).x, ph_old, P.k[0], P.c[0], lc);

    float del[PF_NSTENCIL];
#pragma unroll
    for (int ii = 0; ii < PF_NSTENCIL; ii++) {
        del[ii] = 0.f;
        if (ii < num) {
            const int pi = sph[ii];
            const float ci = pf_sel3(pi, lc[0], lc[1], lc[2]);
            float acc = 0.f;
#pragma unroll
            for (int jj = 0; jj < PF_NSTENCIL; jj++) {
                if (jj < num && jj != ii) {
                    const int e = (pi - 1) + 3 * (sph[jj] - 1);
                    acc += P.A[e] * (s2[ii] * s1[jj] - s2[jj] * s1[ii]) + P.B[e] * (s1[ii] - s1[jj]) +
                           P.G[e] * sqrtf(s1[ii] * s1[jj]) * (ci - P.E[e]);
                }
            }
            float d = s1[ii] + acc;
            if (d > 1.0f) d = 1.0f;
            else if (d < cutoff) d = 0.f;
            del[ii] = d;
        }
    }
    // Top four, first maximum wins (solver.cpp:426-432 truncated to 4 slots).
#pragma unroll
    for (int a = 0; a < PF_NSLOT32; a++) {
        int mx = a;
        float mv = del[a];
#pragma unroll
        for (int b = a + 1; b < PF_NSTENCIL; b++) {
            if (del[b] > mv) { mv = del[b]; mx = b; }
        }
#pragma unroll
        for (int b = a + 1; b < PF_NSTENCIL; b++) {
            if (b == mx) {
                float tv = del[a]; del[a] = del[b]; del[b] = tv;
                int ti = sid[a]; sid[a] = sid[b]; sid[b] = ti;
            }
        }
    }
    float ph[3] = {0.f, 0.f, 0.f};
    float sum = 0.f;
    int kid[4];
    float kv[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        if (del[a] > cutoff) {
            kid[a] = sid[a];
            kv[a] = del[a];
            const int p = pf_lphase(sid[a], b1, b2);
            if (p == 1) ph[0] += del[a];
            else if (p == 2) ph[1] += del[a];
            else ph[2] += del[a];
            sum += del[a];
        } else {
            kid[a] = 0;
            kv[a] = 0.f;
        }
    }
    const float inv = 1.f / sum;
    gid2[n] = make_ushort4((unsigned short)kid[0], (unsigned short)kid[1], (unsigned short)kid[2],
                           (unsigned short)kid[3]);
    phi2[n] = make_float4(kv[0] * inv, kv[1] * inv, kv[2] * inv, kv[3] * inv);
    phase[n] = ph[0] * inv;
    phase[P.N + n] = ph[1] * inv;
    phase[2 * P.N + n] = ph[2] * inv;
}

// ---------------------------------------------------------------------------
// One diffusion sub-step (solver.cpp:343-372) for all solutes.
//
// Every cell contributes two derived quantities to its neighbours' fluxes:
// s_p = sqrt(phi_p) (the flux weight sqrt(phi_p^nb phi_p) = s_p^nb s_p) and the
// partitioned phase concentrations c_p (solver.cpp:389-405).  They are computed
// once per cell: a block owns a TX x TY tile of the x-y plane and marches up a
// chunk of z planes.  The derived values of the current plane, with a one-cell
// in-plane halo, sit in shared memory; those of the planes below and above the
// thread's own column sit in registers.  Each thread then loads its cell's raw
// data once (phase fractions + solute totals), halo cells are re-read from L2.
// The solute total is advanced with a Kahan-compensated sum; D already
// carries dt_sub/dx^2.
// ---------------------------------------------------------------------------
template <int NSOL>
struct pf_der {
    float s[3];
    float c[NSOL][3];
};

template <int NSOL>
__device__ __forceinline__ void pf_load_raw(const float *__restrict__ phase, const float2 *__restrict__ sol,
                                            long long N, long long n, float ph[3], float2 so[NSOL]) {
    ph[0] = __ldg(phase + n);
    ph[1] = __ldg(phase + N + n);
    ph[2] = __ldg(phase + 2 * N + n);
    if (NSOL == 2) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(sol) + n);
        so[0] = make_float2(v.x, v.y);
        so[NSOL - 1] = make_float2(v.z, v.w);
    } else {
        so[0] = __ldg(sol + n);
    }
}

template <int NSOL>
__device__ __forceinline__ void pf_derive(const pf_f32_params &P, const float ph[3], const float2 so[NSOL],
                                          pf_der<NSOL> &d) {
#pragma unroll
    for (int p = 0; p < 3; p++) d.s[p] = sqrtf(ph[p]);
#pragma unroll
    for (int q = 0; q < NSOL; q++) pf_partition_f32(so[q].x, ph, P.k[q], P.c[q], d.c[q]);
}

__device__ __forceinline__ int pf_mod(int v, int L) {
    v %= L;
    return v < 0 ? v + L : v;
}

// Asynchronous global -> shared copies (cp.async): raw plane data is staged two
// planes ahead so its latency overlaps the flux computation.  Each thread only
// ever reads back what it copied itself, so the stages need no barrier.
__device__ __forceinline__ void pf_cp_async4(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void pf_cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void pf_cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void pf_cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void pf_cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }

template <int NSOL>
struct pf_solvec;
template <>
struct pf_solvec<1> { using T = float2; };
template <>
struct pf_solvec<2> { using T = float4; };

template <int NSOL, int TX, int TY, int NST>
struct pf_diff_smem {
    using SV = typename pf_solvec<NSOL>::T;
    static constexpr int NT = TX * TY, NH = 2 * TX + 2 * TY, W = TX + 2, H = TY + 2;
    SV so[NST][NT];          // raw solute totals, own cells
    SV hso[NST][NH];         // raw solute totals, halo cells
    float ph[NST][3][NT];    // raw phase fractions, own cells
    float hph[NST][3][NH];   // raw phase fractions, halo cells
    float ds[3][H][W];       // derived sqrt(phi_p), current plane with halo
    float dc[NSOL][3][H][W]; // derived phase concentrations, current plane with halo
};

template <int NSOL>
__device__ __forceinline__ void pf_unpack_sol(const typename pf_solvec<NSOL>::T &v, float2 so[NSOL]);
template <>
__device__ __forceinline__ void pf_unpack_sol<1>(const float2 &v, float2 so[1]) { so[0] = v; }
template <>
__device__ __forceinline__ void pf_unpack_sol<2>(const float4 &v, float2 so[2]) {
    so[0] = make_float2(v.x, v.y);
    so[1] = make_float2(v.z, v.w);
}

template <int NSOL, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, 4) k_diffuse_f32(const __grid_constant__ pf_f32_params P,
                                                           const float *__restrict__ phase,
                                                           const float2 *__restrict__ sol_in,
                                                           float2 *__restrict__ sol_out, int zchunk) {
    constexpr int NST = 3;
    using SM = pf_diff_smem<NSOL, TX, TY, NST>;
    using SV = typename pf_solvec<NSOL>::T;
    static_assert(SM::NH <= SM::NT, "halo needs one thread per halo cell");
    extern __shared__ __align__(16) unsigned char pf_smem_raw[];
    SM &sm = *reinterpret_cast<SM *>(pf_smem_raw);
    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const long long N = P.N;
    const long long plane = (long long)ix * iy;
    const int tiles_x = (ix + TX - 1) / TX;
    const int tx0 = (int)(blockIdx.x % tiles_x) * TX;
    const int ty0 = (int)(blockIdx.x / tiles_x) * TY;
    const int tid = threadIdx.x;
    const int lx = tid % TX, ly = tid / TX;
    const bool valid = (tx0 + lx < ix) && (ty0 + ly < iy);
    // Every shared slot holds the cell at the wrapped coordinates, so partial
    // tiles and periodic neighbours need no special case.
    const long long col = pf_mod(tx0 + lx, ix) + (long long)ix * pf_mod(ty0 + ly, iy);
    const bool has_halo = tid < SM::NH;
    int hx = 0, hy = 0;
    if (tid < TX) { hx = tid; hy = -1; }
    else if (tid < 2 * TX) { hx = tid - TX; hy = TY; }
    else if (tid < 2 * TX + TY) { hx = -1; hy = tid - 2 * TX; }
    else { hx = TX; hy = tid - 2 * TX - TY; }
    const long long hcol = pf_mod(tx0 + hx, ix) + (long long)ix * pf_mod(ty0 + hy, iy);
    const bool use_y = P.nnb >= 4, use_z = P.nnb >= 6;
    const int z0 = blockIdx.y * zchunk;
    const int z1 = min(z0 + zchunk, iz);
    // Planes this block reads: z0-1 .. z1 with z neighbours, z0 .. z1-1 without.
    const int zlo = use_z ? z0 - 1 : z0, zhi = use_z ? z1 : z1 - 1;
    const SV *solv = reinterpret_cast<const SV *>(sol_in);

    auto issue = [&](int zz) {  // stage raw data of plane zz (if needed), always commit a group
        if (zz >= zlo && zz <= zhi) {
            const int st = (zz - zlo) % NST;
            const long long pz = plane * pf_mod(zz, iz);
            const long long n = col + pz;
            pf_cp_async4(&sm.ph[st][0][tid], phase + n);
            pf_cp_async4(&sm.ph[st][1][tid], phase + N + n);
            pf_cp_async4(&sm.ph[st][2][tid], phase + 2 * N + n);
            if (NSOL == 2) pf_cp_async16(&sm.so[st][tid], solv + n);
            else pf_cp_async8(&sm.so[st][tid], solv + n);
            if (has_halo && zz >= z0 && zz < z1) {
                const long long h = hcol + pz;
                pf_cp_async4(&sm.hph[st][0][tid], phase + h);
                pf_cp_async4(&sm.hph[st][1][tid], phase + N + h);
                pf_cp_async4(&sm.hph[st][2][tid], phase + 2 * N + h);
                if (NSOL == 2) pf_cp_async16(&sm.hso[st][tid], solv + h);
                else pf_cp_async8(&sm.hso[st][tid], solv + h);
            }
        }
        pf_cp_commit();
    };
    auto own_raw = [&](int zz, float ph[3], float2 so[NSOL]) {
        const int st = (zz - zlo) % NST;
        ph[0] = sm.ph[st][0][tid];
        ph[1] = sm.ph[st][1][tid];
        ph[2] = sm.ph[st][2][tid];
        pf_unpack_sol<NSOL>(sm.so[st][tid], so);
    };

    pf_der<NSOL> dprev, dcur, dnext;
    float2 so_cur[NSOL];
    issue(zlo);
    issue(zlo + 1);
    if (use_z) issue(zlo + 2);
    pf_cp_wait1();  // planes zlo and zlo+1 have landed (each thread's own copies)
    {
        float ph[3];
        float2 so[NSOL];
        if (use_z) {
            own_raw(z0 - 1, ph, so);
            pf_derive<NSOL>(P, ph, so, dprev);
        }
        own_raw(z0, ph, so_cur);
        pf_derive<NSOL>(P, ph, so_cur, dcur);
    }
    for (int z = z0; z < z1; z++) {
        // Raw data of plane z (halo) and z+1 (own) must have landed; plane z+2
        // goes in flight into the stage plane z-1 used.
        issue(z + 2);
        pf_cp_wait1();
#pragma unroll
        for (int p = 0; p < 3; p++) {
            sm.ds[p][ly + 1][lx + 1] = dcur.s[p];
#pragma unroll
            for (int q = 0; q < NSOL; q++) sm.dc[q][p][ly + 1][lx + 1] = dcur.c[q][p];
        }
        if (has_halo) {
            const int st = (z - zlo) % NST;
            const float hph[3] = {sm.hph[st][0][tid], sm.hph[st][1][tid], sm.hph[st][2][tid]};
            float2 hso[NSOL];
            pf_unpack_sol<NSOL>(sm.hso[st][tid], hso);
            pf_der<NSOL> dh;
            pf_derive<NSOL>(P, hph, hso, dh);
#pragma unroll
            for (int p = 0; p < 3; p++) {
                sm.ds[p][hy + 1][hx + 1] = dh.s[p];
#pragma unroll
                for (int q = 0; q < NSOL; q++) sm.dc[q][p][hy + 1][hx + 1] = dh.c[q][p];
            }
        }
        __syncthreads();
        float2 so_nxt[NSOL];
        const bool have_next = z + 1 <= zhi;
        if (have_next) {
            float nph[3];
            own_raw(z + 1, nph, so_nxt);
            pf_derive<NSOL>(P, nph, so_nxt, dnext);
        }
        float acc[NSOL][3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                const float c0 = dcur.c[q][p];
                float a = sm.ds[p][ly + 1][lx] * (sm.dc[q][p][ly + 1][lx] - c0);
                a += sm.ds[p][ly + 1][lx + 2] * (sm.dc[q][p][ly + 1][lx + 2] - c0);
                if (use_y) {
                    a += sm.ds[p][ly][lx + 1] * (sm.dc[q][p][ly][lx + 1] - c0);
                    a += sm.ds[p][ly + 2][lx + 1] * (sm.dc[q][p][ly + 2][lx + 1] - c0);
                }
                if (use_z) {
                    a += dprev.s[p] * (dprev.c[q][p] - c0);
                    a += dnext.s[p] * (dnext.c[q][p] - c0);
                }
                acc[q][p] = a;
            }
        }
        if (valid) {
            const long long n = col + plane * z;
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                const float flux = dcur.s[0] * P.D[q][0] * acc[q][0] + dcur.s[1] * P.D[q][1] * acc[q][1] +
                                   dcur.s[2] * P.D[q][2] * acc[q][2];
                const float y = flux - so_cur[q].y;
                const float t = so_cur[q].x + y;
                const float comp = (t - so_cur[q].x) - y;
                so_cur[q] = make_float2(t, comp);
            }
            if (NSOL == 2)
                reinterpret_cast<float4 *>(sol_out)[n] =
                    make_float4(so_cur[0].x, so_cur[0].y, so_cur[NSOL - 1].x, so_cur[NSOL - 1].y);
            else
                sol_out[n] = so_cur[0];
        }
        __syncthreads();
        dprev = dcur;
        dcur = dnext;
#pragma unroll
        for (int q = 0; q < NSOL; q++) so_cur[q] = so_nxt[q];
    }
}

// Per-class maximum of (id mod 100000) over all slots, for the local id map.
__global__ void __launch_bounds__(256) k_id_span(const int *__restrict__ ids64, long long N,
                                                 int *__restrict__ span5) {
    __shared__ int smax[5];
    if (threadIdx.x < 5) smax[threadIdx.x] = 0;
    __syncthreads();
    int lm[5] = {0, 0, 0, 0, 0};
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N;
         n += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 6; a++) {
            const int id = ids64[6 * n + a];
            if (id < 0) lm[4] = 1;
            else if (id > 0) {
                const int c = id / PF_MAXGRAIN_PER_PHASE;
                const int r = id - c * PF_MAXGRAIN_PER_PHASE;
                if (c > 3) lm[4] = 1;
                else {
                    const int s = c == 0 ? r : r + 1;
                    if (c == 0) lm[0] = max(lm[0], s);
                    else if (c == 1) lm[1] = max(lm[1], s);
                    else if (c == 2) lm[2] = max(lm[2], s);
                    else lm[3] = max(lm[3], s);
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 5; c++) {
        int m = __reduce_max_sync(0xffffffffu, lm[c]);
        if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(&smax[c], m);
    }
    __syncthreads();
    if (threadIdx.x < 5 && smax[threadIdx.x] > 0) atomicMax(&span5[threadIdx.x], smax[threadIdx.x]);
}

__device__ __forceinline__ int pf_to_local(int id, const pf_f32_map &map) {
    if (id <= 0) return 0;
    const int c = id / PF_MAXGRAIN_PER_PHASE;
    const int r = id - c * PF_MAXGRAIN_PER_PHASE;
    return map.off[c] + r + (c > 0 ? 1 : 0);
}

__device__ __forceinline__ int pf_to_global(int l, const pf_f32_map &map) {
    if (l == 0) return 0;
    const int c = l <= map.off[1] ? 0 : (l <= map.off[2] ? 1 : (l <= map.off[3] ? 2 : 3));
    return c * PF_MAXGRAIN_PER_PHASE + (l - map.off[c]) - (c > 0 ? 1 : 0);
}

// Reference layout (FP64, 6 slots) -> compact FP32 layout.  A cell with more
// than four non-zero slots keeps its four largest (first maximum wins) and is
// renormalised; such cells are counted in n_truncated.
__global__ void __launch_bounds__(256) k_pack_f32(long long N, int nsol, const pf_f32_map map,
                                                  const int *__restrict__ ids64,
                                                  const double *__restrict__ phi64,
                                                  const double *__restrict__ phase64,
                                                  const double *__restrict__ C64,
                                                  ushort4 *__restrict__ gid, float4 *__restrict__ phi,
                                                  float *__restrict__ phase, float2 *__restrict__ sol,
                                                  unsigned int *__restrict__ n_truncated) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    int id[6];
    double v[6];
#pragma unroll
    for (int a = 0; a < 6; a++) {
        id[a] = ids64[6 * n + a];
        v[a] = phi64[6 * n + a];
    }
#pragma unroll
    for (int a = 0; a < 4; a++) {
        int mx = a;
#pragma unroll
        for (int b = a + 1; b < 6; b++)
            if (v[b] > v[mx]) mx = b;
#pragma unroll
        for (int b = a + 1; b < 6; b++)
            if (b == mx) {
                double t = v[a]; v[a] = v[b]; v[b] = t;
                int ti = id[a]; id[a] = id[b]; id[b] = ti;
            }
    }
    const bool trunc = (v[4] > 0.0 && id[4] != 0) || (v[5] > 0.0 && id[5] != 0);
    double ph[3] = {phase64[3 * n], phase64[3 * n + 1], phase64[3 * n + 2]};
    if (trunc) {
        atomicAdd(n_truncated, 1u);
        double s = v[0] + v[1] + v[2] + v[3];
        ph[0] = ph[1] = ph[2] = 0.0;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            v[a] /= s;
            const int c = id[a] / PF_MAXGRAIN_PER_PHASE;
            const int p = id[a] == 0 ? 0 : (c > 0 ? c : 1);
            if (p >= 1 && p <= 3) ph[p - 1] += v[a];
        }
    }
    int l[4];
#pragma unroll
    for (int a = 0; a < 4; a++) l[a] = pf_to_local(id[a], map);
    gid[n] = make_ushort4((unsigned short)l[0], (unsigned short)l[1], (unsigned short)l[2],
                          (unsigned short)l[3]);
    phi[n] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
    phase[n] = (float)ph[0];
    phase[N + n] = (float)ph[1];
    phase[2 * N + n] = (float)ph[2];
    for (int q = 0; q < nsol; q++) {
        const double c = C64[q * N + n];
        const float f = (float)c;
        sol[n * nsol + q] = make_float2(f, (float)((double)f - c));
    }
}

// Compact FP32 layout -> reference layout (FP64, 6 slots); phase
// concentrations re-partitioned in FP64 from the compensated solute totals.
__global__ void __launch_bounds__(256) k_unpack_f32(const __grid_constant__ pf_step_params P,
                                                    const pf_f32_map map,
                                                    const ushort4 *__restrict__ gid,
                                                    const float4 *__restrict__ phi,
                                                    const float *__restrict__ phase,
                                                    const float2 *__restrict__ sol,
                                                    int *__restrict__ ids64, double *__restrict__ phi64,
                                                    double *__restrict__ phase64,
                                                    double *__restrict__ conc64,
                                                    double *__restrict__ C64) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long N = P.N;
    if (n >= N) return;
    const ushort4 g = gid[n];
    const float4 v = phi[n];
    const int l[4] = {g.x, g.y, g.z, g.w};
    const float fv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int a = 0; a < 4; a++) {
        ids64[6 * n + a] = pf_to_global(l[a], map);
        phi64[6 * n + a] = (double)fv[a];
    }
    ids64[6 * n + 4] = 0; ids64[6 * n + 5] = 0;
    phi64[6 * n + 4] = 0.0; phi64[6 * n + 5] = 0.0;
    double ph[3] = {(double)phase[n], (double)phase[N + n], (double)phase[2 * N + n]};
    phase64[3 * n] = ph[0]; phase64[3 * n + 1] = ph[1]; phase64[3 * n + 2] = ph[2];
    for (int q = 0; q < P.nsol; q++) {
        const float2 s = sol[n * P.nsol + q];
        const double c = (double)s.x - (double)s.y;
        C64[q * N + n] = c;
        if (conc64) {
            for (int i = 0; i < 3; i++) {
                double t1 = 0., t2 = 0.;
                for (int j = 0; j < 3; j++) {
                    t1 += ph[j] * P.k[q][i + 3 * j];
                    t2 += ph[j] * P.c[q][i + 3 * j];
                }
                conc64[q * 3 * N + 3 * n + i] = (c - t2) / t1;
            }
        }
    }
}

inline unsigned pf_blocks(long long N, int threads) { return (unsigned)((N + threads - 1) / threads); }

}  // namespace

cudaError_t pf_launch_id_span(const int *ids64, long long N, int *span5, cudaStream_t s) {
    long long blocks = (N + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    k_id_span<<<(unsigned)blocks, 256, 0, s>>>(ids64, N, span5);
    return cudaGetLastError();
}

cudaError_t pf_launch_pack_f32(long long N, int nsol, const pf_f32_map &map, const int *ids64,
                               const double *phi64, const double *phase64, const double *C64,
                               ushort4 *gid, float4 *phi, float *phase, float2 *sol,
                               unsigned int *n_truncated, cudaStream_t s) {
    k_pack_f32<<<pf_blocks(N, 256), 256, 0, s>>>(N, nsol, map, ids64, phi64, phase64, C64, gid, phi,
                                                 phase, sol, n_truncated);
    return cudaGetLastError();
}

cudaError_t pf_launch_unpack_f32(const pf_step_params &P, const pf_f32_map &map, const ushort4 *gid,
                                 const float4 *phi, const float *phase, const float2 *sol, int *ids64,
                                 double *phi64, double *phase64, double *conc64, double *C64,
                                 cudaStream_t s) {
    k_unpack_f32<<<pf_blocks(P.N, 256), 256, 0, s>>>(P, map, gid, phi, phase, sol, ids64, phi64, phase64,
                                                   conc64, C64);
    return cudaGetLastError();
}

cudaError_t pf_launch_phase_f32(const pf_f32_params &P, const ushort4 *gid1, const float4 *phi1,
                                ushort4 *gid2, float4 *phi2, float *phase, const float2 *sol,
                                cudaStream_t s) {
    if (P.nsol == 2)
        k_phase_f32<2><<<pf_blocks(P.N, 256), 256, 0, s>>>(P, gid1, phi1, gid2, phi2, phase, sol);
    else
        k_phase_f32<1><<<pf_blocks(P.N, 256), 256, 0, s>>>(P, gid1, phi1, gid2, phi2, phase, sol);
    return cudaGetLastError();
}

template <int NSOL, int TX, int TY>
static cudaError_t pf_launch_diffuse_tiled(const pf_f32_params &P, const float *phase, const float2 *sol_in,
                                           float2 *sol_out, cudaStream_t s) {
    const int tiles = ((P.ix + TX - 1) / TX) * ((P.iy + TY - 1) / TY);
    // z chunk: enough blocks for several waves on 152 SMs, at least 8 planes
    // per block to amortise the extra planes of the prologue.
    int zchunk = P.iz;
    while (zchunk > 8 && (long long)tiles * ((P.iz + zchunk - 1) / zchunk) < 152 * 16) zchunk = (zchunk + 1) / 2;
    const dim3 grid((unsigned)tiles, (unsigned)((P.iz + zchunk - 1) / zchunk));
    const size_t smem = sizeof(pf_diff_smem<NSOL, TX, TY, 3>);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_diffuse_f32<NSOL, TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    k_diffuse_f32<NSOL, TX, TY><<<grid, TX * TY, smem, s>>>(P, phase, sol_in, sol_out, zchunk);
    return cudaGetLastError();
}

cudaError_t pf_launch_diffuse_f32(const pf_f32_params &P, const float *phase, const float2 *sol_in,
                                  float2 *sol_out, cudaStream_t s) {
    if (P.nsol == 2) return pf_launch_diffuse_tiled<2, 32, 8>(P, phase, sol_in, sol_out, s);
    return pf_launch_diffuse_tiled<1, 32, 8>(P, phase, sol_in, sol_out, s);
}
