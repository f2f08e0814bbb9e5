// pf_f32_diffuse.cu -- the diffusion sub-step (solver.cpp:343-372) on the
// compact FP32 layout, all solutes at once, sm_103a.
//
// Each cell contributes to its neighbours' fluxes through two derived
// quantities: s_p = sqrt(phi_p) (stored directly in the phase planes, so the
// flux weight sqrt(phi_p^nb phi_p) is the product s_p^nb s_p) and the
// partitioned phase concentrations c_p (solver.cpp:389-405).  Both are formed
// once per cell per sub-step:
//
// * A block owns a TX x TY tile of the x-y plane and marches up a chunk of z
//   planes.  Raw data (s_p and the solute totals) of the cell column and of the
//   tile's one-cell in-plane halo is staged into shared memory with cp.async two
//   planes ahead, so its HBM latency overlaps the arithmetic of the current
//   plane.  Every thread reads back only what it copied itself, so the stages
//   need no barrier.
// * The derived records of the current plane (s_p, c_p per solute, packed in
//   one 16-byte record per phase) sit in shared memory for the in-plane
//   neighbours; those of the planes below and above the thread's own cell sit in
//   registers, rotated without copies by a three-way unrolled z loop.
// * The solute total is advanced with a Kahan-compensated sum.  D carries
//   dt_sub/dx^2.
#include <type_traits>
#include "pf_f32.cuh"
#include "pf_kernels.h"

namespace {

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int PENDING>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING)); }

template <int NSOL> struct Vec;
template <> struct Vec<1> { using T = float2; };
template <> struct Vec<2> { using T = float4; };

// Derived record of one cell.
template <int NSOL>
struct Der {
    float s[3];
    float c[NSOL][3];
};

template <int NSOL>
__device__ __forceinline__ void unpack_sol(const typename Vec<NSOL>::T &v, float C[NSOL], float comp[NSOL]);
template <>
__device__ __forceinline__ void unpack_sol<1>(const float2 &v, float C[1], float comp[1]) { C[0] = v.x; comp[0] = v.y; }
template <>
__device__ __forceinline__ void unpack_sol<2>(const float4 &v, float C[2], float comp[2]) {
    C[0] = v.x; comp[0] = v.y; C[1] = v.z; comp[1] = v.w;
}

// Shared record per phase: (s_p, c_p of each solute).
template <int NSOL>
__device__ __forceinline__ typename Vec<NSOL>::T pack_rec(float s, const float c[NSOL]);
template <>
__device__ __forceinline__ float2 pack_rec<1>(float s, const float c[1]) { return make_float2(s, c[0]); }
template <>
__device__ __forceinline__ float4 pack_rec<2>(float s, const float c[2]) { return make_float4(s, c[0], c[1], 0.f); }
__device__ __forceinline__ float rec_c(const float2 &v, int) { return v.y; }
__device__ __forceinline__ float rec_c(const float4 &v, int q) { return q == 0 ? v.y : v.z; }

template <int NSOL>
__device__ __forceinline__ void derive(const pf_f32_params &P, const float s[3], const float C[NSOL], Der<NSOL> &d) {
    const float ph[3] = {s[0] * s[0], s[1] * s[1], s[2] * s[2]};
#pragma unroll
    for (int p = 0; p < 3; p++) d.s[p] = s[p];
#pragma unroll
    for (int q = 0; q < NSOL; q++) pf_partition_q(P, q, C[q], ph, d.c[q]);
}

// Variant 0.  Raw data is prefetched two planes ahead (three stages); the
// first NH threads also stage and derive the tile's halo cells.
template <int NSOL, int TX, int TY>
struct Smem {
    static constexpr int NT = TX * TY, NH = 2 * TX + 2 * TY, W = TX + 2, H = TY + 2, NST = 3;
    using SV = typename Vec<NSOL>::T;
    SV so[NST][NT];       // raw solute totals (+ compensation), own cells
    SV hso[NST][NH];      // raw solute totals, halo cells
    float sp[NST][3][NT];  // raw s_p, own cells
    float hsp[NST][3][NH]; // raw s_p, halo cells
    SV rec[3][H][W];      // derived records of the current plane, with halo
};

template <int NSOL, int NNB, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, 1024 / (TX * TY)) k_diffuse(const __grid_constant__ pf_f32_params P,
                                                                     const float *__restrict__ sphase,
                                                                     const float2 *__restrict__ sol_in,
                                                                     float2 *__restrict__ sol_out, int zchunk) {
    using S = Smem<NSOL, TX, TY>;
    using SV = typename Vec<NSOL>::T;
    static_assert(S::NH <= S::NT, "halo needs one thread per halo cell");
    constexpr bool use_y = NNB >= 4, use_z = NNB >= 6;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S &sm = *reinterpret_cast<S *>(smem_raw);

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
    // Halo cells go to the first NH threads: whole rows to whole warps, so the
    // halo copies stay coalesced.
    const int hid = tid;
    const bool has_halo = hid < S::NH;
    int hx, hy;
    if (hid < TX) { hx = hid; hy = -1; }
    else if (hid < 2 * TX) { hx = hid - TX; hy = TY; }
    else if (hid < 2 * TX + TY) { hx = -1; hy = hid - 2 * TX; }
    else { hx = TX; hy = hid - 2 * TX - TY; }
    const long long hcol = pf_mod(tx0 + hx, ix) + (long long)ix * pf_mod(ty0 + hy, iy);
    const int z0 = blockIdx.y * zchunk;
    const int z1 = min(z0 + zchunk, iz);
    const int zlo = use_z ? z0 - 1 : z0, zhi = use_z ? z1 : z1 - 1;
    const SV *solv = reinterpret_cast<const SV *>(sol_in);
    const float *own_s = sphase + col;
    const float *halo_s = sphase + hcol;
    const SV *own_v = solv + col;
    const SV *halo_v = solv + hcol;

    // Plane zz lives in stage (zz - zlo) % 3.  Every call site below knows that
    // stage at compile time: the z loop is unrolled by three and zlo - z0 is
    // fixed by use_z, so no integer division appears in the loop.
    constexpr int OFF = use_z ? 1 : 0;  // z0 - zlo
    auto issue = [&](int zz, int st) {
        if (zz >= zlo && zz <= zhi) {
            const int zw = zz < 0 ? zz + iz : (zz >= iz ? zz - iz : zz);  // |wrap| <= 1 plane
            const long long off = plane * zw;
            cp_async4(&sm.sp[st][0][tid], own_s + off);
            cp_async4(&sm.sp[st][1][tid], own_s + N + off);
            cp_async4(&sm.sp[st][2][tid], own_s + 2 * N + off);
            if (NSOL == 2) cp_async16(&sm.so[st][tid], own_v + off);
            else cp_async8(&sm.so[st][tid], own_v + off);
            if (has_halo && zz >= z0 && zz < z1) {
                cp_async4(&sm.hsp[st][0][hid], halo_s + off);
                cp_async4(&sm.hsp[st][1][hid], halo_s + N + off);
                cp_async4(&sm.hsp[st][2][hid], halo_s + 2 * N + off);
                if (NSOL == 2) cp_async16(&sm.hso[st][hid], halo_v + off);
                else cp_async8(&sm.hso[st][hid], halo_v + off);
            }
        }
        cp_commit();
    };
    auto derive_own = [&](int st, Der<NSOL> &d) {
        const float s3[3] = {sm.sp[st][0][tid], sm.sp[st][1][tid], sm.sp[st][2][tid]};
        float C[NSOL], comp[NSOL];
        unpack_sol<NSOL>(sm.so[st][tid], C, comp);
        derive<NSOL>(P, s3, C, d);
    };

    // One plane; J is the position in the three-way unrolled loop, so the
    // stages of planes z, z+1, z+2 are constants.  prev/cur/next rotate.
    auto body = [&](int z, auto J, const Der<NSOL> &prev, const Der<NSOL> &cur, Der<NSOL> &next) {
        constexpr int j = decltype(J)::value;
        constexpr int st_z = (OFF + j) % 3, st_z1 = (OFF + j + 1) % 3, st_z2 = (OFF + j + 2) % 3;
        issue(z + 2, st_z2);
        cp_wait<1>();  // planes z (halo) and z+1 (own) have landed
#pragma unroll
        for (int p = 0; p < 3; p++) {
            float cp[NSOL];
#pragma unroll
            for (int q = 0; q < NSOL; q++) cp[q] = cur.c[q][p];
            sm.rec[p][ly + 1][lx + 1] = pack_rec<NSOL>(cur.s[p], cp);
        }
        if (has_halo) {
            const float s3[3] = {sm.hsp[st_z][0][hid], sm.hsp[st_z][1][hid], sm.hsp[st_z][2][hid]};
            float C[NSOL], comp[NSOL];
            unpack_sol<NSOL>(sm.hso[st_z][hid], C, comp);
            Der<NSOL> dh;
            derive<NSOL>(P, s3, C, dh);
#pragma unroll
            for (int p = 0; p < 3; p++) {
                float cp[NSOL];
#pragma unroll
                for (int q = 0; q < NSOL; q++) cp[q] = dh.c[q][p];
                sm.rec[p][hy + 1][hx + 1] = pack_rec<NSOL>(dh.s[p], cp);
            }
        }
        __syncthreads();
        if (z + 1 <= zhi) derive_own(st_z1, next);
        float acc[NSOL][3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const SV l = sm.rec[p][ly + 1][lx], r = sm.rec[p][ly + 1][lx + 2];
            SV d, u;
            if (use_y) { d = sm.rec[p][ly][lx + 1]; u = sm.rec[p][ly + 2][lx + 1]; }
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                const float c0 = cur.c[q][p];
                float a = l.x * (rec_c(l, q) - c0);
                a += r.x * (rec_c(r, q) - c0);
                if (use_y) {
                    a += d.x * (rec_c(d, q) - c0);
                    a += u.x * (rec_c(u, q) - c0);
                }
                if (use_z) {
                    a += prev.s[p] * (prev.c[q][p] - c0);
                    a += next.s[p] * (next.c[q][p] - c0);
                }
                acc[q][p] = a;
            }
        }
        if (valid) {
            float C[NSOL], comp[NSOL];
            unpack_sol<NSOL>(sm.so[st_z][tid], C, comp);
            float o[2 * NSOL];
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                const float flux = cur.s[0] * P.D[q][0] * acc[q][0] + cur.s[1] * P.D[q][1] * acc[q][1] +
                                   cur.s[2] * P.D[q][2] * acc[q][2];
                const float y = flux - comp[q];
                const float t = C[q] + y;
                o[2 * q] = t;
                o[2 * q + 1] = (t - C[q]) - y;
            }
            const long long n = col + plane * z;
            if (NSOL == 2) reinterpret_cast<float4 *>(sol_out)[n] = make_float4(o[0], o[1], o[2], o[2 * NSOL - 1]);
            else sol_out[n] = make_float2(o[0], o[1]);
        }
        __syncthreads();
    };

    Der<NSOL> A, B, Cd;
    // Planes zlo .. z0+1 in flight (stages 0, 1[, 2]); zlo and z0 must have landed.
    issue(zlo, 0);
    issue(zlo + 1, 1);
    if (use_z) issue(zlo + 2, 2);
    cp_wait<1>();
    if (use_z) derive_own(0, A);
    derive_own(OFF, B);
    for (int z = z0; z < z1; z += 3) {
        body(z, std::integral_constant<int, 0>{}, A, B, Cd);
        if (z + 1 < z1) body(z + 1, std::integral_constant<int, 1>{}, B, Cd, A);
        if (z + 2 < z1) body(z + 2, std::integral_constant<int, 2>{}, Cd, A, B);
    }
}

// ---------------------------------------------------------------------------
// Variant 1: halo warps.  A block holds TY interior warps (one 32-cell row of
// the tile each) and three halo warps: the row above, the row below, and the
// two halo columns (lanes 0..TY-1 and TY..2TY-1).  Every thread owns one cell
// column of the tile with its halo, stages that column's raw data and forms
// that column's derived record for every plane, so each warp does exactly one
// batch of derived records per plane and no warp waits at the barrier for
// another's halo work.  Only interior threads compute fluxes.
// ---------------------------------------------------------------------------
template <int NSOL, int TY>
struct SmemHW {
    static constexpr int TX = 32, NT = 32 * (TY + 3), W = TX + 2, H = TY + 2, NST = 3;
    using SV = typename Vec<NSOL>::T;
    SV so[NST][NT];
    float sp[NST][3][NT];
    SV rec[3][H][W];
};

template <int NSOL, int NNB, int TY>
__global__ void __launch_bounds__(32 * (TY + 3), (TY <= 4 ? 4 : (TY <= 8 ? 2 : 1)))
    k_diffuse_hw(const __grid_constant__ pf_f32_params P, const float *__restrict__ sphase,
                 const float2 *__restrict__ sol_in, float2 *__restrict__ sol_out, int zchunk) {
    using S = SmemHW<NSOL, TY>;
    using SV = typename Vec<NSOL>::T;
    constexpr int TX = S::TX;
    constexpr bool use_y = NNB >= 4, use_z = NNB >= 6;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S &sm = *reinterpret_cast<S *>(smem_raw);

    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const long long N = P.N;
    const long long plane = (long long)ix * iy;
    const int tiles_x = (ix + TX - 1) / TX;
    const int tx0 = (int)(blockIdx.x % tiles_x) * TX;
    const int ty0 = (int)(blockIdx.x / tiles_x) * TY;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    int sx = 0, sy = 0;  // slot in the record tile
    bool active = true;
    if (w < TY) { sx = l + 1; sy = w + 1; }
    else if (w == TY) { sx = l + 1; sy = 0; }
    else if (w == TY + 1) { sx = l + 1; sy = TY + 1; }
    else if (l < TY) { sx = 0; sy = l + 1; }
    else if (l < 2 * TY) { sx = TX + 1; sy = l - TY + 1; }
    else active = false;
    const bool interior = w < TY;
    const bool valid = interior && (tx0 + l < ix) && (ty0 + w < iy);
    const long long col = pf_mod(tx0 + sx - 1, ix) + (long long)ix * pf_mod(ty0 + sy - 1, iy);
    const int z0 = blockIdx.y * zchunk;
    const int z1 = min(z0 + zchunk, iz);
    const int zlo = use_z ? z0 - 1 : z0, zhi = use_z ? z1 : z1 - 1;
    const SV *own_v = reinterpret_cast<const SV *>(sol_in) + col;
    const float *own_s = sphase + col;

    auto stage = [&](int zz) { return (zz - zlo) % S::NST; };
    auto issue = [&](int zz) {
        if (active && zz >= zlo && zz <= zhi) {
            const int st = stage(zz);
            const long long off = plane * pf_mod(zz, iz);
            cp_async4(&sm.sp[st][0][tid], own_s + off);
            cp_async4(&sm.sp[st][1][tid], own_s + N + off);
            cp_async4(&sm.sp[st][2][tid], own_s + 2 * N + off);
            if (NSOL == 2) cp_async16(&sm.so[st][tid], own_v + off);
            else cp_async8(&sm.so[st][tid], own_v + off);
        }
        cp_commit();
    };
    auto derive_own = [&](int zz, Der<NSOL> &d) {
        const int st = stage(zz);
        const float s3[3] = {sm.sp[st][0][tid], sm.sp[st][1][tid], sm.sp[st][2][tid]};
        float C[NSOL], comp[NSOL];
        unpack_sol<NSOL>(sm.so[st][tid], C, comp);
        derive<NSOL>(P, s3, C, d);
    };
    auto body = [&](int z, const Der<NSOL> &prev, const Der<NSOL> &cur, Der<NSOL> &next) {
        issue(z + 2);
        cp_wait<1>();
        if (active) {
#pragma unroll
            for (int p = 0; p < 3; p++) {
                float cp[NSOL];
#pragma unroll
                for (int q = 0; q < NSOL; q++) cp[q] = cur.c[q][p];
                sm.rec[p][sy][sx] = pack_rec<NSOL>(cur.s[p], cp);
            }
        }
        __syncthreads();
        if (active && z + 1 <= zhi) derive_own(z + 1, next);
        if (valid) {
            float acc[NSOL][3];
#pragma unroll
            for (int p = 0; p < 3; p++) {
                const SV lr = sm.rec[p][sy][sx - 1], rr = sm.rec[p][sy][sx + 1];
                SV d, u;
                if (use_y) { d = sm.rec[p][sy - 1][sx]; u = sm.rec[p][sy + 1][sx]; }
#pragma unroll
                for (int q = 0; q < NSOL; q++) {
                    const float c0 = cur.c[q][p];
                    float a = lr.x * (rec_c(lr, q) - c0);
                    a += rr.x * (rec_c(rr, q) - c0);
                    if (use_y) {
                        a += d.x * (rec_c(d, q) - c0);
                        a += u.x * (rec_c(u, q) - c0);
                    }
                    if (use_z) {
                        a += prev.s[p] * (prev.c[q][p] - c0);
                        a += next.s[p] * (next.c[q][p] - c0);
                    }
                    acc[q][p] = a;
                }
            }
            float C[NSOL], comp[NSOL];
            unpack_sol<NSOL>(sm.so[stage(z)][tid], C, comp);
            float o[2 * NSOL];
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                const float flux = cur.s[0] * P.D[q][0] * acc[q][0] + cur.s[1] * P.D[q][1] * acc[q][1] +
                                   cur.s[2] * P.D[q][2] * acc[q][2];
                const float y = flux - comp[q];
                const float t = C[q] + y;
                o[2 * q] = t;
                o[2 * q + 1] = (t - C[q]) - y;
            }
            const long long n = col + plane * z;
            if (NSOL == 2) reinterpret_cast<float4 *>(sol_out)[n] = make_float4(o[0], o[1], o[2], o[2 * NSOL - 1]);
            else sol_out[n] = make_float2(o[0], o[1]);
        }
        __syncthreads();
    };

    Der<NSOL> A, B, Cd;
    for (int zz = zlo; zz <= z0 + 1; zz++) issue(zz);
    cp_wait<1>();
    if (active) {
        if (use_z) derive_own(z0 - 1, A);
        derive_own(z0, B);
    }
    for (int z = z0; z < z1; z += 3) {
        body(z, A, B, Cd);
        if (z + 1 < z1) body(z + 1, B, Cd, A);
        if (z + 2 < z1) body(z + 2, Cd, A, B);
    }
}

template <int NSOL, int NNB, int TY>
cudaError_t launch_hw(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                      cudaStream_t s, int zchunk) {
    using S = SmemHW<NSOL, TY>;
    const int tiles = ((P.ix + 31) / 32) * ((P.iy + TY - 1) / TY);
    const dim3 grid((unsigned)tiles, (unsigned)((P.iz + zchunk - 1) / zchunk));
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_diffuse_hw<NSOL, NNB, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(S));
        if (e != cudaSuccess) return e;
        configured = true;
    }
    k_diffuse_hw<NSOL, NNB, TY><<<grid, S::NT, sizeof(S), s>>>(P, sphase, sol_in, sol_out, zchunk);
    return cudaGetLastError();
}

template <int NSOL, int NNB, int TY>
cudaError_t launch_one(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int zchunk) {
    constexpr int TX = 32;
    using S = Smem<NSOL, TX, TY>;
    const int tiles = ((P.ix + TX - 1) / TX) * ((P.iy + TY - 1) / TY);
    const dim3 grid((unsigned)tiles, (unsigned)((P.iz + zchunk - 1) / zchunk));
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_diffuse<NSOL, NNB, TX, TY>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(S));
        if (e != cudaSuccess) return e;
        configured = true;
    }
    k_diffuse<NSOL, NNB, TX, TY><<<grid, TX * TY, sizeof(S), s>>>(P, sphase, sol_in, sol_out, zchunk);
    return cudaGetLastError();
}

template <int NSOL, int NNB>
cudaError_t launch_ty(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                      cudaStream_t s, int ty, int zchunk, int variant) {
    if (variant == 1) {
        switch (ty) {
            case 4: return launch_hw<NSOL, NNB, 4>(P, sphase, sol_in, sol_out, s, zchunk);
            case 16: return launch_hw<NSOL, NNB, 16>(P, sphase, sol_in, sol_out, s, zchunk);
            default: return launch_hw<NSOL, NNB, 8>(P, sphase, sol_in, sol_out, s, zchunk);
        }
    }
    switch (ty) {
        case 4: return launch_one<NSOL, NNB, 4>(P, sphase, sol_in, sol_out, s, zchunk);
        case 16: return launch_one<NSOL, NNB, 16>(P, sphase, sol_in, sol_out, s, zchunk);
        default: return launch_one<NSOL, NNB, 8>(P, sphase, sol_in, sol_out, s, zchunk);
    }
}

template <int NSOL>
cudaError_t launch_nnb(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int ty, int zchunk, int variant) {
    if (P.nnb >= 6) return launch_ty<NSOL, 6>(P, sphase, sol_in, sol_out, s, ty, zchunk, variant);
    if (P.nnb >= 4) return launch_ty<NSOL, 4>(P, sphase, sol_in, sol_out, s, ty, zchunk, variant);
    return launch_ty<NSOL, 2>(P, sphase, sol_in, sol_out, s, ty, zchunk, variant);
}

}  // namespace

pf_diff_cfg pf_diffuse_default_cfg(const pf_f32_params &P) {
    pf_diff_cfg c;
    c.ty = 8;
    c.variant = 0;
    const int tiles = ((P.ix + 31) / 32) * ((P.iy + 7) / 8);
    // About two waves of 4 resident blocks on 152 SMs, at least 8 planes per block.
    int z = P.iz;
    while (z > 8 && (long long)tiles * ((P.iz + z - 1) / z) < 152 * 4 * 2) z = (z + 1) / 2;
    c.zchunk = z < 1 ? 1 : z;
    return c;
}

int pf_diffuse_candidates(const pf_f32_params &P, pf_diff_cfg *out, int max) {
    const int tys[3] = {4, 8, 16};
    const int zcs[5] = {8, 16, 32, 64, 128};
    int n = 0;
    for (int d = 0; d <= 1; d++)
        for (int a = 0; a < 3; a++) {
            if (P.iz == 1) {
                if (n < max) out[n++] = {tys[a], 1, d};
                continue;
            }
            for (int b = 0; b < 5; b++) {
                if (zcs[b] > P.iz && b > 0) break;
                if (n < max) out[n++] = {tys[a], zcs[b] < P.iz ? zcs[b] : P.iz, d};
            }
        }
    return n;
}

cudaError_t pf_launch_diffuse_f32(const pf_f32_params &P, const float *sphase, const float2 *sol_in,
                                  float2 *sol_out, cudaStream_t s, const pf_diff_cfg *cfg) {
    const pf_diff_cfg c = cfg ? *cfg : pf_diffuse_default_cfg(P);
    if (P.nsol == 2) return launch_nnb<2>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk, c.variant);
    return launch_nnb<1>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk, c.variant);
}
