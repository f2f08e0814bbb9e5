// pf_f32_diffuse.cu -- the diffusion sub-step (solver.cpp:343-372) on the
// compact FP32 layout, all solutes at once, sm_103a.
//
// Each cell enters its neighbours' fluxes through a derived record formed once
// per cell per sub-step:
//   s_p = sqrt(phi_p)   stored directly in the phase planes, so the flux weight
//                       sqrt(phi_p^nb phi_p) (solver.cpp:363) is s_p^nb s_p;
//   c_p                 the partitioned carbon of phase p (solver.cpp:389-405);
//   r                   for the second solute (Mn), whose partition is separable
//                       (c_Mn,p = a_p r with r = C_Mn / sum_j phi_j a_j), so
//                       c_Mn,p^nb - c_Mn,p = a_p (r^nb - r).
// A record is 32 bytes: R1 = (s_0, s_1, s_2, r), R2 = (c_0, c_1, c_2, -).
//
// * A block owns a 32 x TY tile of the x-y plane and marches up a chunk of z
//   planes.  Raw data (s_p and the solute totals) of the cell column and of the
//   tile's one-cell in-plane halo is staged into shared memory with cp.async two
//   planes ahead, so its HBM latency overlaps the arithmetic of the current
//   plane.  Every thread reads back only what it copied itself, so the stages
//   need no barrier; the stage of each plane is a compile-time constant of the
//   three-way unrolled z loop.
// * The records of the current plane (with halo) sit in shared memory for the
//   in-plane neighbours; those of the planes below and above the thread's own
//   cell sit in registers, rotated without copies by the unrolled loop.
//   Shared-memory bandwidth, not HBM, limits this stencil, so records are kept
//   at 32 bytes.
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

template <int NSOL>
__device__ __forceinline__ void unpack_sol(const typename Vec<NSOL>::T &v, float C[NSOL], float comp[NSOL]);
template <>
__device__ __forceinline__ void unpack_sol<1>(const float2 &v, float C[1], float comp[1]) { C[0] = v.x; comp[0] = v.y; }
template <>
__device__ __forceinline__ void unpack_sol<2>(const float4 &v, float C[2], float comp[2]) {
    C[0] = v.x; comp[0] = v.y; C[1] = v.z; comp[1] = v.w;
}

// Derived record of one cell (register form).
struct Rec {
    float s[3], c[3], r;
};

template <int NSOL>
__device__ __forceinline__ void derive(const pf_f32_params &P, const float s[3], const float C[NSOL], Rec &d) {
    const float ph[3] = {s[0] * s[0], s[1] * s[1], s[2] * s[2]};
#pragma unroll
    for (int p = 0; p < 3; p++) d.s[p] = s[p];
    pf_partition_q(P, 0, C[0], ph, d.c);
    if (NSOL == 2) {
        const float S = ph[0] * P.a[1][0] + ph[1] * P.a[1][1] + ph[2] * P.a[1][2];
        d.r = __fdividef(C[NSOL - 1], S);
    } else {
        d.r = 0.f;
    }
}

// Flux sums of the cell: aC[p] += s_p^nb (c_p^nb - c_p), aM[p] += s_p^nb (r^nb - r).
template <int NSOL>
__device__ __forceinline__ void accumulate(const float4 &r1, const float4 &r2, const Rec &cur, float aC[3],
                                           float aM[3]) {
    aC[0] += r1.x * (r2.x - cur.c[0]);
    aC[1] += r1.y * (r2.y - cur.c[1]);
    aC[2] += r1.z * (r2.z - cur.c[2]);
    if (NSOL == 2) {
        const float dr = r1.w - cur.r;
        aM[0] += r1.x * dr;
        aM[1] += r1.y * dr;
        aM[2] += r1.z * dr;
    }
}
__device__ __forceinline__ float4 rec1(const Rec &d) { return make_float4(d.s[0], d.s[1], d.s[2], d.r); }
__device__ __forceinline__ float4 rec2(const Rec &d) { return make_float4(d.c[0], d.c[1], d.c[2], 0.f); }

template <int NSOL, int TX, int TY>
struct Smem {
    static constexpr int NT = TX * TY, NH = 2 * TX + 2 * TY, W = TX + 2, H = TY + 2, NST = 3;
    using SV = typename Vec<NSOL>::T;
    SV so[NST][NT];        // raw solute totals (+ compensation), own cells
    SV hso[NST][NH];       // raw solute totals, halo cells
    float sp[NST][3][NT];  // raw s_p, own cells
    float hsp[NST][3][NH]; // raw s_p, halo cells
    float4 r1[H][W];       // records of the current plane, with halo
    float4 r2[H][W];
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
    // Flux coefficients of the cell's own side: D_p (carbon) and D_p a_p (Mn).
    float DC[3], DM[3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        DC[p] = P.D[0][p];
        DM[p] = NSOL == 2 ? P.D[NSOL - 1][p] * P.a[NSOL - 1][p] : 0.f;
    }

    // Plane zz lives in stage (zz - zlo) % 3; every call site knows it at
    // compile time (OFF = z0 - zlo).
    constexpr int OFF = use_z ? 1 : 0;
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
    auto derive_own = [&](int st, Rec &d) {
        const float s3[3] = {sm.sp[st][0][tid], sm.sp[st][1][tid], sm.sp[st][2][tid]};
        float C[NSOL], comp[NSOL];
        unpack_sol<NSOL>(sm.so[st][tid], C, comp);
        derive<NSOL>(P, s3, C, d);
    };

    // One plane; J is the position in the unrolled loop.  prev/cur/next rotate.
    auto body = [&](int z, auto J, const Rec &prev, const Rec &cur, Rec &next) {
        constexpr int j = decltype(J)::value;
        constexpr int st_z = (OFF + j) % 3, st_z1 = (OFF + j + 1) % 3, st_z2 = (OFF + j + 2) % 3;
        issue(z + 2, st_z2);
        cp_wait<1>();  // planes z (halo) and z+1 (own) have landed
        sm.r1[ly + 1][lx + 1] = rec1(cur);
        sm.r2[ly + 1][lx + 1] = rec2(cur);
        if (has_halo) {
            const float s3[3] = {sm.hsp[st_z][0][hid], sm.hsp[st_z][1][hid], sm.hsp[st_z][2][hid]};
            float C[NSOL], comp[NSOL];
            unpack_sol<NSOL>(sm.hso[st_z][hid], C, comp);
            Rec dh;
            derive<NSOL>(P, s3, C, dh);
            sm.r1[hy + 1][hx + 1] = rec1(dh);
            sm.r2[hy + 1][hx + 1] = rec2(dh);
        }
        __syncthreads();
        if (z + 1 <= zhi) derive_own(st_z1, next);
        // Neighbours in the reference order x-, x+, y-, y+, z-, z+.
        float aC[3] = {0.f, 0.f, 0.f}, aM[3] = {0.f, 0.f, 0.f};
        accumulate<NSOL>(sm.r1[ly + 1][lx], sm.r2[ly + 1][lx], cur, aC, aM);
        accumulate<NSOL>(sm.r1[ly + 1][lx + 2], sm.r2[ly + 1][lx + 2], cur, aC, aM);
        if (use_y) {
            accumulate<NSOL>(sm.r1[ly][lx + 1], sm.r2[ly][lx + 1], cur, aC, aM);
            accumulate<NSOL>(sm.r1[ly + 2][lx + 1], sm.r2[ly + 2][lx + 1], cur, aC, aM);
        }
        if (use_z) {
            accumulate<NSOL>(rec1(prev), rec2(prev), cur, aC, aM);
            accumulate<NSOL>(rec1(next), rec2(next), cur, aC, aM);
        }
        if (valid) {
            float C[NSOL], comp[NSOL];
            unpack_sol<NSOL>(sm.so[st_z][tid], C, comp);
            float o[2 * NSOL];
            {
                const float flux = cur.s[0] * DC[0] * aC[0] + cur.s[1] * DC[1] * aC[1] + cur.s[2] * DC[2] * aC[2];
                const float y = flux - comp[0];
                const float t = C[0] + y;
                o[0] = t;
                o[1] = (t - C[0]) - y;
            }
            if (NSOL == 2) {
                const float flux = cur.s[0] * DM[0] * aM[0] + cur.s[1] * DM[1] * aM[1] + cur.s[2] * DM[2] * aM[2];
                const float y = flux - comp[NSOL - 1];
                const float t = C[NSOL - 1] + y;
                o[2 * NSOL - 2] = t;
                o[2 * NSOL - 1] = (t - C[NSOL - 1]) - y;
            }
            const long long n = col + plane * z;
            if (NSOL == 2) reinterpret_cast<float4 *>(sol_out)[n] = make_float4(o[0], o[1], o[2], o[2 * NSOL - 1]);
            else sol_out[n] = make_float2(o[0], o[1]);
        }
        __syncthreads();
    };

    Rec A, B, Cd;
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

template <int NSOL, int NNB, int TY>
cudaError_t launch_one(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int zchunk) {
    constexpr int TX = 32;
    using S = Smem<NSOL, TX, TY>;
    const int tiles = ((P.ix + TX - 1) / TX) * ((P.iy + TY - 1) / TY);
    const dim3 grid((unsigned)tiles, (unsigned)((P.iz + zchunk - 1) / zchunk));
    // The shared-memory opt-in is a per-device, per-context attribute: set it
    // on every launch (a host-side driver call, far below the kernel's time) so
    // a second device or a re-created context is never launched without it.
    cudaError_t e = cudaFuncSetAttribute(k_diffuse<NSOL, NNB, TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(S));
    if (e != cudaSuccess) return e;
    k_diffuse<NSOL, NNB, TX, TY><<<grid, TX * TY, sizeof(S), s>>>(P, sphase, sol_in, sol_out, zchunk);
    return cudaGetLastError();
}

template <int NSOL, int NNB>
cudaError_t launch_ty(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                      cudaStream_t s, int ty, int zchunk) {
    switch (ty) {
        case 4: return launch_one<NSOL, NNB, 4>(P, sphase, sol_in, sol_out, s, zchunk);
        case 16: return launch_one<NSOL, NNB, 16>(P, sphase, sol_in, sol_out, s, zchunk);
        default: return launch_one<NSOL, NNB, 8>(P, sphase, sol_in, sol_out, s, zchunk);
    }
}

template <int NSOL>
cudaError_t launch_nnb(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int ty, int zchunk) {
    if (P.nnb >= 6) return launch_ty<NSOL, 6>(P, sphase, sol_in, sol_out, s, ty, zchunk);
    if (P.nnb >= 4) return launch_ty<NSOL, 4>(P, sphase, sol_in, sol_out, s, ty, zchunk);
    return launch_ty<NSOL, 2>(P, sphase, sol_in, sol_out, s, ty, zchunk);
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
    for (int a = 0; a < 3; a++) {
        if (P.iz == 1) {
            if (n < max) out[n++] = {tys[a], 1, 0};
            continue;
        }
        for (int b = 0; b < 5; b++) {
            if (zcs[b] > P.iz && b > 0) break;
            if (n < max) out[n++] = {tys[a], zcs[b] < P.iz ? zcs[b] : P.iz, 0};
        }
    }
    return n;
}

cudaError_t pf_launch_diffuse_f32(const pf_f32_params &P, const float *sphase, const float2 *sol_in,
                                  float2 *sol_out, cudaStream_t s, const pf_diff_cfg *cfg) {
    const pf_diff_cfg c = cfg ? *cfg : pf_diffuse_default_cfg(P);
    // The packed record carries the second solute as one value: its partition
    // must be separable (always so for the Mn ratios of pf_model).
    if (P.nsol == 2 && !P.sep[1]) return cudaErrorInvalidValue;
    if (P.nsol == 2) return launch_nnb<2>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk);
    return launch_nnb<1>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk);
}
