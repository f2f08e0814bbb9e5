// pf_f32_diffuse.cu -- the diffusion sub-step (solver.cpp:343-372) on the
// compact FP32 layout, all solutes at once, sm_103a.
//
// The reference sums, for every cell A and each neighbour B, the flux
//   F(A,B) = sum_p sqrt(phi_p^A phi_p^B) * (c_p^B - c_p^A) * D_p
// (solver.cpp:363).  F(B,A) = -F(A,B), so each face's flux is a quantity of the
// face: here it is evaluated once per face where both cells live in one
// thread, and the receiving side uses its negation.  The phase planes hold
// s_p = sqrt(phi_p) (pf_f32.cuh), so the weight is s_p^A s_p^B; D carries
// dt_sub/dx^2.  A cell enters its faces through a derived record
//   s_p, c_p    square-root phase fraction and partitioned carbon
//               (solver.cpp:389-405) of each phase that carries flux,
//   r           the second solute (Mn) reduced to C_Mn / sum_j phi_j a_j: its
//               partition is separable (c_Mn,p = a_p r), so its flux is
//               (r^B - r^A) sum_p s_p^A s_p^B D_p a_p.
// Phases whose diffusivity is zero for every solute (cementite in the steel
// workloads) carry no flux and are left out of the records (NPF = 2).
//
// Work decomposition:
// * A block owns a 64 x BY tile of the x-y plane and marches up a chunk of z
//   planes.  Each thread owns a 2 x RY micro-tile of cells: the x faces inside
//   it and, for RY = 2, the y face inside it are evaluated once; the z face
//   between consecutive planes of the thread's column is evaluated once and
//   kept in a register for the next plane.
// * Records of the current plane (own cells and a one-cell halo ring, derived
//   by the first 128 + 2*BY threads) sit in shared memory, split by x parity
//   so that every warp-wide record load is contiguous (no bank conflicts);
//   the buffer alternates between planes, so one barrier per plane suffices.
// * Raw data of the next plane (s_p planes and solute totals) is loaded into
//   registers one plane ahead, so its HBM latency overlaps the current plane.
// * The solute total is advanced with a Kahan-compensated sum.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <type_traits>
#include <vector>
#include "pf_f32.cuh"
#include "pf_kernels.h"

namespace {

constexpr int kBX = 64;           // tile width in cells (two per lane of a warp)
constexpr int kCols = kBX / 2 + 2;  // record columns per parity, halo included

template <int NSOL> struct SolVec;
template <> struct SolVec<1> { using T = float2; };
template <> struct SolVec<2> { using T = float4; };

// Raw solute vector -> value and compensation per solute.
__device__ __forceinline__ void sol_split(const float2 &v, float C[1], float K[1]) { C[0] = v.x; K[0] = v.y; }
__device__ __forceinline__ void sol_split(const float4 &v, float C[2], float K[2]) {
    C[0] = v.x; K[0] = v.y; C[1] = v.z; K[1] = v.w;
}

// Record of one cell: s_p, c_p for the NPF flux phases, r for Mn.
template <int NPF>
struct Rec {
    float s[NPF], c[NPF], r;
};

// Shared record slots: part A = (s_0, s_1, c_0, c_1) for NPF = 2 or
// (s_0, s_1, s_2, r) for NPF = 3; part B = r (NPF = 2, two solutes) or
// (c_0, c_1, c_2, -) (NPF = 3).
template <int NSOL, int NPF> struct RecB;
template <> struct RecB<1, 2> { using T = float; static constexpr bool used = false; };
template <> struct RecB<2, 2> { using T = float; static constexpr bool used = true; };
template <int NSOL> struct RecB<NSOL, 3> { using T = float4; static constexpr bool used = true; };

template <int NSOL, int NPF>
__device__ __forceinline__ void rec_store(const Rec<NPF> &R, float4 *a, typename RecB<NSOL, NPF>::T *b) {
    if constexpr (NPF == 2) {
        *a = make_float4(R.s[0], R.s[1], R.c[0], R.c[1]);
        if constexpr (NSOL == 2) *b = R.r;
    } else {
        *a = make_float4(R.s[0], R.s[1], R.s[2], R.r);
        *b = make_float4(R.c[0], R.c[1], R.c[2], 0.f);
    }
}
template <int NSOL, int NPF>
__device__ __forceinline__ Rec<NPF> rec_load(const float4 *a, const typename RecB<NSOL, NPF>::T *b) {
    Rec<NPF> R;
    const float4 x = *a;
    if constexpr (NPF == 2) {
        R.s[0] = x.x; R.s[1] = x.y; R.c[0] = x.z; R.c[1] = x.w;
        R.r = NSOL == 2 ? *b : 0.f;
    } else {
        const float4 y = *b;
        R.s[0] = x.x; R.s[1] = x.y; R.s[2] = x.z; R.r = x.w;
        R.c[0] = y.x; R.c[1] = y.y; R.c[2] = y.z;
    }
    return R;
}

// Record from raw data: the partition of carbon (solver.cpp:389-405) for the
// flux phases and the reduced Mn value.
template <int NSOL, int NPF>
__device__ __forceinline__ Rec<NPF> derive(const pf_f32_params &P, const float s3[3], const float C[NSOL]) {
    Rec<NPF> R;
    const float ph[3] = {s3[0] * s3[0], s3[1] * s3[1], s3[2] * s3[2]};
#pragma unroll
    for (int p = 0; p < NPF; p++) R.s[p] = s3[p];
    // Every sum is written as explicit fused multiply-adds (the file is built
    // with -fmad=false): no contraction is left to the compiler, so each
    // kernel variant that derives records rounds them identically.
    if (P.sep[0]) {
        const float S = fmaf(ph[2], P.a[0][2], fmaf(ph[1], P.a[0][1], ph[0] * P.a[0][0]));
        const float r = __fdividef(C[0], S);
#pragma unroll
        for (int p = 0; p < NPF; p++) R.c[p] = P.a[0][p] * r;
    } else {
#pragma unroll
        for (int i = 0; i < NPF; i++) {
            const float t1 = fmaf(ph[2], P.k[0][i + 6], fmaf(ph[1], P.k[0][i + 3], ph[0] * P.k[0][i]));
            const float t2 = fmaf(ph[2], P.c[0][i + 6], fmaf(ph[1], P.c[0][i + 3], ph[0] * P.c[0][i]));
            R.c[i] = __fdividef(C[0] - t2, t1);
        }
    }
    if constexpr (NSOL == 2) {
        const float S = fmaf(ph[2], P.a[1][2], fmaf(ph[1], P.a[1][1], ph[0] * P.a[1][0]));
        R.r = __fdividef(C[1], S);
    } else {
        R.r = 0.f;
    }
    return R;
}

// Flux through the face between cells A and B as seen from A (add to A,
// subtract from B).  Exactly antisymmetric: F(B,A) == -F(A,B) bit for bit.
template <int NSOL, int NPF>
__device__ __forceinline__ void face(const Rec<NPF> &A, const Rec<NPF> &B, const float DC[NPF],
                                     const float DM[NPF], float f[NSOL]) {
    float w[NPF];
#pragma unroll
    for (int p = 0; p < NPF; p++) w[p] = A.s[p] * B.s[p];
    float fc = (w[0] * DC[0]) * (B.c[0] - A.c[0]);
#pragma unroll
    for (int p = 1; p < NPF; p++) fc = fmaf(w[p] * DC[p], B.c[p] - A.c[p], fc);
    f[0] = fc;
    if constexpr (NSOL == 2) {
        float m = w[0] * DM[0];
#pragma unroll
        for (int p = 1; p < NPF; p++) m = fmaf(w[p], DM[p], m);
        f[1] = m * (B.r - A.r);
    }
}

// Raw data of one cell.
template <int NSOL>
struct Raw {
    float s[3];
    typename SolVec<NSOL>::T v;
};

template <int NSOL, int NPF, int NNB, int RY, int NTY>
struct Shape {
    static constexpr int BY = RY * NTY, NT = 32 * NTY, NH = 2 * kBX + 2 * BY, ROWS = BY + 2;
    static constexpr size_t bytes_a = 2ull * ROWS * 2 * kCols * sizeof(float4);
    static constexpr size_t bytes_b = RecB<NSOL, NPF>::used ? 2ull * ROWS * 2 * kCols * sizeof(typename RecB<NSOL, NPF>::T) : 0;
    static constexpr size_t bytes = bytes_a + bytes_b;
};

template <int NSOL, int NPF, int NNB, int RY, int NTY>
__global__ void __launch_bounds__(32 * NTY, (32 * NTY) >= 512 ? 1 : 2)
    k_diffuse(const __grid_constant__ pf_f32_params P, const float *__restrict__ sphase,
              const float2 *__restrict__ sol_in, float2 *__restrict__ sol_out, int zchunk) {
    using S = Shape<NSOL, NPF, NNB, RY, NTY>;
    using SV = typename SolVec<NSOL>::T;
    using RB = typename RecB<NSOL, NPF>::T;
    constexpr int BY = S::BY, ROWS = S::ROWS;
    constexpr bool use_y = NNB >= 4, use_z = NNB >= 6;
    static_assert(S::NH <= S::NT, "one halo cell per thread at most");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // recA[buf][row][parity][col], recB likewise
    float4 *recA = reinterpret_cast<float4 *>(smem_raw);
    RB *recB = reinterpret_cast<RB *>(smem_raw + S::bytes_a);
    auto slot = [](int buf, int row, int par, int col) { return ((buf * ROWS + row) * 2 + par) * kCols + col; };

    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const long long N = P.N;
    const long long plane = (long long)ix * iy;
    const int tiles_x = (ix + kBX - 1) / kBX;
    const int x0 = (int)(blockIdx.x % tiles_x) * kBX;
    const int y0 = (int)(blockIdx.x / tiles_x) * BY;
    const int tid = threadIdx.x;
    const int tx = tid & 31, ty = tid >> 5;
    const SV *solv = reinterpret_cast<const SV *>(sol_in);
    SV *solo = reinterpret_cast<SV *>(sol_out);

    // Own cells: (xa + rx, ya + ry), rx = 0, 1; ry < RY.  Every slot holds the
    // cell at the wrapped coordinates, so partial tiles and periodic
    // neighbours need no special case.
    const int xg = x0 + 2 * tx, yg = y0 + RY * ty;
    const bool vx[2] = {xg < ix, xg + 1 < ix};
    long long col[RY][2];
    bool valid[RY][2];
#pragma unroll
    for (int ry = 0; ry < RY; ry++) {
        const long long yo = (long long)ix * pf_mod(yg + ry, iy);
#pragma unroll
        for (int rx = 0; rx < 2; rx++) {
            col[ry][rx] = pf_mod(xg + rx, ix) + yo;
            valid[ry][rx] = vx[rx] && (yg + ry < iy);
        }
    }
    // s_p of the cell pair (xa, xa+1) is one aligned float2 when ix is even.
    const bool pair_load = (ix & 1) == 0;

    // Halo ring: bottom row, top row (64 cells each), left and right columns.
    const bool has_halo = tid < S::NH && (use_y || tid >= 2 * kBX);
    int hrow, hpar, hcol;
    long long hcolg;
    {
        int hx, hy;
        if (tid < kBX) { hx = tid; hy = -1; }
        else if (tid < 2 * kBX) { hx = tid - kBX; hy = BY; }
        else if (tid < 2 * kBX + BY) { hx = -1; hy = tid - 2 * kBX; }
        else { hx = kBX; hy = tid - 2 * kBX - BY; }
        hrow = hy + 1;
        hpar = hx & 1;
        hcol = (hx >> 1) + 1;
        hcolg = pf_mod(x0 + hx, ix) + (long long)ix * pf_mod(y0 + hy, iy);
    }

    float DC[NPF], DM[NPF];
#pragma unroll
    for (int p = 0; p < NPF; p++) {
        DC[p] = P.D[0][p];
        DM[p] = NSOL == 2 ? P.D[NSOL - 1][p] * P.a[NSOL - 1][p] : 0.f;
    }

    auto wrapz = [&](int z) { return z < 0 ? z + iz : (z >= iz ? z - iz : z); };  // |overshoot| <= 1 plane
    auto load_own = [&](int z, Raw<NSOL> (&R)[RY][2]) {
        const long long off = plane * wrapz(z);
#pragma unroll
        for (int ry = 0; ry < RY; ry++) {
#pragma unroll
            for (int p = 0; p < 3; p++) {
                const float *sp = sphase + p * N + off;
                if (pair_load) {
                    const float2 v = __ldg(reinterpret_cast<const float2 *>(sp + col[ry][0]));
                    R[ry][0].s[p] = v.x;
                    R[ry][1].s[p] = v.y;
                } else {
                    R[ry][0].s[p] = __ldg(sp + col[ry][0]);
                    R[ry][1].s[p] = __ldg(sp + col[ry][1]);
                }
            }
#pragma unroll
            for (int rx = 0; rx < 2; rx++) R[ry][rx].v = __ldg(solv + off + col[ry][rx]);
        }
    };
    auto load_halo = [&](int z, Raw<NSOL> &H) {
        const long long off = plane * wrapz(z) + hcolg;
#pragma unroll
        for (int p = 0; p < 3; p++) H.s[p] = __ldg(sphase + p * N + off);
        H.v = __ldg(solv + off);
    };
    auto derive_raw = [&](const Raw<NSOL> &R) {
        float C[NSOL], K[NSOL];
        sol_split(R.v, C, K);
        return derive<NSOL, NPF>(P, R.s, C);
    };

    const int z0 = blockIdx.y * zchunk;
    const int z1 = min(z0 + zchunk, iz);

    Raw<NSOL> raw[RY][2];   // next plane's raw data
    SV cur_v[RY][2];        // current plane's solute totals (for the update)
    Rec<NPF> cur[RY][2];    // current plane's records
    float zdn[RY][2][NSOL]; // flux through the face below each own cell
    Raw<NSOL> hraw;

#pragma unroll
    for (int ry = 0; ry < RY; ry++)
#pragma unroll
        for (int rx = 0; rx < 2; rx++)
#pragma unroll
            for (int q = 0; q < NSOL; q++) zdn[ry][rx][q] = 0.f;
    if (use_z) {
        load_own(z0 - 1, raw);
        Rec<NPF> below[RY][2];
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) below[ry][rx] = derive_raw(raw[ry][rx]);
        load_own(z0, raw);
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                cur[ry][rx] = derive_raw(raw[ry][rx]);
                cur_v[ry][rx] = raw[ry][rx].v;
                face<NSOL, NPF>(cur[ry][rx], below[ry][rx], DC, DM, zdn[ry][rx]);
            }
        if (z0 + 1 <= z1) load_own(z0 + 1, raw);
    } else {
        load_own(z0, raw);
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                cur[ry][rx] = derive_raw(raw[ry][rx]);
                cur_v[ry][rx] = raw[ry][rx].v;
            }
        if (z0 + 1 < z1) load_own(z0 + 1, raw);
    }
    if (has_halo) load_halo(z0, hraw);

    for (int z = z0; z < z1; z++) {
        const int buf = (z - z0) & 1;
        // 1. Publish the records of this plane: own cells and the halo ring.
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                const int s = slot(buf, RY * ty + ry + 1, rx, tx + 1);
                rec_store<NSOL, NPF>(cur[ry][rx], recA + s, recB + s);
            }
        if (has_halo) {
            const Rec<NPF> h = derive_raw(hraw);
            const int s = slot(buf, hrow, hpar, hcol);
            rec_store<NSOL, NPF>(h, recA + s, recB + s);
            if (z + 1 < z1) load_halo(z + 1, hraw);
        }
        __syncthreads();
        // 2. Next plane's records (z face above), then prefetch the one after.
        Rec<NPF> nxt[RY][2];
        SV nxt_v[RY][2];
        const bool more = use_z ? true : (z + 1 < z1);
        if (more) {
#pragma unroll
            for (int ry = 0; ry < RY; ry++)
#pragma unroll
                for (int rx = 0; rx < 2; rx++) {
                    nxt[ry][rx] = derive_raw(raw[ry][rx]);
                    nxt_v[ry][rx] = raw[ry][rx].v;
                }
            if (z + 2 <= (use_z ? z1 : z1 - 1)) load_own(z + 2, raw);
        }
        // 3. Face fluxes.
        float acc[RY][2][NSOL];
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++)
#pragma unroll
                for (int q = 0; q < NSOL; q++) acc[ry][rx][q] = zdn[ry][rx][q];
        float f[NSOL];
#pragma unroll
        for (int ry = 0; ry < RY; ry++) {
            const int row = RY * ty + ry + 1;
            // x faces: outer left, inner, outer right
            face<NSOL, NPF>(cur[ry][0], rec_load<NSOL, NPF>(recA + slot(buf, row, 1, tx), recB + slot(buf, row, 1, tx)),
                            DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) acc[ry][0][q] += f[q];
            face<NSOL, NPF>(cur[ry][0], cur[ry][1], DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                acc[ry][0][q] += f[q];
                acc[ry][1][q] -= f[q];
            }
            face<NSOL, NPF>(cur[ry][1],
                            rec_load<NSOL, NPF>(recA + slot(buf, row, 0, tx + 2), recB + slot(buf, row, 0, tx + 2)),
                            DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) acc[ry][1][q] += f[q];
        }
        if (use_y) {
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                const int rlo = RY * ty, rhi = RY * ty + RY + 1;
                face<NSOL, NPF>(cur[0][rx],
                                rec_load<NSOL, NPF>(recA + slot(buf, rlo, rx, tx + 1), recB + slot(buf, rlo, rx, tx + 1)),
                                DC, DM, f);
#pragma unroll
                for (int q = 0; q < NSOL; q++) acc[0][rx][q] += f[q];
#pragma unroll
                for (int ry = 0; ry + 1 < RY; ry++) {
                    face<NSOL, NPF>(cur[ry][rx], cur[ry + 1][rx], DC, DM, f);
#pragma unroll
                    for (int q = 0; q < NSOL; q++) {
                        acc[ry][rx][q] += f[q];
                        acc[ry + 1][rx][q] -= f[q];
                    }
                }
                face<NSOL, NPF>(cur[RY - 1][rx],
                                rec_load<NSOL, NPF>(recA + slot(buf, rhi, rx, tx + 1), recB + slot(buf, rhi, rx, tx + 1)),
                                DC, DM, f);
#pragma unroll
                for (int q = 0; q < NSOL; q++) acc[RY - 1][rx][q] += f[q];
            }
        }
        if (use_z) {
#pragma unroll
            for (int ry = 0; ry < RY; ry++)
#pragma unroll
                for (int rx = 0; rx < 2; rx++) {
                    face<NSOL, NPF>(cur[ry][rx], nxt[ry][rx], DC, DM, f);
#pragma unroll
                    for (int q = 0; q < NSOL; q++) {
                        acc[ry][rx][q] += f[q];
                        zdn[ry][rx][q] = -f[q];
                    }
                }
        }
        // 4. Kahan-compensated update of the solute totals.
        const long long off = plane * z;
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                if (valid[ry][rx]) {
                    float C[NSOL], K[NSOL], o[2 * NSOL];
                    sol_split(cur_v[ry][rx], C, K);
#pragma unroll
                    for (int q = 0; q < NSOL; q++) {
                        const float y = acc[ry][rx][q] - K[q];
                        const float t = C[q] + y;
                        o[2 * q] = t;
                        o[2 * q + 1] = (t - C[q]) - y;
                    }
                    if constexpr (NSOL == 2) solo[off + col[ry][rx]] = make_float4(o[0], o[1], o[2], o[3]);
                    else solo[off + col[ry][rx]] = make_float2(o[0], o[1]);
                }
            }
        if (more) {
#pragma unroll
            for (int ry = 0; ry < RY; ry++)
#pragma unroll
                for (int rx = 0; rx < 2; rx++) {
                    cur[ry][rx] = nxt[ry][rx];
                    cur_v[ry][rx] = nxt_v[ry][rx];
                }
        }
    }
}


// ---------------------------------------------------------------------------
// Variant 1: the same sub-step with the tile interior staged by TMA.
//
// For 3D grids whose x extent is a multiple of 64 and y extent a multiple of
// the tile height, every tile's interior box lies inside the domain, so one
// cp.async.bulk.tensor per array per plane brings it into shared memory: the
// square-root phase planes as a (64, BY, 1, 3) box and the solute totals as a
// (64 x BY) box.  A ring of 3 or 4 planes is kept in flight, each completing
// on its own mbarrier, so HBM latency is covered by copies in flight rather
// than by registers or resident warps.  The halo ring is loaded with plain
// loads one plane ahead, as in variant 0.  Arithmetic, and so every result bit,
// is identical to variant 0.
//
// Every mbarrier wait is bounded (%globaltimer, kWaitNs): a wait that runs out
// sets g_diffuse_timeout, the block carries on with whatever the buffer holds
// (no thread leaves early, so no barrier is left waiting), and before exiting
// waits once more, again bounded, for its own copies still in flight.
// ---------------------------------------------------------------------------
constexpr unsigned long long kWaitNs = 2000000000ull;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for one phase of a stage barrier; false when it ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer() - t0 > kWaitNs) return false;
    return true;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ int g_diffuse_timeout;

// NST planes in the ring; NRB record buffers (2: one barrier per plane, 1: a
// second barrier per plane but half the record storage, which lets two
// 16-row blocks share an SM).
template <int NSOL, int NPF, int RY, int NTY, int NST, int NRB>
struct TmaShape {
    using B = Shape<NSOL, NPF, 6, RY, NTY>;
    static constexpr int BY = B::BY;
    static constexpr size_t s_bytes = 3ull * BY * kBX * sizeof(float);                 // phase planes of one plane
    static constexpr size_t v_bytes = (size_t)BY * kBX * sizeof(typename SolVec<NSOL>::T);  // solute totals
    static constexpr size_t stage = ((s_bytes + v_bytes + 127) / 128) * 128;
    static constexpr size_t rec_off = NST * stage;
    static constexpr size_t bar_off = rec_off + ((B::bytes * NRB / 2 + 127) / 128) * 128;
    static constexpr size_t bytes = bar_off + NST * sizeof(unsigned long long) + 128;  // + alignment slack
};

template <int NSOL, int NPF, int RY, int NTY, int NST, int NRB>
__global__ void __launch_bounds__(32 * NTY, 2)
    k_diffuse_tma(const __grid_constant__ pf_f32_params P, const __grid_constant__ CUtensorMap tm_s,
                  const __grid_constant__ CUtensorMap tm_v, const float *__restrict__ sphase,
                  const float2 *__restrict__ sol_in, float2 *__restrict__ sol_out, int zchunk) {
    using T = TmaShape<NSOL, NPF, RY, NTY, NST, NRB>;
    using S = typename T::B;
    constexpr int kStages = NST;
    using SV = typename SolVec<NSOL>::T;
    using RB = typename RecB<NSOL, NPF>::T;
    constexpr int BY = S::BY, ROWS = S::ROWS;
    extern __shared__ unsigned char smem_dyn[];
    // TMA destinations want 128-byte alignment.
    unsigned char *smem_raw =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_dyn) + 127) & ~uintptr_t(127));
    float4 *recA = reinterpret_cast<float4 *>(smem_raw + T::rec_off);
    RB *recB = reinterpret_cast<RB *>(smem_raw + T::rec_off + S::bytes_a * NRB / 2);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem_raw + T::bar_off);
    auto slot = [](int buf, int row, int par, int col) { return ((buf * ROWS + row) * 2 + par) * kCols + col; };
    auto stage_s = [&](int st) { return reinterpret_cast<const float *>(smem_raw + st * T::stage); };
    auto stage_v = [&](int st) { return reinterpret_cast<const SV *>(smem_raw + st * T::stage + T::s_bytes); };

    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const long long N = P.N;
    const long long plane = (long long)ix * iy;
    const int tiles_x = ix / kBX;
    const int x0 = (int)(blockIdx.x % tiles_x) * kBX;
    const int y0 = (int)(blockIdx.x / tiles_x) * BY;
    const int tid = threadIdx.x;
    const int tx = tid & 31, ty = tid >> 5;
    const SV *solv = reinterpret_cast<const SV *>(sol_in);
    SV *solo = reinterpret_cast<SV *>(sol_out);
    const int z0 = blockIdx.y * zchunk;
    const int z1 = min(z0 + zchunk, iz);
    const int npl = z1 - z0 + 2;  // planes z0-1 .. z1
    auto wrapz = [&](int z) { return z < 0 ? z + iz : (z >= iz ? z - iz : z); };

    if (tid == 0) {
        for (int st = 0; st < kStages; st++) mbar_init(&bars[st], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int pl) {  // plane z0 - 1 + pl into stage pl % kStages (thread 0)
        const int st = pl % kStages;
        const int zw = wrapz(z0 - 1 + pl);
        unsigned char *dst = smem_raw + st * T::stage;
        mbar_expect_tx(&bars[st], (unsigned)(T::s_bytes + T::v_bytes));
        tma_load_4d(dst, &tm_s, x0, y0, zw, 0, &bars[st]);
        if constexpr (NSOL == 2) tma_load_4d(dst + T::s_bytes, &tm_v, 0, x0, y0, zw, &bars[st]);
        else tma_load_3d(dst + T::s_bytes, &tm_v, x0, y0, zw, &bars[st]);
    };
    if (tid == 0)
        for (int pl = 0; pl < kStages && pl < npl; pl++) issue(pl);
    bool ok = true;
    auto wait_plane = [&](int pl) {
        if (!mbar_wait(&bars[pl % kStages], (unsigned)((pl / kStages) & 1))) ok = false;
    };

    // Own cells of the thread: rows RY*ty + ry, columns 2tx, 2tx + 1 of the tile.
    long long col[RY][2];
#pragma unroll
    for (int ry = 0; ry < RY; ry++)
#pragma unroll
        for (int rx = 0; rx < 2; rx++) col[ry][rx] = (x0 + 2 * tx + rx) + (long long)ix * (y0 + RY * ty + ry);
    auto read_own = [&](int pl, int ry, int rx, float s3[3], SV &v) {
        const float *Ss = stage_s(pl % kStages);
        const int r = RY * ty + ry, c = 2 * tx + rx;
#pragma unroll
        for (int p = 0; p < 3; p++) s3[p] = Ss[(p * BY + r) * kBX + c];
        v = stage_v(pl % kStages)[r * kBX + c];
    };
    auto derive_own = [&](int pl, Rec<NPF> (&R)[RY][2]) {
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                float s3[3], C[NSOL], K[NSOL];
                SV v;
                read_own(pl, ry, rx, s3, v);
                sol_split(v, C, K);
                R[ry][rx] = derive<NSOL, NPF>(P, s3, C);
            }
    };

    // Halo ring, as in variant 0 (plain loads one plane ahead).
    const bool has_halo = tid < S::NH;
    int hrow, hpar, hcol;
    long long hcolg;
    {
        int hx, hy;
        if (tid < kBX) { hx = tid; hy = -1; }
        else if (tid < 2 * kBX) { hx = tid - kBX; hy = BY; }
        else if (tid < 2 * kBX + BY) { hx = -1; hy = tid - 2 * kBX; }
        else { hx = kBX; hy = tid - 2 * kBX - BY; }
        hrow = hy + 1;
        hpar = hx & 1;
        hcol = (hx >> 1) + 1;
        hcolg = pf_mod(x0 + hx, ix) + (long long)ix * pf_mod(y0 + hy, iy);
    }
    Raw<NSOL> hraw;
    auto load_halo = [&](int z) {
        const long long off = plane * wrapz(z) + hcolg;
#pragma unroll
        for (int p = 0; p < 3; p++) hraw.s[p] = __ldg(sphase + p * N + off);
        hraw.v = __ldg(solv + off);
    };
    if (has_halo) load_halo(z0);

    float DC[NPF], DM[NPF];
#pragma unroll
    for (int p = 0; p < NPF; p++) {
        DC[p] = P.D[0][p];
        DM[p] = NSOL == 2 ? P.D[NSOL - 1][p] * P.a[NSOL - 1][p] : 0.f;
    }

    Rec<NPF> cur[RY][2];
    float zdn[RY][2][NSOL];
    {
        Rec<NPF> below[RY][2];
        wait_plane(0);
        derive_own(0, below);
        wait_plane(1);
        derive_own(1, cur);
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) face<NSOL, NPF>(cur[ry][rx], below[ry][rx], DC, DM, zdn[ry][rx]);
    }

    for (int z = z0; z < z1; z++) {
        const int pl = z - z0 + 1;
        const int buf = NRB == 2 ? (z - z0) & 1 : 0;
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                const int s = slot(buf, RY * ty + ry + 1, rx, tx + 1);
                rec_store<NSOL, NPF>(cur[ry][rx], recA + s, recB + s);
            }
        if (has_halo) {
            float C[NSOL], K[NSOL];
            sol_split(hraw.v, C, K);
            const Rec<NPF> h = derive<NSOL, NPF>(P, hraw.s, C);
            const int s = slot(buf, hrow, hpar, hcol);
            rec_store<NSOL, NPF>(h, recA + s, recB + s);
            if (z + 1 < z1) load_halo(z + 1);
        }
        __syncthreads();
        // Every thread is past plane pl - 1: its stage takes plane pl - 1 + kStages.
        if (tid == 0 && pl - 1 + kStages < npl) issue(pl - 1 + kStages);
        Rec<NPF> nxt[RY][2];
        wait_plane(pl + 1);
        derive_own(pl + 1, nxt);
        float acc[RY][2][NSOL];
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++)
#pragma unroll
                for (int q = 0; q < NSOL; q++) acc[ry][rx][q] = zdn[ry][rx][q];
        float f[NSOL];
#pragma unroll
        for (int ry = 0; ry < RY; ry++) {
            const int row = RY * ty + ry + 1;
            face<NSOL, NPF>(cur[ry][0], rec_load<NSOL, NPF>(recA + slot(buf, row, 1, tx), recB + slot(buf, row, 1, tx)),
                            DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) acc[ry][0][q] += f[q];
            face<NSOL, NPF>(cur[ry][0], cur[ry][1], DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) {
                acc[ry][0][q] += f[q];
                acc[ry][1][q] -= f[q];
            }
            face<NSOL, NPF>(cur[ry][1],
                            rec_load<NSOL, NPF>(recA + slot(buf, row, 0, tx + 2), recB + slot(buf, row, 0, tx + 2)),
                            DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) acc[ry][1][q] += f[q];
        }
#pragma unroll
        for (int rx = 0; rx < 2; rx++) {
            const int rlo = RY * ty, rhi = RY * ty + RY + 1;
            face<NSOL, NPF>(cur[0][rx],
                            rec_load<NSOL, NPF>(recA + slot(buf, rlo, rx, tx + 1), recB + slot(buf, rlo, rx, tx + 1)),
                            DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) acc[0][rx][q] += f[q];
#pragma unroll
            for (int ry = 0; ry + 1 < RY; ry++) {
                face<NSOL, NPF>(cur[ry][rx], cur[ry + 1][rx], DC, DM, f);
#pragma unroll
                for (int q = 0; q < NSOL; q++) {
                    acc[ry][rx][q] += f[q];
                    acc[ry + 1][rx][q] -= f[q];
                }
            }
            face<NSOL, NPF>(cur[RY - 1][rx],
                            rec_load<NSOL, NPF>(recA + slot(buf, rhi, rx, tx + 1), recB + slot(buf, rhi, rx, tx + 1)),
                            DC, DM, f);
#pragma unroll
            for (int q = 0; q < NSOL; q++) acc[RY - 1][rx][q] += f[q];
        }
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                face<NSOL, NPF>(cur[ry][rx], nxt[ry][rx], DC, DM, f);
#pragma unroll
                for (int q = 0; q < NSOL; q++) {
                    acc[ry][rx][q] += f[q];
                    zdn[ry][rx][q] = -f[q];
                }
            }
        const long long off = plane * z;
#pragma unroll
        for (int ry = 0; ry < RY; ry++)
#pragma unroll
            for (int rx = 0; rx < 2; rx++) {
                float s3[3], C[NSOL], K[NSOL], o[2 * NSOL];
                SV v;
                read_own(pl, ry, rx, s3, v);
                sol_split(v, C, K);
#pragma unroll
                for (int q = 0; q < NSOL; q++) {
                    const float y = acc[ry][rx][q] - K[q];
                    const float t = C[q] + y;
                    o[2 * q] = t;
                    o[2 * q + 1] = (t - C[q]) - y;
                }
                if constexpr (NSOL == 2) solo[off + col[ry][rx]] = make_float4(o[0], o[1], o[2], o[3]);
                else solo[off + col[ry][rx]] = make_float2(o[0], o[1]);
                cur[ry][rx] = nxt[ry][rx];
            }
        if (NRB == 1) __syncthreads();  // the single record buffer is rewritten next plane
    }
    if (!ok) {
        atomicExch(&g_diffuse_timeout, 1);
        // Own copies still in flight: wait for them once more (bounded).
        if (tid == 0)
            for (int pl = (npl > kStages ? npl - kStages : 0); pl < npl; pl++)
                mbar_wait(&bars[pl % kStages], (unsigned)((pl / kStages) & 1));
    }
}

// ---- tensor maps of variant 1 (host) ----
using EncodeTiled = PFN_cuTensorMapEncodeTiled_v12000;

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// Maps are a function of (base address, grid, tile height, kind): kept in a
// small process-wide cache so each launch only looks one up.
struct MapEntry {
    const void *ptr;
    int ix, iy, iz, by, kind;
    CUtensorMap map;
};
std::mutex g_map_mutex;
std::vector<MapEntry> g_maps;

bool tensor_map(const void *ptr, int ix, int iy, int iz, int by, int kind, CUtensorMap *out) {
    std::lock_guard<std::mutex> lock(g_map_mutex);
    for (const MapEntry &e : g_maps)
        if (e.ptr == ptr && e.ix == ix && e.iy == iy && e.iz == iz && e.by == by && e.kind == kind) {
            *out = e.map;
            return true;
        }
    EncodeTiled enc = encode_fn();
    if (!enc) return false;
    MapEntry e{ptr, ix, iy, iz, by, kind, {}};
    const cuuint64_t X = (cuuint64_t)ix, Y = (cuuint64_t)iy, Z = (cuuint64_t)iz;
    CUresult r;
    if (kind == 0) {  // square-root phase planes [3][iz][iy][ix] float: box (64, by, 1, 3)
        const cuuint64_t dims[4] = {X, Y, Z, 3};
        const cuuint64_t strides[3] = {X * 4, X * Y * 4, X * Y * Z * 4};
        const cuuint32_t box[4] = {(cuuint32_t)kBX, (cuuint32_t)by, 1, 3};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        r = enc(&e.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void *>(ptr), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else if (kind == 2) {  // two solutes: float4 per cell as (4, ix, iy, iz) floats, box (4, 64, by, 1)
        const cuuint64_t dims[4] = {4, X, Y, Z};
        const cuuint64_t strides[3] = {16, X * 16, X * Y * 16};
        const cuuint32_t box[4] = {4, (cuuint32_t)kBX, (cuuint32_t)by, 1};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        r = enc(&e.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void *>(ptr), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else {  // one solute: float2 per cell as one 8-byte element, box (64, by, 1)
        const cuuint64_t dims[3] = {X, Y, Z};
        const cuuint64_t strides[2] = {X * 8, X * Y * 8};
        const cuuint32_t box[3] = {(cuuint32_t)kBX, (cuuint32_t)by, 1};
        const cuuint32_t es[3] = {1, 1, 1};
        r = enc(&e.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(ptr), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    }
    if (r != CUDA_SUCCESS) return false;
    if (g_maps.size() >= 64) g_maps.erase(g_maps.begin());
    g_maps.push_back(e);
    *out = e.map;
    return true;
}

// Variant 1 needs a 3D grid whose tiles all lie inside it.
bool tma_ok(const pf_f32_params &P, int by) {
    return P.nnb >= 6 && P.ix % kBX == 0 && P.iy % by == 0 && P.iz >= 2 && encode_fn() != nullptr;
}

template <int NSOL, int NPF, int BY>
cudaError_t launch_tma(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int zchunk) {
    // A 4-plane ring with double-buffered records: about 85 KB of shared
    // memory for 8-row tiles (two blocks per SM), 164 KB for 16-row tiles (one
    // block per SM; measured faster on GB300 than a 3-plane ring with a single
    // record buffer, which fits two).
    constexpr int RY = BY == 8 ? 1 : 2, NTY = 8, NST = 4, NRB = 2;
    using T = TmaShape<NSOL, NPF, RY, NTY, NST, NRB>;
    CUtensorMap ms, mv;
    if (!tensor_map(sphase, P.ix, P.iy, P.iz, BY, 0, &ms) || !tensor_map(sol_in, P.ix, P.iy, P.iz, BY, NSOL, &mv))
        return cudaErrorInvalidValue;
    const int tiles = (P.ix / kBX) * (P.iy / BY);
    const dim3 grid((unsigned)tiles, (unsigned)((P.iz + zchunk - 1) / zchunk));
    auto kern = k_diffuse_tma<NSOL, NPF, RY, NTY, NST, NRB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::bytes);
    if (e != cudaSuccess) return e;
    kern<<<grid, 32 * NTY, T::bytes, s>>>(P, ms, mv, sphase, sol_in, sol_out, zchunk);
    return cudaGetLastError();
}

template <int NSOL, int NPF>
cudaError_t launch_tma_ty(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                          cudaStream_t s, int ty, int zchunk) {
    if (ty == 8) return launch_tma<NSOL, NPF, 8>(P, sphase, sol_in, sol_out, s, zchunk);
    return launch_tma<NSOL, NPF, 16>(P, sphase, sol_in, sol_out, s, zchunk);
}

// Tile height -> (cells per thread in y, warps per block).
template <int BY> struct TileOf;
template <> struct TileOf<8> { static constexpr int RY = 1, NTY = 8; };
template <> struct TileOf<16> { static constexpr int RY = 2, NTY = 8; };
template <> struct TileOf<32> { static constexpr int RY = 2, NTY = 16; };

template <int NSOL, int NPF, int NNB, int BY>
cudaError_t launch_one(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int zchunk) {
    constexpr int RY = TileOf<BY>::RY, NTY = TileOf<BY>::NTY;
    using S = Shape<NSOL, NPF, NNB, RY, NTY>;
    const int tiles = ((P.ix + kBX - 1) / kBX) * ((P.iy + BY - 1) / BY);
    const dim3 grid((unsigned)tiles, (unsigned)((P.iz + zchunk - 1) / zchunk));
    // The shared-memory opt-in is a per-device, per-context attribute: set it
    // on every launch (a host-side driver call, far below the kernel's time) so
    // a second device or a re-created context is never launched without it.
    auto kern = k_diffuse<NSOL, NPF, NNB, RY, NTY>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bytes);
    if (e != cudaSuccess) return e;
    kern<<<grid, S::NT, S::bytes, s>>>(P, sphase, sol_in, sol_out, zchunk);
    return cudaGetLastError();
}

template <int NSOL, int NPF, int NNB>
cudaError_t launch_ty(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                      cudaStream_t s, int ty, int zchunk) {
    switch (ty) {
        case 8: return launch_one<NSOL, NPF, NNB, 8>(P, sphase, sol_in, sol_out, s, zchunk);
        case 32: return launch_one<NSOL, NPF, NNB, 32>(P, sphase, sol_in, sol_out, s, zchunk);
        default: return launch_one<NSOL, NPF, NNB, 16>(P, sphase, sol_in, sol_out, s, zchunk);
    }
}

template <int NSOL, int NPF>
cudaError_t launch_nnb(const pf_f32_params &P, const float *sphase, const float2 *sol_in, float2 *sol_out,
                       cudaStream_t s, int ty, int zchunk) {
    if (P.nnb >= 6) return launch_ty<NSOL, NPF, 6>(P, sphase, sol_in, sol_out, s, ty, zchunk);
    if (P.nnb >= 4) return launch_ty<NSOL, NPF, 4>(P, sphase, sol_in, sol_out, s, ty, zchunk);
    return launch_ty<NSOL, NPF, 2>(P, sphase, sol_in, sol_out, s, ty, zchunk);
}

// Number of phases that carry flux: cementite drops out when every solute's
// diffusivity in it is zero.
int flux_phases(const pf_f32_params &P) {
    for (int q = 0; q < P.nsol; q++)
        if (P.D[q][2] != 0.f) return 3;
    return 2;
}

}  // namespace

pf_diff_cfg pf_diffuse_default_cfg(const pf_f32_params &P) {
    pf_diff_cfg c;
    c.ty = 16;
    // The TMA-staged variant where the grid allows it (the autotuner's usual
    // pick on GB300), else plain loads.
    c.variant = tma_ok(P, 16) ? 1 : 0;
    const int tiles = ((P.ix + kBX - 1) / kBX) * ((P.iy + 15) / 16);
    // About 1024 blocks (several waves on 152 SMs), at least 8 planes per block.
    int z = P.iz;
    while (z > 8 && (long long)tiles * ((P.iz + z - 1) / z) < 1024) z = (z + 1) / 2;
    c.zchunk = z < 1 ? 1 : z;
    return c;
}

int pf_diffuse_candidates(const pf_f32_params &P, pf_diff_cfg *out, int max) {
    const int tys[3] = {8, 16, 32};
    const int zcs[5] = {8, 16, 32, 64, 128};
    int n = 0;
    for (int var = 0; var < 2; var++)
        for (int a = 0; a < 3; a++) {
            if (var == 1 && (tys[a] == 32 || !tma_ok(P, tys[a]))) continue;
            if (P.iz == 1) {
                if (n < max) out[n++] = {tys[a], 1, var};
                continue;
            }
            for (int b = 0; b < 5; b++) {
                if (zcs[b] > P.iz && b > 0) break;
                if (n < max) out[n++] = {tys[a], zcs[b] < P.iz ? zcs[b] : P.iz, var};
            }
        }
    return n;
}

bool pf_diffuse_variant_ok(const pf_f32_params &P, int ty, int variant) {
    if (variant == 0) return ty == 8 || ty == 16 || ty == 32;
    if (variant == 1) return (ty == 8 || ty == 16) && tma_ok(P, ty);
    return false;
}

int pf_diffuse_take_timeout() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_diffuse_timeout, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_diffuse_timeout, &zero, sizeof(int));
    }
    return v;
}

cudaError_t pf_launch_diffuse_f32(const pf_f32_params &P, const float *sphase, const float2 *sol_in,
                                  float2 *sol_out, cudaStream_t s, const pf_diff_cfg *cfg) {
    const pf_diff_cfg c = cfg ? *cfg : pf_diffuse_default_cfg(P);
    // The record carries the second solute as one value: its partition must
    // be separable (always so for the Mn ratios of pf_model).
    if (P.nsol == 2 && !P.sep[1]) return cudaErrorInvalidValue;
    const bool three = flux_phases(P) == 3;
    if (c.variant == 1) {
        if (!pf_diffuse_variant_ok(P, c.ty, 1)) return cudaErrorInvalidValue;
        if (P.nsol == 2)
            return three ? launch_tma_ty<2, 3>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk)
                         : launch_tma_ty<2, 2>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk);
        return three ? launch_tma_ty<1, 3>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk)
                     : launch_tma_ty<1, 2>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk);
    }
    if (P.nsol == 2)
        return three ? launch_nnb<2, 3>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk)
                     : launch_nnb<2, 2>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk);
    return three ? launch_nnb<1, 3>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk)
                 : launch_nnb<1, 2>(P, sphase, sol_in, sol_out, s, c.ty, c.zchunk);
}

