// pf_f32.cu -- compact FP32 phase sweep and the layout conversions (sm_103a).
//
// Model: the Steinbach pairwise phase update of zhubq/PhaseField
// (C++-openmp-cuda/src/solver.cpp:147-304) on the compact layout of
// pf_f32.cuh: up to 4 grains per cell with uint16 local ids, FP32 values, the
// phase planes holding sqrt(phase fraction).  The local grain id encodes the
// phase by range: id <= b1 -> ferrite(1), <= b2 -> austenite(2), else
// cementite(3).  Phase concentrations are never stored: the sweep re-partitions
// the cell's carbon where the driving force needs it.
//
// Built with -prec-div=false -prec-sqrt=false: divisions and square roots are
// the approximate (<= 2 ulp) forms.
#include "pf_f32.cuh"
#include "pf_kernels.h"

namespace {

constexpr int kPX = 32, kPY = 8, kPT = kPX * kPY;  // phase-sweep block: 32 x 8 cells of one plane
// Each warp takes a compact patch (not a 32-cell row): a compact patch is
// more often all bulk or all interface, so fewer lanes idle while others run
// the list update.  2D: 8 x 4 patches of a 32 x 8 block.  3D (Z2): 8 x 2 x 2
// patches of a 32 x 4 x 2 block (eight consecutive cells per row keep the
// warp's loads to few sectors; measured faster than 4 x 4 x 2).
constexpr int kWX = 8, kWY = 4;
static_assert(kPX % kWX == 0 && kPY % kWY == 0 && kWX * kWY == 32, "warp patches tile the block");
constexpr int kZX = 32, kZY = 4;  // Z2 block: 32 x 4 cells on each of two planes

// Phase sweep, one thread per cell, 2D blocks of 32x8 cells of one plane (x-y
// neighbours mostly in the same block's L1 footprint).  Every cell whose
// merged stencil list fits four entries is updated with the list in
// registers (pf_phase_cell_reg); the few others are appended to a work list
// (one atomic per warp) and updated by k_phase_f32_rest with the ten-entry
// shared-memory list of pf_phase_cell.  The sweep reads buffer 1 and writes
// buffer 2 only, so deferring a cell changes nothing it reads.
__device__ __forceinline__ void pf_defer(bool defer, unsigned n, unsigned int *rest, unsigned int *rest_count) {
    const unsigned m = __ballot_sync(0xffffffffu, defer);
    if (m) {
        const int lane = threadIdx.x & 31;
        unsigned base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(rest_count, (unsigned)__popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        if (defer) rest[base + __popc(m & ((1u << lane) - 1u))] = (unsigned)n;
    }
}

// Four resident blocks per SM (64 registers): measured faster than three
// (75 registers, no spills) or five and six (heavy spills).
template <int NSOL, int MINB, bool Z2>
__global__ void __launch_bounds__(kPT, MINB) k_phase_f32(const __grid_constant__ pf_f32_params P,
                                                         const ushort4 *__restrict__ gid1,
                                                         const float4 *__restrict__ phi1,
                                                         ushort4 *__restrict__ gid2, float4 *__restrict__ phi2,
                                                         float *__restrict__ sphase,
                                                         const float2 *__restrict__ sol,
                                                         unsigned int *__restrict__ rest,
                                                         unsigned int *__restrict__ rest_count) {
    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const int warp = threadIdx.y, lane = threadIdx.x;  // blockDim = (32, 8): one warp per y index
    int i, j, k;
    if (Z2) {
        i = blockIdx.x * kZX + (warp % (kZX / 8)) * 8 + (lane & 7);
        j = blockIdx.y * kZY + (warp / (kZX / 8)) * 2 + ((lane >> 3) & 1);
        k = 2 * blockIdx.z + (lane >> 4);
    } else {
        i = blockIdx.x * kPX + (warp % (kPX / kWX)) * kWX + lane % kWX;
        j = blockIdx.y * kPY + (warp / (kPX / kWX)) * kWY + lane / kWX;
        k = blockIdx.z;
    }
    __shared__ float4 coef[9];
    pf_coef_table(P, coef);
    __syncthreads();
    const unsigned plane = (unsigned)ix * (unsigned)iy;
    const unsigned n = (unsigned)i + (unsigned)ix * (unsigned)j + plane * (unsigned)k;
    bool defer = false;
    if (i < ix && j < iy && k < iz) {
        unsigned nb[6];
        nb[0] = n - i + pf_wrap(i, ix, -1);
        nb[1] = n - i + pf_wrap(i, ix, 1);
        nb[2] = n + (unsigned)ix * (pf_wrap(j, iy, -1) - j);
        nb[3] = n + (unsigned)ix * (pf_wrap(j, iy, 1) - j);
        nb[4] = n + plane * (pf_wrap(k, iz, -1) - k);
        nb[5] = n + plane * (pf_wrap(k, iz, 1) - k);
        defer = !pf_phase_cell_reg<NSOL>(P, coef, n, nb, gid1, phi1, gid2, phi2, sphase, sol);
    }
    // Every lane of the warp reaches the vote.
    pf_defer(defer, n, rest, rest_count);
}

// The deferred cells of k_phase_f32, one per thread: lists of up to eight
// grains in registers, longer ones (or own slots that are not a prefix) with
// the general ten-entry list (solver.cpp:147-304) in the thread's local
// memory -- no shared memory, so occupancy is set by registers alone.
template <int NSOL>
__global__ void __launch_bounds__(kPT, 3) k_phase_f32_rest(const __grid_constant__ pf_f32_params P,
                                                        const ushort4 *__restrict__ gid1,
                                                        const float4 *__restrict__ phi1,
                                                        ushort4 *__restrict__ gid2, float4 *__restrict__ phi2,
                                                        float *__restrict__ sphase,
                                                        const float2 *__restrict__ sol,
                                                        const unsigned int *__restrict__ rest,
                                                        const unsigned int *__restrict__ rest_count) {
    __shared__ float4 coef[9];
    pf_coef_table(P, coef);
    __syncthreads();
    const unsigned cnt = *rest_count;
    const unsigned ix = (unsigned)P.ix, iy = (unsigned)P.iy, iz = (unsigned)P.iz;
    const unsigned plane = ix * iy;
    for (unsigned q = blockIdx.x * kPT + threadIdx.x; q < cnt; q += gridDim.x * kPT) {
        const unsigned n = rest[q];
        const unsigned r = n / ix;
        const int i = (int)(n - r * ix), j = (int)(r % iy), k = (int)(r / iy);
        unsigned nb[6];
        nb[0] = n - i + pf_wrap(i, (int)ix, -1);
        nb[1] = n - i + pf_wrap(i, (int)ix, 1);
        nb[2] = n + ix * (pf_wrap(j, (int)iy, -1) - j);
        nb[3] = n + ix * (pf_wrap(j, (int)iy, 1) - j);
        nb[4] = n + plane * (pf_wrap(k, (int)iz, -1) - k);
        nb[5] = n + plane * (pf_wrap(k, (int)iz, 1) - k);
        if (!pf_phase_cell_reg<NSOL, false, 8>(P, coef, n, nb, gid1, phi1, gid2, phi2, sphase, sol)) {
            pf_plist<1> L;
            pf_phase_cell<NSOL, 1>(P, i, j, k, 0, gid1, phi1, gid2, phi2, sphase, sol, L);
        }
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
                                                  float *__restrict__ sphase, float2 *__restrict__ sol,
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
        const double s = v[0] + v[1] + v[2] + v[3];
        double q[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int a = 0; a < 4; a++) {
            v[a] /= s;
            const int c = id[a] / PF_MAXGRAIN_PER_PHASE;
            const int p = id[a] == 0 ? 0 : (c > 0 ? c : 1);
            if (p == 1) q[0] += v[a];
            else if (p == 2) q[1] += v[a];
            else if (p == 3) q[2] += v[a];
        }
        ph[0] = q[0]; ph[1] = q[1]; ph[2] = q[2];
    }
    int l[4];
#pragma unroll
    for (int a = 0; a < 4; a++) l[a] = pf_to_local(id[a], map);
    gid[n] = make_ushort4((unsigned short)l[0], (unsigned short)l[1], (unsigned short)l[2],
                          (unsigned short)l[3]);
    phi[n] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
    sphase[n] = (float)sqrt(ph[0]);
    sphase[N + n] = (float)sqrt(ph[1]);
    sphase[2 * N + n] = (float)sqrt(ph[2]);
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (q < nsol) {
            const double c = C64[q * N + n];
            const float f = (float)c;
            sol[n * nsol + q] = make_float2(f, (float)((double)f - c));
        }
    }
}

// Compact FP32 layout -> reference layout (FP64, 6 slots); phase
// concentrations re-partitioned in FP64 from the compensated solute totals.
__global__ void __launch_bounds__(256) k_unpack_f32(const __grid_constant__ pf_step_params P,
                                                    const pf_f32_map map,
                                                    const ushort4 *__restrict__ gid,
                                                    const float4 *__restrict__ phi,
                                                    const float *__restrict__ sphase,
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
    double ph[3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const double s = (double)sphase[p * N + n];
        ph[p] = s * s;
        phase64[3 * n + p] = ph[p];
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (q < P.nsol) {
            const float2 s = sol[n * P.nsol + q];
            const double c = (double)s.x - (double)s.y;
            C64[q * N + n] = c;
            if (conc64) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    double t1 = 0., t2 = 0.;
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        t1 += ph[j] * P.k[q][i + 3 * j];
                        t2 += ph[j] * P.c[q][i + 3 * j];
                    }
                    conc64[q * 3 * N + 3 * n + i] = (c - t2) / t1;
                }
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
                               ushort4 *gid, float4 *phi, float *sphase, float2 *sol,
                               unsigned int *n_truncated, cudaStream_t s) {
    k_pack_f32<<<pf_blocks(N, 256), 256, 0, s>>>(N, nsol, map, ids64, phi64, phase64, C64, gid, phi,
                                                 sphase, sol, n_truncated);
    return cudaGetLastError();
}

cudaError_t pf_launch_unpack_f32(const pf_step_params &P, const pf_f32_map &map, const ushort4 *gid,
                                 const float4 *phi, const float *sphase, const float2 *sol, int *ids64,
                                 double *phi64, double *phase64, double *conc64, double *C64,
                                 cudaStream_t s) {
    k_unpack_f32<<<pf_blocks(P.N, 256), 256, 0, s>>>(P, map, gid, phi, sphase, sol, ids64, phi64, phase64,
                                                   conc64, C64);
    return cudaGetLastError();
}

cudaError_t pf_launch_phase_f32(const pf_f32_params &P, const ushort4 *gid1, const float4 *phi1,
                                ushort4 *gid2, float4 *phi2, float *sphase, const float2 *sol,
                                unsigned int *rest, unsigned int *rest_count, cudaStream_t s) {
    const dim3 block(kPX, kPY);
    const bool z2 = P.iz > 1;
    const dim3 grid = z2 ? dim3((unsigned)((P.ix + kZX - 1) / kZX), (unsigned)((P.iy + kZY - 1) / kZY),
                                (unsigned)((P.iz + 1) / 2))
                         : dim3((unsigned)((P.ix + kPX - 1) / kPX), (unsigned)((P.iy + kPY - 1) / kPY), 1u);
    long long rb = (P.N / 32 + kPT - 1) / kPT;  // the rest kernel loops if more than 1/32 of the cells wait
    if (rb > 152 * 8) rb = 152 * 8;
    if (rb < 1) rb = 1;
    cudaError_t e = cudaMemsetAsync(rest_count, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    if (P.nsol == 2) {
        if (z2) k_phase_f32<2, 4, true><<<grid, block, 0, s>>>(P, gid1, phi1, gid2, phi2, sphase, sol, rest, rest_count);
        else k_phase_f32<2, 4, false><<<grid, block, 0, s>>>(P, gid1, phi1, gid2, phi2, sphase, sol, rest, rest_count);
        k_phase_f32_rest<2><<<(unsigned)rb, kPT, 0, s>>>(P, gid1, phi1, gid2, phi2, sphase, sol, rest, rest_count);
    } else {
        if (z2) k_phase_f32<1, 4, true><<<grid, block, 0, s>>>(P, gid1, phi1, gid2, phi2, sphase, sol, rest, rest_count);
        else k_phase_f32<1, 4, false><<<grid, block, 0, s>>>(P, gid1, phi1, gid2, phi2, sphase, sol, rest, rest_count);
        k_phase_f32_rest<1><<<(unsigned)rb, kPT, 0, s>>>(P, gid1, phi1, gid2, phi2, sphase, sol, rest, rest_count);
    }
    return cudaGetLastError();
}
