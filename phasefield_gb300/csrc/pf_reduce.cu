// pf_reduce.cu -- FP64 reductions over the grid (sm_103a).
//
// The statistics that write_data.cpp:13-18 prints every output step (the
// volume fraction of each phase and the fraction carried by grain ids below
// 100000) plus the solute totals used for the conservation check and a count of
// non-finite values.  Each block accumulates in FP64 registers, reduces with
// warp shuffles and shared memory, and writes one row of 8 partials; a
// single-block second pass sums the rows in a fixed order, so the result is
// deterministic run to run.
#include "pf_dev.cuh"
#include "pf_kernels.h"

namespace {

constexpr int kRedThreads = 256;

__device__ __forceinline__ void block_store_partials(double acc[PF_RED_NOUT], double *row) {
    __shared__ double sm[kRedThreads / 32][PF_RED_NOUT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 0; o < PF_RED_NOUT; o++) {
        double v = acc[o];
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
        if (lane == 0) sm[warp][o] = v;
    }
    __syncthreads();
    if (threadIdx.x < PF_RED_NOUT) {
        double v = 0.;
        for (int w = 0; w < kRedThreads / 32; w++) v += sm[w][threadIdx.x];
        row[threadIdx.x] = v;
    }
}

__device__ __forceinline__ double nf(double x) { return isfinite(x) ? 0. : 1.; }

__global__ void __launch_bounds__(kRedThreads) k_reduce_f64(long long N, int nsol, const int *__restrict__ ids,
                                                            const double *__restrict__ phi,
                                                            const double *__restrict__ phase,
                                                            const double *__restrict__ C,
                                                            double *__restrict__ partials) {
    double acc[PF_RED_NOUT] = {0., 0., 0., 0., 0., 0., 0., 0.};
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N;
         n += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const double v = phase[3 * n + p];
            acc[p] += v;
            acc[7] += nf(v);
        }
#pragma unroll
        for (int a = 0; a < 6; a++) {
            const double v = phi[6 * n + a];
            acc[3] += (ids[6 * n + a] < PF_MAXGRAIN_PER_PHASE) ? v : 0.;
            acc[7] += nf(v);
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (q < nsol) {
                const double v = C[q * N + n];
                acc[4 + q] += v;
                acc[7] += nf(v);
            }
        }
    }
    block_store_partials(acc, partials + (long long)blockIdx.x * PF_RED_NOUT);
}

__global__ void __launch_bounds__(kRedThreads) k_reduce_f32(long long N, int nsol, int deformed_max_local,
                                                            const ushort4 *__restrict__ gid,
                                                            const float4 *__restrict__ phi,
                                                            const float *__restrict__ phase,
                                                            const float2 *__restrict__ sol,
                                                            double *__restrict__ partials) {
    // Each thread sums its few dozen cells in FP32 with Kahan compensation
    // (error ~ eps^2 of the partial), then the partials go to FP64: the sums
    // keep FP64 accuracy without per-cell FP64 arithmetic.
    float s[9], c[9];
#pragma unroll
    for (int o = 0; o < 9; o++) { s[o] = 0.f; c[o] = 0.f; }
    auto kadd = [&](int o, float v) {
        const float y = v - c[o];
        const float t = s[o] + y;
        c[o] = (t - s[o]) - y;
        s[o] = t;
    };
    int bad = 0;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N;
         n += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const float sq = phase[p * N + n];  // planes hold sqrt(phase fraction)
            bad += !isfinite(sq);
            kadd(p, sq * sq);
        }
        const ushort4 g = gid[n];
        const float4 v4 = phi[n];
        const int l[4] = {g.x, g.y, g.z, g.w};
        const float fv[4] = {v4.x, v4.y, v4.z, v4.w};
        float def = 0.f;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            bad += !isfinite(fv[a]);
            def += (l[a] <= deformed_max_local) ? fv[a] : 0.f;
        }
        kadd(3, def);
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (q < nsol) {
                const float2 v = sol[n * nsol + q];
                bad += !isfinite(v.x) + !isfinite(v.y);
                kadd(4 + q, v.x);
                kadd(6 + q, v.y);
            }
        }
    }
    double acc[PF_RED_NOUT];
#pragma unroll
    for (int o = 0; o < 4; o++) acc[o] = (double)s[o] - (double)c[o];
    // Solute totals: true value = sum(x) - sum(compensation).
    acc[4] = ((double)s[4] - (double)c[4]) - ((double)s[6] - (double)c[6]);
    acc[5] = ((double)s[5] - (double)c[5]) - ((double)s[7] - (double)c[7]);
    acc[6] = 0.;
    acc[7] = (double)bad;
    block_store_partials(acc, partials + (long long)blockIdx.x * PF_RED_NOUT);
}

// Second pass: one block sums the per-block rows in a fixed order.
__global__ void __launch_bounds__(kRedThreads) k_reduce_final(const double *__restrict__ partials, int nblocks,
                                                              double *__restrict__ out) {
    double acc[PF_RED_NOUT] = {0., 0., 0., 0., 0., 0., 0., 0.};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int o = 0; o < PF_RED_NOUT; o++) acc[o] += partials[(long long)b * PF_RED_NOUT + o];
    block_store_partials(acc, out);
}

}  // namespace

int pf_reduce_blocks(long long N) {
    long long b = (N + kRedThreads - 1) / kRedThreads;
    const long long cap = 152 * 8;  // 8 resident blocks on each of the 152 SMs
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

cudaError_t pf_launch_reduce_f64(long long N, int nsol, const int *ids, const double *phi,
                                 const double *phase, const double *C, double *partials, int nblocks,
                                 double *out, cudaStream_t s) {
    k_reduce_f64<<<nblocks, kRedThreads, 0, s>>>(N, nsol, ids, phi, phase, C, partials);
    k_reduce_final<<<1, kRedThreads, 0, s>>>(partials, nblocks, out);
    return cudaGetLastError();
}

cudaError_t pf_launch_reduce_f32(long long N, int nsol, int deformed_max_local, const ushort4 *gid,
                                 const float4 *phi, const float *phase, const float2 *sol,
                                 double *partials, int nblocks, double *out, cudaStream_t s) {
    k_reduce_f32<<<nblocks, kRedThreads, 0, s>>>(N, nsol, deformed_max_local, gid, phi, phase, sol,
                                                 partials);
    k_reduce_final<<<1, kRedThreads, 0, s>>>(partials, nblocks, out);
    return cudaGetLastError();
}
