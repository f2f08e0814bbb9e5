// pf_reduce_noalloc.cu -- the grid statistics of pf_reduce, computed on
// caller-owned device arrays without allocating any memory.
//
// Some callers cannot call cudaMalloc: an application whose own memory pool
// owns all device memory, a framework whose caching allocator must not be
// bypassed, or a latency-critical loop that cannot afford the implicit device
// synchronisation of cudaMalloc/cudaFree.  For them this file keeps the
// reduction's scratch -- one row of 8 partial sums per chunk of
// PF_NOALLOC_CHUNK cells plus a completion counter -- in a file-scope
// __device__ array of fixed size (256 KiB).  Every GPU that loads the library
// holds that array until the process exits.
//
// The host-side name of a __device__ array is only a stand-in, not a device
// address: a kernel handed it would fault or, where the GPU can reach host
// memory, silently use the wrong memory.  The device address is therefore
// taken with cudaGetSymbolAddress once per device, with that device current,
// the first time the entry point runs on it; that first call should come
// before any stream capture.  The address is kept for the life of the process:
// cudaDeviceReset unloads the module, so the entry point is not to be called
// on a device after that device has been reset.
//
// All calls share the one array and it keeps the last call's contents.  The
// completion counter is cleared on the call's stream before the kernel runs and
// every chunk row is rewritten, so no state leaks from call to call; calls that
// overlap on the GPU (different streams, or different host threads on the same
// device) race on the array and must be serialised by the caller.
#include <mutex>
#include <string>
#include "pf_dev.cuh"
#include "pf_host.h"

#define PF_NOALLOC_CHUNK 4096
#define PF_NOALLOC_MAX_CHUNKS 4096
#define PF_NOALLOC_ROWS_DOUBLES (PF_NOALLOC_MAX_CHUNKS * 8)
#define PF_NOALLOC_MAX_DEVICES 64

// Rows of partial sums, then one 8-byte completion counter.
static __device__ __align__(256) double g_noalloc_scratch[PF_NOALLOC_ROWS_DOUBLES + 1];

namespace {

std::mutex g_setup_mutex;
double *g_scratch_dev[PF_NOALLOC_MAX_DEVICES] = {nullptr};

constexpr int kThreads = 256;

__device__ __forceinline__ double nf(double x) { return isfinite(x) ? 0. : 1.; }

// Warp shuffles + shared memory; thread o < 8 returns the block total of acc[o].
__device__ __forceinline__ double block_sum(double acc[8], double (*sm)[8]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 0; o < 8; o++) {
        double v = acc[o];
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
        if (lane == 0) sm[warp][o] = v;
    }
    __syncthreads();
    double v = 0.;
    if (threadIdx.x < 8)
        for (int w = 0; w < kThreads / 32; w++) v += sm[w][threadIdx.x];
    return v;
}

// One block per chunk; the last block to finish sums the rows in chunk order.
__global__ void __launch_bounds__(kThreads) k_reduce_noalloc(long long N, int nsol, const int *__restrict__ ids,
                                                             const double *__restrict__ phi,
                                                             const double *__restrict__ phase,
                                                             const double *__restrict__ C, double *scratch,
                                                             int nchunks, double *__restrict__ out) {
    __shared__ double sm[kThreads / 32][8];
    __shared__ bool last;
    double acc[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
    const long long begin = (long long)blockIdx.x * PF_NOALLOC_CHUNK;
    const long long end = begin + PF_NOALLOC_CHUNK < N ? begin + PF_NOALLOC_CHUNK : N;
    for (long long n = begin + threadIdx.x; n < end; n += kThreads) {
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
    const double row = block_sum(acc, sm);
    if (threadIdx.x < 8) scratch[(long long)blockIdx.x * 8 + threadIdx.x] = row;
    __threadfence();
    __syncthreads();
    unsigned long long *counter = reinterpret_cast<unsigned long long *>(scratch + PF_NOALLOC_ROWS_DOUBLES);
    if (threadIdx.x == 0) last = (atomicAdd(counter, 1ull) == (unsigned long long)(nchunks - 1));
    __syncthreads();
    if (!last) return;
    __threadfence();
    double tot[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
    for (int b = threadIdx.x; b < nchunks; b += kThreads)
#pragma unroll
        for (int o = 0; o < 8; o++) tot[o] += __ldcg(scratch + (long long)b * 8 + o);
    __syncthreads();
    const double t = block_sum(tot, sm);
    if (threadIdx.x < 8) out[threadIdx.x] = t;
    if (threadIdx.x == 0) *counter = 0ull;  // ready for the next call
}

int setup_device(double **scratch) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return pf_fail(PF_ERR_CUDA, std::string("pf_reduce_noalloc: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= PF_NOALLOC_MAX_DEVICES) return pf_fail(PF_ERR_RANGE, "pf_reduce_noalloc: device ordinal too large");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_dev[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return pf_fail(PF_ERR_CUDA, std::string("pf_reduce_noalloc: cudaGetSymbolAddress failed: ") +
                                            cudaGetErrorString(e));
        g_scratch_dev[dev] = static_cast<double *>(p);
    }
    *scratch = g_scratch_dev[dev];
    return PF_OK;
}

}  // namespace

extern "C" int pf_reduce_noalloc(long long N, int nsol, const int32_t *d_ids, const double *d_phi,
                                 const double *d_phase, const double *d_C, double *d_out, void *cuda_stream) {
    if (!d_ids || !d_phi || !d_phase || !d_C || !d_out) return pf_fail(PF_ERR_ARG, "pf_reduce_noalloc: null pointer");
    if (nsol < 1 || nsol > 2) return pf_fail(PF_ERR_ARG, "pf_reduce_noalloc: nsol must be 1 or 2");
    if (N < 1 || N > (long long)PF_NOALLOC_CHUNK * PF_NOALLOC_MAX_CHUNKS)
        return pf_fail(PF_ERR_RANGE, "pf_reduce_noalloc: N must be between 1 and PF_NOALLOC_MAX_CELLS (16777216) cells");
    double *scratch = nullptr;
    int st = setup_device(&scratch);
    if (st != PF_OK) return st;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    const int nchunks = (int)((N + PF_NOALLOC_CHUNK - 1) / PF_NOALLOC_CHUNK);
    cudaError_t e = cudaMemsetAsync(scratch + PF_NOALLOC_ROWS_DOUBLES, 0, sizeof(double), s);
    if (e != cudaSuccess) return pf_fail(PF_ERR_CUDA, std::string("pf_reduce_noalloc: ") + cudaGetErrorString(e));
    k_reduce_noalloc<<<nchunks, kThreads, 0, s>>>(N, nsol, d_ids, d_phi, d_phase, d_C, scratch, nchunks, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return pf_fail(PF_ERR_CUDA, std::string("pf_reduce_noalloc: ") + cudaGetErrorString(e));
    return PF_OK;
}
