// pf_batch.cu -- many independent 2D domains advanced by one persistent launch.
//
// Each domain is a compact-FP32 state (its own size, temperature, time step and
// number of diffusion sub-steps).  The grid is launched cooperatively, so every
// block is resident; the blocks are split into one group per domain (sized by
// the domain's work), and each group runs that domain's whole sequence of
// sweeps -- phase sweep (solver.cpp:147-304), then n_sub diffusion sub-steps
// (solver.cpp:343-372) -- for nsteps time steps, separated by a barrier among
// the group's blocks only.  Domains never wait for each other.
//
// The group barrier is a counter per domain.  Its wait is bounded by a
// wall-clock limit read from %globaltimer: a block that waits longer sets the
// error flag and every block of the launch returns at its next barrier, so a
// fault can never hang the device.  Data written by other blocks inside the
// launch is read with ld.global.cg (L2, the coherence point), never through
// the non-coherent L1 path.
#include "pf_f32.cuh"
#include "pf_kernels.h"

namespace {

constexpr int kBX = 32;  // tile width; the tile height BY (4 or 8) is chosen by pf_batch_autotune

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Group barrier: returns false when the launch is being abandoned.
__device__ __forceinline__ bool group_barrier(unsigned long long *ctr, unsigned long long target, int *err,
                                              unsigned long long timeout_ns) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1ull);
        const unsigned long long t0 = globaltimer();
        int good = 1;
        while (true) {
            const unsigned long long v = atomicAdd(ctr, 0ull);
            if (v >= target) break;
            if (*(volatile int *)err) { good = 0; break; }
            if (globaltimer() - t0 > timeout_ns) {
                atomicExch(err, 1);
                good = 0;
                break;
            }
            __nanosleep(128);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

template <int NSOL> struct BVec;
template <> struct BVec<1> { using T = float2; };
template <> struct BVec<2> { using T = float4; };

template <int NSOL, int BY>
struct BRec {
    typename BVec<NSOL>::T rec[3][BY + 2][kBX + 2];
};

template <int NSOL>
__device__ __forceinline__ void load_raw_cg(const float *sph, const float2 *sol, long long N, long long n, float s[3],
                                            float C[NSOL], float comp[NSOL]) {
    s[0] = __ldcg(sph + n);
    s[1] = __ldcg(sph + N + n);
    s[2] = __ldcg(sph + 2 * N + n);
#pragma unroll
    for (int q = 0; q < NSOL; q++) {
        const float2 v = __ldcg(sol + n * NSOL + q);
        C[q] = v.x;
        comp[q] = v.y;
    }
}

template <int BY>
__device__ __forceinline__ void store_rec(BRec<1, BY> &R, int y, int x, const float s[3], const float c[1][3]) {
#pragma unroll
    for (int p = 0; p < 3; p++) R.rec[p][y][x] = make_float2(s[p], c[0][p]);
}
template <int BY>
__device__ __forceinline__ void store_rec(BRec<2, BY> &R, int y, int x, const float s[3], const float c[2][3]) {
#pragma unroll
    for (int p = 0; p < 3; p++) R.rec[p][y][x] = make_float4(s[p], c[0][p], c[1][p], 0.f);
}
__device__ __forceinline__ float rec_conc(const float2 &v, int) { return v.y; }
__device__ __forceinline__ float rec_conc(const float4 &v, int q) { return q == 0 ? v.y : v.z; }

// One 32 x BY tile of one diffusion sub-step of a 2D domain.
template <int NSOL, int BY>
__device__ __forceinline__ void diffuse_tile(const pf_f32_params &P, int tx0, int ty0, const float *sph,
                                             const float2 *sol_in, float2 *sol_out, BRec<NSOL, BY> &R) {
    const int tid = threadIdx.x;
    const int lx = tid % kBX, ly = tid / kBX;
    const int ix = P.ix, iy = P.iy;
    const long long N = P.N;
    const bool valid = (tx0 + lx < ix) && (ty0 + ly < iy);
    const long long n = pf_mod(tx0 + lx, ix) + (long long)ix * pf_mod(ty0 + ly, iy);
    float s[3], C[NSOL], comp[NSOL], c[NSOL][3];
    load_raw_cg<NSOL>(sph, sol_in, N, n, s, C, comp);
    {
        const float ph[3] = {s[0] * s[0], s[1] * s[1], s[2] * s[2]};
#pragma unroll
        for (int q = 0; q < NSOL; q++) pf_partition_q(P, q, C[q], ph, c[q]);
    }
    store_rec(R, ly + 1, lx + 1, s, c);
    // Halo ring: 2*kBX + 2*BY cells, one or two per thread.
    constexpr int NH = 2 * kBX + 2 * BY, NT = kBX * BY;
    for (int hid = tid; hid < NH; hid += NT) {
        int hx, hy;
        if (hid < kBX) { hx = hid; hy = -1; }
        else if (hid < 2 * kBX) { hx = hid - kBX; hy = BY; }
        else if (hid < 2 * kBX + BY) { hx = -1; hy = hid - 2 * kBX; }
        else { hx = kBX; hy = hid - 2 * kBX - BY; }
        const long long h = pf_mod(tx0 + hx, ix) + (long long)ix * pf_mod(ty0 + hy, iy);
        float hs[3], hC[NSOL], hcomp[NSOL], hc[NSOL][3];
        load_raw_cg<NSOL>(sph, sol_in, N, h, hs, hC, hcomp);
        const float hph[3] = {hs[0] * hs[0], hs[1] * hs[1], hs[2] * hs[2]};
#pragma unroll
        for (int q = 0; q < NSOL; q++) pf_partition_q(P, q, hC[q], hph, hc[q]);
        store_rec(R, hy + 1, hx + 1, hs, hc);
    }
    __syncthreads();
    if (valid) {
        const bool use_y = P.nnb >= 4;
        float o[2 * NSOL];
#pragma unroll
        for (int q = 0; q < NSOL; q++) {
            float flux = 0.f;
#pragma unroll
            for (int p = 0; p < 3; p++) {
                const float c0 = c[q][p];
                const auto l = R.rec[p][ly + 1][lx];
                const auto r = R.rec[p][ly + 1][lx + 2];
                float a = l.x * (rec_conc(l, q) - c0);
                a += r.x * (rec_conc(r, q) - c0);
                if (use_y) {
                    const auto d = R.rec[p][ly][lx + 1];
                    const auto u = R.rec[p][ly + 2][lx + 1];
                    a += d.x * (rec_conc(d, q) - c0);
                    a += u.x * (rec_conc(u, q) - c0);
                }
                flux += s[p] * P.D[q][p] * a;
            }
            const float y = flux - comp[q];
            const float t = C[q] + y;
            o[2 * q] = t;
            o[2 * q + 1] = (t - C[q]) - y;
        }
#pragma unroll
        for (int q = 0; q < NSOL; q++) sol_out[n * NSOL + q] = make_float2(o[2 * q], o[2 * q + 1]);
    }
    __syncthreads();
}

template <int NSOL, int BY>
__global__ void __launch_bounds__(kBX * BY, 1024 / (kBX * BY)) k_batch(const pf_batch_dom *__restrict__ doms,
                                               const pf_f32_params *__restrict__ params,
                                               const int *__restrict__ block_dom, int nsteps,
                                               unsigned long long *ctr, int *err, unsigned long long timeout_ns) {
    constexpr int kBT = kBX * BY;
    __shared__ union U {
        pf_plist<kBT> L;
        BRec<NSOL, BY> R;
    } sm;
    __shared__ pf_f32_params P;
    const int d = block_dom[blockIdx.x];
    const pf_batch_dom D = doms[d];
    if (threadIdx.x == 0) P = params[d];
    __syncthreads();
    const int lb = blockIdx.x - D.nb_first;
    const int nb = D.nb;
    int g = D.cur, sidx = D.curs;
    unsigned long long target = (unsigned long long)D.extra_target;
    for (int step = 0; step < nsteps; step++) {
        // Phase sweep of the group's tiles.
        for (int tile = lb; tile < D.tiles; tile += nb) {
            const int tx0 = (tile % D.tiles_x) * kBX, ty0 = (tile / D.tiles_x) * BY;
            // each warp takes an 8 x 4 patch of the tile (lanes more often all bulk or all interface)
            const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
            const int i = tx0 + (w % (kBX / 8)) * 8 + (lane & 7), j = ty0 + (w / (kBX / 8)) * 4 + (lane >> 3);
            if (i < P.ix && j < P.iy)
                pf_phase_cell<NSOL, kBT, true>(P, i, j, 0, threadIdx.x, D.gid[g], D.phi[g], D.gid[g ^ 1],
                                               D.phi[g ^ 1], D.sph, D.sol[sidx], sm.L);
        }
        target += nb;
        if (!group_barrier(ctr + d, target, err, timeout_ns)) return;
        g ^= 1;
        for (int sub = 0; sub < P.n_sub; sub++) {
            for (int tile = lb; tile < D.tiles; tile += nb)
                diffuse_tile<NSOL, BY>(P, (tile % D.tiles_x) * kBX, (tile / D.tiles_x) * BY, D.sph, D.sol[sidx],
                                   D.sol[sidx ^ 1], sm.R);
            target += nb;
            if (!group_barrier(ctr + d, target, err, timeout_ns)) return;
            sidx ^= 1;
        }
    }
}


template <int NSOL>
int blocks_per_sm_ty(int by) {
    int nblk = 0;
    cudaError_t e = by == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_batch<NSOL, 4>, kBX * 4, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_batch<NSOL, 8>, kBX * 8, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nblk;
}

template <int NSOL>
cudaError_t launch_ty(int by, const cudaLaunchConfig_t &cfg, const pf_batch_dom *doms, const pf_f32_params *params,
                      const int *block_dom, int nsteps, unsigned long long *ctr, int *err,
                      unsigned long long timeout_ns) {
    if (by == 4) return cudaLaunchKernelEx(&cfg, k_batch<NSOL, 4>, doms, params, block_dom, nsteps, ctr, err, timeout_ns);
    return cudaLaunchKernelEx(&cfg, k_batch<NSOL, 8>, doms, params, block_dom, nsteps, ctr, err, timeout_ns);
}

}  // namespace

int pf_batch_blocks_per_sm(int nsol, int tile_y) {
    return nsol == 2 ? blocks_per_sm_ty<2>(tile_y) : blocks_per_sm_ty<1>(tile_y);
}

bool pf_batch_tile_ok(int tile_y) { return tile_y == 4 || tile_y == 8; }

cudaError_t pf_launch_batch(int nsol, int tile_y, int nblocks, const pf_batch_dom *doms, const pf_f32_params *params,
                            const int *block_dom, int nsteps, unsigned long long *ctr, int *err,
                            unsigned long long timeout_ns, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)nblocks);
    cfg.blockDim = dim3(kBX * tile_y);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (nsol == 2) return launch_ty<2>(tile_y, cfg, doms, params, block_dom, nsteps, ctr, err, timeout_ns);
    return launch_ty<1>(tile_y, cfg, doms, params, block_dom, nsteps, ctr, err, timeout_ns);
}
