// pf_dev.cuh -- small device helpers shared by the FP64 and FP32 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "pf_types.h"

// Periodic neighbour (phase_field.h:58-68 restated 0-based; also gpu_solver.cpp:123-126).
__device__ __forceinline__ int pf_wrap(int i, int len, int d) {
    int g = i + d;
    if (g >= len) g -= len;
    else if (g < 0) g += len;
    return g;
}

// v mod L in [0, L) for any int v.
__device__ __forceinline__ int pf_mod(int v, int L) {
    v %= L;
    return v < 0 ? v + L : v;
}

// phase_field.h:25-29: grain id -> phase (0 for an empty slot).
__device__ __forceinline__ int pf_phase_of_grain(int g) {
    if (g == 0) return 0;
    int q = g / PF_MAXGRAIN_PER_PHASE;
    return q > 0 ? q : 1;
}

// One-thread-per-cell kernels run on a (ceil(ix/256), iy, iz) grid of 256-thread
// blocks: the cell's coordinates come from the block coordinates (no integer
// division), and a thread with i >= ix has no cell.
constexpr int PF_CELL_THREADS = 256;

inline dim3 pf_cell_grid(int ix, int iy, int iz) {
    return dim3((unsigned)((ix + PF_CELL_THREADS - 1) / PF_CELL_THREADS), (unsigned)iy, (unsigned)iz);
}

__device__ __forceinline__ bool pf_cell(int ix, int iy, int &i, int &j, int &k, long long &n) {
    i = blockIdx.x * PF_CELL_THREADS + threadIdx.x;
    j = blockIdx.y;
    k = blockIdx.z;
    n = i + (long long)ix * (j + (long long)iy * k);
    return i < ix;
}

// The same cells with each warp on an 8 x 4 patch of a 32 x 8 block (grids
// of at least 8 rows): kernels whose lanes branch on bulk versus interface
// cells find a compact patch more often uniform than a 32-cell row.
// 3D grids (iz > 1, map 2): 8 x 2 x 2 patches of 32 x 4 x 2 blocks instead.
inline int pf_use_patch(int iy, int iz = 1) { return iy < 8 ? 0 : (iz > 1 ? 2 : 1); }
inline dim3 pf_map_grid(int patch, int ix, int iy, int iz) {
    if (patch == 2) return dim3((unsigned)((ix + 31) / 32), (unsigned)((iy + 3) / 4), (unsigned)((iz + 1) / 2));
    return patch ? dim3((unsigned)((ix + 31) / 32), (unsigned)((iy + 7) / 8), (unsigned)iz) : pf_cell_grid(ix, iy, iz);
}
__device__ __forceinline__ bool pf_cell_map(int patch, int ix, int iy, int iz, int &i, int &j, int &k,
                                            long long &n) {
    if (!patch) return pf_cell(ix, iy, i, j, k, n);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (patch == 2) {
        i = blockIdx.x * 32 + (w & 3) * 8 + (lane & 7);
        j = blockIdx.y * 4 + (w >> 2) * 2 + ((lane >> 3) & 1);
        k = blockIdx.z * 2 + (lane >> 4);
    } else {
        i = blockIdx.x * 32 + (w & 3) * 8 + (lane & 7);
        j = blockIdx.y * 8 + (w >> 2) * 4 + (lane >> 3);
        k = blockIdx.z;
    }
    n = i + (long long)ix * (j + (long long)iy * k);
    return i < ix && j < iy && k < iz;
}

// Neighbours of (i,j,k) in the reference order x-, x+, y-, y+, z-, z+
// (solver.cpp:159-166, :353-358).
__device__ __forceinline__ void pf_neighbours3(int i, int j, int k, long long n, int ix, int iy, int iz,
                                               long long nbr[6]) {
    const long long plane = (long long)ix * iy;
    nbr[0] = n - i + pf_wrap(i, ix, -1);
    nbr[1] = n - i + pf_wrap(i, ix, 1);
    nbr[2] = n + (long long)ix * (pf_wrap(j, iy, -1) - j);
    nbr[3] = n + (long long)ix * (pf_wrap(j, iy, 1) - j);
    nbr[4] = n + plane * (pf_wrap(k, iz, -1) - k);
    nbr[5] = n + plane * (pf_wrap(k, iz, 1) - k);
}

#define PF_CUDA_OK(call)                                  \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return pf_cuda_fail(e_);   \
    } while (0)
