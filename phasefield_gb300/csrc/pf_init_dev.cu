// pf_init_dev.cu -- the seeded initial microstructure generated on the GPU.
//
// One thread per cell runs pfinit::cell (pf_init_cell.h), the same code the
// host generator runs, over seeds and bucket grids drawn on the host
// (pf_init_prepare) and copied to the device; the state is written straight
// into device arrays in the reference layout.  Built with -fmad=false, so the
// double arithmetic rounds as the host build (-ffp-contract=off) does; only
// tanh may differ by a few ulp between the two.  At 512^3 with 1000 grains and
// 20000 nuclei this replaces seconds of host work and a 15 GB upload.
#include <cuda_runtime.h>

#include <vector>

#include "pf_init_cell.h"
#include "pf_init_setup.h"
#include "pf_kernels.h"

namespace {

struct Part {
    double k[2][9], c[2][9];
};

__global__ void __launch_bounds__(256) k_init(const __grid_constant__ pfinit::Setup S, const __grid_constant__ Part T,
                                              long long N, int32_t *__restrict__ ids, double *__restrict__ phi,
                                              double *__restrict__ phase, double *__restrict__ conc,
                                              double *__restrict__ C, int *__restrict__ crowded, bool patch) {
    // patch (grids of at least 8 rows): 32 x 8 cells of one plane per block,
    // each warp an 8 x 4 patch, whose lanes search the same seed buckets;
    // else consecutive cells.
    long long n;
    int i, j, k;
    if (patch) {
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        i = blockIdx.x * 32 + (w & 3) * 8 + (lane & 7);
        j = blockIdx.y * 8 + (w >> 2) * 4 + (lane >> 3);
        k = blockIdx.z;
        if (i >= S.ix || j >= S.iy) return;
        n = i + (long long)S.ix * (j + (long long)S.iy * k);
    } else {
        n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (n >= N) return;
        i = (int)(n % S.ix);
        const long long r = n / S.ix;
        j = (int)(r % S.iy);
        k = (int)(r / S.iy);
    }
    int32_t id[6];
    double ph6[6], ph[3], Cv[2];
    if (!pfinit::cell(S, i, j, k, id, ph6, ph, Cv)) atomicExch(crowded, 1);
#pragma unroll
    for (int a = 0; a < 6; a++) {
        ids[6 * n + a] = id[a];
        phi[6 * n + a] = ph6[a];
    }
#pragma unroll
    for (int p = 0; p < 3; p++) phase[3 * n + p] = ph[p];
    for (int q = 0; q < S.nsol; q++) {
        C[q * N + n] = Cv[q];
        if (conc) {
            double out[3];
            pfinit::partition(ph, Cv[q], T.k[q], T.c[q], out);
#pragma unroll
            for (int a = 0; a < 3; a++) conc[q * 3 * N + 3 * n + a] = out[a];
        }
    }
}

template <class T>
bool upload(const std::vector<T> &v, T **d, std::vector<void *> &owned) {
    *d = nullptr;
    if (v.empty()) return true;
    if (cudaMalloc(d, v.size() * sizeof(T)) != cudaSuccess) return false;
    owned.push_back(*d);
    return cudaMemcpy(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

}  // namespace

int pf_init_generate_device(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec,
                            const double *kq, const double *cq, int32_t *d_ids, double *d_phi, double *d_phase,
                            double *d_conc, double *d_C, cudaStream_t s, const char **msg) {
    PfInitHost H;
    int st = pf_init_prepare(ix, iy, iz, nsol, cutoff, spec, H, msg);
    if (st != PF_OK) return st;
    pfinit::Setup S = H.S;
    std::vector<void *> owned;
    bool ok = true;
    double *dv[9];
    const std::vector<double> *hv[9] = {&H.gx, &H.gy, &H.gz, &H.nx, &H.ny, &H.nz, &H.px, &H.py, &H.pz};
    for (int a = 0; a < 9 && ok; a++) ok = upload(*hv[a], &dv[a], owned);
    int *bs[3] = {nullptr, nullptr, nullptr}, *bi[3] = {nullptr, nullptr, nullptr};
    const PfHostBuckets *hb[3] = {&H.bgr, &H.bnuc, &H.bpar};
    for (int a = 0; a < 3 && ok; a++) ok = upload(hb[a]->start, &bs[a], owned) && upload(hb[a]->items, &bi[a], owned);
    int *d_crowded = nullptr;
    if (ok) ok = cudaMalloc(&d_crowded, sizeof(int)) == cudaSuccess;
    if (ok) owned.push_back(d_crowded);
    if (ok) ok = cudaMemsetAsync(d_crowded, 0, sizeof(int), s) == cudaSuccess;
    int crowded = 0;
    if (ok) {
        S.gx = dv[0]; S.gy = dv[1]; S.gz = dv[2];
        S.nx = dv[3]; S.ny = dv[4]; S.nz = dv[5];
        S.px = dv[6]; S.py = dv[7]; S.pz = dv[8];
        S.bgr = H.bgr.view(bs[0], bi[0]);
        S.bnuc = H.bnuc.view(bs[1], bi[1]);
        S.bpar = H.bpar.view(bs[2], bi[2]);
        Part T{};
        for (int q = 0; q < nsol; q++)
            for (int a = 0; a < 9; a++) {
                T.k[q][a] = kq ? kq[q * 9 + a] : 0.0;
                T.c[q][a] = cq ? cq[q * 9 + a] : 0.0;
            }
        const long long N = (long long)ix * iy * iz;
        const bool patch = iy >= 8;
        const dim3 grid = patch ? dim3((unsigned)((ix + 31) / 32), (unsigned)((iy + 7) / 8), (unsigned)iz)
                                : dim3((unsigned)((N + 255) / 256));
        k_init<<<grid, 256, 0, s>>>(S, T, N, d_ids, d_phi, d_phase, d_conc, d_C, d_crowded, patch);
        ok = cudaGetLastError() == cudaSuccess &&
             cudaMemcpyAsync(&crowded, d_crowded, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
             cudaStreamSynchronize(s) == cudaSuccess;
    }
    for (void *p : owned) cudaFree(p);
    if (!ok) {
        cudaGetLastError();
        if (msg) *msg = "device generation failed (allocation or launch)";
        return PF_ERR_CUDA;
    }
    if (crowded) {
        if (msg) *msg = "more than 256 inclusions near one cell";
        return PF_ERR_RANGE;
    }
    if (msg) *msg = nullptr;
    return PF_OK;
}
