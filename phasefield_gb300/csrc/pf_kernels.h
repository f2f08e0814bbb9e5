// pf_kernels.h -- host-side launchers of the sm_103a kernels (internal to libpfstep).
#pragma once
#include <cuda_runtime.h>
#include "pf_types.h"

// ---- FP64 reference layout (pf_f64.cu) ----
// avg: 3N doubles of scratch for the interface-averaged concentrations
// (used when P.avg_range > 0; may be null otherwise).  flags: N bytes of
// scratch for the coherent-mobility flags, coh: the coherent-partner table of
// n_coh austenite grains (used when P.coh_model; may be null otherwise).
cudaError_t pf_launch_phase_f64(const pf_step_params &P, const int *ids1, const double *phi1, int *ids2,
                                double *phi2, double *phase, double *conc1, const double *C, double *avg,
                                unsigned char *flags, const int *coh, int n_coh, cudaStream_t s);
// 1 if a solute-drag velocity iteration of the FP64 sweep found no root since
// the last call (then cleared).
int pf_drag_take_failure();
// links: 9N doubles, the flux weights of every cell's forward links; tpart:
// 6N doubles per solute, the partition sums; both valid while the phase
// fractions are unchanged (pf_launch_links_f64).
cudaError_t pf_launch_links_f64(const pf_step_params &P, int nnb, const double *phase, double *links,
                                double *tpart, cudaStream_t s);
cudaError_t pf_launch_diffuse_f64(const pf_step_params &P, int nnb, double coef, const double *links,
                                  const double *tpart, const double *conc1, double *conc2, double *C,
                                  cudaStream_t s);
cudaError_t pf_launch_partition_f64(const pf_step_params &P, const double *phase, const double *C,
                                    double *conc, cudaStream_t s);

// ---- compact FP32 layout (pf_f32.cu) ----
// gid: ushort4 per cell (local grain ids, 0 = empty), phi: float4 per cell,
// phase: three float planes [3][N], sol: float2 (value, Kahan compensation)
// per cell and solute, interleaved [N][nsol].
struct pf_f32_map {
    int off[4];    // local id offsets of grain classes 0..3 (id/100000)
    int total;     // largest local id
};
cudaError_t pf_launch_id_span(const int *ids64, long long N, int *span4, cudaStream_t s);
cudaError_t pf_launch_pack_f32(long long N, int nsol, const pf_f32_map &map, const int *ids64,
                               const double *phi64, const double *phase64, const double *C64,
                               ushort4 *gid, float4 *phi, float *phase, float2 *sol,
                               unsigned int *n_truncated, cudaStream_t s);
cudaError_t pf_launch_unpack_f32(const pf_step_params &P, const pf_f32_map &map, const ushort4 *gid,
                                 const float4 *phi, const float *phase, const float2 *sol, int *ids64,
                                 double *phi64, double *phase64, double *conc64, double *C64,
                                 cudaStream_t s);
// 'rest' holds N cell indices and 'rest_count' one counter: the cells whose
// stencil list exceeds four entries wait there between the sweep's two kernels.
cudaError_t pf_launch_phase_f32(const pf_f32_params &P, const ushort4 *gid1, const float4 *phi1,
                                ushort4 *gid2, float4 *phi2, float *phase, const float2 *sol,
                                unsigned int *rest, unsigned int *rest_count, cudaStream_t s);
// Tile shape of the diffusion kernel: TX = 32 cells in x, ty in y, zchunk z
// planes per block, kernel variant (chosen by the autotuner or the default rule).
struct pf_diff_cfg {
    int ty;
    int zchunk;
    int variant; // 0: plain loads one plane ahead; 1: tile interior staged by TMA (same results)
};
pf_diff_cfg pf_diffuse_default_cfg(const pf_f32_params &P);
int pf_diffuse_candidates(const pf_f32_params &P, pf_diff_cfg *out, int max);
// Whether (tile height, variant) can run on this grid.
bool pf_diffuse_variant_ok(const pf_f32_params &P, int ty, int variant);
// 1 if a bounded wait of the TMA variant ran out since the last call (then cleared).
int pf_diffuse_take_timeout();
// 'sphase' holds the square roots of the phase fractions (pf_f32.cuh).
cudaError_t pf_launch_diffuse_f32(const pf_f32_params &P, const float *sphase, const float2 *sol_in,
                                  float2 *sol_out, cudaStream_t s, const pf_diff_cfg *cfg);

// ---- batched 2D domains, one persistent cooperative launch (pf_batch.cu) ----
struct pf_batch_dom {
    ushort4 *gid[2];
    float4 *phi[2];
    float *sph;
    float2 *sol[2];
    int cur, curs;          // buffer roles at the start of the launch
    int nb_first, nb;       // the domain's block group
    int tiles_x, tiles;     // 32 x tile_y tiles of the domain
    int extra_target;       // test knob: > 0 makes the group barriers unreachable
};
// Tiles are 32 x tile_y cells, tile_y 4 or 8 (pf_batch_tile_ok).
int pf_batch_blocks_per_sm(int nsol, int tile_y);
bool pf_batch_tile_ok(int tile_y);
cudaError_t pf_launch_batch(int nsol, int tile_y, int nblocks, const pf_batch_dom *doms, const pf_f32_params *params,
                            const int *block_dom, int nsteps, unsigned long long *ctr, int *err,
                            unsigned long long timeout_ns, cudaStream_t s);

// ---- FP64 reductions (pf_reduce.cu) ----
// out[0..2]  sum of phase fractions, out[3] sum of phi over slots whose grain
// id is below 100000 (write_data.cpp:18), out[4..5] solute sums, out[6]
// number of non-finite values seen.  'partials' holds 8 doubles per block.
#define PF_RED_NOUT 8
int pf_reduce_blocks(long long N);
cudaError_t pf_launch_reduce_f64(long long N, int nsol, const int *ids, const double *phi,
                                 const double *phase, const double *C, double *partials, int nblocks,
                                 double *out, cudaStream_t s);
cudaError_t pf_launch_reduce_f32(long long N, int nsol, int deformed_max_local, const ushort4 *gid,
                                 const float4 *phi, const float *phase, const float2 *sol,
                                 double *partials, int nblocks, double *out, cudaStream_t s);

// ---- seeded initial state on the device (pf_init_dev.cu) ----
int pf_init_generate_device(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec,
                            const double *kq, const double *cq, int32_t *d_ids, double *d_phi, double *d_phase,
                            double *d_conc, double *d_C, cudaStream_t s, const char **msg);
