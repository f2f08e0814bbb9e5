/*
 * pfstep.h -- C ABI of libpfstep, the GB300 (sm_103a) Steinbach
 * multi-phase-field time step.
 *
 * Two groups of entry points:
 *
 *  1. A drop-in for the reference's GPU plug-in, zhubq/PhaseField
 *     C++-openmp-cuda/src/gpu_solver.h:18-23.  Same names, same argument
 *     meaning, same return convention, so phase_field.cpp links against this
 *     library unchanged.
 *
 *  2. A full-step API (pf_*) that keeps the whole state resident in HBM and
 *     advances complete time steps (phase sweep + sub-cycled diffusion +
 *     partitioning) on the GPU: phase_field::Update
 *     (C++-openmp-cuda/src/phase_field.cpp:243-305) and its per-cell solvers
 *     (solver.cpp:147-432).  Every pf_* call returns an int status (PF_OK = 0,
 *     negative on error; pf_last_error() gives a message).  One context per
 *     host thread; contexts share nothing.
 *
 * Layout at the boundary is the reference's (phase_field.h:81-89): Blitz
 * fortranArray order with the slot / phase index fastest, then x, y, z.
 *   ids   int32  [N*6]        grain ids (phase = id/100000, ids < 100000 are phase 1)
 *   phi   double [N*6]        phase-field value of each slot
 *   phase double [N*3]        phase fractions (ferrite, austenite, cementite)
 *   conc  double [nsol][N*3]  solute concentration of each phase
 *   C     double [nsol][N]    total solute concentration (solute 0 = carbon, 1 = Mn)
 * with N = ix*iy*iz and cell n = i + ix*(j + iy*k).
 */
#ifndef PFSTEP_H
#define PFSTEP_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* 1. Drop-in for gpu_solver.h                                              */
/* ------------------------------------------------------------------------ */

/* Replaces GPU_Init, gpu_solver.h:18 / gpu_solver.cpp:26-99.  Selects device 0
 * and allocates the device buffers for an x*y*z grid.  Returns 1 when the GPU
 * can be used, 0 when there is no device or not enough memory (the caller then
 * falls back to its CPU solver, phase_field.cpp:364). */
int GPU_Init(const int x, const int y, const int z);

/* Replaces GPU_Diffusion_solver, gpu_solver.h:19 / gpu_solver.cpp:204-218.
 * Copies the phase fractions and total carbon to the device, advances the
 * multiphase diffusion over the interval dt in num_loop = ceil(dt/del_t)
 * sub-steps with del_t = dx*dx/max(D)/dims*0.2f (dims = 3 if z > 1 else 2),
 * each sub-step partitioning C into phase concentrations with
 * c_i = (C - sum_j phase_j*c_ij)/(sum_j phase_j*k_ij) and applying the
 * 6-neighbour flux sum_nb sum_p sqrt(phase_p^nb*phase_p)*(c_p^nb - c_p)*D_p,
 * then copies C back into htotal_conc.  k and c are 3x3 column-major. */
void GPU_Diffusion_solver(double *hdiffusivity, double *hpartition_k, double *hpartition_c,
                          double *hvalue_phase, double *htotal_conc, int x, int y, int z, double dt,
                          double dx);

/* Replaces GPU_Cleanup, gpu_solver.h:23 / gpu_solver.cpp:223-239.  Frees the
 * buffers of GPU_Init.  Unlike the reference it neither calls
 * cudaDeviceReset (which would tear down every other user of the device in the
 * process) nor exit(0) on a failed free. */
void GPU_Cleanup(void);

/* ------------------------------------------------------------------------ */
/* 2. Full-step API                                                         */
/* ------------------------------------------------------------------------ */

#define PF_OK 0
#define PF_ERR_ARG (-1)       /* invalid argument / state                   */
#define PF_ERR_NOMEM (-2)     /* device or pinned-host allocation failed     */
#define PF_ERR_CUDA (-3)      /* CUDA runtime error                          */
#define PF_ERR_TIMEOUT (-4)   /* a bounded device-side wait ran out          */
#define PF_ERR_NONFINITE (-5) /* NaN / Inf found in the state                */
#define PF_ERR_IO (-6)        /* file missing / malformed                    */
#define PF_ERR_NODEV (-7)     /* no CUDA device                              */
#define PF_ERR_RANGE (-8)     /* value outside what the layout can hold      */
#define PF_ERR_DRIFT (-9)     /* a solute total drifted beyond the tolerance */

#define PF_PREC_FP64 0   /* reference layout, FP64, bit-matching the CPU solver      */
#define PF_PREC_FP32C 1  /* compact layout: 4 slots, uint16 ids, FP32 + Kahan solutes */

#define PF_MAXT 64

/* Parsed model: the configuration file (phase_field.cpp:166-330) and the
 * thermodynamic file (thermo_functor.cpp:11-53).  3x3 tables are column-major
 * with phase pair (i,j), 1-based, at (i-1)+3*(j-1). */
typedef struct {
    char directory[256];
    int ix, iy, iz;
    double dx;                 /* cell size, um */
    int i_intf;                /* interface thickness in cells; eta = dx*i_intf */
    double cutoff;
    int num_grain[3];
    double phase_fraction[3];
    double init_conc[3];
    int nT;                    /* temperature path: nT (time, T) points */
    double T_time[PF_MAXT], T_temp[PF_MAXT];
    double reduction;
    int num_init_iteration;
    double timestep_output;
    int micro_out;
    double num_nuclei;
    double m0[9], mQ[9];       /* mobility prefactor (um^4/J/s) and activation energy (J/mol) */
    double sigma[9];           /* interface energy, J/um^2 */
    double D0[2][3], DQ[2][3]; /* solute diffusivity per phase: [0] carbon, [1] Mn */
    char thermo_file[256];
    int gpu_flag;
    int nsol;                  /* 1 = carbon (reference); 2 when the Mn extension is present */
    double mn_ratio[3];        /* Mn partition: c_Mn,p proportional to mn_ratio[p] */
    double ent_a[9], ent_b[9];                 /* entropy k_ij = a*T + b */
    double nple1_a[9], nple1_b[9], nple1_c[9]; /* parsed, unused by the step */
    double nple2_a[9], nple2_b[9], nple2_c[9]; /* parsed, unused by the step */
    double eq_a[9], eq_b[9], eq_c[9];          /* PARA equilibrium wt% = a*T^2 + b*T + c */
    /* 0: the thermo file's linear entropy and quadratic PARA lines
     * (thermo_data.cpp:24-41, driving force solver.cpp:374-387).
     * 1: the Fortran model's piecewise polynomial para lines and its linear
     * driving force (Fortran_openmp_phase_field/PFM/src/sparse.f90:500-528,
     * 797-923), selected by a thermo file whose first word is F90_POLYNOMIAL. */
    int thermo_model;
    /* 1: the driving force reads the phase concentrations averaged over the
     * interface neighbourhood (Fortran model, sparse.f90:184-255; FP64 path
     * only), selected by the keyword AVERAGED_INTERFACE_CARBON after
     * F90_POLYNOMIAL in the thermo file. */
    int avg_carbon;
    /* 1: the Fortran model's Purdy-Brechet solute drag on ferrite/austenite
     * interfaces (sparse.f90:326-360, 538-671, 958-1041; FP64 path only),
     * selected by "SOLUTE_DRAG binding_energy v_max0 q_sd" after
     * F90_POLYNOMIAL in the thermo file (J/mol, um/s, J/mol). */
    int drag;
    double drag_binding, drag_vmax0, drag_qsd;
    /* 1: the Fortran model's coherent-grain mobility (sparse.f90:298-315;
     * FP64 path only): a ferrite/austenite pair whose austenite grain nucleated
     * coherent with that ferrite grain (pf_set_coherent_grains) moves at 0.02
     * of its mobility in a cell with one own ferrite grain whose interface
     * neighbourhood holds bulk ferrite and no recrystallisation front.
     * Selected by "COHERENT_MOBILITY npp0" after F90_POLYNOMIAL in the thermo
     * file; ferrite ids <= npp0 are the initial (deformed) grains, larger ones
     * recrystallised (0: a single class, no recrystallisation fronts). */
    int coherent;
    int coh_npp0;
} pf_model;

/* Per-step parameters evaluated on the host (Update_parameter,
 * phase_field.cpp:307-315; thermo_data::Get_data, thermo_data.cpp:24-41). */
typedef struct {
    int ix, iy, iz;
    int nnb;            /* 2*dimensions */
    int nsol;
    int n_sub;          /* diffusion sub-steps per phase step */
    long long N;
    double T, time;
    double dx, cutoff, eta;
    double pfm_dt, diff_dt, dt_sub;
    double factor1, factor2, factor3;
    double coef_diff;
    double m[9], sigma[9];
    double entropy[9], eq[9], dcdT[9];
    double D[2][3];
    double k[2][9], c[2][9];
    /* Driving force form: 0 = entropy*(c_i - eq_ij)/dcdT_ij; 1 (thermo_model 1)
     * = -df_ratio_ij * (max(c_i, c_j) - df_ref) */
    int df_model;
    double df_ratio[9], df_ref;
    /* > 0: half-width (i_intf + 1 cells) of the interface neighbourhood
     * scanned before the sweep (averaged carbon, coherent-mobility flags);
     * avg_conc = 1: the driving force reads the averaged phase
     * concentrations, 0: the cell's own */
    int avg_range;
    int avg_conc;
    /* Solute drag at the step's temperature (PARAMETER_DRAG_PB,
     * sparse.f90:958-1003): v_max, E0 = binding/RT, the Mn segregation
     * parameters of heating / cooling and the bulk fraction of the first
     * species, the correction factors and zero-velocity drags [heating, cooling]. */
    int drag_model;
    double drag_vmax, drag_ex0, drag_de_heat, drag_de_cool, drag_u0;
    double drag_corr[2], drag_drag0[2];
    /* Coherent-grain mobility (pf_model.coherent) and the last id of the
     * initial ferrite class */
    int coh_model;
    int coh_npp0;
} pf_step_params;

/* Seeded synthetic microstructure (replaces the reference's unseeded
 * Construct/Nucleate1in2, MicrostructureConstruction.cpp:4-65 and
 * nucleation.cpp:3-43): periodic Voronoi ferrite grains (ids 100000+g),
 * spherical austenite nuclei (ids 200000+n) and cementite particles
 * (ids 300000+n) with tanh interfaces, uniform solutes plus uniform noise. */
typedef struct {
    uint64_t seed;
    int n_grains;
    int n_nuclei;
    double nucleus_radius;    /* cells */
    int n_particles;
    double particle_radius;   /* cells */
    double width;             /* interface width, cells */
    double C0[2];             /* total solute, wt% */
    double C_noise[2];        /* half-width of the uniform noise, wt% */
    int max_slots;            /* slots filled per cell (<= 6) */
} pf_init_spec;

const char *pf_status_string(int status);
const char *pf_last_error(void);
/* sizeof(pf_model), sizeof(pf_step_params), sizeof(pf_init_spec): lets a
 * binding check its struct mirrors against the library it loaded. */
int pf_abi_sizes(long long out[3]);

/* Parse the reference configuration file and the thermodynamic file it names
 * (looked up relative to the working directory, then the config's directory). */
int pf_model_read(const char *config_path, pf_model *out);
int pf_thermo_read(const char *thermo_path, pf_model *out);
/* Parameters of the step that starts at 'time'. */
int pf_params_at(const pf_model *model, double time, pf_step_params *out);
/* Fill host arrays (reference layout) with a seeded initial state at 'time'. */
int pf_init_microstructure(const pf_model *model, const pf_init_spec *spec, double time, int32_t *ids,
                           double *phi, double *phase, double *conc, double *C);
/* The same state restricted to planes [z0, z0+nz) of the model's grid (arrays
 * sized for ix*iy*nz cells): equal to those planes of the whole domain. */
int pf_init_microstructure_box(const pf_model *model, const pf_init_spec *spec, double time, int z0, int nz,
                               int32_t *ids, double *phi, double *phase, double *conc, double *C);

typedef struct pf_ctx pf_ctx;
int pf_create(const pf_model *model, int precision, pf_ctx **out);
int pf_destroy(pf_ctx *ctx);
/* Run on a caller-owned cudaStream_t (NULL = the context's own stream). */
int pf_set_stream(pf_ctx *ctx, void *cuda_stream);
int pf_upload_state(pf_ctx *ctx, const int32_t *ids, const double *phi, const double *phase,
                    const double *conc, const double *C, double time);
/* conc may be NULL. */
int pf_download_state(pf_ctx *ctx, int32_t *ids, double *phi, double *phase, double *conc, double *C,
                      double *time);
/* Advance nsteps full time steps (asynchronous on the context's stream). */
int pf_step(pf_ctx *ctx, int nsteps);
/* Only the diffusion sub-cycle: nsub sub-steps with the parameters of the
 * current time, phases fixed, time not advanced (phase_field.cpp:408-418 alone). */
int pf_diffuse(pf_ctx *ctx, int nsub);
/* FP64 statistics: out[0..2] sum of phase fractions over cells, out[3] sum of
 * phi over slots with grain id < 100000, out[4..5] solute totals, out[6] 0,
 * out[7] count of non-finite values.  Divide by N for write_data.cpp:14-18. */
int pf_reduce(pf_ctx *ctx, double out[8]);
/* Failure check on the FP64 statistics: PF_ERR_NONFINITE if any value of the
 * state is NaN/Inf; otherwise PF_ERR_DRIFT if a solute total differs from
 * reference_totals[q] by more than max_rel_drift (relative; skipped when
 * reference_totals is NULL or max_rel_drift <= 0).  out (may be NULL) receives
 * the pf_reduce statistics. */
int pf_check_state(pf_ctx *ctx, const double reference_totals[2], double max_rel_drift, double out[8]);
/* Waits for the context's stream; PF_ERR_TIMEOUT if a bounded device-side
 * wait of the staged diffusion kernel ran out since the last check. */
int pf_synchronize(pf_ctx *ctx);
int pf_get_time(pf_ctx *ctx, double *time);
int pf_last_params(pf_ctx *ctx, pf_step_params *out);
/* Number of cells whose upload kept only the 4 largest of >4 slots (FP32C). */
int pf_truncated_cells(pf_ctx *ctx, long long *out);
/* Bracket every kernel launch with CUDA events; read back accumulated times. */
int pf_enable_kernel_timing(pf_ctx *ctx, int on);
/* times[0]/counts[0]: phase sweep, [1]: diffusion sub-step. Synchronises. */
int pf_kernel_times(pf_ctx *ctx, double times_ms[2], long long counts[2]);
/* Capture steps with constant parameters in a CUDA graph and replay it. */
int pf_use_graph(pf_ctx *ctx, int on);
/* Time every candidate tile shape of the FP32C diffusion kernel on the
 * context's own state and keep the fastest (state unchanged); reports the
 * chosen tile height, z chunk, kernel variant (0: plain loads one plane
 * ahead; 1: tile interior staged by TMA, 3D tile-aligned grids only -- both
 * give identical results) and mean launch time.  No-op for FP64. */
int pf_autotune(pf_ctx *ctx, int *tile_y, int *zchunk, int *variant, float *ms);
/* Fix the FP32C diffusion tile shape: tile_y 8/16/32 rows of a 64-cell-wide
 * tile with variant 0, or 8/16 with variant 1 on a 3D grid whose x extent is a
 * multiple of 64 and y extent a multiple of tile_y; z chunk >= 1; anything
 * else is PF_ERR_ARG.  tile_y = 0 returns to the default rule. */
int pf_set_diffusion_tile(pf_ctx *ctx, int tile_y, int zchunk, int variant);
/* The autotuner's candidates as (tile_y, zchunk, variant) triples; returns
 * how many were written (at most max). */
int pf_diffusion_candidates(pf_ctx *ctx, int *out, int max);
/* Batched ensemble (no reference counterpart): many independent 2D domains
 * (own size, constant temperature, time step, sub-step count), each stored
 * like a PF_PREC_FP32C context, advanced together by one persistent
 * cooperative kernel launch replayed from a CUDA graph.  Blocks are grouped per
 * domain; a group's barrier waits are bounded (default 2 s), and a launch whose
 * wait runs out is abandoned and reported as PF_ERR_TIMEOUT (the device stays
 * usable; the domains' states must then be uploaded again). */
typedef struct pf_batch pf_batch;
int pf_batch_create(const pf_model *models, int ndomains, pf_batch **out);
int pf_batch_upload(pf_batch *b, int domain, const int32_t *ids, const double *phi, const double *phase,
                    const double *C, double time);
int pf_batch_run(pf_batch *b, int nsteps);
int pf_batch_download(pf_batch *b, int domain, int32_t *ids, double *phi, double *phase, double *conc,
                      double *C, double *time);
int pf_batch_reduce(pf_batch *b, int domain, double out[8]);
/* out[0] total cells, out[1] resident blocks used, out[2] domains, out[3] largest n_sub. */
int pf_batch_info(pf_batch *b, long long out[4]);
/* Barrier wait limit; unreachable_barrier != 0 makes every group barrier wait
 * for one block too many (to exercise the timeout path in tests). */
int pf_batch_set_timeout(pf_batch *b, unsigned long long timeout_ns, int unreachable_barrier);
/* Tile shape of the persistent kernel: 32 x tile_y cells (tile_y 4 or 8), using
 * 1/occupancy_divisor (1..4) of the resident-block capacity. */
int pf_batch_set_tile(pf_batch *b, int tile_y, int occupancy_divisor);
/* Time every tile shape on nsteps of the current ensemble (the states are
 * restored afterwards) and keep the fastest; reports it and its time. */
int pf_batch_autotune(pf_batch *b, int nsteps, int *tile_y, int *occupancy_divisor, float *ms);
int pf_batch_destroy(pf_batch *b);

/* Adjoint of the explicit step (no reference counterpart), for calibration.
 * The calibration model is the four-slot compact step (carbon only: Mn does
 * not enter the phase update or the carbon field), in FP64 (PF_PREC_FP64) or
 * FP32 with FP64 reductions (PF_PREC_FP32C).  Parameters are scale factors
 * s[4] on the interface mobilities, the interface energies, D_C and D_Mn; the
 * time step and sub-step count are those of s = 1 and stay fixed.
 * pf_adj_forward runs nsteps from the uploaded state, keeping a checkpoint
 * every checkpoint_every steps, and returns J[0] = mean ferrite fraction and
 * J[1] = mean austenite carbon (sum phi_2 c_2 / sum phi_2) at the end.
 * pf_adj_gradient(objective 0 or 1) then returns dJ/ds by the hand-written
 * reverse sweep (segments recomputed from the checkpoints, discrete decisions
 * of every step held fixed).  checkpoint_every = 0 is the record mode: the
 * forward keeps every step's record on the device ((72 + 4*n_sub) bytes per
 * cell and step in FP32, (136 + 8*n_sub) in FP64; PF_ERR_NOMEM when it does
 * not fit) and the gradient only sweeps backwards.  pf_adj_timings: ms of the last forward and of the last gradient
 * (recomputation included). */
typedef struct pf_adj pf_adj;
int pf_adj_create(const pf_model *model, int precision, int checkpoint_every, pf_adj **out);
int pf_adj_upload(pf_adj *a, const int32_t *ids, const double *phi, const double *phase, const double *C,
                  double time);
int pf_adj_set_scales(pf_adj *a, const double scales[4]);
int pf_adj_forward(pf_adj *a, int nsteps, double J[2]);
int pf_adj_gradient(pf_adj *a, int objective, double grad[4]);
int pf_adj_timings(pf_adj *a, double ms[2]);
/* Phase fractions [N*3] and total carbon [N] at the end of the last forward run
 * (the four-slot model: the FP64 reference for the FP32 compact path). */
int pf_adj_final_state(pf_adj *a, double *phase, double *C);
int pf_adj_destroy(pf_adj *a);

/* Reference output writers (write_data.cpp:3-82).  pf_write_data appends a
 * fraction_time.txt row under 'directory' when the reference would (or when
 * forced) and, if the model's micro_out flag is set, writes a VTI file. */
int pf_write_data(pf_ctx *ctx, const char *directory, int forced, int *written);
int pf_write_vti(const char *path, int ix, int iy, int iz, double dx, const int32_t *ids,
                 const double *C);

/* The seeded initial state of 'spec' at 'time' generated on the device,
 * straight into the context (replaces pf_init_microstructure + upload; no
 * host arrays).  The same generator code as pf_init_microstructure, run one
 * cell per thread: the grain ids and solutes equal the host's, the phase
 * values agree to a few ulp (the device's tanh).  PF_ERR_RANGE if more than
 * 256 nuclei or particles lie near one cell. */
int pf_init_device(pf_ctx *ctx, const pf_init_spec *spec, double time);

/* Coherent partners of the austenite grains (Fortran model's Coherent_grain,
 * sparse.f90:298-315, set at nucleation by module_nucleation.f90:357-367):
 * partners[2*n + k], k = 0, 1, is a ferrite grain id coherent with austenite
 * grain 200001 + n, or 0; n_austenite <= 100000 entries (later austenite ids
 * have none).  Copied to the device; replaces any earlier table.  Used by a
 * model with coherent = 1 (PF_ERR_ARG otherwise). */
int pf_set_coherent_grains(pf_ctx *ctx, const int32_t *partners, int n_austenite);
/* The table of the seeded state of 'spec', by the Fortran's rule for
 * nucleation in a grain boundary (module_nucleation.f90:357-367): at the cell
 * of nucleus n, before any nucleus is laid, Or_num = min(2, number of ferrite
 * grains - 1) partners, the largest ferrite ids there.  partners[2*n_nuclei]. */
int pf_init_coherent(const pf_model *model, const pf_init_spec *spec, int32_t *partners);

/* Microstructure files in appended raw binary VTK image data, written from
 * the device state while stepping continues (the MPI variant's piece files and
 * .pvti index, C++-MPI/source/write_data.cpp:30-110, with the fields of
 * write_data.cpp:42-82: Int32 "korn" = 0 where the second slot is occupied,
 * else the phase of the first grain; Float32 "conc" = total carbon).  The
 * fields are formed by a kernel on the context's stream, copied to pinned
 * memory on a stream of their own and written by a host thread as 'pieces'
 * z slabs (neighbours share a plane) named <index:07d>_<piece>.vti, plus
 * <index:07d>.pvti.  Returns once the kernel is enqueued; a later call (or
 * pf_write_wait) first waits for the write in flight.  pf_write_wait returns
 * that write's status. */
int pf_write_vti_binary(pf_ctx *ctx, const char *directory, int index, int pieces);
int pf_write_wait(pf_ctx *ctx);
/* The same files from host arrays korn[N], conc[N] (synchronous). */
int pf_write_vti_binary_host(const char *directory, int index, int pieces, int ix, int iy, int iz, double dx,
                             const int32_t *korn, const float *conc);

/* No counterpart in the reference.  The statistics of pf_reduce (same 8
 * outputs, written to the device array d_out) for caller-owned device arrays in
 * the reference layout, computed without allocating anything: for callers that
 * cannot call cudaMalloc -- an application pool that owns all device memory, a
 * framework caching allocator, or a loop that cannot take cudaMalloc's implicit
 * device synchronisation.  The scratch is a fixed 256 KiB __device__ array
 * held by every GPU that loads the library; N is limited to
 * PF_NOALLOC_MAX_CELLS (PF_ERR_RANGE beyond it).  The first call on a device
 * looks up the array's device address (once per device, kept for the life of
 * the process) and should come before any stream capture; a cudaDeviceReset
 * invalidates that address, so calls on a device after it has been reset are
 * not supported.  Asynchronous on cuda_stream (NULL = the legacy default
 * stream); calls that overlap on the GPU share the array and race. */
#define PF_NOALLOC_MAX_CELLS 16777216LL
int pf_reduce_noalloc(long long N, int nsol, const int32_t *d_ids, const double *d_phi,
                      const double *d_phase, const double *d_C, double *d_out, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
