/*
 * pf_oracle.h -- CPU oracle for the Steinbach multi-phase-field time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: it is linked by the
 * tests, by __graft_entry__.smoke() and by bench.py's cpu_baseline / reference
 * arm, never by the product library.  It is a plain-C FP64 restatement of the
 * reference's OpenMP CPU path (zhubq/PhaseField, C++-openmp-cuda/src/), with
 * the reference's operation order kept literally so that the product's FP64
 * GPU path can be compared bit-for-bit.
 *
 * Parity status: the reference ships no tests, golden vectors or recorded
 * outputs, and its C++ needs Blitz++ (absent here); its unmodified CPU sources
 * are built against a minimal Blitz++ stand-in (oracle/blitz_shim), and full
 * time steps of that build (phase sweep, driver, thermo, diffusion) are the
 * golden vectors this oracle matches bit for bit (tests/test_golden.py).  The
 * partition and diffusion sub-step are also checked against the reference's
 * own CUDA kernels (gpu_solver.cpp) compiled from source.
 *
 * Layout (the reference's, phase_field.h:81-89): Blitz fortranArray with the
 * slot / phase index fastest, then x, y, z.  Here 0-based and flat:
 *   ids[s + 6*n], phi[s + 6*n], phase[p + 3*n], conc[q][p + 3*n], C[q][n]
 * with n = i + ix*(j + iy*k) and q the solute (0 = carbon, 1 = Mn).
 * 3x3 matrices are column-major: (i,j) (1-based) at (i-1) + 3*(j-1).
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFO_NSLOT 6      /* max_num_coexist, constant.h:5 */
#define PFO_NPHASE 3     /* max_num_phase, constant.h:6 */
#define PFO_NSTENCIL 10  /* max_num_nonzero_stencil, solver.cpp:148 */
#define PFO_MAXSOL 2
#define PFO_MAXT 64

typedef struct {
    int ix, iy, iz;
    double dx;
    int i_intf;
    double cutoff;
    int nT;
    double T_time[PFO_MAXT], T_temp[PFO_MAXT];
    double m0[9], mQ[9];          /* interface mobility prefactor / activation energy */
    double sigma[9];              /* interface energy */
    int nsol;                     /* 1 = carbon only (reference), 2 = carbon + Mn */
    double D0[PFO_MAXSOL][3], DQ[PFO_MAXSOL][3];
    double ent_a[9], ent_b[9];    /* entropy functor a*T+b  (thermo_functor.cpp:20-25) */
    double eq_a[9], eq_b[9], eq_c[9]; /* PARA functor a*T^2+b*T+c (thermo_functor.cpp:45-50) */
    double mn_ratio[3];           /* Mn partition ratios r_p: c_p = r_p * c_ref (solute 2 only) */
    int thermo_model;             /* 1: the Fortran model's polynomial thermodynamics (sparse.f90:797-923) */
    int avg_carbon;               /* 1: interface-averaged concentrations in the driving force (sparse.f90:184-255) */
    int drag;                     /* 1: Purdy-Brechet solute drag (sparse.f90:326-360, 538-671, 958-1041) */
    double drag_binding, drag_vmax0, drag_qsd;
    int coherent;                 /* 1: coherent-grain mobility (sparse.f90:298-315) */
    int coh_npp0;                 /* last id of the initial ferrite class (Npp0) */
} pfo_model;

typedef struct {
    double T;
    double m[9];
    double D[PFO_MAXSOL][3];
    double pfm_dt, diff_dt;
    int n_sub;
    double dt_sub;
    double entropy[9], eq[9], dcdT[9];
    double k[PFO_MAXSOL][9], c[PFO_MAXSOL][9];
    double dims;                  /* 'dimensions' is a real in the reference */
    double eta;
    int df_model;                 /* 1: driving force -ratio_ij*(max(c_i,c_j) - ref) (sparse.f90:512-515) */
    double df_ratio[9], df_ref;
    int avg_range;                /* > 0: half-width of the scanned neighbourhood (i_intf + 1) */
    int avg_conc;                 /* 1: the driving force reads the averaged concentrations */
    int drag_model;
    double drag_vmax, drag_ex0, drag_de_heat, drag_de_cool, drag_u0;
    double drag_corr[2], drag_drag0[2];
    int coh_model, coh_npp0;
} pfo_params;

typedef struct {
    int32_t *ids1, *ids2;   /* [N*6] */
    double *phi1, *phi2;    /* [N*6] */
    double *phase;          /* [N*3] */
    double *conc1, *conc2;  /* [nsol][N*3] */
    double *C;              /* [nsol][N] */
} pfo_state;

/* phase_field.h:25-29 */
int pfo_phase_of_grain(int grain);
/* phase_field.cpp:232-242 (Temperature_function) */
double pfo_temperature(const pfo_model *m, double time);
/* phase_field.cpp:307-315 + thermo_data.cpp:24-41 + phase_field.cpp:247-248 */
void pfo_params_at(const pfo_model *m, double time, pfo_params *p);
/* solver.cpp:389-405 */
void pfo_partition(double C, const double *phase3, const double *k9, const double *c9, double *out3);
/* Partition every cell: conc[q] = Partitioning(C[q], phase) (MicrostructureConstruction.cpp:53-62) */
void pfo_partition_all(const pfo_model *m, const pfo_params *p, const double *phase,
                       const double *C, double *conc);
/* solver.cpp:147-304 over all cells (phase_field.cpp:252-257) */
void pfo_phase_sweep(const pfo_model *m, const pfo_params *p, const int32_t *ids1, const double *phi1,
                     int32_t *ids2, double *phi2, double *phase, double *conc1, const double *C);
/* sparse.f90:184-255: interface-averaged phase concentrations of every cell;
 * flags (may be NULL): bit 0 Has_ferrite, bit 1 Rex_intf of the same scan */
void pfo_avg_conc(const pfo_model *m, const pfo_params *p, const int32_t *ids1, const double *phase,
                  const double *conc1, double *avg, unsigned char *flags);
/* Coherent_grain: partners[2n + k] of austenite grain 200001 + n (copied) */
void pfo_set_coherent(const int32_t *partners, int n_austenite);
/* solver.cpp:343-372 over all cells (phase_field.cpp:274-280) */
void pfo_diffusion_substep(const pfo_model *m, const pfo_params *p, double dt_sub, const double *phase,
                           const double *conc1, double *conc2, double *C);
/* phase_field.cpp:243-305 (Update(false)), nsteps times.  time is advanced as
 * Update_parameter does.  On return the current state is in the "1" buffers. */
void pfo_run(const pfo_model *m, pfo_state *s, double *time, int nsteps);
/* gpu_solver.cpp:204-218 semantics (0.2f stability factor, 6 neighbours,
 * partition-then-flux per sub-step); C updated in place, conc_out = final
 * partition (what phase_field.cpp:291-297 recomputes on the host). */
int pfo_gpu_diffusion_solver(const double *D3, const double *k9, const double *c9,
                             const double *phase, double *C, int x, int y, int z,
                             double dt, double dx, double *conc_out);
/* write_data.cpp:14-18: out[0..2] = sum(value_phase(p))/N, out[3] = deformed fraction */
void pfo_fractions(const pfo_model *m, const int32_t *ids, const double *phi, const double *phase,
                   double *out4);
int pfo_num_threads(void);
/* Nonzero once a solute-drag iteration found no root (cleared by the caller). */
extern int pfo_drag_failures;
double pfo_dissipation(double unchanged, double driv, double drag, double norm, int heating, const pfo_params *p);
double pfo_exp(double x);
double pfo_log(double x);
void pfo_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
