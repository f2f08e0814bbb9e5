/*
 * pf_oracle.c -- FP64 CPU oracle of the Steinbach multi-phase-field step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle; never linked into the product).
 * Pinned: tests/test_golden.py checks it bit for bit against full time steps
 * of the reference's own CPU code (built unmodified against the minimal
 * Blitz++ stand-in of oracle/blitz_shim; tests/golden/ref_cpu_steps.npz) and
 * against the reference's CUDA diffusion kernels (ref_gpu_diffusion.npz); the
 * Fortran-model options are checked against literal restatements of the
 * Fortran loops in the tests (no Fortran compiler here).  Every function cites
 * the reference file:line (paths inside zhubq/PhaseField) it restates.  The
 * arithmetic follows the reference's evaluation order operation by operation;
 * build with -ffp-contract=off so that no multiply-add is fused.
 */
#include "pf_oracle.h"
#include <math.h>

#include "pf_math.h" /* exp/log shared with the product's GPU kernel (identical rounding) */

int pfo_drag_failures; /* set when a solute-drag iteration finds no root (the Fortran stops) */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PFO_PI = 3.1415926; /* constant.h:7 (truncated on purpose) */
static const double PFO_R = 8.314;      /* constant.h:8 */
#define MAXGRAIN_PER_PHASE 100000       /* phase_field.h:19 */

#define M3(a, i, j) ((a)[((i)-1) + 3 * ((j)-1)]) /* 1-based column-major 3x3 */

int pfo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void pfo_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* phase_field.h:25-29 */
int pfo_phase_of_grain(int grain) {
    if (grain == 0) return 0;
    return (grain / MAXGRAIN_PER_PHASE > 0 ? grain / MAXGRAIN_PER_PHASE : 1);
}

/* phase_field.h:58-68 (Get_neighbor), restated 0-based */
static inline int nb(int i, int len, int d) {
    int g = i + d;
    if (g >= len) g -= len;
    else if (g < 0) g += len;
    return g;
}

/* phase_field.cpp:232-242.  The reference leaves Temp uninitialised when no
 * segment matches; the oracle returns the last profile temperature then. */
double pfo_temperature(const pfo_model *m, double t) {
    double Temp = m->T_temp[m->nT - 1];
    for (int i = 0; i < m->nT - 1; i++)
        if (t >= m->T_time[i] && t < m->T_time[i + 1])
            Temp = (m->T_temp[i + 1] - m->T_temp[i]) / (m->T_time[i + 1] - m->T_time[i]) *
                       (t - m->T_time[i]) + m->T_temp[i];
    return Temp;
}

static double model_dims(const pfo_model *m) {
    /* phase_field.cpp:354-362 */
    double d = 3;
    if (m->iz == 1) d -= 1;
    if (m->iy == 1) d -= 1;
    return d;
}

/* phase_field.cpp:307-315 (Update_parameter, without the time increment),
 * thermo_data.cpp:24-41 (Get_data), phase_field.cpp:247-248 (sub-cycling). */
/* The Fortran intercritical-annealing model's thermodynamics
 * (Fortran_openmp_phase_field/PFM/src/sparse.f90:797-923 THERMO_DATA, with
 * poly4 / diff_poly4 of util_func.f90:491-503): para equilibrium lines
 * Ref_c_para and slopes 1/diff_poly4; Ref_c_para(1,3) = (1,2), (3,1) = (2,3)
 * = (3,2) = (2,1) (sparse.f90:882-889); the diagonal keeps the initial
 * Ref_c_para = 0, Slope_para = 1 (pre_process.f90:139-140).  In the C++
 * model's terms eq_ij = Ref_c_para(i,j) and dcdT_ij = diff_poly4, so the
 * partition of thermo_data.cpp:34-40 that follows is Partition_k_para(j,i),
 * Partition_c_para(j,i).  Ratio_k_para (sparse.f90:916-921) drives the
 * austenite pairs: driving_force = -Ratio_k_para(i,j) (max(c_i, c_j) -
 * Ref_c_para(2,1)) (sparse.f90:512-515; the stored energy of deformed grains
 * is not modelled).  Double precision (the Fortran declares default REAL). */
static double f90_poly4(double x, double a, double b, double c, double d) {
    return a * x + b * x * x + c * x * x * x + d * x * x * x * x;
}
static double f90_diff_poly4(double x, double a, double b, double c, double d) {
    return a + 2 * b * x + 3 * c * x * x + 4 * d * x * x * x;
}
static void f90_thermo(double T, pfo_params *p) {
    double ref[9], slope_d[9], ratio[9];
    for (int e = 0; e < 9; e++) {
        ref[e] = 0.;
        slope_d[e] = 1.;
        ratio[e] = 0.;
    }
    if (T < 1086.52) {
        M3(ref, 1, 2) = f90_poly4(T - 273.15, -8.309e-5, 0., 0., 0.) + 6.883e-2;
        M3(ref, 2, 1) = f90_poly4(T - 273.15, 2.607e-2, -6.58e-5, 3.984e-8, 0.) + 0.9115;
        M3(slope_d, 1, 2) = f90_diff_poly4(T - 273.15, -8.309e-5, 0., 0., 0.);
        M3(slope_d, 2, 1) = f90_diff_poly4(T - 273.15, 2.607e-2, -6.58e-5, 3.984e-8, 0.);
    } else {
        M3(ref, 1, 2) = f90_poly4(T - 1086.52, -1.1428e-4, 0., 0., 0.);
        M3(ref, 2, 1) = f90_poly4(T - 1086.52, -0.00325, 0., 0., 0.);
        M3(slope_d, 1, 2) = f90_diff_poly4(0., -1.1428e-4, -1.78883e-7, -3.66186e-10, 2.53049e-12);
        M3(slope_d, 2, 1) = f90_diff_poly4(0., -0.00325, 1.13712e-5, -2.88193e-8, 1.05482e-10);
    }
    M3(ref, 1, 3) = M3(ref, 1, 2);
    M3(ref, 3, 1) = M3(ref, 2, 1);
    M3(slope_d, 1, 3) = M3(slope_d, 1, 2);
    M3(slope_d, 3, 1) = M3(slope_d, 2, 1);
    M3(ref, 2, 3) = M3(ref, 2, 1);
    M3(ref, 3, 2) = M3(ref, 2, 1);
    M3(slope_d, 2, 3) = M3(slope_d, 2, 1);
    M3(slope_d, 3, 2) = M3(slope_d, 2, 1);
    const double x = T - 273.15;
    M3(ratio, 1, 2) = (0.000264 * x * x - 0.4466 * x + 243.4713) * 1.03e-12;
    M3(ratio, 2, 1) = -M3(ratio, 1, 2);
    M3(ratio, 3, 2) = M3(ratio, 1, 2);
    M3(ratio, 2, 3) = -M3(ratio, 3, 2);
    M3(ratio, 2, 2) = 0.;
    for (int e = 0; e < 9; e++) {
        p->entropy[e] = 0.;
        p->eq[e] = ref[e];
        p->dcdT[e] = slope_d[e];
        p->df_ratio[e] = ratio[e];
    }
    p->df_ref = M3(ref, 2, 1);
    p->df_model = 1;
}

/* SOLUTE_DRAG_PB (sparse.f90:1005-1037), literally. */
static double f90_solute_drag_pb(double V0, double E0, double De, double U0, double V_max, double Temperature) {
    const double V = V0 / V_max;
    const double A = (De - E0) + V;
    const double B = (De + E0) + V;
    const double D0 = 1. - U0;
    const double Vu0 = V * U0;
    const double D1_d0 = (A - Vu0) / (A * D0 + (A - V) * U0 * pf_exp(-(A - Vu0)));
    const double D1 = D0 * D1_d0;
    const double U1 = 1. - D1;
    const double D2_d1 = (B - Vu0) / (B * D1 + (B * U1 - Vu0) * pf_exp(-(B - Vu0)));
    return (2. * De * U0 - ((A - V) / A * (Vu0 + pf_log(D1_d0)) + (B - V) / B * (Vu0 + pf_log(D2_d1)))) * 8.314 *
           Temperature / 7.2e12;
}

/* DISSIPATION_ITERATION (sparse.f90:538-605; heating) and _R (607-660;
 * cooling), literally; Solution enters with the caller's value and keeps it
 * when no bracket is found (the _R variant stops the Fortran program there:
 * counted in pfo_drag_failures).  The bisection gets a limit of 200 halvings
 * the Fortran loop lacks (reached only for a root at exactly zero). */
static double f90_dissipation(double Solution, double Driv, double Drag, double Norm, int heating,
                              const pfo_params *p) {
    const double drag0 = heating ? p->drag_drag0[0] : p->drag_drag0[1];
    const double De = heating ? p->drag_de_heat : p->drag_de_cool;
    const double Cf = heating ? p->drag_corr[0] : p->drag_corr[1];
    double Err1, Err2 = Driv - Drag * drag0, Dv, V, X1, X2, Tmp_v, Tmp_err;
    if (Err2 < 0.) return 0.;
    Dv = 0.1 * p->drag_vmax;
    V = 0.;
    for (int J = 1; J <= 2; J++) {
        for (int I = 1; I <= 40; I++) {
            Err1 = Err2;
            V = V + Dv;
            Err2 = Driv - V * Norm - Drag * (f90_solute_drag_pb(V, p->drag_ex0, De, p->drag_u0, p->drag_vmax, p->T) * Cf);
            if (Err1 * Err2 <= 0.) {
                X1 = V - Dv;
                X2 = V;
                int it = 0;
                while ((X2 - X1) > 0.01 * X2) {
                    if (++it > 200) {
                        pfo_drag_failures = 1;
                        break;
                    }
                    Tmp_v = 0.5 * (X1 + X2);
                    Tmp_err = Driv - Tmp_v * Norm -
                              Drag * (f90_solute_drag_pb(Tmp_v, p->drag_ex0, De, p->drag_u0, p->drag_vmax, p->T) * Cf);
                    if (Err1 * Tmp_err <= 0.) {
                        X2 = Tmp_v;
                        Err2 = Tmp_err;
                    } else {
                        X1 = Tmp_v;
                        Err1 = Tmp_err;
                    }
                }
                return 0.5 * (X1 + X2) * Norm;
            }
        }
        V = Driv / Norm;
        Dv = -0.2 * V;
        Err2 = -1.;
    }
    if (!heating) pfo_drag_failures = 1;
    return Solution;
}

/* DISSIPATION_ITERATION / _R as the sweep calls them, exported so the tests
 * can check the velocity solve against a literal restatement of the Fortran. */
double pfo_dissipation(double unchanged, double driv, double drag, double norm, int heating, const pfo_params *p) {
    return f90_dissipation(unchanged, driv, drag, norm, heating, p);
}

/* The shared exp/log, exported so the tests can check them against the C
 * library and against the GPU build. */
double pfo_exp(double x) { return pf_exp(x); }
double pfo_log(double x) { return pf_log(x); }

/* PARAMETER_DRAG_PB (sparse.f90:958-1003) restated: V_max, M_nple, N_nple,
 * Ux0, De_heat, De_cool, Ex0, Driv_f (with Ref_c_nple(2,1) and
 * Ref_c_nple_r(2,1) of THERMO_DATA, sparse.f90:844-880; the latter stays at
 * its initial 0 below 1041.3 K), Drag0 and Correct_factor.  exp/log are
 * pf_exp/pf_log, as in the product, so both round alike. */
static double f90_max(double a, double b) { return a > b ? a : b; }
static void f90_drag(const pfo_model *m, double T, pfo_params *p) {
    p->drag_vmax = m->drag_vmax0 * pf_exp(-m->drag_qsd / (8.314 * T));
    const double x = T - 273.15;
    double M_nple[3], N_nple[3];
    M_nple[0] = f90_max(1.E-10, 3.9793e-5 * x - 2.3163e-2);
    M_nple[1] = f90_max(1.E-10, -2.928e-8 * (x * x) + 5.629e-5 * x - 2.35e-2);
    M_nple[2] = f90_max(1.E-10, 2.253e-8 * (x * x) - 4.255e-5 * x + 2.351e-2);
    N_nple[0] = f90_max(1.E-10, -3.818e-9 * (x * x * x) + 9.055e-6 * (x * x) - 7.408e-3 * x + 2.118);
    N_nple[1] = f90_max(1.E-10, -7.1227e-10 * (x * x * x) + 1.6307e-6 * (x * x) - 1.2584e-3 * x + 3.3166e-1);
    N_nple[2] = 3.E-3;
    const double Ux0[3] = {1.887e-2, 3.65e-3, 3.12e-3};
    double De_heat[3], De_cool[3];
    for (int i = 0; i < 3; i++) {
        De_heat[i] = -0.5 * pf_log(M_nple[i] * (1. - Ux0[i]) / (Ux0[i] * (1. - M_nple[i])));
        De_cool[i] = -0.5 * pf_log(N_nple[i] * (1. - Ux0[i]) / (Ux0[i] * (1. - N_nple[i])));
    }
    const double Ex0 = m->drag_binding / (8.314 * T);
    const double ref_nple21 = T < 1110.64 ? f90_poly4(T - 1110.64, -3.3441e-3, 1.0406e-5, -5.6345e-8, 0.0)
                                          : f90_poly4(T - 1110.64, -3.23154e-3, 0., 0., 0.);
    const double ref_nple_r21 = T < 1041.3 ? 0. : -2.39e-3 * (T - 1041.3);
    const double Driv_f1 = fabs(M3(p->df_ratio, 2, 1) * (M3(p->eq, 2, 1) - ref_nple21));
    const double Driv_f2 = fabs(M3(p->df_ratio, 2, 1) * (M3(p->eq, 2, 1) - ref_nple_r21));
    const double vm = p->drag_vmax;
    double Drag0_1 = f90_solute_drag_pb(0., Ex0, De_heat[0], Ux0[0], vm, T) + f90_solute_drag_pb(0., 0., De_heat[1], Ux0[1], vm, T) +
                     f90_solute_drag_pb(0., 0., De_heat[2], Ux0[2], vm, T);
    double Drag0_2 = f90_solute_drag_pb(0., Ex0, De_cool[0], Ux0[0], vm, T) + f90_solute_drag_pb(0., 0., De_cool[1], Ux0[1], vm, T) +
                     f90_solute_drag_pb(0., 0., De_cool[2], Ux0[2], vm, T);
    const double Correct_factor1 = Driv_f1 / Drag0_1, Correct_factor2 = Driv_f2 / Drag0_2;
    Drag0_1 = f90_solute_drag_pb(0., Ex0, De_heat[0], Ux0[0], vm, T) * Correct_factor1;
    Drag0_2 = f90_solute_drag_pb(0., Ex0, De_cool[0], Ux0[0], vm, T) * Correct_factor2;
    p->drag_ex0 = Ex0;
    p->drag_de_heat = De_heat[0];
    p->drag_de_cool = De_cool[0];
    p->drag_u0 = Ux0[0];
    p->drag_corr[0] = Correct_factor1;
    p->drag_corr[1] = Correct_factor2;
    p->drag_drag0[0] = Drag0_1;
    p->drag_drag0[1] = Drag0_2;
    p->drag_model = 1;
}

void pfo_params_at(const pfo_model *m, double time, pfo_params *p) {
    memset(p, 0, sizeof(*p));
    const double T = pfo_temperature(m, time);
    p->T = T;
    p->dims = model_dims(m);
    p->eta = m->dx * m->i_intf; /* phase_field.cpp:363 */
    const double RT = PFO_R * T;
    double maxms = -INFINITY;
    for (int e = 0; e < 9; e++) {
        p->m[e] = m->m0[e] * exp(-m->mQ[e] / RT);
        double ms = p->m[e] * m->sigma[e];
        if (ms > maxms) maxms = ms;
    }
    double maxD = -INFINITY;
    for (int q = 0; q < m->nsol; q++)
        for (int ph = 0; ph < 3; ph++) {
            p->D[q][ph] = m->D0[q][ph] * exp(-m->DQ[q][ph] / RT);
            if (p->D[q][ph] > maxD) maxD = p->D[q][ph];
        }
    p->pfm_dt = m->dx * m->dx / p->dims * 0.2 / maxms;
    p->diff_dt = m->dx * m->dx / maxD / p->dims * 0.2;

    p->df_model = 0;
    p->drag_model = 0;
    p->avg_range = (m->avg_carbon || m->coherent) ? m->i_intf + 1 : 0; /* sparse.f90:186 */
    p->avg_conc = m->avg_carbon;
    p->coh_model = m->coherent;
    p->coh_npp0 = m->coh_npp0;
    if (m->thermo_model == 1) {
        f90_thermo(T, p);
        if (m->drag) f90_drag(m, T, p);
    } else {
        /* thermo_data.cpp:25-32: functor evaluation; linear_functor.h:11-13,
         * quadratic_functor.h:12-14.  Unset functors are zero. */
        for (int j = 1; j <= 3; j++)
            for (int i = 1; i <= 3; i++) {
                const double x = T;
                M3(p->entropy, i, j) = M3(m->ent_a, i, j) * x + M3(m->ent_b, i, j);
                M3(p->eq, i, j) = M3(m->eq_a, i, j) * x * x + M3(m->eq_b, i, j) * x + M3(m->eq_c, i, j);
                M3(p->dcdT, i, j) = (2 * M3(m->eq_a, i, j)) * x + M3(m->eq_b, i, j);
            }
    }
    /* thermo_data.cpp:34-40 */
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            if (i == j) M3(p->dcdT, i, j) = 1.;
            M3(p->k[0], i, j) = M3(p->dcdT, j, i) / M3(p->dcdT, i, j);
            M3(p->c[0], i, j) = M3(p->eq, j, i) - M3(p->k[0], i, j) * M3(p->eq, i, j);
        }
    /* Mn (no reference counterpart): c_p proportional to r_p.  In the sense of
     * solver.cpp:389-405, k_ij is defined by c_j = k_ij*c_i + c_ij, so
     * k_ij = r_j/r_i and c_ij = 0. */
    if (m->nsol > 1)
        for (int i = 1; i <= 3; i++)
            for (int j = 1; j <= 3; j++) {
                M3(p->k[1], i, j) = m->mn_ratio[j - 1] / m->mn_ratio[i - 1];
                M3(p->c[1], i, j) = 0.;
            }
    /* phase_field.cpp:247-248 */
    int n = (int)ceil(p->pfm_dt / p->diff_dt);
    p->n_sub = n > 1 ? n : 1;
    p->dt_sub = p->pfm_dt / p->n_sub;
}

/* solver.cpp:389-405 */
void pfo_partition(double C, const double *phase3, const double *k9, const double *c9, double *out3) {
    for (int i = 1; i <= 3; i++) {
        double t1 = 0., t2 = 0.;
        for (int j = 1; j <= 3; j++) {
            t1 += phase3[j - 1] * M3(k9, i, j);
            t2 += phase3[j - 1] * M3(c9, i, j);
        }
        out3[i - 1] = (C - t2) / t1;
    }
}

void pfo_partition_all(const pfo_model *m, const pfo_params *p, const double *phase,
                       const double *C, double *conc) {
    const long N = (long)m->ix * m->iy * m->iz;
    for (int q = 0; q < m->nsol; q++) {
#pragma omp parallel for schedule(static)
        for (long n = 0; n < N; n++)
            pfo_partition(C[q * N + n], phase + 3 * n, p->k[q], p->c[q], conc + q * 3 * N + 3 * n);
    }
}

/* solver.cpp:374-387 (Driving_force); uses only the carbon concentration of
 * phase ii -- or, with the Fortran model's thermodynamics, the larger of the
 * two phases' carbon (sparse.f90:512-515). */
static inline double driving_force(const pfo_params *p, int phii, int phjj, double concii, double concjj) {
    double df = 0.;
    if (phii != phjj) {
        if (p->df_model == 1)
            df -= M3(p->df_ratio, phii, phjj) * (fmax(concii, concjj) - p->df_ref);
        else
            df += M3(p->entropy, phii, phjj) * (concii - M3(p->eq, phii, phjj)) / M3(p->dcdT, phii, phjj);
    }
    return df;
}

/* solver.cpp:147-304 (Phase_field_solver) for cell (i,j,k), 0-based. */
/* Coherent_grain (pre_process.f90:238, module_nucleation.f90:357-367):
 * two ferrite ids per austenite grain; Any(Coherent_grain(aus,:) == other) */
static int32_t *pfo_coh = NULL;
static int pfo_n_coh = 0;
static int coherent_with(int aus, int other) {
    const int k = aus - 200001;
    if (k < 0 || k >= pfo_n_coh || other == 0) return 0;
    return pfo_coh[2 * k] == other || pfo_coh[2 * k + 1] == other;
}

static void phase_cell(const pfo_model *m, const pfo_params *p, int i, int j, int k,
                       const int32_t *ids1, const double *phi1, int32_t *ids2, double *phi2,
                       double *phase, double *conc1, const double *C, const double *dfconc,
                       const unsigned char *flags) {
    const int ix = m->ix, iy = m->iy, iz = m->iz;
    const long N = (long)ix * iy * iz;
    const long n = i + (long)ix * (j + (long)iy * k);
    const double cutoff = m->cutoff;
    /* solver.cpp:149-157: 1-based arrays of length 10, zero-initialised */
    int sid[PFO_NSTENCIL + 1] = {0}, sph[PFO_NSTENCIL + 1] = {0};
    double sv1[PFO_NSTENCIL + 1] = {0}, sv2[PFO_NSTENCIL + 1] = {0};
    int num_local = 0, num = 0;
    /* solver.cpp:159-166: neighbour order x-, x+, y-, y+, z-, z+ */
    long nbr[6];
    nbr[0] = nb(i, ix, -1) + (long)ix * (j + (long)iy * k);
    nbr[1] = nb(i, ix, 1) + (long)ix * (j + (long)iy * k);
    nbr[2] = i + (long)ix * (nb(j, iy, -1) + (long)iy * k);
    nbr[3] = i + (long)ix * (nb(j, iy, 1) + (long)iy * k);
    nbr[4] = i + (long)ix * (j + (long)iy * nb(k, iz, -1));
    nbr[5] = i + (long)ix * (j + (long)iy * nb(k, iz, 1));

    /* solver.cpp:168-175: own slots above cutoff, stored at their slot position */
    for (int ii = 1; ii <= PFO_NSLOT; ii++) {
        if (phi1[6 * n + ii - 1] > cutoff) {
            num_local += 1;
            sid[ii] = ids1[6 * n + ii - 1];
            sph[ii] = pfo_phase_of_grain(ids1[6 * n + ii - 1]);
            sv1[ii] = phi1[6 * n + ii - 1];
        }
    }
    num = num_local;
    /* solver.cpp:179-205: merge the neighbours' lists (break at id 0) */
    for (int ii = 1; ii <= 2 * p->dims; ii++) {
        const long q = nbr[ii - 1];
        for (int jj = 1; jj <= PFO_NSLOT; jj++) {
            int tid = ids1[6 * q + jj - 1];
            if (tid == 0) break;
            double tv = phi1[6 * q + jj - 1];
            int kk;
            for (kk = 1; kk <= PFO_NSTENCIL; kk++) {
                if (tid == sid[kk]) {
                    sv2[kk] += tv;
                    break;
                }
            }
            if (kk > PFO_NSTENCIL && num < PFO_NSTENCIL) {
                num += 1;
                sid[num] = tid;
                sph[num] = pfo_phase_of_grain(tid);
                sv2[num] += tv;
            }
        }
    }
    /* solver.cpp:207-216: bulk fast path */
    if (num == 1) {
        for (int ii = 0; ii < PFO_NSLOT; ii++) {
            ids2[6 * n + ii] = ids1[6 * n + ii];
            phi2[6 * n + ii] = phi1[6 * n + ii];
        }
        return;
    }
    /* solver.cpp:224-266 */
    double del[PFO_NSTENCIL + 1] = {0};
    const double factor1 = 1. / (m->dx * m->dx);
    const double factor2 = PFO_PI * PFO_PI / (2. * p->eta * p->eta);
    const double factor3 = PFO_PI / p->eta;
    double local_conc[4];
    for (int ii = 1; ii <= 3; ii++) local_conc[ii] = dfconc[3 * n + ii - 1]; /* carbon */
    double drag[PFO_NSTENCIL + 1];
    for (int ii = 0; ii <= PFO_NSTENCIL; ii++) drag[ii] = 0.;
    /* sparse.f90:300-306: Count(Phase_index(Ind_ph1(1:N_nonzero))==1) == 1,
     * .Not. Rex_intf, Has_ferrite */
    int coh_cell = 0;
    if (p->coh_model && flags) {
        int n_nonzero = 0, n_ferrite = 0;
        for (int a = 0; a < PFO_NSLOT; a++)
            if (phi1[6 * n + a] > cutoff) n_nonzero++;
        for (int a = 0; a < n_nonzero; a++)
            if (pfo_phase_of_grain(ids1[6 * n + a]) == 1) n_ferrite++;
        coh_cell = (flags[n] & 1) && !(flags[n] & 2) && n_ferrite == 1;
    }
    for (int ii = 1; ii <= num; ii++) {
        const int gi = sid[ii], phi_ = sph[ii];
        for (int jj = 1; jj <= num; jj++) {
            if (ii == jj) continue;
            const int phj = sph[jj];
            if (abs(phi_ - phj) == 2) continue;
            double d = 0.;
            d = (sv2[ii] * sv1[jj] - sv2[jj] * sv1[ii]) * factor1;
            d += (sv1[ii] - sv1[jj]) * factor2;
            d *= M3(m->sigma, phi_, phj);
            d += factor3 * sqrt(sv1[ii] * sv1[jj]) *
                 driving_force(p, phi_, phj, local_conc[phi_], local_conc[phj]);
            /* sparse.f90:298-315: a pair whose austenite grain is coherent
             * with the other grain moves at 0.02 of the mobility */
            const int coherent = coh_cell && ((phi_ == 2 && coherent_with(gi, sid[jj])) ||
                                              (phj == 2 && coherent_with(sid[jj], gi)));
            if (coherent) d = 0.02 * M3(p->m, phi_, phj) * d;
            else d *= M3(p->m, phi_, phj);
            del[ii] += d;
            /* sparse.f90:287-292: Drag_ij = Factor3 sqrt(phi_i phi_j) for
             * ferrite/austenite, times the mobility */
            if (p->drag_model && phi_ + phj == 3) {
                const double drag_ij = factor3 * sqrt(sv1[ii] * sv1[jj]);
                if (coherent) drag[ii] += 0.02 * M3(p->m, phi_, phj) * drag_ij;
                else drag[ii] += M3(p->m, phi_, phj) * drag_ij;
            }
        }
    }
    /* sparse.f90:326-360: the Fortran model's solute drag.  Only in a cell
     * with ferrite and austenite (Flag_coexist(2)) and without ferrite and
     * cementite (Flag_coexist(1)) above the cutoff, only for the cell's own
     * grains (Ii <= N_nonzero); positive rates of austenite and negative ones
     * of ferrite are growth (DISSIPATION_ITERATION), the others shrinkage
     * (_R); a rate of zero stays zero; with two entries the second rate is
     * the negative of the first (sparse.f90:363-366). */
    if (p->drag_model) {
        const int co1 = phase[3 * n] > cutoff && phase[3 * n + 2] > cutoff;
        const int co2 = phase[3 * n] > cutoff && phase[3 * n + 1] > cutoff;
        int n_nonzero = 0;
        for (int a = 0; a < PFO_NSLOT; a++)
            if (phi1[6 * n + a] > cutoff) n_nonzero++;
        for (int ii = 1; ii <= num; ii++) {
            if (!co1 && co2 && ii <= n_nonzero) {
                const double driv = del[ii];
                const double norm = factor3 * sqrt(sv1[ii] * (1. - sv1[ii])); /* Normal_vec, sparse.f90:263-264 */
                double lst = driv;                                            /* Lst_tmp(Ii) = Driv_matrix(Ii) */
                if (driv > 0.) {
                    if (sph[ii] == 2)
                        lst = f90_dissipation(lst, driv, drag[ii], norm, 1, p);
                    else if (sph[ii] == 1)
                        lst = f90_dissipation(lst, driv, drag[ii], norm, 0, p);
                } else if (driv < 0.) {
                    if (sph[ii] == 1)
                        lst = f90_dissipation(lst, -driv, drag[ii], norm, 1, p);
                    else if (sph[ii] == 2)
                        lst = f90_dissipation(lst, -driv, drag[ii], norm, 0, p);
                    lst = -lst;
                } else {
                    lst = 0.;
                }
                del[ii] = lst;
            }
            if (num == 2) {
                del[2] = -del[1];
                break;
            }
        }
    }
    for (int ii = 1; ii <= num; ii++) {
        del[ii] *= p->pfm_dt;
        del[ii] += sv1[ii];
        if (del[ii] > 1.0) del[ii] = 1.0;
        else if (del[ii] < cutoff) del[ii] = 0.;
    }
    /* solver.cpp:270-271 */
    for (int ii = 0; ii < 3; ii++) phase[3 * n + ii] = 0.;
    /* solver.cpp:273 + 426-432: selection sort, first maximum wins */
    for (int a = 1; a <= PFO_NSTENCIL; a++) {
        int mx = a;
        for (int b = a + 1; b <= PFO_NSTENCIL; b++)
            if (del[b] > del[mx]) mx = b;
        double tv = del[a]; del[a] = del[mx]; del[mx] = tv;
        int ti = sid[a]; sid[a] = sid[mx]; sid[mx] = ti;
    }
    /* solver.cpp:276-296 */
    double sum = 0.;
    for (int ii = 1; ii <= PFO_NSLOT; ii++) {
        if (del[ii] > cutoff) {
            ids2[6 * n + ii - 1] = sid[ii];
            phi2[6 * n + ii - 1] = del[ii];
            int ph = pfo_phase_of_grain(sid[ii]);
            phase[3 * n + ph - 1] += del[ii];
            sum += del[ii];
        } else {
            ids2[6 * n + ii - 1] = 0;
            phi2[6 * n + ii - 1] = 0.;
        }
    }
    for (int ii = 0; ii < PFO_NSLOT; ii++) phi2[6 * n + ii] *= 1. / sum;
    for (int ii = 0; ii < 3; ii++) phase[3 * n + ii] *= 1. / sum;
    /* solver.cpp:299: partition in place (every solute) */
    for (int q = 0; q < m->nsol; q++)
        pfo_partition(C[q * N + n], phase + 3 * n, p->k[q], p->c[q], conc1 + q * 3 * N + 3 * n);
}

/* MYNGB (util_func.f90:33-47) restated 0-based: the cell n places away along
 * an axis of length len, periodic. */
static inline int f90_ngb(int c, int len, int n) {
    int nn = n % len;
    if (nn < 0) nn += len;
    int r = c + nn;
    if (r >= len) r -= len;
    return r;
}

/* The Fortran model's interface-averaged phase concentrations for every
 * cell (sparse.f90:141-146 and 184-255), from the phase fractions and phase
 * concentrations of the start of the sweep (the Fortran loop reads values
 * its own sweep may already have updated; here none are). */
void pfo_avg_conc(const pfo_model *m, const pfo_params *p, const int32_t *ids1, const double *phase,
                  const double *conc1, double *avg, unsigned char *flags) {
    const int ix = m->ix, iy = m->iy, iz = m->iz;
    const double cutoff = m->cutoff;
    const int R = p->avg_range;
#define PH1(x, y, z) phase[3 * ((long)(x) + (long)ix * ((y) + (long)iy * (z)))]
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < iz; k++)
        for (int j = 0; j < iy; j++)
            for (int i = 0; i < ix; i++) {
                const long n = i + (long)ix * (j + (long)iy * k);
                double out[3] = {conc1[3 * n], conc1[3 * n + 1], conc1[3 * n + 2]};
                int has_ferrite = 0, rex_intf = 0; /* sparse.f90:137-139 */
                if (phase[3 * n] > cutoff && phase[3 * n + 1] > cutoff) { /* Flag_coexist(2) */
                    double G[3];
                    G[0] = PH1(f90_ngb(i, ix, 1), j, k) - PH1(f90_ngb(i, ix, -1), j, k);
                    G[1] = PH1(i, f90_ngb(j, iy, 1), k) - PH1(i, f90_ngb(j, iy, -1), k);
                    G[2] = PH1(i, j, f90_ngb(k, iz, 1)) - PH1(i, j, f90_ngb(k, iz, -1));
                    for (int d = 0; d < 3; d++) G[d] = G[d] / 2.;
                    double g2 = 0.;
                    for (int d = 0; d < 3; d++) g2 += G[d] * G[d];
                    const int rz = (iz - 1) / 2 < R ? (iz - 1) / 2 : R;
                    const int ry = (iy - 1) / 2 < R ? (iy - 1) / 2 : R;
                    const int rx = (ix - 1) / 2 < R ? (ix - 1) / 2 : R;
                    double sum[3] = {0., 0., 0.}, num = 0.;
                    for (int kk = -rz; kk <= rz; kk++) {
                        const int z = f90_ngb(k, iz, kk);
                        for (int jj = -ry; jj <= ry; jj++) {
                            const int y = f90_ngb(j, iy, jj);
                            for (int ii = -rx; ii <= rx; ii++) {
                                const int x = f90_ngb(i, ix, ii);
                                const double a = jj * G[2] - kk * G[1], b = kk * G[0] - ii * G[2],
                                             c = ii * G[1] - jj * G[0];
                                const double distance = a * a + b * b + c * c;
                                if (distance > g2 * 1.0) continue;
                                const long q = x + (long)ix * (y + (long)iy * z);
                                const double p1 = phase[3 * q], p2 = phase[3 * q + 1];
                                if (p1 > 1. - cutoff) has_ferrite = 1; /* sparse.f90:214-215 */
                                if (p1 < cutoff || p2 < cutoff) continue;
                                { /* sparse.f90:218-222: a deformed and a recrystallised ferrite grain */
                                    int lo = 0, hi = 0;
                                    for (int a = 0; a < PFO_NSLOT; a++) {
                                        const int g = ids1[6 * q + a];
                                        if (pfo_phase_of_grain(g) == 1 && g <= p->coh_npp0) lo = 1;
                                        if (pfo_phase_of_grain(g) == 1 && g > p->coh_npp0) hi = 1;
                                    }
                                    rex_intf = rex_intf || (lo && hi);
                                }
                                const double h[3] = {PH1(f90_ngb(x, ix, 1), y, z) - PH1(f90_ngb(x, ix, -1), y, z),
                                                     PH1(x, f90_ngb(y, iy, 1), z) - PH1(x, f90_ngb(y, iy, -1), z),
                                                     PH1(x, y, f90_ngb(z, iz, 1)) - PH1(x, y, f90_ngb(z, iz, -1))};
                                double dot = 0.;
                                for (int d = 0; d < 3; d++) dot += G[d] * h[d];
                                if (dot < 0.) continue;
                                if (p1 < 0.4 * p2 || p1 > 2.5 * p2) continue;
                                for (int d = 0; d < 3; d++) sum[d] += conc1[3 * q + d];
                                num += 1.;
                            }
                        }
                    }
                    if (num > 0.)
                        for (int d = 0; d < 3; d++) out[d] = sum[d] / num;
                }
                for (int d = 0; d < 3; d++) avg[3 * n + d] = out[d];
                if (flags) flags[n] = (unsigned char)(has_ferrite | (rex_intf << 1));
            }
#undef PH1
}

void pfo_set_coherent(const int32_t *partners, int n_austenite) {
    free(pfo_coh);
    pfo_coh = NULL;
    pfo_n_coh = 0;
    if (n_austenite > 0 && partners) {
        pfo_coh = (int32_t *)malloc(2 * (size_t)n_austenite * sizeof(int32_t));
        memcpy(pfo_coh, partners, 2 * (size_t)n_austenite * sizeof(int32_t));
        pfo_n_coh = n_austenite;
    }
}

void pfo_phase_sweep(const pfo_model *m, const pfo_params *p, const int32_t *ids1, const double *phi1,
                     int32_t *ids2, double *phi2, double *phase, double *conc1, const double *C) {
    double *avg = NULL;
    unsigned char *flags = NULL;
    if (p->avg_range > 0) {
        const long N = (long)m->ix * m->iy * m->iz;
        avg = (double *)malloc(3 * N * sizeof(double));
        if (p->coh_model) flags = (unsigned char *)malloc(N);
        pfo_avg_conc(m, p, ids1, phase, conc1, avg, flags);
    }
    /* phase_field.cpp:252-257 */
#pragma omp parallel for schedule(guided, 1) collapse(2)
    for (int k = 0; k < m->iz; k++)
        for (int j = 0; j < m->iy; j++)
            for (int i = 0; i < m->ix; i++)
                phase_cell(m, p, i, j, k, ids1, phi1, ids2, phi2, phase, conc1, C,
                           (avg && p->avg_conc) ? avg : conc1, flags);
    free(avg);
    free(flags);
}

/* solver.cpp:343-372 (Diffusion_solver) for every solute */
void pfo_diffusion_substep(const pfo_model *m, const pfo_params *p, double dt_sub, const double *phase,
                           const double *conc1, double *conc2, double *C) {
    const int ix = m->ix, iy = m->iy, iz = m->iz;
    const long N = (long)ix * iy * iz;
    const int nnb = (int)(2 * p->dims);
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < iz; k++)
        for (int j = 0; j < iy; j++)
            for (int i = 0; i < ix; i++) {
                const long n = i + (long)ix * (j + (long)iy * k);
                long nbr[6];
                nbr[0] = nb(i, ix, -1) + (long)ix * (j + (long)iy * k);
                nbr[1] = nb(i, ix, 1) + (long)ix * (j + (long)iy * k);
                nbr[2] = i + (long)ix * (nb(j, iy, -1) + (long)iy * k);
                nbr[3] = i + (long)ix * (nb(j, iy, 1) + (long)iy * k);
                nbr[4] = i + (long)ix * (j + (long)iy * nb(k, iz, -1));
                nbr[5] = i + (long)ix * (j + (long)iy * nb(k, iz, 1));
                for (int q = 0; q < m->nsol; q++) {
                    const double *c1 = conc1 + q * 3 * N;
                    double del = 0.;
                    for (int ii = 0; ii < nnb; ii++)
                        for (int jj = 0; jj < 3; jj++)
                            del += sqrt(phase[3 * nbr[ii] + jj] * phase[3 * n + jj]) *
                                   (c1[3 * nbr[ii] + jj] - c1[3 * n + jj]) * p->D[q][jj];
                    del *= (dt_sub / (m->dx * m->dx));
                    C[q * N + n] += del;
                    pfo_partition(C[q * N + n], phase + 3 * n, p->k[q], p->c[q],
                                  conc2 + q * 3 * N + 3 * n);
                }
            }
}

/* phase_field.cpp:243-305, Update(false) on the CPU branch (GPU_Flag == 0). */
void pfo_run(const pfo_model *m, pfo_state *s, double *time, int nsteps) {
    const long N = (long)m->ix * m->iy * m->iz;
    int32_t *ids_a = s->ids1, *ids_b = s->ids2;
    double *phi_a = s->phi1, *phi_b = s->phi2;
    double *conc_a = s->conc1, *conc_b = s->conc2;
    for (int st = 0; st < nsteps; st++) {
        pfo_params p;
        pfo_params_at(m, *time, &p);
        *time += p.pfm_dt; /* phase_field.cpp:314 */
        pfo_phase_sweep(m, &p, ids_a, phi_a, ids_b, phi_b, s->phase, conc_a, s->C);
        { int32_t *t = ids_a; ids_a = ids_b; ids_b = t; }
        { double *t = phi_a; phi_a = phi_b; phi_b = t; }
        for (int it = 1; it <= p.n_sub; it++) {
            pfo_diffusion_substep(m, &p, p.dt_sub, s->phase, conc_a, conc_b, s->C);
            double *t = conc_a; conc_a = conc_b; conc_b = t;
        }
    }
    if (ids_a != s->ids1) {
        memcpy(s->ids1, ids_a, sizeof(int32_t) * 6 * N);
        memcpy(s->phi1, phi_a, sizeof(double) * 6 * N);
        memcpy(s->ids2, ids_b, sizeof(int32_t) * 6 * N);
        memcpy(s->phi2, phi_b, sizeof(double) * 6 * N);
    }
    if (conc_a != s->conc1) {
        memcpy(s->conc1, conc_a, sizeof(double) * 3 * N * m->nsol);
        memcpy(s->conc2, conc_b, sizeof(double) * 3 * N * m->nsol);
    }
}

/* gpu_solver.cpp:204-218 with GPU_Partitioning (:131-154) and Diff3D (:160-188). */
int pfo_gpu_diffusion_solver(const double *D3, const double *k9, const double *c9,
                             const double *phase, double *C, int x, int y, int z,
                             double dt, double dx, double *conc_out) {
    const long N = (long)x * y * z;
    int dims = (z > 1) ? 3 : 2; /* gpu_solver.cpp:93-94 */
    double max_diff = D3[0];
    for (int p = 1; p < 3; p++)
        if (D3[p] > max_diff) max_diff = D3[p];
    double del_t = dx * dx / max_diff / dims * 0.2f; /* 0.2f as in gpu_solver.cpp:207 */
    int num_loop = (int)ceil(dt / del_t);
    double dt_dxdx = dt / num_loop / (dx * dx);
    double *conc = (double *)malloc(sizeof(double) * 3 * N);
    if (!conc) return -1;
    for (int it = 1; it <= num_loop; it++) {
#pragma omp parallel for schedule(static)
        for (long n = 0; n < N; n++) pfo_partition(C[n], phase + 3 * n, k9, c9, conc + 3 * n);
#pragma omp parallel for schedule(static) collapse(2)
        for (int sl = 0; sl < z; sl++)
            for (int row = 0; row < y; row++)
                for (int col = 0; col < x; col++) {
                    const long n = col + (long)x * (row + (long)y * sl);
                    long nbr[6] = {nb(col, x, -1) + (long)x * (row + (long)y * sl),
                                   nb(col, x, 1) + (long)x * (row + (long)y * sl),
                                   col + (long)x * (nb(row, y, -1) + (long)y * sl),
                                   col + (long)x * (nb(row, y, 1) + (long)y * sl),
                                   col + (long)x * (row + (long)y * nb(sl, z, -1)),
                                   col + (long)x * (row + (long)y * nb(sl, z, 1))};
                    double del = 0.;
                    for (int ii = 0; ii < 6; ii++)
                        for (int jj = 0; jj < 3; jj++)
                            del += sqrt(phase[3 * nbr[ii] + jj] * phase[3 * n + jj]) *
                                   (conc[3 * nbr[ii] + jj] - conc[3 * n + jj]) * D3[jj];
                    C[n] += (del * dt_dxdx);
                }
    }
    if (conc_out)
        for (long n = 0; n < N; n++) pfo_partition(C[n], phase + 3 * n, k9, c9, conc_out + 3 * n);
    free(conc);
    return num_loop;
}

/* write_data.cpp:14-18 */
void pfo_fractions(const pfo_model *m, const int32_t *ids, const double *phi, const double *phase,
                   double *out4) {
    const long N = (long)m->ix * m->iy * m->iz;
    const double vol = (double)m->ix * m->iy * m->iz;
    for (int p = 0; p < 3; p++) {
        double s = 0.;
        for (long n = 0; n < N; n++) s += phase[3 * n + p];
        out4[p] = s / vol;
    }
    double s = 0.;
    for (long e = 0; e < 6 * N; e++) s += (ids[e] < MAXGRAIN_PER_PHASE) ? phi[e] : 0.;
    out4[3] = s / vol;
}
