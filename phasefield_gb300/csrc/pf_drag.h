/* pf_drag.h -- the Fortran model's Purdy-Brechet solute drag
 * (Fortran_openmp_phase_field/PFM/src/sparse.f90:538-671 DISSIPATION_ITERATION
 * and _R, 958-1041 PARAMETER_DRAG_PB and SOLUTE_DRAG_PB), restated in double
 * with pf_exp / pf_log so the host parameters, the GPU kernel and the oracle
 * round identically.  C and C++ (host and device) alike; the parameter block
 * is passed as plain values. */
#ifndef PF_DRAG_H
#define PF_DRAG_H
#include "pf_math.h"

#if defined(__CUDACC__)
#define PF_DRAG_FN static __host__ __device__ __forceinline__
#else
#define PF_DRAG_FN static inline
#endif

/* SOLUTE_DRAG_PB (sparse.f90:1008-1037): drag pressure at velocity v0 for a
 * species of segregation energy e0 (/RT), parameter de (/RT) and bulk
 * fraction u0, at temperature T with the velocity scale vmax. */
PF_DRAG_FN double pf_solute_drag_pb(double v0, double e0, double de, double u0, double vmax, double T) {
    const double V = v0 / vmax;
    const double A = (de - e0) + V;
    const double B = (de + e0) + V;
    const double D0 = 1. - u0;
    const double Vu0 = V * u0;
    const double D1_d0 = (A - Vu0) / (A * D0 + (A - V) * u0 * pf_exp(-(A - Vu0)));
    const double D1 = D0 * D1_d0;
    const double U1 = 1. - D1;
    const double D2_d1 = (B - Vu0) / (B * D1 + (B * U1 - Vu0) * pf_exp(-(B - Vu0)));
    return (2. * de * u0 - ((A - V) / A * (Vu0 + pf_log(D1_d0)) + (B - V) / B * (Vu0 + pf_log(D2_d1)))) * 8.314 * T /
           7.2e12;
}

/* DISSIPATION_ITERATION (heating = 1) / DISSIPATION_ITERATION_R (heating = 0):
 * the interface rate where driv - v*norm = drag * (drag pressure at v), by
 * stepping v up from 0 in tenths of vmax (40 steps), then down from driv/norm
 * in fifths, and bisecting the first bracket to 1%.  'unchanged' is what the
 * Fortran leaves in place when no bracket is found (the caller's rate); the
 * cooling variant stops the Fortran program there -- here *fail is set.  The
 * Fortran bisection has no iteration limit; 200 halvings (reached only for a
 * root at exactly zero) end it here with *fail set. */
PF_DRAG_FN double pf_drag_solve(double driv, double drag, double norm, int heating, double unchanged, double vmax,
                                double ex0, double de, double u0, double corr, double drag0, double T, int *fail) {
    double err2 = driv - drag * drag0;
    if (err2 < 0.) return 0.;
    double dv = 0.1 * vmax, v = 0.;
    for (int J = 0; J < 2; J++) {
        for (int I = 0; I < 40; I++) {
            double err1 = err2;
            v = v + dv;
            err2 = driv - v * norm - drag * (pf_solute_drag_pb(v, ex0, de, u0, vmax, T) * corr);
            if (err1 * err2 <= 0.) {
                double x1 = v - dv, x2 = v;
                int it = 0;
                while ((x2 - x1) > 0.01 * x2) {
                    if (++it > 200) {
                        *fail = 1;
                        break;
                    }
                    const double tv = 0.5 * (x1 + x2);
                    const double te = driv - tv * norm - drag * (pf_solute_drag_pb(tv, ex0, de, u0, vmax, T) * corr);
                    if (err1 * te <= 0.) {
                        x2 = tv;
                        err2 = te;
                    } else {
                        x1 = tv;
                        err1 = te;
                    }
                }
                return 0.5 * (x1 + x2) * norm;
            }
        }
        v = driv / norm;
        dv = -0.2 * v;
        err2 = -1.;
    }
    if (!heating) *fail = 1;
    return unchanged;
}

#endif
