// pf_types.h -- parameter blocks shared by the host code and the sm_103a kernels.
//
// One time step of the Steinbach multi-phase-field model (zhubq/PhaseField,
// C++-openmp-cuda/src/phase_field.cpp:243-315) needs a handful of
// temperature-dependent scalars and 3x3 phase-pair tables.  The host evaluates
// them once per step (exp, thermo polynomials) and hands them to the kernels by
// value as a __grid_constant__ block, so no device exp/pow is ever evaluated and
// a captured CUDA graph carries its parameters with it.
#pragma once
#include <stdint.h>
#include "pfstep.h"

#define PF_NSLOT64 6      // slots per cell, FP64 reference layout (constant.h:5)
#define PF_NSLOT32 4      // slots per cell, compact FP32 layout
#define PF_NPHASE 3       // constant.h:6
#define PF_NSTENCIL 10    // merged stencil list length (solver.cpp:148)
#define PF_MAXSOL 2       // carbon + Mn
#define PF_MAXGRAIN_PER_PHASE 100000  // phase_field.h:19

// pf_step_params (the per-step parameters in the reference's FP64 form) is
// part of the public ABI, declared in pfstep.h.

// The same step folded for the compact FP32 kernels.  The pair term of
// solver.cpp:249-256 is regrouped as
//   dphi_ij = dt*m_ij*[ sigma_ij*(f1*(S_i phi_j - S_j phi_i) + f2*(phi_i - phi_j))
//                       + f3*sqrt(phi_i phi_j)*entropy_ij*(c_i - eq_ij)/dcdT_ij ]
// with every phase-pair product precomputed in FP64 and rounded once.
typedef struct {
    int ix, iy, iz, nnb, nsol, n_sub;
    long long N;
    int b1, b2;                 // local grain id -> phase: id<=b1 ->1, <=b2 ->2, else 3
    float cutoff;
    int dfmax;                  // 1: pair driving term G*(max(c_i, c_j) - E) (Fortran thermodynamics)
    float A[9];                 // dt*m*sigma*f1
    float B[9];                 // dt*m*sigma*f2
    float G[9];                 // dt*m*f3*entropy/dcdT
    float E[9];                 // eq_ij
    // A, B and G are zero for pairs that do not interact (|p_i-p_j| == 2,
    // solver.cpp:246) and G is zero on the diagonal (solver.cpp:381).
    float D[PF_MAXSOL][3];      // D * dt_sub/dx^2
    float k[PF_MAXSOL][9], c[PF_MAXSOL][9];
    // Separable partition of solute q (c_ij = 0, k_ij = a_j/a_i): c_i = a_i C / sum_j phi_j a_j.
    int sep[PF_MAXSOL];
    float a[PF_MAXSOL][3];
} pf_f32_params;
