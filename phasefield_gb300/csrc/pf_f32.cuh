// pf_f32.cuh -- device helpers shared by the compact FP32 kernels.
//
// Compact layout (see pf_f32.cu):
//   gid   ushort4 / cell   up to 4 local grain ids (0 = empty)
//   phi   float4  / cell   their phase-field values
//   phase float[3][N]      SQUARE ROOTS of the phase fractions, one plane per
//                          phase: the diffusion flux weight sqrt(phi_p^nb phi_p)
//                          is then a product, and phi_p = s_p^2 where needed
//   sol   float2[N][nsol]  solute total and its Kahan compensation (x - y)
#pragma once
#include "pf_dev.cuh"

__device__ __forceinline__ int pf_lphase(int l, int b1, int b2) {
    return l == 0 ? 0 : (l <= b1 ? 1 : (l <= b2 ? 2 : 3));
}

// Partitioning (solver.cpp:389-405) in FP32 for solute q, from the phase
// fractions ph.  A separable partition (c_ij = 0 and k_ij = a_j/a_i, the Mn
// case) collapses to c_i = a_i * C / sum_j phi_j a_j.
__device__ __forceinline__ void pf_partition_q(const pf_f32_params &P, int q, float C, const float ph[3],
                                               float out[3]) {
    if (P.sep[q]) {
        const float S = ph[0] * P.a[q][0] + ph[1] * P.a[q][1] + ph[2] * P.a[q][2];
        const float r = __fdividef(C, S);
#pragma unroll
        for (int i = 0; i < 3; i++) out[i] = P.a[q][i] * r;
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float t1 = ph[0] * P.k[q][i] + ph[1] * P.k[q][i + 3] + ph[2] * P.k[q][i + 6];
            const float t2 = ph[0] * P.c[q][i] + ph[1] * P.c[q][i + 3] + ph[2] * P.c[q][i + 6];
            out[i] = __fdividef(C - t2, t1);
        }
    }
}

__device__ __forceinline__ int pf_mod(int v, int L) {
    v %= L;
    return v < 0 ? v + L : v;
}
