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

// The list storage of the phase sweep: one column per thread, PF_NSTENCIL
// entries (grain id, own phi, neighbour phi sum, updated value).
template <int NT>
struct pf_plist {
    int id[PF_NSTENCIL][NT];
    float v1[PF_NSTENCIL][NT];
    float v2[PF_NSTENCIL][NT];
    float del[PF_NSTENCIL][NT];
};

// Read-only loads: through the non-coherent path within one sweep, or through
// L2 (CG) where other blocks of the same launch rewrote the data earlier.
template <bool CG, typename T>
__device__ __forceinline__ T pf_ld(const T *p) {
    if (CG) return __ldcg(p);
    return __ldg(p);
}

// Phase_field_solver (solver.cpp:147-304) for cell (i,j,k) on the compact FP32
// layout; t is the thread's column in the shared list storage L.  Bulk cells
// (a single grain in the stencil) are copied and keep their phase planes.
template <int NSOL, int NT, bool CG = false>
__device__ __forceinline__ void pf_phase_cell(const pf_f32_params &P, int i, int j, int k, int t,
                                              const ushort4 *__restrict__ gid1, const float4 *__restrict__ phi1,
                                              ushort4 *__restrict__ gid2, float4 *__restrict__ phi2,
                                              float *__restrict__ sphase, const float2 *__restrict__ sol,
                                              pf_plist<NT> &L) {
    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const long long plane = (long long)ix * iy;
    const long long n = i + (long long)ix * j + plane * k;
    const float cutoff = P.cutoff;
    const int b1 = P.b1, b2 = P.b2;

    const ushort4 g = pf_ld<CG>(gid1 + n);
    const float4 v = pf_ld<CG>(phi1 + n);
    const int oid[4] = {g.x, g.y, g.z, g.w};
    const float ov[4] = {v.x, v.y, v.z, v.w};
    long long nb[6];
    nb[0] = n - i + pf_wrap(i, ix, -1);
    nb[1] = n - i + pf_wrap(i, ix, 1);
    nb[2] = n + (long long)ix * (pf_wrap(j, iy, -1) - j);
    nb[3] = n + (long long)ix * (pf_wrap(j, iy, 1) - j);
    nb[4] = n + plane * (pf_wrap(k, iz, -1) - k);
    nb[5] = n + plane * (pf_wrap(k, iz, 1) - k);
    // Fast path for the common bulk cell: one grain above the cutoff here and
    // the same single grain (and nothing else) in every neighbour -- the merged
    // stencil list would hold one entry (solver.cpp:207-216), so copy.
    ushort4 ngid[6];
#pragma unroll
    for (int b = 0; b < 6; b++)
        if (b < P.nnb) ngid[b] = pf_ld<CG>(gid1 + nb[b]);
    if (g.y == 0 && g.z == 0 && g.w == 0 && v.x > cutoff) {
        bool bulk = true;
#pragma unroll
        for (int b = 0; b < 6; b++)
            if (b < P.nnb) bulk = bulk && ngid[b].x == g.x && ngid[b].y == 0;
        if (bulk) {
            gid2[n] = g;
            phi2[n] = v;
            return;
        }
    }
    // solver.cpp:168-177: own slots above the cutoff (a sorted prefix).
    int num = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        if (ov[a] > cutoff) {
            L.id[num][t] = oid[a];
            L.v1[num][t] = ov[a];
            L.v2[num][t] = 0.f;
            num++;
        }
    }
    // solver.cpp:179-205: merge the neighbours' lists (x-, x+, y-, y+, z-, z+),
    // each scanned until its first empty slot.
#pragma unroll
    for (int b = 0; b < 6; b++) {
        if (b < P.nnb) {
            const ushort4 ng = ngid[b];
            const float4 nv4 = pf_ld<CG>(phi1 + nb[b]);
            const int nid[4] = {ng.x, ng.y, ng.z, ng.w};
            const float nv[4] = {nv4.x, nv4.y, nv4.z, nv4.w};
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int tid = nid[a];
                if (tid == 0) break;
                int kk = 0;
                while (kk < num && L.id[kk][t] != tid) kk++;
                if (kk < num) {
                    L.v2[kk][t] += nv[a];
                } else if (num < PF_NSTENCIL) {
                    L.id[num][t] = tid;
                    L.v1[num][t] = 0.f;
                    L.v2[num][t] = nv[a];
                    num++;
                }
            }
        }
    }
    if (num == 1) {  // solver.cpp:207-216: bulk, copy and leave the phase planes untouched
        gid2[n] = g;
        phi2[n] = v;
        return;
    }
    // Carbon concentration of each phase in this cell (for the driving force),
    // partitioned with the phase fractions of the current slots.
    float ph_old[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int p = pf_lphase(oid[a], b1, b2);
        if (p == 1) ph_old[0] += ov[a];
        else if (p == 2) ph_old[1] += ov[a];
        else if (p == 3) ph_old[2] += ov[a];
    }
    float lc[3];
    pf_partition_q(P, 0, pf_ld<CG>(sol + n * NSOL).x, ph_old, lc);

    // Pair terms (solver.cpp:235-258), each unordered pair once:
    //   X = S_i phi_j - S_j phi_i and Y = phi_i - phi_j flip sign between (i,j)
    //   and (j,i), Z = sqrt(phi_i phi_j) does not; A, B are symmetric in the
    //   phase pair, G and E are not.  A = B = G = 0 for pairs that do not interact.
    for (int a = 0; a < num; a++) L.del[a][t] = 0.f;
    for (int a = 0; a < num; a++) {
        const int ia = L.id[a][t];
        const int pa = pf_lphase(ia, b1, b2);
        const float va1 = L.v1[a][t], va2 = L.v2[a][t];
        const float ca = pa == 1 ? lc[0] : (pa == 2 ? lc[1] : lc[2]);
        float da = L.del[a][t];
        for (int b = a + 1; b < num; b++) {
            const int pb = pf_lphase(L.id[b][t], b1, b2);
            const float vb1 = L.v1[b][t], vb2 = L.v2[b][t];
            const int e = (pa - 1) + 3 * (pb - 1), ee = (pb - 1) + 3 * (pa - 1);
            const float X = va2 * vb1 - vb2 * va1;
            const float Y = va1 - vb1;
            const float Z = sqrtf(va1 * vb1);
            const float sym = P.A[e] * X + P.B[e] * Y;
            const float cb = pb == 1 ? lc[0] : (pb == 2 ? lc[1] : lc[2]);
            da += sym + P.G[e] * Z * (ca - P.E[e]);
            L.del[b][t] += -sym + P.G[ee] * Z * (cb - P.E[ee]);
        }
        float d = va1 + da;
        if (d > 1.0f) d = 1.0f;
        else if (d < cutoff) d = 0.f;
        L.del[a][t] = d;
    }
    // Top four, first maximum wins (solver.cpp:426-432), keep > cutoff,
    // normalise with x * (1/sum) (solver.cpp:276-296).
    float ph[3] = {0.f, 0.f, 0.f};
    float sum = 0.f;
    int kid[4];
    float kv[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        kid[a] = 0;
        kv[a] = 0.f;
        if (a < num) {
            int mx = a;
            float mv = L.del[a][t];
            for (int b = a + 1; b < num; b++) {
                const float x = L.del[b][t];
                if (x > mv) { mv = x; mx = b; }
            }
            const int mid = L.id[mx][t];
            if (mx != a) {
                L.del[mx][t] = L.del[a][t];
                L.id[mx][t] = L.id[a][t];
            }
            if (mv > cutoff) {
                kid[a] = mid;
                kv[a] = mv;
                const int p = pf_lphase(mid, b1, b2);
                if (p == 1) ph[0] += mv;
                else if (p == 2) ph[1] += mv;
                else ph[2] += mv;
                sum += mv;
            }
        }
    }
    const float inv = 1.f / sum;
    gid2[n] = make_ushort4((unsigned short)kid[0], (unsigned short)kid[1], (unsigned short)kid[2],
                           (unsigned short)kid[3]);
    phi2[n] = make_float4(kv[0] * inv, kv[1] * inv, kv[2] * inv, kv[3] * inv);
    const long long N = P.N;
    sphase[n] = sqrtf(ph[0] * inv);
    sphase[N + n] = sqrtf(ph[1] * inv);
    sphase[2 * N + n] = sqrtf(ph[2] * inv);
}
