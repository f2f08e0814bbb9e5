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
    //   The driving term is G (c_i - E), or G (max(c_i, c_j) - E) with the
    //   Fortran model's thermodynamics (P.dfmax).
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
            const float xa = P.dfmax ? fmaxf(ca, cb) : ca, xb = P.dfmax ? fmaxf(ca, cb) : cb;
            da += sym + P.G[e] * Z * (xa - P.E[e]);
            L.del[b][t] += -sym + P.G[ee] * Z * (xb - P.E[ee]);
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

// The same update for a cell whose merged stencil list has at most K grains
// (K = 4 covers about 98% of the cells of 3D Voronoi/nucleus
// microstructures) with the list held in registers: the merge compares each
// neighbour slot with the K entries at once, the pair loop, the clamps and
// the top-four selection are unrolled over the K entries with the list
// length as a predicate, so the lanes of a warp stay together.  The entry order, the
// summation order of every pair term and the selection rule are those of
// pf_phase_cell, so both routes give the same values for such a cell.
// Returns false, having written nothing, for a cell the register list cannot
// hold (a (K+1)-th grain in the stencil, or own slots above the cutoff that
// are not a prefix); the caller routes that cell to pf_phase_cell.  Cell indices
// are 32-bit (grids of fewer than 2^32 cells).
// The pair coefficients (A, B, G, E) of the nine phase pairs as one float4
// each, for a shared-memory copy: a warp whose lanes need different pairs
// reads them in one pass (indexed constant-bank loads serialise over the
// distinct addresses of a warp).
__device__ __forceinline__ void pf_coef_table(const pf_f32_params &P, float4 *tab) {
    if (threadIdx.x + blockDim.x * threadIdx.y < 9) {
        const int e = threadIdx.x + blockDim.x * threadIdx.y;
        tab[e] = make_float4(P.A[e], P.B[e], P.G[e], P.E[e]);
    }
}

template <int NSOL, bool CG = false, int K = 4>
__device__ __forceinline__ bool pf_phase_cell_reg(const pf_f32_params &P, const float4 *__restrict__ coef,
                                                  unsigned n, const unsigned nb[6],
                                                  const ushort4 *__restrict__ gid1,
                                                  const float4 *__restrict__ phi1, ushort4 *__restrict__ gid2,
                                                  float4 *__restrict__ phi2, float *__restrict__ sphase,
                                                  const float2 *__restrict__ sol) {
    const float cutoff = P.cutoff;
    const int b1 = P.b1, b2 = P.b2, nnb = P.nnb;
    const ushort4 g = pf_ld<CG>(gid1 + n);
    const float4 v = pf_ld<CG>(phi1 + n);
    ushort4 ng[6];
    float4 nv[6];
#pragma unroll
    for (int b = 0; b < 6; b++) {
        if (b < nnb) {
            ng[b] = pf_ld<CG>(gid1 + nb[b]);
            nv[b] = pf_ld<CG>(phi1 + nb[b]);
        } else {
            ng[b] = make_ushort4(0, 0, 0, 0);
            nv[b] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    // Bulk cell: one grain here and the same single grain in every neighbour.
    if (g.y == 0 && g.z == 0 && g.w == 0 && v.x > cutoff) {
        bool bulk = true;
#pragma unroll
        for (int b = 0; b < 6; b++)
            if (b < nnb) bulk = bulk && ng[b].x == g.x && ng[b].y == 0;
        if (bulk) {
            gid2[n] = g;
            phi2[n] = v;
            return true;
        }
    }
    // solver.cpp:168-177: own slots above the cutoff, in slot order.
    const bool ok0 = v.x > cutoff, ok1 = v.y > cutoff, ok2 = v.z > cutoff, ok3 = v.w > cutoff;
    if ((ok1 && !ok0) || (ok2 && !ok1) || (ok3 && !ok2)) return false;
    static_assert(K >= 4 && K <= PF_NSTENCIL, "the register list holds the own slots");
    int lid[K];
    float v1[K], v2[K];
#pragma unroll
    for (int e = 0; e < K; e++) {
        lid[e] = 0;
        v1[e] = 0.f;
        v2[e] = 0.f;
    }
    lid[0] = ok0 ? (int)g.x : 0; lid[1] = ok1 ? (int)g.y : 0; lid[2] = ok2 ? (int)g.z : 0; lid[3] = ok3 ? (int)g.w : 0;
    v1[0] = ok0 ? v.x : 0.f; v1[1] = ok1 ? v.y : 0.f; v1[2] = ok2 ? v.z : 0.f; v1[3] = ok3 ? v.w : 0.f;
    int num = (int)ok0 + (int)ok1 + (int)ok2 + (int)ok3;
    // solver.cpp:179-205: neighbours x-, x+, y-, y+, z-, z+, each scanned to
    // its first empty slot; an id already listed adds its value, a new id is
    // appended.  Entries past num hold id 0, which no live slot carries.
    bool full = false;
#pragma unroll
    for (int b = 0; b < 6; b++) {
        if (b < nnb) {
            const int nid[4] = {ng[b].x, ng[b].y, ng[b].z, ng[b].w};
            const float nvv[4] = {nv[b].x, nv[b].y, nv[b].z, nv[b].w};
            bool live = true;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int tid = nid[a];
                live = live && tid != 0;
                if (live) {
                    const float tv = nvv[a];
                    bool hit = false;
#pragma unroll
                    for (int e = 0; e < K; e++) {
                        const bool m = lid[e] == tid;
                        if (m) v2[e] += tv;
                        hit = hit || m;
                    }
                    if (!hit) {
                        if (num < K) {
#pragma unroll
                            for (int e = 0; e < K; e++)
                                if (e == num) {
                                    lid[e] = tid;
                                    v2[e] = tv;
                                }
                            num++;
                        } else {
                            full = true;
                        }
                    }
                }
            }
        }
    }
    if (full) return false;
    if (num == 1) {  // solver.cpp:207-216
        gid2[n] = g;
        phi2[n] = v;
        return true;
    }
    float ph_old[3] = {0.f, 0.f, 0.f};
    {
        const int oid[4] = {g.x, g.y, g.z, g.w};
        const float ov[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int p = pf_lphase(oid[a], b1, b2);
            if (p == 1) ph_old[0] += ov[a];
            else if (p == 2) ph_old[1] += ov[a];
            else if (p == 3) ph_old[2] += ov[a];
        }
    }
    float lc[3];
    pf_partition_q(P, 0, pf_ld<CG>(sol + n * NSOL).x, ph_old, lc);
    int pe[K];
    float ce[K];
#pragma unroll
    for (int e = 0; e < K; e++) {
        pe[e] = pf_lphase(lid[e], b1, b2);
        ce[e] = pe[e] == 1 ? lc[0] : (pe[e] == 2 ? lc[1] : lc[2]);
    }
    // Pair terms, each unordered pair once, in the order of pf_phase_cell.
    float del[K];
#pragma unroll
    for (int e = 0; e < K; e++) del[e] = 0.f;
#pragma unroll
    for (int a = 0; a < K; a++) {
        if (a < num) {
            float da = del[a];
#pragma unroll
            for (int b = a + 1; b < K; b++) {
                if (b < num) {
                    const int e = (pe[a] - 1) + 3 * (pe[b] - 1), ee = (pe[b] - 1) + 3 * (pe[a] - 1);
                    const float X = v2[a] * v1[b] - v2[b] * v1[a];
                    const float Y = v1[a] - v1[b];
                    const float Z = sqrtf(v1[a] * v1[b]);
                    const float4 ce_ = coef[e], cee = coef[ee];
                    const float sym = ce_.x * X + ce_.y * Y;
                    const float xa = P.dfmax ? fmaxf(ce[a], ce[b]) : ce[a], xb = P.dfmax ? fmaxf(ce[a], ce[b]) : ce[b];
                    da += sym + ce_.z * Z * (xa - ce_.w);
                    del[b] += -sym + cee.z * Z * (xb - cee.w);
                }
            }
            float d = v1[a] + da;
            if (d > 1.0f) d = 1.0f;
            else if (d < cutoff) d = 0.f;
            del[a] = d;
        }
    }
    // Top four, first maximum wins, the maximum swapped into place.
    float ph[3] = {0.f, 0.f, 0.f};
    float sum = 0.f;
    int kid[4];
    float kv[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        kid[a] = 0;
        kv[a] = 0.f;
        if (a < num) {
            int mx = a, mid = lid[a];
            float mv = del[a];
#pragma unroll
            for (int b = a + 1; b < K; b++)
                if (b < num && del[b] > mv) {
                    mv = del[b];
                    mx = b;
                    mid = lid[b];
                }
#pragma unroll
            for (int b = a + 1; b < K; b++)
                if (b == mx) {
                    del[b] = del[a];
                    lid[b] = lid[a];
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
    return true;
}
