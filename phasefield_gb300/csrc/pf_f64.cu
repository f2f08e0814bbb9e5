// pf_f64.cu -- plain FP64 step kernels in the reference layout (sm_103a).
//
// These kernels are the parity path: they evaluate every floating-point
// operation of the reference's CPU solver (zhubq/PhaseField,
// C++-openmp-cuda/src/solver.cpp) in the same order, and this file is compiled
// with -fmad=false so that no multiply-add is contracted.  IEEE sqrt and
// division are correctly rounded on the device, so the results are
// bit-identical to a -ffp-contract=off host build of the same arithmetic.
//
// Layout (phase_field.h:81-89): slot/phase fastest, then x, y, z.
//   ids[6n+s] int32, phi[6n+s] f64, phase[3n+p] f64,
//   conc[q*3N + 3n+p] f64, C[q*N + n] f64.
#include "pf_dev.cuh"
#include "pf_drag.h"
#include "pf_kernels.h"

__device__ int g_drag_fail;  // a solute-drag iteration found no root (the Fortran stops there)

namespace {

// Driving_force (solver.cpp:374-387) for a phase pair, given the cell's carbon
// concentrations of phases pi and pj.  df = 0.; df += ... is kept literally.
// With the Fortran model's thermodynamics (df_model 1) it is
// -Ratio_k_para(pi,pj) * (max(c_pi, c_pj) - Ref_c_para(2,1)) (sparse.f90:512-515).
__device__ __forceinline__ double pf_df(const pf_step_params &P, int pi, int pj, double conc_pi, double conc_pj) {
    double df = 0.;
    if (pi != pj) {
        const int e = (pi - 1) + 3 * (pj - 1);
        if (P.df_model == 1) df -= P.df_ratio[e] * (fmax(conc_pi, conc_pj) - P.df_ref);
        else df += P.entropy[e] * (conc_pi - P.eq[e]) / P.dcdT[e];
    }
    return df;
}

// solver.cpp:389-405
__device__ __forceinline__ void pf_partition(double C, const double ph[3], const double *k9,
                                             const double *c9, double out[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double t1 = 0., t2 = 0.;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            t1 += ph[j] * k9[i + 3 * j];
            t2 += ph[j] * c9[i + 3 * j];
        }
        out[i] = (C - t2) / t1;
    }
}

// The Fortran model's interface-averaged phase concentrations
// (sparse.f90:184-255), one thread per cell, from the phase fractions and
// phase concentrations before the sweep.  In a cell holding ferrite and
// austenite above the cutoff (Flag_coexist(2), sparse.f90:141-146) the
// average runs over the cells of the (2R+1)^dims neighbourhood (R = i_intf+1,
// clipped to half the grid) that lie within one cell of the line through
// the cell along G = grad(phi_ferrite)/2 (|r x G|^2 <= |G|^2), hold both
// phases above the cutoff, whose own ferrite gradient does not point against
// G, and whose ferrite/austenite ratio lies in [0.4, 2.5]; with no such cell,
// and elsewhere, the cell's own concentrations.  The Fortran loop updates the
// phase fractions in place as it goes (an order the OpenMP schedule decides);
// here every cell reads the values of the start of the sweep.
// flags (may be null): the same scan's Has_ferrite (bit 0: a cell of the line
// holds ferrite above 1 - cutoff) and Rex_intf (bit 1: a cell of the line with
// both phases above the cutoff holds a ferrite grain of the initial class,
// id <= coh_npp0, and a recrystallised one), sparse.f90:214-222; 0 outside
// Flag_coexist(2).
__global__ void __launch_bounds__(256) k_avg_conc_f64(const __grid_constant__ pf_step_params P,
                                                      const int *__restrict__ ids1,
                                                      const double *__restrict__ phase,
                                                      const double *__restrict__ conc1,
                                                      double *__restrict__ avg,
                                                      unsigned char *__restrict__ flags) {
    int ci, cj, ck;
    long long n;
    if (!pf_cell(P.ix, P.iy, ci, cj, ck, n)) return;
    const int ix = P.ix, iy = P.iy, iz = P.iz;
    const double cutoff = P.cutoff;
    double out[3] = {conc1[3 * n], conc1[3 * n + 1], conc1[3 * n + 2]};
    int fl = 0;
    auto at = [&](int i, int j, int k) { return (long long)i + (long long)ix * (j + (long long)iy * k); };
    auto ph1 = [&](int i, int j, int k) { return phase[3 * at(i, j, k)]; };
    if (phase[3 * n] > cutoff && phase[3 * n + 1] > cutoff) {
        double G[3];
        G[0] = ph1(pf_wrap(ci, ix, 1), cj, ck) - ph1(pf_wrap(ci, ix, -1), cj, ck);
        G[1] = ph1(ci, pf_wrap(cj, iy, 1), ck) - ph1(ci, pf_wrap(cj, iy, -1), ck);
        G[2] = ph1(ci, cj, pf_wrap(ck, iz, 1)) - ph1(ci, cj, pf_wrap(ck, iz, -1));
        G[0] = G[0] / 2.; G[1] = G[1] / 2.; G[2] = G[2] / 2.;
        double g2 = 0.;
        g2 += G[0] * G[0];
        g2 += G[1] * G[1];
        g2 += G[2] * G[2];
        const int R = P.avg_range;
        const int rz = min((iz - 1) / 2, R), ry = min((iy - 1) / 2, R), rx = min((ix - 1) / 2, R);
        double sum[3] = {0., 0., 0.}, num = 0.;
        bool has_ferrite = false, rex = false;
        const double bulk = 1. - cutoff;
        const int npp0 = P.coh_npp0;
        for (int kk = -rz; kk <= rz; kk++) {
            const int z = pf_mod(ck + kk, iz);
            for (int jj = -ry; jj <= ry; jj++) {
                const int y = pf_mod(cj + jj, iy);
                for (int ii = -rx; ii <= rx; ii++) {
                    const int x = pf_mod(ci + ii, ix);
                    const double a = jj * G[2] - kk * G[1], b = kk * G[0] - ii * G[2], c = ii * G[1] - jj * G[0];
                    const double dist = a * a + b * b + c * c;
                    if (dist > g2 * 1.0) continue;
                    const long long m = at(x, y, z);
                    const double p1 = phase[3 * m], p2 = phase[3 * m + 1];
                    if (p1 > bulk) has_ferrite = true;
                    if (p1 < cutoff || p2 < cutoff) continue;
                    if (flags) {
                        bool lo = false, hi = false;
#pragma unroll
                        for (int a = 0; a < 6; a++) {
                            const int g = ids1[6 * m + a];
                            if (pf_phase_of_grain(g) == 1) {
                                if (g <= npp0) lo = true;
                                else hi = true;
                            }
                        }
                        rex = rex || (lo && hi);
                    }
                    const double h0 = ph1(pf_wrap(x, ix, 1), y, z) - ph1(pf_wrap(x, ix, -1), y, z);
                    const double h1 = ph1(x, pf_wrap(y, iy, 1), z) - ph1(x, pf_wrap(y, iy, -1), z);
                    const double h2 = ph1(x, y, pf_wrap(z, iz, 1)) - ph1(x, y, pf_wrap(z, iz, -1));
                    double dot = 0.;
                    dot += G[0] * h0;
                    dot += G[1] * h1;
                    dot += G[2] * h2;
                    if (dot < 0.) continue;
                    if (p1 < 0.4 * p2 || p1 > 2.5 * p2) continue;
                    sum[0] += conc1[3 * m];
                    sum[1] += conc1[3 * m + 1];
                    sum[2] += conc1[3 * m + 2];
                    num += 1.;
                }
            }
        }
        if (num > 0.) {
            out[0] = sum[0] / num;
            out[1] = sum[1] / num;
            out[2] = sum[2] / num;
        }
        fl = (has_ferrite ? 1 : 0) | (rex ? 2 : 0);
    }
    if (flags) flags[n] = (unsigned char)fl;
    avg[3 * n] = out[0];
    avg[3 * n + 1] = out[1];
    avg[3 * n + 2] = out[2];
}

// Whether austenite grain 'aus' nucleated coherent with ferrite grain 'fer'
// (Coherent_grain(aus, :) holds fer): coh[2k], coh[2k+1] for aus = 200001 + k.
__device__ __forceinline__ bool pf_coh_has(const int *coh, int n_coh, int aus, int fer) {
    const int k = aus - (2 * PF_MAXGRAIN_PER_PHASE + 1);
    if (k < 0 || k >= n_coh || fer == 0) return false;
    return coh[2 * k] == fer || coh[2 * k + 1] == fer;
}

// Phase_field_solver (solver.cpp:147-304), one thread per cell.  avg (may be
// null): the phase concentrations the driving force reads instead of the
// cell's own (k_avg_conc_f64), when P.avg_conc is set.  flags, coh (null
// unless P.coh_model): the scan's Has_ferrite / Rex_intf bits and the
// coherent-partner table of the Fortran model's coherent-grain mobility.
// EXT: compiled with the solute drag and the coherent mobility (the plain
// model's instance carries neither, and keeps its register budget).
template <bool EXT>
__global__ void __launch_bounds__(256) k_phase_f64(const __grid_constant__ pf_step_params P, int patch,
                                                   const int *__restrict__ ids1,
                                                   const double *__restrict__ phi1,
                                                   int *__restrict__ ids2, double *__restrict__ phi2,
                                                   double *__restrict__ phase,
                                                   double *__restrict__ conc1,
                                                   const double *__restrict__ C,
                                                   const double *__restrict__ avg,
                                                   const unsigned char *__restrict__ flags,
                                                   const int *__restrict__ coh, int n_coh) {
    int ci, cj, ck;
    long long n;
    if (!pf_cell_map(patch, P.ix, P.iy, P.iz, ci, cj, ck, n)) return;
    long long nbr[6];
    pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nbr);
    const double cutoff = P.cutoff;

    // 1-based stencil arrays of the reference become 0-based position arrays.
    int sid[PF_NSTENCIL], sph[PF_NSTENCIL];
    double s1[PF_NSTENCIL], s2[PF_NSTENCIL];
#pragma unroll
    for (int a = 0; a < PF_NSTENCIL; a++) {
        sid[a] = 0; sph[a] = 0; s1[a] = 0.; s2[a] = 0.;
    }
    int own_id[6];
    double own_v[6];
    {
        const int2 *ip = reinterpret_cast<const int2 *>(ids1 + 6 * n);
        const double2 *vp = reinterpret_cast<const double2 *>(phi1 + 6 * n);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            int2 t = __ldg(ip + a);
            double2 v = __ldg(vp + a);
            own_id[2 * a] = t.x; own_id[2 * a + 1] = t.y;
            own_v[2 * a] = v.x; own_v[2 * a + 1] = v.y;
        }
    }
    // solver.cpp:168-175: own slots above the cutoff keep their slot position.
    int num = 0;
#pragma unroll
    for (int a = 0; a < 6; a++) {
        if (own_v[a] > cutoff) {
            num += 1;
            sid[a] = own_id[a];
            sph[a] = pf_phase_of_grain(own_id[a]);
            s1[a] = own_v[a];
        }
    }
    // solver.cpp:179-205: merge the neighbours' lists, stopping at id 0.
#pragma unroll
    for (int b = 0; b < 6; b++) {
        if (b < P.nnb) {
            const long long q = nbr[b];
            int nid[6];
            double nv[6];
            const int2 *ip = reinterpret_cast<const int2 *>(ids1 + 6 * q);
            const double2 *vp = reinterpret_cast<const double2 *>(phi1 + 6 * q);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                int2 t = __ldg(ip + a);
                double2 v = __ldg(vp + a);
                nid[2 * a] = t.x; nid[2 * a + 1] = t.y;
                nv[2 * a] = v.x; nv[2 * a + 1] = v.y;
            }
            bool live = true;
#pragma unroll
            for (int a = 0; a < 6; a++) {
                const int tid = nid[a];
                live = live && (tid != 0);
                if (live) {
                    bool found = false;
#pragma unroll
                    for (int kk = 0; kk < PF_NSTENCIL; kk++) {
                        if (!found && tid == sid[kk]) {
                            s2[kk] += nv[a];
                            found = true;
                        }
                    }
                    if (!found && num < PF_NSTENCIL) {
#pragma unroll
                        for (int kk = 0; kk < PF_NSTENCIL; kk++) {
                            if (kk == num) {
                                sid[kk] = tid;
                                sph[kk] = pf_phase_of_grain(tid);
                                s2[kk] += nv[a];
                            }
                        }
                        num += 1;
                    }
                }
            }
        }
    }
    // solver.cpp:207-216: a single field in the stencil -> copy and return.
    if (num == 1) {
        int2 *op = reinterpret_cast<int2 *>(ids2 + 6 * n);
        double2 *ov = reinterpret_cast<double2 *>(phi2 + 6 * n);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            op[a] = make_int2(own_id[2 * a], own_id[2 * a + 1]);
            ov[a] = make_double2(own_v[2 * a], own_v[2 * a + 1]);
        }
        return;
    }
    // Driving forces depend only on the phase pair and the cell's carbon
    // concentration (solver.cpp:231-232, 374-387): evaluate the six ordered
    // off-diagonal pairs once.
    const double *lcp = (avg && P.avg_conc) ? avg : conc1;
    double lc[3];
    lc[0] = lcp[3 * n + 0]; lc[1] = lcp[3 * n + 1]; lc[2] = lcp[3 * n + 2];
    double df[9];
#pragma unroll
    for (int a = 1; a <= 3; a++)
#pragma unroll
        for (int b = 1; b <= 3; b++) df[(a - 1) + 3 * (b - 1)] = pf_df(P, a, b, lc[a - 1], lc[b - 1]);

    const double factor1 = P.factor1, factor2 = P.factor2, factor3 = P.factor3;
    // sparse.f90:300-306: the coherent-mobility gate of the cell -- the scan
    // saw bulk ferrite and no recrystallisation front, and exactly one of the
    // cell's own grains above the cutoff (Ind_ph1(1:N_nonzero)) is ferrite.
    bool coh_cell = false;
    if (EXT && P.coh_model && flags && coh) {
        const int fl = flags[n];
        int nown = 0, nfer = 0;
#pragma unroll
        for (int a = 0; a < 6; a++) nown += own_v[a] > cutoff ? 1 : 0;
#pragma unroll
        for (int a = 0; a < 6; a++) nfer += (a < nown && pf_phase_of_grain(own_id[a]) == 1) ? 1 : 0;
        coh_cell = (fl & 1) && !(fl & 2) && nfer == 1;
    }
    double del[PF_NSTENCIL];
    double drag[PF_NSTENCIL];  // sum over ferrite/austenite partners of m_ij f3 sqrt(phi_i phi_j) (solute drag)
#pragma unroll
    for (int ii = 0; ii < PF_NSTENCIL; ii++) {
        del[ii] = 0.;
        drag[ii] = 0.;
        if (ii < num) {
            const int pi = sph[ii];
#pragma unroll
            for (int jj = 0; jj < PF_NSTENCIL; jj++) {
                if (jj < num && jj != ii) {
                    const int pj = sph[jj];
                    if (abs(pi - pj) != 2) {
                        const int e = (pi - 1) + 3 * (pj - 1);
                        double d = 0.;
                        d = (s2[ii] * s1[jj] - s2[jj] * s1[ii]) * factor1;
                        d += (s1[ii] - s1[jj]) * factor2;
                        d *= P.sigma[e];
                        double dfe = 0.;
#pragma unroll
                        for (int t = 0; t < 9; t++)
                            if (t == e) dfe = df[t];
                        d += factor3 * sqrt(s1[ii] * s1[jj]) * dfe;
                        // sparse.f90:298-315: 0.02 of the mobility for a coherent pair
                        const bool cp = coh_cell && ((pi == 2 && pf_coh_has(coh, n_coh, sid[ii], sid[jj])) ||
                                                     (pj == 2 && pf_coh_has(coh, n_coh, sid[jj], sid[ii])));
                        const double mob = cp ? 0.02 * P.m[e] : P.m[e];
                        d = cp ? mob * d : d * mob;
                        del[ii] += d;
                        if (EXT && P.drag_model && pi + pj == 3) drag[ii] += mob * (factor3 * sqrt(s1[ii] * s1[jj]));
                    }
                }
            }
        }
    }
    // The Fortran model's solute drag (sparse.f90:326-360): in a cell holding
    // ferrite and austenite but not ferrite and cementite above the cutoff,
    // each of the cell's own grains moves at the rate that balances its
    // driving rate against the drag; a two-entry stencil keeps the second
    // rate the negative of the first.
    if (EXT && P.drag_model) {
        const double f = phase[3 * n], a = phase[3 * n + 1], c = phase[3 * n + 2];
        const bool co1 = f > cutoff && c > cutoff, co2 = f > cutoff && a > cutoff;
        int nown = 0;
#pragma unroll
        for (int a6 = 0; a6 < 6; a6++) nown += own_v[a6] > cutoff ? 1 : 0;
        int fail = 0;
        // With two entries only the first is solved; the second takes its
        // negative.  Entries are picked by static index so the stencil arrays
        // stay in registers.
        const int nsolve = num == 2 ? 1 : num;
        for (int ii = 0; ii < nsolve; ii++) {
            if (!co1 && co2 && ii < nown) {
                double drv = 0., dg = 0., v1 = 0.;
                int ph_ii = 0;
#pragma unroll
                for (int t = 0; t < PF_NSTENCIL; t++)
                    if (t == ii) {
                        drv = del[t]; dg = drag[t]; v1 = s1[t]; ph_ii = sph[t];
                    }
                const double norm = factor3 * sqrt(v1 * (1. - v1));
                // growth (austenite up, ferrite down) uses the heating branch
                const bool active = (drv > 0. && (ph_ii == 1 || ph_ii == 2)) || (drv < 0. && (ph_ii == 1 || ph_ii == 2));
                const bool heat = (drv > 0.) ? (ph_ii == 2) : (ph_ii == 1);
                double r = drv;
                if (active)
                    r = pf_drag_solve(drv > 0. ? drv : -drv, dg, norm, heat ? 1 : 0, drv, P.drag_vmax, P.drag_ex0,
                                      heat ? P.drag_de_heat : P.drag_de_cool, P.drag_u0,
                                      P.drag_corr[heat ? 0 : 1], P.drag_drag0[heat ? 0 : 1], P.T, &fail);
                if (drv < 0.) r = -r;
                else if (!(drv > 0.)) r = 0.;
#pragma unroll
                for (int t = 0; t < PF_NSTENCIL; t++)
                    if (t == ii) del[t] = r;
            }
        }
        if (num == 2) del[1] = -del[0];
        if (fail) atomicExch(&g_drag_fail, 1);
    }
#pragma unroll
    for (int ii = 0; ii < PF_NSTENCIL; ii++) {
        if (ii < num) {
            del[ii] *= P.pfm_dt;
            del[ii] += s1[ii];
            if (del[ii] > 1.0) del[ii] = 1.0;
            else if (del[ii] < cutoff) del[ii] = 0.;
        }
    }
    // Sort_xyz (solver.cpp:426-432): selection sort, first maximum wins.  Only
    // the first six positions are read afterwards.
#pragma unroll
    for (int a = 0; a < PF_NSLOT64; a++) {
        int mx = a;
        double mv = del[a];
#pragma unroll
        for (int b = a + 1; b < PF_NSTENCIL; b++) {
            if (del[b] > mv) { mv = del[b]; mx = b; }
        }
#pragma unroll
        for (int b = a + 1; b < PF_NSTENCIL; b++) {
            if (b == mx) {
                double tv = del[a]; del[a] = del[b]; del[b] = tv;
                int ti = sid[a]; sid[a] = sid[b]; sid[b] = ti;
            }
        }
    }
    // solver.cpp:270-296
    double ph[3] = {0., 0., 0.};
    double sum = 0.;
    int oid[6];
    double ov[6];
#pragma unroll
    for (int a = 0; a < PF_NSLOT64; a++) {
        if (del[a] > cutoff) {
            oid[a] = sid[a];
            ov[a] = del[a];
            const int p = pf_phase_of_grain(sid[a]);
            if (p == 1) ph[0] += del[a];
            else if (p == 2) ph[1] += del[a];
            else if (p == 3) ph[2] += del[a];
            sum += del[a];
        } else {
            oid[a] = 0;
            ov[a] = 0.;
        }
    }
#pragma unroll
    for (int a = 0; a < PF_NSLOT64; a++) ov[a] *= 1. / sum;
#pragma unroll
    for (int p = 0; p < 3; p++) ph[p] *= 1. / sum;
    {
        int2 *op = reinterpret_cast<int2 *>(ids2 + 6 * n);
        double2 *vp = reinterpret_cast<double2 *>(phi2 + 6 * n);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            op[a] = make_int2(oid[2 * a], oid[2 * a + 1]);
            vp[a] = make_double2(ov[2 * a], ov[2 * a + 1]);
        }
    }
    phase[3 * n + 0] = ph[0];
    phase[3 * n + 1] = ph[1];
    phase[3 * n + 2] = ph[2];
    // solver.cpp:299: partition in place, every solute.
    for (int q = 0; q < P.nsol; q++) {
        double out[3];
        pf_partition(C[q * P.N + n], ph, P.k[q], P.c[q], out);
        double *cp = conc1 + (long long)q * 3 * P.N + 3 * n;
        cp[0] = out[0]; cp[1] = out[1]; cp[2] = out[2];
    }
}

// Flux weights of the forward links of every cell (solver.cpp:363):
// links[9n + 3d + p] = sqrt(phase_p(n + e_d) * phase_p(n)) for d = x+, y+, z+
// (the directions the stencil uses).  The phase fractions stay fixed through
// a step's diffusion sub-steps, so the sub-steps read these instead of taking
// 18 FP64 square roots per cell each (FP64 arithmetic is scarce on GB300).  A
// link is shared by its two cells and a*b == b*a exactly, so both read the
// weight the reference computes for them.
// tpart[6(qN + n) + i], tpart[6(qN + n) + 3 + i]: the sums t1_i, t2_i of the
// partition (solver.cpp:389-405) of solute q, also fixed through the
// sub-steps; a sub-step then only divides, (C - t2_i) / t1_i.
__global__ void __launch_bounds__(256) k_links_f64(const __grid_constant__ pf_step_params P, int nnb,
                                                   const double *__restrict__ phase,
                                                   double *__restrict__ links, double *__restrict__ tpart) {
    int ci, cj, ck;
    long long n;
    if (!pf_cell(P.ix, P.iy, ci, cj, ck, n)) return;
    long long nbr[6];
    pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nbr);
    double ph[3];
    ph[0] = __ldg(phase + 3 * n + 0);
    ph[1] = __ldg(phase + 3 * n + 1);
    ph[2] = __ldg(phase + 3 * n + 2);
#pragma unroll
    for (int d = 0; d < 3; d++)
        if (2 * d + 1 < nnb) {
#pragma unroll
            for (int p = 0; p < 3; p++)
                links[9 * n + 3 * d + p] = sqrt(__ldg(phase + 3 * nbr[2 * d + 1] + p) * ph[p]);
        }
    for (int q = 0; q < P.nsol; q++) {
        double *tp = tpart + 6 * ((long long)q * P.N + n);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            double t1 = 0., t2 = 0.;
#pragma unroll
            for (int j = 0; j < 3; j++) {
                t1 += ph[j] * P.k[q][i + 3 * j];
                t2 += ph[j] * P.c[q][i + 3 * j];
            }
            tp[i] = t1;
            tp[3 + i] = t2;
        }
    }
}

// Diffusion_solver (solver.cpp:343-372) for every solute, one thread per cell:
// reads phase/conc1 of the cell and its nnb neighbours, updates C in place and
// writes the re-partitioned concentrations to conc2.  The flux weight of
// neighbour b, sqrt(phase_p^nb * phase_p), comes from links (k_links_f64): the
// cell's own forward link for x+, y+, z+, the neighbour's for x-, y-, z-;
// the partition's sums come from tpart (same arithmetic, done once per step).
// With nnb = 6 and coef = dt/num_loop/dx^2 it is also one sub-step of the
// reference's GPU plug-in (gpu_solver.cpp:131-188): the partition written here
// is exactly what GPU_Partitioning computes at the start of the next sub-step.
__global__ void __launch_bounds__(256) k_diffuse_f64(const __grid_constant__ pf_step_params P, int nnb,
                                                     double coef, const double *__restrict__ links,
                                                     const double *__restrict__ tpart,
                                                     const double *__restrict__ conc1,
                                                     double *__restrict__ conc2,
                                                     double *__restrict__ C) {
    int ci, cj, ck;
    long long n;
    if (!pf_cell(P.ix, P.iy, ci, cj, ck, n)) return;
    long long nbr[6];
    pf_neighbours3(ci, cj, ck, n, P.ix, P.iy, P.iz, nbr);
    double w[6][3];
#pragma unroll
    for (int b = 0; b < 6; b++)
        if (b < nnb) {
            const long long at = (b & 1) ? 9 * n + 3 * (b >> 1) : 9 * nbr[b] + 3 * (b >> 1);
#pragma unroll
            for (int p = 0; p < 3; p++) w[b][p] = __ldg(links + at + p);
        }
    for (int q = 0; q < P.nsol; q++) {
        const double *c1 = conc1 + (long long)q * 3 * P.N;
        double cs[3];
        cs[0] = __ldg(c1 + 3 * n + 0);
        cs[1] = __ldg(c1 + 3 * n + 1);
        cs[2] = __ldg(c1 + 3 * n + 2);
        double del = 0.;
#pragma unroll
        for (int b = 0; b < 6; b++)
            if (b < nnb) {
#pragma unroll
                for (int p = 0; p < 3; p++)
                    del += w[b][p] * (__ldg(c1 + 3 * nbr[b] + p) - cs[p]) * P.D[q][p];
            }
        del *= coef;
        const double cn = C[q * P.N + n] + del;
        C[q * P.N + n] = cn;
        const double *tp = tpart + 6 * ((long long)q * P.N + n);
        double *cp = conc2 + (long long)q * 3 * P.N + 3 * n;
#pragma unroll
        for (int i = 0; i < 3; i++) cp[i] = (cn - __ldg(tp + 3 + i)) / __ldg(tp + i);
    }
}

// Partitioning of every cell and solute (MicrostructureConstruction.cpp:53-62,
// gpu_solver.cpp:131-154).
__global__ void __launch_bounds__(256) k_partition_f64(const __grid_constant__ pf_step_params P,
                                                       const double *__restrict__ phase,
                                                       const double *__restrict__ C,
                                                       double *__restrict__ conc) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.N) return;
    double ph[3] = {phase[3 * n], phase[3 * n + 1], phase[3 * n + 2]};
    for (int q = 0; q < P.nsol; q++) {
        double out[3];
        pf_partition(C[q * P.N + n], ph, P.k[q], P.c[q], out);
        double *cp = conc + (long long)q * 3 * P.N + 3 * n;
        cp[0] = out[0]; cp[1] = out[1]; cp[2] = out[2];
    }
}

inline unsigned pf_blocks(long long N, int threads) { return (unsigned)((N + threads - 1) / threads); }

}  // namespace

cudaError_t pf_launch_phase_f64(const pf_step_params &P, const int *ids1, const double *phi1, int *ids2,
                                double *phi2, double *phase, double *conc1, const double *C, double *avg,
                                unsigned char *flags, const int *coh, int n_coh, cudaStream_t s) {
    const bool scanned = P.avg_range > 0 && avg;
    const bool coherent = scanned && P.coh_model && flags && coh;
    if (scanned) {
        k_avg_conc_f64<<<pf_cell_grid(P.ix, P.iy, P.iz), PF_CELL_THREADS, 0, s>>>(P, ids1, phase, conc1, avg,
                                                                                  coherent ? flags : nullptr);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int pt = pf_use_patch(P.iy, P.iz);  // warps on compact cell patches
    const dim3 gp = pf_map_grid(pt, P.ix, P.iy, P.iz);
    if (P.drag_model || coherent)
        k_phase_f64<true><<<gp, PF_CELL_THREADS, 0, s>>>(P, pt, ids1, phi1, ids2, phi2, phase, conc1, C,
                                                         scanned ? avg : nullptr, coherent ? flags : nullptr,
                                                         coherent ? coh : nullptr, n_coh);
    else
        k_phase_f64<false><<<gp, PF_CELL_THREADS, 0, s>>>(P, pt, ids1, phi1, ids2, phi2, phase, conc1, C,
                                                          scanned ? avg : nullptr, nullptr, nullptr, 0);
    return cudaGetLastError();
}

cudaError_t pf_launch_links_f64(const pf_step_params &P, int nnb, const double *phase, double *links,
                                double *tpart, cudaStream_t s) {
    k_links_f64<<<pf_cell_grid(P.ix, P.iy, P.iz), PF_CELL_THREADS, 0, s>>>(P, nnb, phase, links, tpart);
    return cudaGetLastError();
}

cudaError_t pf_launch_diffuse_f64(const pf_step_params &P, int nnb, double coef, const double *links,
                                  const double *tpart, const double *conc1, double *conc2, double *C,
                                  cudaStream_t s) {
    k_diffuse_f64<<<pf_cell_grid(P.ix, P.iy, P.iz), PF_CELL_THREADS, 0, s>>>(P, nnb, coef, links, tpart, conc1,
                                                                             conc2, C);
    return cudaGetLastError();
}

cudaError_t pf_launch_partition_f64(const pf_step_params &P, const double *phase, const double *C,
                                    double *conc, cudaStream_t s) {
    k_partition_f64<<<pf_blocks(P.N, 256), 256, 0, s>>>(P, phase, C, conc);
    return cudaGetLastError();
}

int pf_drag_take_failure() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_drag_fail, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_drag_fail, &zero, sizeof(int));
    }
    return v;
}
