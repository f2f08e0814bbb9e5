// pf_init.cpp -- seeded synthetic initial microstructure (host, OpenMP).
//
// The per-cell generator is pf_init_cell.h (shared with the device generator
// pf_init_dev.cu); this file draws the seeds, builds their bucket grids and
// runs the cells of a z slab.  Every value is a function of the global cell
// index and the seed alone, so any z slab of the domain can be generated by
// itself and the result does not depend on the thread count.
//
// The nearest Voronoi seeds of a cell are found on a periodic bucket grid,
// searching growing cubes of buckets until no unvisited seed can be closer
// than the sixth found; candidates are ranked by (distance, seed index), so
// the result equals a scan over every seed in index order.
//
// Compiled into libpfstep and, unchanged, into the CPU oracle library (the
// CPU baseline must step the same state as the GPU).
#include "pf_init.h"

#include <algorithm>
#include <cmath>
#include <vector>

#include "pf_init_setup.h"

void PfHostBuckets::build(const std::vector<double> &x, const std::vector<double> &y, const std::vector<double> &z,
                          const int len[3], double target_edge) {
    for (int d = 0; d < 3; d++) {
        n[d] = std::max(1, (int)std::floor(len[d] / std::max(target_edge, 1.0)));
        edge[d] = (double)len[d] / n[d];
    }
    const size_t nb = (size_t)n[0] * n[1] * n[2];
    std::vector<int> cnt(nb + 1, 0);
    std::vector<size_t> where(x.size());
    for (size_t g = 0; g < x.size(); g++) {
        const int b[3] = {std::min(n[0] - 1, (int)(x[g] / edge[0])), std::min(n[1] - 1, (int)(y[g] / edge[1])),
                          std::min(n[2] - 1, (int)(z[g] / edge[2]))};
        where[g] = b[0] + (size_t)n[0] * (b[1] + (size_t)n[1] * b[2]);
        cnt[where[g] + 1]++;
    }
    for (size_t b = 0; b < nb; b++) cnt[b + 1] += cnt[b];
    start = cnt;
    items.assign(x.size(), 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (size_t g = 0; g < x.size(); g++) items[fill[where[g]]++] = (int)g;
}

pfinit::Buckets PfHostBuckets::view(const int *start_ptr, const int *items_ptr) const {
    pfinit::Buckets b;
    for (int d = 0; d < 3; d++) {
        b.n[d] = n[d];
        b.edge[d] = edge[d];
    }
    b.start = start_ptr;
    b.items = items_ptr;
    return b;
}

int pf_init_prepare(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec, PfInitHost &H,
                    const char **msg) {
    auto fail = [&](int st, const char *m) {
        if (msg) *msg = m;
        return st;
    };
    if (!spec) return fail(PF_ERR_ARG, "null argument");
    if (ix < 1 || iy < 1 || iz < 1 || nsol < 1 || nsol > 2) return fail(PF_ERR_ARG, "bad grid");
    if (spec->n_grains < 1) return fail(PF_ERR_ARG, "need at least one grain");
    if (spec->n_grains >= pfinit::kGrainsPerPhase || spec->n_nuclei >= pfinit::kGrainsPerPhase ||
        spec->n_particles >= pfinit::kGrainsPerPhase)
        return fail(PF_ERR_RANGE, "too many grains");
    const double W = spec->width > 0 ? spec->width : 6.0;
    const double kk = 3.0 / W;  // tanh(3*h/W): 5%..95% over one interface width
    uint64_t s = spec->seed;
    auto draw = [&](int n, std::vector<double> &X, std::vector<double> &Y, std::vector<double> &Z) {
        X.resize(n); Y.resize(n); Z.resize(n);
        for (int g = 0; g < n; g++) {
            X[g] = pfinit::u01(s) * ix; Y[g] = pfinit::u01(s) * iy; Z[g] = pfinit::u01(s) * iz;
        }
    };
    draw(spec->n_grains, H.gx, H.gy, H.gz);
    draw(spec->n_nuclei, H.nx, H.ny, H.nz);
    draw(spec->n_particles, H.px, H.py, H.pz);
    const bool zflat = (iz == 1), yflat = (iy == 1);
    const int len[3] = {ix, yflat ? 1 : iy, zflat ? 1 : iz};
    // Voronoi seed buckets: about two seeds per bucket.
    const int dims = 1 + (yflat ? 0 : 1) + (zflat ? 0 : 1);
    const double vol = (double)ix * (yflat ? 1 : iy) * (zflat ? 1 : iz);
    const double spacing = std::pow(vol / spec->n_grains, 1.0 / dims);
    std::vector<double> gyb = H.gy, gzb = H.gz;
    if (yflat) std::fill(gyb.begin(), gyb.end(), 0.0);
    if (zflat) std::fill(gzb.begin(), gzb.end(), 0.0);
    H.bgr.build(H.gx, gyb, gzb, len, std::max(1.0, spacing * std::pow(2.0, 1.0 / dims)));
    const int blen[3] = {ix, iy, iz};
    H.bnuc.build(H.nx, H.ny, H.nz, blen, spec->nucleus_radius + 3.0 / kk + 1.0);
    H.bpar.build(H.px, H.py, H.pz, blen, spec->particle_radius + 3.0 / kk + 1.0);
    pfinit::Setup &S = H.S;
    S.ix = ix; S.iy = iy; S.iz = iz;
    S.K = spec->max_slots < 1 ? 1 : (spec->max_slots > 6 ? 6 : spec->max_slots);
    S.nsol = nsol;
    S.yflat = yflat; S.zflat = zflat;
    S.gx = H.gx.data(); S.gy = H.gy.data(); S.gz = H.gz.data();
    S.nx = H.nx.data(); S.ny = H.ny.data(); S.nz = H.nz.data();
    S.px = H.px.data(); S.py = H.py.data(); S.pz = H.pz.data();
    S.bgr = H.bgr.view(H.bgr.start.data(), H.bgr.items.data());
    S.bnuc = H.bnuc.view(H.bnuc.start.data(), H.bnuc.items.data());
    S.bpar = H.bpar.view(H.bpar.start.data(), H.bpar.items.data());
    S.kk = kk;
    S.nucleus_radius = spec->nucleus_radius;
    S.particle_radius = spec->particle_radius;
    S.cutoff = cutoff;
    for (int q = 0; q < 2; q++) {
        S.C0[q] = spec->C0[q];
        S.C_noise[q] = spec->C_noise[q];
    }
    S.seed = spec->seed;
    if (msg) *msg = nullptr;
    return PF_OK;
}

extern "C" int pf_init_state(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec,
                             const double *kq, const double *cq, int z0, int nzb, int32_t *ids, double *phi,
                             double *phase, double *conc, double *C, const char **msg) {
    auto fail = [&](int st, const char *m) {
        if (msg) *msg = m;
        return st;
    };
    if (!spec || !ids || !phi || !phase || !C) return fail(PF_ERR_ARG, "null argument");
    if (ix < 1 || iy < 1 || iz < 1 || z0 < 0 || nzb < 1 || z0 + nzb > iz || nsol < 1 || nsol > 2)
        return fail(PF_ERR_ARG, "bad grid or slab");
    if (conc && (!kq || !cq)) return fail(PF_ERR_ARG, "partition coefficients needed for conc");
    PfInitHost H;
    const int st = pf_init_prepare(ix, iy, iz, nsol, cutoff, spec, H, msg);
    if (st != PF_OK) return st;
    const pfinit::Setup &S = H.S;
    const long long Nb = (long long)ix * iy * nzb;  // cells of the slab
    int crowded = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : crowded)
    for (long long n = 0; n < Nb; n++) {
        const int i = (int)(n % ix);
        const int j = (int)((n / ix) % iy);
        const int k = z0 + (int)(n / ((long long)ix * iy));
        double Cv[2], ph[3];
        if (!pfinit::cell(S, i, j, k, ids + 6 * n, phi + 6 * n, ph, Cv)) crowded = 1;
        for (int p = 0; p < 3; p++) phase[3 * n + p] = ph[p];
        for (long long q = 0; q < nsol; q++) {
            C[q * Nb + n] = Cv[q];
            if (conc) {
                double out[3];
                pfinit::partition(ph, Cv[q], kq + q * 9, cq + q * 9, out);
                for (int a = 0; a < 3; a++) conc[q * 3 * Nb + 3 * n + a] = out[a];
            }
        }
    }
    if (crowded) return fail(PF_ERR_RANGE, "more than 256 inclusions near one cell");
    if (msg) *msg = nullptr;
    return PF_OK;
}

extern "C" int pf_init_coherent_table(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec,
                                      int32_t *partners, const char **msg) {
    auto fail = [&](int st, const char *m) {
        if (msg) *msg = m;
        return st;
    };
    if (!spec || (spec->n_nuclei > 0 && !partners)) return fail(PF_ERR_ARG, "null argument");
    PfInitHost H;
    const int st = pf_init_prepare(ix, iy, iz, nsol, cutoff, spec, H, msg);
    if (st != PF_OK) return st;
    // The matrix before nucleation: the same set-up with no nucleus near any cell.
    const std::vector<double> none;
    PfHostBuckets empty;
    const int blen[3] = {ix, iy, iz};
    empty.build(none, none, none, blen, 1.0);
    pfinit::Setup S = H.S;
    S.bnuc = empty.view(empty.start.data(), empty.items.data());
    auto site = [](double v, int L) {
        const long long c = (long long)std::floor(v + 0.5);
        return (int)(((c % L) + L) % L);
    };
    int crowded = 0;
#pragma omp parallel for schedule(static) reduction(| : crowded)
    for (int n = 0; n < spec->n_nuclei; n++) {
        const int i = site(H.nx[n], ix), j = S.yflat ? 0 : site(H.ny[n], iy), k = S.zflat ? 0 : site(H.nz[n], iz);
        int32_t ids[6];
        double phi[6], ph[3], Cv[2];
        if (!pfinit::cell(S, i, j, k, ids, phi, ph, Cv)) crowded = 1;
        int fer[6], nf = 0;
        for (int a = 0; a < 6; a++)
            if (ids[a] / pfinit::kGrainsPerPhase == 1) fer[nf++] = ids[a];
        std::sort(fer, fer + nf, [](int a, int b) { return a > b; });
        const int or_num = std::min(2, nf - 1);
        partners[2 * n] = or_num >= 1 ? fer[0] : 0;
        partners[2 * n + 1] = or_num >= 2 ? fer[1] : 0;
    }
    if (crowded) return fail(PF_ERR_RANGE, "more than 256 inclusions near one cell");
    if (msg) *msg = nullptr;
    return PF_OK;
}
