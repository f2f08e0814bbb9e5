// pf_init.cpp -- seeded synthetic initial microstructure (host, OpenMP).
//
// Replaces the reference's unseeded Construct / Nucleate1in2
// (zhubq/PhaseField C++-openmp-cuda/src/MicrostructureConstruction.cpp:4-109,
// nucleation.cpp:3-43) with a reproducible generator: a periodic Voronoi
// ferrite matrix (ids 100000+g) with a tanh profile across every bisector,
// spherical austenite nuclei (ids 200000+n) and cementite particles
// (ids 300000+n) laid over it with the same profile, uniform solutes plus
// counter-based uniform noise.  Every value is a function of the global cell
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

namespace {

constexpr int kGrainsPerPhase = 100000;  // phase_field.h:19

inline uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double u01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }
// Counter-based uniform for per-cell noise: independent of thread count.
inline double u01_at(uint64_t seed, uint64_t stream, uint64_t n) {
    uint64_t s = seed ^ (stream * 0xD1B54A32D192ED03ull) ^ (n * 0x9E3779B97F4A7C15ull);
    splitmix64(s);
    return u01(s);
}
// Minimum-image separation along one periodic axis (|d| < len on entry).
inline double mi(double d, int len) {
    const double L = (double)len;
    if (d > 0.5 * L) d -= L;
    else if (d < -0.5 * L) d += L;
    return d;
}

struct Cand {
    int id;
    double w;
};

// Periodic bucket grid over points (CSR lists, ascending point index).
struct Buckets {
    int n[3] = {1, 1, 1};
    double edge[3] = {1, 1, 1};
    std::vector<int> start, items;

    void build(const std::vector<double> &x, const std::vector<double> &y, const std::vector<double> &z,
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
    int cell_of(double p, int d) const { return std::min(n[d] - 1, std::max(0, (int)(p / edge[d]))); }
    // Points in the buckets within Chebyshev radius r of the bucket holding p
    // (unordered unless 'sorted'); covered[d] tells whether dimension d is
    // searched entirely.
    void gather(const double p[3], int r, std::vector<int> &out, bool covered[3], bool sorted) const {
        out.clear();
        int lo[3], cnt[3];
        for (int d = 0; d < 3; d++) {
            covered[d] = 2 * r + 1 >= n[d];
            lo[d] = covered[d] ? 0 : cell_of(p[d], d) - r;
            cnt[d] = covered[d] ? n[d] : 2 * r + 1;
        }
        for (int a = 0; a < cnt[2]; a++) {
            const int bz = ((lo[2] + a) % n[2] + n[2]) % n[2];
            for (int b = 0; b < cnt[1]; b++) {
                const int by = ((lo[1] + b) % n[1] + n[1]) % n[1];
                for (int cc = 0; cc < cnt[0]; cc++) {
                    const int bx = ((lo[0] + cc) % n[0] + n[0]) % n[0];
                    const size_t bk = bx + (size_t)n[0] * (by + (size_t)n[1] * bz);
                    out.insert(out.end(), items.begin() + start[bk], items.begin() + start[bk + 1]);
                }
            }
        }
        if (sorted) std::sort(out.begin(), out.end());
    }
    // Distance from p to the outside of the searched cube along dimension d.
    double margin(const double p[3], int r, int d) const {
        const int c = cell_of(p[d], d);
        return std::min(p[d] - (c - r) * edge[d], (c + r + 1) * edge[d] - p[d]);
    }
};

}  // namespace

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
    const long long Nb = (long long)ix * iy * nzb;  // cells of the slab
    const int K = spec->max_slots < 1 ? 1 : (spec->max_slots > 6 ? 6 : spec->max_slots);
    if (spec->n_grains < 1) return fail(PF_ERR_ARG, "need at least one grain");
    if (spec->n_grains >= kGrainsPerPhase || spec->n_nuclei >= kGrainsPerPhase ||
        spec->n_particles >= kGrainsPerPhase)
        return fail(PF_ERR_RANGE, "too many grains");
    const double W = spec->width > 0 ? spec->width : 6.0;
    const double kk = 3.0 / W;  // tanh(3*h/W): 5%..95% over one interface width
    uint64_t s = spec->seed;
    std::vector<double> gx(spec->n_grains), gy(spec->n_grains), gz(spec->n_grains);
    for (int g = 0; g < spec->n_grains; g++) {
        gx[g] = u01(s) * ix; gy[g] = u01(s) * iy; gz[g] = u01(s) * iz;
    }
    std::vector<double> nx(spec->n_nuclei), ny(spec->n_nuclei), nz(spec->n_nuclei);
    for (int g = 0; g < spec->n_nuclei; g++) {
        nx[g] = u01(s) * ix; ny[g] = u01(s) * iy; nz[g] = u01(s) * iz;
    }
    std::vector<double> px(spec->n_particles), py(spec->n_particles), pz(spec->n_particles);
    for (int g = 0; g < spec->n_particles; g++) {
        px[g] = u01(s) * ix; py[g] = u01(s) * iy; pz[g] = u01(s) * iz;
    }
    const uint64_t seed = spec->seed;
    const bool zflat = (iz == 1), yflat = (iy == 1);
    const int len[3] = {ix, yflat ? 1 : iy, zflat ? 1 : iz};
    // Voronoi seed buckets: about two seeds per bucket.
    const int dims = 1 + (yflat ? 0 : 1) + (zflat ? 0 : 1);
    const double vol = (double)ix * (yflat ? 1 : iy) * (zflat ? 1 : iz);
    const double spacing = std::pow(vol / spec->n_grains, 1.0 / dims);
    std::vector<double> gyb = gy, gzb = gz;
    if (yflat) std::fill(gyb.begin(), gyb.end(), 0.0);
    if (zflat) std::fill(gzb.begin(), gzb.end(), 0.0);
    Buckets bgr, bnuc, bpar;
    bgr.build(gx, gyb, gzb, len, std::max(1.0, spacing * std::pow(2.0, 1.0 / dims)));
    const int blen[3] = {ix, iy, iz};
    bnuc.build(nx, ny, nz, blen, spec->nucleus_radius + 3.0 / kk + 1.0);
    bpar.build(px, py, pz, blen, spec->particle_radius + 3.0 / kk + 1.0);

#pragma omp parallel
    {
    std::vector<int> near;
    near.reserve(256);
#pragma omp for schedule(dynamic, 256)
    for (long long n = 0; n < Nb; n++) {
        const int i = (int)(n % ix);
        const int j = (int)((n / ix) % iy);
        const int k = z0 + (int)(n / ((long long)ix * iy));
        const long long ng = i + (long long)ix * (j + (long long)iy * k);  // global cell index
        const double x = i, y = j, z = k;
        // Ferrite matrix: periodic Voronoi with a tanh profile across each
        // bisector.  Keep the few nearest seeds (first seed wins ties).
        constexpr int KN = 6;
        int best[KN];
        double bd2[KN], bvx[KN], bvy[KN], bvz[KN];
        int nb = 0;
        const double pg[3] = {x, yflat ? 0.0 : y, zflat ? 0.0 : z};
        for (int r = 1;; r++) {
            bool covered[3];
            bgr.gather(pg, r, near, covered, false);
            nb = 0;
            // Ranked by (distance, seed index): the order of a scan over the
            // seeds in index order that keeps the first of equal distances.
            for (int g : near) {
                const double vx = mi(gx[g] - x, ix), vy = yflat ? 0 : mi(gy[g] - y, iy), vz = zflat ? 0 : mi(gz[g] - z, iz);
                const double d2 = vx * vx + vy * vy + vz * vz;
                if (nb < KN || d2 < bd2[nb - 1] || (d2 == bd2[nb - 1] && g < best[nb - 1])) {
                    int pos = nb < KN ? nb++ : KN - 1;
                    while (pos > 0 && (bd2[pos - 1] > d2 || (bd2[pos - 1] == d2 && best[pos - 1] > g))) {
                        best[pos] = best[pos - 1]; bd2[pos] = bd2[pos - 1];
                        bvx[pos] = bvx[pos - 1]; bvy[pos] = bvy[pos - 1]; bvz[pos] = bvz[pos - 1];
                        pos--;
                    }
                    best[pos] = g; bd2[pos] = d2; bvx[pos] = vx; bvy[pos] = vy; bvz[pos] = vz;
                }
            }
            double margin = 1e300;
            bool all = true;
            for (int d = 0; d < 3; d++)
                if (!covered[d]) {
                    all = false;
                    margin = std::min(margin, bgr.margin(pg, r, d));
                }
            if (all) break;
            if (nb == KN && bd2[KN - 1] < margin * margin) break;
        }
        // Signed distance to each candidate's Voronoi cell boundary facing the
        // nearest seed: h_g = (|b|^2 - |a|^2) / (2|b - a|) for g != nearest,
        // and the nearest grain's depth -min_g h_g.
        Cand cand[16];
        int nc = 0;
        double hmin = 1e30;
        double hg[KN];
        for (int t = 1; t < nb; t++) {
            const double dx_ = bvx[t] - bvx[0], dy_ = bvy[t] - bvy[0], dz_ = bvz[t] - bvz[0];
            const double sep = std::sqrt(dx_ * dx_ + dy_ * dy_ + dz_ * dz_);
            hg[t] = sep > 0 ? (bd2[t] - bd2[0]) / (2 * sep) : 0.0;
            if (hg[t] < hmin) hmin = hg[t];
        }
        hg[0] = nb > 1 ? -hmin : -1e30;
        double wsum = 0;
        for (int t = 0; t < nb; t++) {
            const double a = kk * hg[t];
            const double w = a >= 3.0 ? 0.0 : (a <= -3.0 ? 1.0 : 0.5 * (1.0 - std::tanh(a)));
            if (w > 0) { cand[nc++] = {100000 + best[t] + 1, w}; wsum += w; }
        }
        for (int t = 0; t < nc; t++) cand[t].w /= wsum;
        // Nuclei and particles: spheres (discs in 2D) with the same profile.
        auto add_spheres = [&](const std::vector<double> &sx, const std::vector<double> &sy,
                               const std::vector<double> &sz, double r, int base, const Buckets &bk) {
            const double p[3] = {x, y, z};
            bool cov[3];
            bk.gather(p, 1, near, cov, true);  // inclusions apply in index order
            for (int g : near) {
                const double vx = mi(sx[g] - x, ix), vy = yflat ? 0 : mi(sy[g] - y, iy), vz = zflat ? 0 : mi(sz[g] - z, iz);
                const double a = kk * (std::sqrt(vx * vx + vy * vy + vz * vz) - r);
                if (a >= 3.0) continue;
                const double w = a <= -3.0 ? 1.0 : 0.5 * (1.0 - std::tanh(a));
                // Insert w for this inclusion, scaling what was there by (1-w).
                double keep = 1.0 - w;
                for (int t = 0; t < nc; t++) cand[t].w *= keep;
                if (nc < 16) cand[nc++] = {base + (int)g + 1, w};
                else {
                    int lo = 0;
                    for (int t = 1; t < nc; t++) if (cand[t].w < cand[lo].w) lo = t;
                    if (cand[lo].w < w) cand[lo] = {base + (int)g + 1, w};
                }
            }
        };
        add_spheres(nx, ny, nz, spec->nucleus_radius, 200000, bnuc);
        add_spheres(px, py, pz, spec->particle_radius, 300000, bpar);
        // Largest K with weight above the cutoff, sorted descending, renormalised.
        for (int a = 0; a < nc; a++)
            for (int b = a + 1; b < nc; b++)
                if (cand[b].w > cand[a].w) std::swap(cand[a], cand[b]);
        int keep = 0;
        double sum = 0;
        for (int a = 0; a < nc && keep < K; a++)
            if (cand[a].w > 10.0 * cutoff) { keep++; sum += cand[a].w; }
        double ph[3] = {0, 0, 0};
        for (int a = 0; a < 6; a++) {
            if (a < keep) {
                const double v = cand[a].w / sum;
                ids[6 * n + a] = cand[a].id;
                phi[6 * n + a] = v;
                ph[cand[a].id / kGrainsPerPhase - 1] += v;
            } else {
                ids[6 * n + a] = 0;
                phi[6 * n + a] = 0.0;
            }
        }
        for (int p = 0; p < 3; p++) phase[3 * n + p] = ph[p];
        for (long long q = 0; q < nsol; q++) {
            const double cv = spec->C0[q] + spec->C_noise[q] * (2.0 * u01_at(seed, 1 + q, (uint64_t)ng) - 1.0);
            C[q * Nb + n] = cv;
            if (conc) {
                // solver.cpp:389-405
                for (int a = 1; a <= 3; a++) {
                    double t1 = 0., t2 = 0.;
                    for (int b = 1; b <= 3; b++) {
                        t1 += ph[b - 1] * kq[q * 9 + (a - 1) + 3 * (b - 1)];
                        t2 += ph[b - 1] * cq[q * 9 + (a - 1) + 3 * (b - 1)];
                    }
                    conc[q * 3 * Nb + 3 * n + a - 1] = (cv - t2) / t1;
                }
            }
        }
    }
    }  // omp parallel
    if (msg) *msg = nullptr;
    return PF_OK;
}
