// pf_init_cell.h -- one cell of the seeded initial microstructure.
//
// Shared, unchanged, by the host generator (pf_init.cpp, OpenMP; also built
// into the CPU oracle library) and the device generator (pf_init_dev.cu, one
// thread per cell), so both place the same grains in the same cells.  The
// two agree bit for bit except where the host's and the device's tanh round
// differently (a few ulp of a weight).
//
// The generator replaces the reference's unseeded Construct / Nucleate1in2
// (zhubq/PhaseField C++-openmp-cuda/src/MicrostructureConstruction.cpp:4-109,
// nucleation.cpp:3-43): a periodic Voronoi ferrite matrix (ids 100000+g) with
// a tanh profile across every bisector, spherical austenite nuclei (ids
// 200000+n) and cementite particles (ids 300000+n) laid over it in index
// order with the same profile, uniform solutes plus counter-based noise.
// Every value is a function of the global cell index and the seed alone.
#pragma once
#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define PF_HD __host__ __device__ __forceinline__
#else
#define PF_HD inline
#endif

namespace pfinit {

constexpr int kGrainsPerPhase = 100000;  // phase_field.h:19
constexpr int kNear = 6;                 // nearest Voronoi seeds ranked per cell
constexpr int kCand = 16;                // weighted candidates per cell
constexpr int kSpheres = 256;            // inclusions near one cell (more: PF_ERR_RANGE)

PF_HD uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
PF_HD double u01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }
// Counter-based uniform for per-cell noise: independent of the thread count.
PF_HD double u01_at(uint64_t seed, uint64_t stream, uint64_t n) {
    uint64_t s = seed ^ (stream * 0xD1B54A32D192ED03ull) ^ (n * 0x9E3779B97F4A7C15ull);
    splitmix64(s);
    return u01(s);
}
// Minimum-image separation along one periodic axis (|d| < len on entry).
PF_HD double mi(double d, int len) {
    const double L = (double)len;
    if (d > 0.5 * L) d -= L;
    else if (d < -0.5 * L) d += L;
    return d;
}

// A periodic bucket grid over points (CSR lists in ascending point index).
struct Buckets {
    int n[3];
    double edge[3];
    const int *start, *items;

    PF_HD int cell_of(double p, int d) const {
        const int c = (int)(p / edge[d]);
        return c < 0 ? 0 : (c > n[d] - 1 ? n[d] - 1 : c);
    }
    // Calls f(point) for every point in the buckets within Chebyshev radius r
    // of the bucket holding p; covered[d] tells whether dimension d is
    // searched entirely (then every bucket of it is visited once).
    template <class F>
    PF_HD void visit(const double p[3], int r, bool covered[3], F &&f) const {
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
                for (int c = 0; c < cnt[0]; c++) {
                    const int bx = ((lo[0] + c) % n[0] + n[0]) % n[0];
                    const long long bk = bx + (long long)n[0] * (by + (long long)n[1] * bz);
                    for (int t = start[bk]; t < start[bk + 1]; t++) f(items[t]);
                }
            }
        }
    }
    // Distance from p to the outside of the searched cube along dimension d.
    PF_HD double margin(const double p[3], int r, int d) const {
        const int c = cell_of(p[d], d);
        const double a = p[d] - (c - r) * edge[d], b = (c + r + 1) * edge[d] - p[d];
        return a < b ? a : b;
    }
};

// Everything a cell needs: seed coordinates, their bucket grids, the profile
// and the solute parameters.
struct Setup {
    int ix, iy, iz, K, nsol;
    bool yflat, zflat;
    const double *gx, *gy, *gz;  // Voronoi seeds
    const double *nx, *ny, *nz;  // nuclei
    const double *px, *py, *pz;  // particles
    Buckets bgr, bnuc, bpar;
    double kk, nucleus_radius, particle_radius, cutoff;
    double C0[2], C_noise[2];
    uint64_t seed;
};

struct Cand {
    int id;
    double w;
};

// One cell (i, j, k): its six slots (largest K weights above 10*cutoff,
// sorted, renormalised), phase fractions and solute values.  Returns false
// when more than kSpheres inclusions lie near the cell.
PF_HD bool cell(const Setup &S, int i, int j, int k, int32_t ids[6], double phi[6], double phase[3],
                double Cv[2]) {
    const long long ng = i + (long long)S.ix * (j + (long long)S.iy * k);  // global cell index
    const double x = i, y = j, z = k;
    const int ix = S.ix, iy = S.iy, iz = S.iz;
    // Ferrite matrix: periodic Voronoi with a tanh profile across each
    // bisector.  The kNear nearest seeds, ranked by (distance, seed index):
    // the order of a scan over the seeds in index order keeping the first of
    // equal distances.
    int best[kNear];
    double bd2[kNear], bvx[kNear], bvy[kNear], bvz[kNear];
    int nb = 0;
    const double pg[3] = {x, S.yflat ? 0.0 : y, S.zflat ? 0.0 : z};
    for (int r = 1;; r++) {
        bool covered[3];
        nb = 0;
        S.bgr.visit(pg, r, covered, [&](int g) {
            const double vx = mi(S.gx[g] - x, ix), vy = S.yflat ? 0 : mi(S.gy[g] - y, iy),
                         vz = S.zflat ? 0 : mi(S.gz[g] - z, iz);
            const double d2 = vx * vx + vy * vy + vz * vz;
            if (nb < kNear || d2 < bd2[nb - 1] || (d2 == bd2[nb - 1] && g < best[nb - 1])) {
                int pos = nb < kNear ? nb++ : kNear - 1;
                while (pos > 0 && (bd2[pos - 1] > d2 || (bd2[pos - 1] == d2 && best[pos - 1] > g))) {
                    best[pos] = best[pos - 1]; bd2[pos] = bd2[pos - 1];
                    bvx[pos] = bvx[pos - 1]; bvy[pos] = bvy[pos - 1]; bvz[pos] = bvz[pos - 1];
                    pos--;
                }
                best[pos] = g; bd2[pos] = d2; bvx[pos] = vx; bvy[pos] = vy; bvz[pos] = vz;
            }
        });
        double margin = 1e300;
        bool all = true;
        for (int d = 0; d < 3; d++)
            if (!covered[d]) {
                all = false;
                const double m = S.bgr.margin(pg, r, d);
                if (m < margin) margin = m;
            }
        if (all) break;
        if (nb == kNear && bd2[kNear - 1] < margin * margin) break;
    }
    // Signed distance to each candidate's Voronoi cell boundary facing the
    // nearest seed: h_g = (|b|^2 - |a|^2) / (2|b - a|) for g != nearest, and
    // the nearest grain's depth -min_g h_g.
    Cand cand[kCand];
    int nc = 0;
    double hmin = 1e30;
    double hg[kNear];
    for (int t = 1; t < nb; t++) {
        const double dx_ = bvx[t] - bvx[0], dy_ = bvy[t] - bvy[0], dz_ = bvz[t] - bvz[0];
        const double sep = sqrt(dx_ * dx_ + dy_ * dy_ + dz_ * dz_);
        hg[t] = sep > 0 ? (bd2[t] - bd2[0]) / (2 * sep) : 0.0;
        if (hg[t] < hmin) hmin = hg[t];
    }
    hg[0] = nb > 1 ? -hmin : -1e30;
    double wsum = 0;
    for (int t = 0; t < nb; t++) {
        const double a = S.kk * hg[t];
        const double w = a >= 3.0 ? 0.0 : (a <= -3.0 ? 1.0 : 0.5 * (1.0 - tanh(a)));
        if (w > 0) { cand[nc++] = {100000 + best[t] + 1, w}; wsum += w; }
    }
    for (int t = 0; t < nc; t++) cand[t].w /= wsum;
    // Nuclei and particles: spheres (discs in 2D) with the same profile,
    // applied in index order.
    bool ok = true;
    auto add_spheres = [&](const double *sx, const double *sy, const double *sz, double rad, int base,
                           const Buckets &bk) {
        int near[kSpheres];
        int cnt = 0;
        const double p[3] = {x, y, z};
        bool cov[3];
        bk.visit(p, 1, cov, [&](int g) {
            if (cnt < kSpheres) near[cnt] = g;
            cnt++;
        });
        if (cnt > kSpheres) {
            ok = false;
            cnt = kSpheres;
        }
        for (int a = 1; a < cnt; a++) {  // ascending index
            const int v = near[a];
            int b = a;
            while (b > 0 && near[b - 1] > v) { near[b] = near[b - 1]; b--; }
            near[b] = v;
        }
        for (int t = 0; t < cnt; t++) {
            const int g = near[t];
            const double vx = mi(sx[g] - x, ix), vy = S.yflat ? 0 : mi(sy[g] - y, iy),
                         vz = S.zflat ? 0 : mi(sz[g] - z, iz);
            const double a = S.kk * (sqrt(vx * vx + vy * vy + vz * vz) - rad);
            if (a >= 3.0) continue;
            const double w = a <= -3.0 ? 1.0 : 0.5 * (1.0 - tanh(a));
            // Insert w for this inclusion, scaling what was there by (1-w).
            const double keep = 1.0 - w;
            for (int c = 0; c < nc; c++) cand[c].w *= keep;
            if (nc < kCand) cand[nc++] = {base + g + 1, w};
            else {
                int lo = 0;
                for (int c = 1; c < nc; c++) if (cand[c].w < cand[lo].w) lo = c;
                if (cand[lo].w < w) cand[lo] = {base + g + 1, w};
            }
        }
    };
    add_spheres(S.nx, S.ny, S.nz, S.nucleus_radius, 200000, S.bnuc);
    add_spheres(S.px, S.py, S.pz, S.particle_radius, 300000, S.bpar);
    // Largest K with weight above 10 * cutoff, sorted descending, renormalised.
    for (int a = 0; a < nc; a++)
        for (int b = a + 1; b < nc; b++)
            if (cand[b].w > cand[a].w) { const Cand t = cand[a]; cand[a] = cand[b]; cand[b] = t; }
    int keep = 0;
    double sum = 0;
    for (int a = 0; a < nc && keep < S.K; a++)
        if (cand[a].w > 10.0 * S.cutoff) { keep++; sum += cand[a].w; }
    phase[0] = phase[1] = phase[2] = 0;
    for (int a = 0; a < 6; a++) {
        if (a < keep) {
            const double v = cand[a].w / sum;
            ids[a] = cand[a].id;
            phi[a] = v;
            phase[cand[a].id / kGrainsPerPhase - 1] += v;
        } else {
            ids[a] = 0;
            phi[a] = 0.0;
        }
    }
    for (int q = 0; q < S.nsol; q++)
        Cv[q] = S.C0[q] + S.C_noise[q] * (2.0 * u01_at(S.seed, 1 + q, (uint64_t)ng) - 1.0);
    return ok;
}

// solver.cpp:389-405: the phase concentrations of solute q from the phase
// fractions (k, c: 3x3 column-major partition tables of solute q).
PF_HD void partition(const double ph[3], double C, const double *k, const double *c, double out[3]) {
    for (int a = 1; a <= 3; a++) {
        double t1 = 0., t2 = 0.;
        for (int b = 1; b <= 3; b++) {
            t1 += ph[b - 1] * k[(a - 1) + 3 * (b - 1)];
            t2 += ph[b - 1] * c[(a - 1) + 3 * (b - 1)];
        }
        out[a - 1] = (C - t2) / t1;
    }
}

}  // namespace pfinit
