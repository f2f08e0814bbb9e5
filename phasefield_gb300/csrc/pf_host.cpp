// pf_host.cpp -- host side of libpfstep: configuration and thermodynamic file
// parsers, per-step parameter evaluation, the seeded initial microstructure and
// the reference output writers.
//
// Compiled with -ffp-contract=off: the per-step parameters must come out
// bit-identical to the reference's host arithmetic (no fused multiply-add).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "pf_host.h"

namespace {
thread_local std::string g_last_error;
constexpr double kPi = 3.1415926;  // constant.h:7 (the reference's truncated pi)
constexpr double kR = 8.314;       // constant.h:8
inline int e3(int i, int j) { return (i - 1) + 3 * (j - 1); }
}  // namespace

int pf_fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

extern "C" const char *pf_last_error(void) { return g_last_error.c_str(); }

extern "C" int pf_abi_sizes(long long out[3]) {
    if (!out) return pf_fail(PF_ERR_ARG, "pf_abi_sizes: null argument");
    out[0] = (long long)sizeof(pf_model);
    out[1] = (long long)sizeof(pf_step_params);
    out[2] = (long long)sizeof(pf_init_spec);
    return PF_OK;
}

extern "C" const char *pf_status_string(int s) {
    switch (s) {
        case PF_OK: return "ok";
        case PF_ERR_ARG: return "invalid argument";
        case PF_ERR_NOMEM: return "out of memory";
        case PF_ERR_CUDA: return "CUDA error";
        case PF_ERR_TIMEOUT: return "device wait timed out";
        case PF_ERR_NONFINITE: return "non-finite value in state";
        case PF_ERR_IO: return "file error";
        case PF_ERR_NODEV: return "no CUDA device";
        case PF_ERR_RANGE: return "value out of range";
        case PF_ERR_DRIFT: return "solute total drifted";
        default: return "unknown status";
    }
}

// ---------------------------------------------------------------------------
// Thermodynamic file: thermo_functor.cpp:11-53.  Three header lines, three
// entropy lines "i j a b" (the (j,i) entry gets -a,-b), four skipped lines, six
// NPLE1 lines "i j a b c", two skipped, six NPLE2 lines, two skipped, six PARA
// lines (equilibrium a,b,c; dc/dT = 2a*T + b).
// ---------------------------------------------------------------------------
extern "C" int pf_thermo_read(const char *path, pf_model *m) {
    if (!path || !m) return pf_fail(PF_ERR_ARG, "pf_thermo_read: null argument");
    std::ifstream f(path);
    if (!f.is_open()) return pf_fail(PF_ERR_IO, std::string("cannot open thermo file ") + path);
    for (int e = 0; e < 9; e++) {
        m->ent_a[e] = m->ent_b[e] = 0.;
        m->nple1_a[e] = m->nple1_b[e] = m->nple1_c[e] = 0.;
        m->nple2_a[e] = m->nple2_b[e] = m->nple2_c[e] = 0.;
        m->eq_a[e] = m->eq_b[e] = m->eq_c[e] = 0.;
    }
    for (int t = 0; t < 3; t++) f.ignore(1000, '\n');
    int i, j;
    double a, b, c;
    auto bad = [&](int i_, int j_) { return i_ < 1 || i_ > 3 || j_ < 1 || j_ > 3; };
    for (int k = 0; k < 3; k++) {
        f >> i >> j >> a >> b;
        if (!f || bad(i, j)) return pf_fail(PF_ERR_IO, "thermo file: bad entropy line");
        m->ent_a[e3(i, j)] = a; m->ent_b[e3(i, j)] = b;
        m->ent_a[e3(j, i)] = -a; m->ent_b[e3(j, i)] = -b;
    }
    for (int t = 0; t < 4; t++) f.ignore(1000, '\n');
    for (int k = 0; k < 6; k++) {
        f >> i >> j >> a >> b >> c;
        if (!f || bad(i, j)) return pf_fail(PF_ERR_IO, "thermo file: bad NPLE1 line");
        m->nple1_a[e3(i, j)] = a; m->nple1_b[e3(i, j)] = b; m->nple1_c[e3(i, j)] = c;
    }
    for (int t = 0; t < 2; t++) f.ignore(1000, '\n');
    for (int k = 0; k < 6; k++) {
        f >> i >> j >> a >> b >> c;
        if (!f || bad(i, j)) return pf_fail(PF_ERR_IO, "thermo file: bad NPLE2 line");
        m->nple2_a[e3(i, j)] = a; m->nple2_b[e3(i, j)] = b; m->nple2_c[e3(i, j)] = c;
    }
    for (int t = 0; t < 2; t++) f.ignore(1000, '\n');
    for (int k = 0; k < 6; k++) {
        f >> i >> j >> a >> b >> c;
        if (!f || bad(i, j)) return pf_fail(PF_ERR_IO, "thermo file: bad PARA line");
        m->eq_a[e3(i, j)] = a; m->eq_b[e3(i, j)] = b; m->eq_c[e3(i, j)] = c;
    }
    return PF_OK;
}

// ---------------------------------------------------------------------------
// Configuration file: phase_field.cpp:166-330.  Every value is preceded by a
// prompt line that is skipped with ignore(1000,'\n'); the field order is the
// drop-in contract.  After the GPU flag an optional extension (no reference
// counterpart) adds Mn as a second solute:
//   prompt / "D0 Q" for each of the three phases / prompt / "r1 r2 r3"
// ---------------------------------------------------------------------------
extern "C" int pf_model_read(const char *config_path, pf_model *m) {
    if (!config_path || !m) return pf_fail(PF_ERR_ARG, "pf_model_read: null argument");
    std::memset(m, 0, sizeof(*m));
    std::ifstream in(config_path);
    if (!in.is_open()) return pf_fail(PF_ERR_IO, std::string("cannot open config file ") + config_path);
    auto skip = [&](int n) { for (int t = 0; t < n; t++) in.ignore(1000, '\n'); };
    auto need = [&](const char *what) -> int {
        if (!in) return pf_fail(PF_ERR_IO, std::string("config file: cannot read ") + what);
        return PF_OK;
    };
    std::string directory;
    skip(1);
    std::getline(in, directory, '\n');
    std::snprintf(m->directory, sizeof(m->directory), "%s", directory.c_str());
    skip(3);
    in >> m->ix >> m->iy >> m->iz;
    if (need("domain size")) return PF_ERR_IO;
    skip(2);
    in >> m->dx;
    if (need("cell size")) return PF_ERR_IO;
    skip(2);
    in >> m->i_intf;
    if (need("interface thickness")) return PF_ERR_IO;
    skip(2);
    in >> m->cutoff;
    if (need("cutoff")) return PF_ERR_IO;
    skip(2);
    for (int i = 0; i < 3; i++) in >> m->num_grain[i];
    if (need("grain numbers")) return PF_ERR_IO;
    skip(2);
    for (int i = 0; i < 3; i++) in >> m->phase_fraction[i];
    if (need("phase fractions")) return PF_ERR_IO;
    skip(2);
    for (int i = 0; i < 3; i++) in >> m->init_conc[i];
    if (need("initial concentrations")) return PF_ERR_IO;
    skip(2);
    in >> m->nT;
    if (need("temperature points") || m->nT < 1 || m->nT > PF_MAXT)
        return pf_fail(PF_ERR_IO, "config file: bad number of temperature points");
    for (int i = 0; i < m->nT; i++) in >> m->T_time[i] >> m->T_temp[i];
    if (need("temperature path")) return PF_ERR_IO;
    skip(2);
    in >> m->reduction;
    skip(2);
    in >> m->num_init_iteration;
    skip(2);
    in >> m->timestep_output;
    skip(2);
    bool micro = false;
    in >> micro;
    m->micro_out = micro ? 1 : 0;
    if (need("output settings")) return PF_ERR_IO;
    skip(1);
    skip(1);
    in >> m->num_nuclei;
    if (need("number of nuclei")) return PF_ERR_IO;
    for (int i = 1; i <= 3; i++)
        for (int j = i; j <= 3; j++) {
            skip(2);
            in >> m->m0[e3(i, j)] >> m->mQ[e3(i, j)];
            m->m0[e3(j, i)] = m->m0[e3(i, j)];
            m->mQ[e3(j, i)] = m->mQ[e3(i, j)];
        }
    if (need("interface mobilities")) return PF_ERR_IO;
    for (int i = 1; i <= 3; i++)
        for (int j = i; j <= 3; j++) {
            skip(2);
            in >> m->sigma[e3(i, j)];
            m->sigma[e3(j, i)] = m->sigma[e3(i, j)];
        }
    if (need("interface energies")) return PF_ERR_IO;
    for (int i = 0; i < 3; i++) {
        skip(2);
        in >> m->D0[0][i] >> m->DQ[0][i];
    }
    if (need("diffusivities")) return PF_ERR_IO;
    skip(2);
    std::string thermo;
    std::getline(in, thermo, '\n');
    std::snprintf(m->thermo_file, sizeof(m->thermo_file), "%s", thermo.c_str());
    skip(1);
    in >> m->gpu_flag;
    if (need("GPU flag")) return PF_ERR_IO;
    // Optional Mn extension.
    m->nsol = 1;
    m->mn_ratio[0] = m->mn_ratio[1] = m->mn_ratio[2] = 1.;
    {
        double d0[3], dq[3], r[3];
        bool ok = true;
        for (int i = 0; i < 3 && ok; i++) {
            skip(2);
            in >> d0[i] >> dq[i];
            ok = bool(in);
        }
        if (ok) {
            skip(2);
            in >> r[0] >> r[1] >> r[2];
            ok = bool(in);
        }
        if (ok) {
            m->nsol = 2;
            for (int i = 0; i < 3; i++) {
                m->D0[1][i] = d0[i];
                m->DQ[1][i] = dq[i];
                m->mn_ratio[i] = r[i];
            }
        }
    }
    if (m->ix < 1 || m->iy < 1 || m->iz < 1) return pf_fail(PF_ERR_ARG, "config file: bad domain size");
    // The thermo file name is relative to the working directory in the
    // reference (thermo_functor.cpp:13); fall back to the config's directory.
    int st = PF_ERR_IO;
    {
        std::ifstream probe(thermo);
        if (probe.is_open()) st = pf_thermo_read(thermo.c_str(), m);
    }
    if (st != PF_OK) {
        std::string cp(config_path);
        size_t slash = cp.find_last_of('/');
        std::string alt = (slash == std::string::npos ? std::string() : cp.substr(0, slash + 1)) + thermo;
        st = pf_thermo_read(alt.c_str(), m);
    }
    return st;
}

// ---------------------------------------------------------------------------
// Per-step parameters.
// ---------------------------------------------------------------------------
static double pf_temperature(const pf_model &m, double t) {
    // phase_field.cpp:232-242.  Outside the path the reference reads an
    // uninitialised value; here the last temperature of the path is used.
    double Temp = m.T_temp[m.nT - 1];
    for (int i = 0; i < m.nT - 1; i++)
        if (t >= m.T_time[i] && t < m.T_time[i + 1])
            Temp = (m.T_temp[i + 1] - m.T_temp[i]) / (m.T_time[i + 1] - m.T_time[i]) * (t - m.T_time[i]) +
                   m.T_temp[i];
    return Temp;
}

void pf_compute_params(const pf_model &m, double time, pf_step_params &p) {
    std::memset(&p, 0, sizeof(p));
    p.ix = m.ix; p.iy = m.iy; p.iz = m.iz;
    p.N = (long long)m.ix * m.iy * m.iz;
    p.nsol = m.nsol;
    double dims = 3;  // phase_field.cpp:354-360
    if (m.iz == 1) dims -= 1;
    if (m.iy == 1) dims -= 1;
    p.nnb = (int)(2 * dims);
    p.time = time;
    p.dx = m.dx;
    p.cutoff = m.cutoff;
    p.eta = m.dx * m.i_intf;
    const double T = pf_temperature(m, time);
    p.T = T;
    // phase_field.cpp:309-312
    const double RT = kR * T;
    double maxms = -INFINITY, maxD = -INFINITY;
    for (int e = 0; e < 9; e++) {
        p.m[e] = m.m0[e] * std::exp(-m.mQ[e] / RT);
        p.sigma[e] = m.sigma[e];
        const double ms = p.m[e] * m.sigma[e];
        if (ms > maxms) maxms = ms;
    }
    for (int q = 0; q < m.nsol; q++)
        for (int ph = 0; ph < 3; ph++) {
            p.D[q][ph] = m.D0[q][ph] * std::exp(-m.DQ[q][ph] / RT);
            if (p.D[q][ph] > maxD) maxD = p.D[q][ph];
        }
    p.pfm_dt = m.dx * m.dx / dims * 0.2 / maxms;
    p.diff_dt = m.dx * m.dx / maxD / dims * 0.2;
    // thermo_data.cpp:25-32 with linear_functor.h / quadratic_functor.h
    for (int j = 1; j <= 3; j++)
        for (int i = 1; i <= 3; i++) {
            const int e = e3(i, j);
            p.entropy[e] = m.ent_a[e] * T + m.ent_b[e];
            p.eq[e] = m.eq_a[e] * T * T + m.eq_b[e] * T + m.eq_c[e];
            p.dcdT[e] = (2 * m.eq_a[e]) * T + m.eq_b[e];
        }
    // thermo_data.cpp:34-40
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            if (i == j) p.dcdT[e3(i, j)] = 1.;
            p.k[0][e3(i, j)] = p.dcdT[e3(j, i)] / p.dcdT[e3(i, j)];
            p.c[0][e3(i, j)] = p.eq[e3(j, i)] - p.k[0][e3(i, j)] * p.eq[e3(i, j)];
        }
    // Mn: c_p proportional to mn_ratio[p].  Partitioning (solver.cpp:389-405)
    // reads k_ij as c_j = k_ij*c_i + c_ij, hence k_ij = r_j/r_i, c_ij = 0.
    if (m.nsol > 1)
        for (int i = 1; i <= 3; i++)
            for (int j = 1; j <= 3; j++) {
                p.k[1][e3(i, j)] = m.mn_ratio[j - 1] / m.mn_ratio[i - 1];
                p.c[1][e3(i, j)] = 0.;
            }
    // phase_field.cpp:247-248
    const int n = (int)std::ceil(p.pfm_dt / p.diff_dt);
    p.n_sub = n > 1 ? n : 1;
    p.dt_sub = p.pfm_dt / p.n_sub;
    // solver.cpp:226-228, :366
    p.factor1 = 1. / (m.dx * m.dx);
    p.factor2 = kPi * kPi / (2. * p.eta * p.eta);
    p.factor3 = kPi / p.eta;
    p.coef_diff = p.dt_sub / (m.dx * m.dx);
}

extern "C" int pf_params_at(const pf_model *m, double time, pf_step_params *out) {
    if (!m || !out) return pf_fail(PF_ERR_ARG, "pf_params_at: null argument");
    if (m->nT < 1 || m->nsol < 1 || m->nsol > 2) return pf_fail(PF_ERR_ARG, "pf_params_at: bad model");
    pf_compute_params(*m, time, *out);
    return PF_OK;
}

void pf_fold_f32(const pf_step_params &p, int b1, int b2, pf_f32_params &f) {
    std::memset(&f, 0, sizeof(f));
    f.ix = p.ix; f.iy = p.iy; f.iz = p.iz; f.nnb = p.nnb; f.nsol = p.nsol; f.n_sub = p.n_sub;
    f.N = p.N;
    f.b1 = b1; f.b2 = b2;
    f.cutoff = (float)p.cutoff;
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            const int e = e3(i, j);
            const bool inter = std::abs(i - j) != 2;
            const double dm = p.pfm_dt * p.m[e];
            f.A[e] = inter ? (float)(dm * p.sigma[e] * p.factor1) : 0.f;
            f.B[e] = inter ? (float)(dm * p.sigma[e] * p.factor2) : 0.f;
            f.G[e] = (inter && i != j) ? (float)(dm * p.factor3 * p.entropy[e] / p.dcdT[e]) : 0.f;
            f.E[e] = (float)p.eq[e];
        }
    for (int q = 0; q < p.nsol; q++) {
        for (int ph = 0; ph < 3; ph++) f.D[q][ph] = (float)(p.D[q][ph] * p.coef_diff);
        for (int e = 0; e < 9; e++) {
            f.k[q][e] = (float)p.k[q][e];
            f.c[q][e] = (float)p.c[q][e];
        }
        // Separable partition?  a_j = k_1j (a_1 = 1); require c_ij = 0 and
        // k_ij = a_j/a_i to 1e-12 relative.
        bool sep = true;
        double a[3];
        for (int j = 1; j <= 3; j++) a[j - 1] = p.k[q][e3(1, j)];
        for (int i = 1; i <= 3 && sep; i++)
            for (int j = 1; j <= 3 && sep; j++) {
                const double kij = p.k[q][e3(i, j)], want = a[j - 1] / a[i - 1];
                if (p.c[q][e3(i, j)] != 0.0 || !(std::abs(kij - want) <= 1e-12 * std::abs(want)) || a[i - 1] <= 0.0)
                    sep = false;
            }
        f.sep[q] = sep ? 1 : 0;
        for (int j = 0; j < 3; j++) f.a[q][j] = sep ? (float)a[j] : 0.f;
    }
}

// ---------------------------------------------------------------------------
// Output: write_data.cpp:3-82.
// ---------------------------------------------------------------------------
bool pf_output_due(double time, double timestep_output, double pfm_dt, double temperature,
                   double last_temperature) {
    return (std::abs(time - timestep_output * std::floor(time / timestep_output + 0.5)) < 0.5 * pfm_dt) ||
           std::abs(temperature - last_temperature) > 10.;
}

std::string pf_format_fraction_line(double time, double temperature, const double frac3[3],
                                    double deformed) {
    std::ostringstream k;
    k << std::setw(8) << std::setprecision(4) << time << " " << temperature << " ";
    for (int i = 0; i < 3; i++) k << std::setprecision(4) << (float)frac3[i] << " ";
    k << deformed << "\n";
    return k.str();
}

extern "C" int pf_write_vti(const char *path, int ix, int iy, int iz, double dx, const int32_t *ids,
                            const double *C) {
    if (!path || !ids || !C || ix < 1 || iy < 1 || iz < 1) return pf_fail(PF_ERR_ARG, "pf_write_vti: bad argument");
    std::ofstream file(path);
    if (!file.is_open()) return pf_fail(PF_ERR_IO, std::string("cannot write ") + path);
    file << "<?xml version=\"1.0\"?>" << '\n'
         << "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">" << "\n"
         << "<ImageData WholeExtent=\"" << 1 << ' ' << ix << ' ' << 1 << ' ' << iy << ' ' << 1 << ' ' << iz << '"'
         << " Origin=" << "\"0 0 0\" Spacing=\"" << dx << ' ' << dx << ' ' << dx << "\">" << std::endl;
    file << "<Piece Extent=\"" << 1 << ' ' << ix << ' ' << 1 << ' ' << iy << ' ' << 1 << ' ' << iz << "\">"
         << std::endl;
    file << "<PointData Scalars=\"energy\">" << std::endl;
    file << "<DataArray type=\"Int32\" Name=\"korn\" format=\"ascii\">" << std::endl;
    const long long N = (long long)ix * iy * iz;
    for (long long n = 0; n < N; n++) {
        // write_data.cpp:60-64: 0 in interfaces (second slot occupied), else the phase.
        if (ids[6 * n + 1] > 0) file << 0 << " ";
        else {
            const int g = ids[6 * n];
            const int ph = g == 0 ? 0 : (g / PF_MAXGRAIN_PER_PHASE > 0 ? g / PF_MAXGRAIN_PER_PHASE : 1);
            file << ph << " ";
        }
    }
    file << "\n</DataArray>" << std::endl;
    file << "<DataArray type=\"Float32\" Name=\"conc\" format=\"ascii\">" << std::endl;
    for (long long n = 0; n < N; n++) file << std::setprecision(3) << C[n] << " ";
    file << "</DataArray>" << std::endl
         << "</PointData>" << std::endl
         << "</Piece>" << std::endl
         << "</ImageData>" << std::endl
         << "</VTKFile>" << std::endl;
    return file ? PF_OK : pf_fail(PF_ERR_IO, std::string("write failed: ") + path);
}

// ---------------------------------------------------------------------------
// Seeded initial microstructure.
// ---------------------------------------------------------------------------
namespace {

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

// Periodic bucket grid over sphere centres with bucket edge >= range, so a
// cell only needs its own and the adjacent buckets.
struct Buckets {
    int n[3] = {1, 1, 1};
    double edge[3] = {1, 1, 1};
    std::vector<std::vector<int>> items;
    void build(const std::vector<double> &x, const std::vector<double> &y, const std::vector<double> &z,
               const int len[3], double range) {
        for (int d = 0; d < 3; d++) {
            n[d] = std::max(1, (int)std::floor(len[d] / std::max(range, 1.0)));
            edge[d] = (double)len[d] / n[d];
        }
        items.assign((size_t)n[0] * n[1] * n[2], {});
        for (size_t g = 0; g < x.size(); g++) {
            int b[3] = {std::min(n[0] - 1, (int)(x[g] / edge[0])), std::min(n[1] - 1, (int)(y[g] / edge[1])),
                        std::min(n[2] - 1, (int)(z[g] / edge[2]))};
            items[b[0] + (size_t)n[0] * (b[1] + (size_t)n[1] * b[2])].push_back((int)g);
        }
    }
    // Candidate indices near point p, ascending (application order is the index order).
    void near(const double p[3], std::vector<int> &out) const {
        out.clear();
        int lists[3][3], cnt[3];
        for (int d = 0; d < 3; d++) {
            const int c = std::min(n[d] - 1, (int)(p[d] / edge[d]));
            if (n[d] >= 3) {
                lists[d][0] = (c + n[d] - 1) % n[d]; lists[d][1] = c; lists[d][2] = (c + 1) % n[d];
                cnt[d] = 3;
            } else {
                for (int t = 0; t < n[d]; t++) lists[d][t] = t;
                cnt[d] = n[d];
            }
        }
        for (int a = 0; a < cnt[0]; a++)
            for (int b = 0; b < cnt[1]; b++)
                for (int c = 0; c < cnt[2]; c++) {
                    const auto &v = items[lists[0][a] + (size_t)n[0] * (lists[1][b] + (size_t)n[1] * lists[2][c])];
                    out.insert(out.end(), v.begin(), v.end());
                }
        std::sort(out.begin(), out.end());
    }
};

}  // namespace

extern "C" int pf_init_microstructure(const pf_model *model, const pf_init_spec *spec, double time,
                                      int32_t *ids, double *phi, double *phase, double *conc, double *C) {
    if (!model || !spec || !ids || !phi || !phase || !C) return pf_fail(PF_ERR_ARG, "pf_init_microstructure: null argument");
    const pf_model &m = *model;
    const int ix = m.ix, iy = m.iy, iz = m.iz;
    const long long N = (long long)ix * iy * iz;
    const int K = spec->max_slots < 1 ? 1 : (spec->max_slots > 6 ? 6 : spec->max_slots);
    if (spec->n_grains < 1) return pf_fail(PF_ERR_ARG, "pf_init_microstructure: need at least one grain");
    if (spec->n_grains >= PF_MAXGRAIN_PER_PHASE || spec->n_nuclei >= PF_MAXGRAIN_PER_PHASE ||
        spec->n_particles >= PF_MAXGRAIN_PER_PHASE)
        return pf_fail(PF_ERR_RANGE, "pf_init_microstructure: too many grains");
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
    pf_step_params P;
    pf_compute_params(m, time, P);
    const uint64_t seed = spec->seed;
    const bool zflat = (iz == 1), yflat = (iy == 1);
    const long long nsol = m.nsol;
    const int len[3] = {ix, iy, iz};
    Buckets bnuc, bpar;
    bnuc.build(nx, ny, nz, len, spec->nucleus_radius + 3.0 / kk + 1.0);
    bpar.build(px, py, pz, len, spec->particle_radius + 3.0 / kk + 1.0);

#pragma omp parallel
    {
    std::vector<int> near;
    near.reserve(256);
#pragma omp for schedule(dynamic, 256)
    for (long long n = 0; n < N; n++) {
        const int i = (int)(n % ix);
        const int j = (int)((n / ix) % iy);
        const int k = (int)(n / ((long long)ix * iy));
        const double x = i, y = j, z = k;
        // Ferrite matrix: periodic Voronoi with a tanh profile across each
        // bisector.  Keep the few nearest seeds.
        constexpr int KN = 6;
        int best[KN];
        double bd2[KN], bvx[KN], bvy[KN], bvz[KN];
        int nb = 0;
        for (int g = 0; g < spec->n_grains; g++) {
            const double vx = mi(gx[g] - x, ix), vy = yflat ? 0 : mi(gy[g] - y, iy), vz = zflat ? 0 : mi(gz[g] - z, iz);
            const double d2 = vx * vx + vy * vy + vz * vz;
            if (nb < KN || d2 < bd2[nb - 1]) {
                int pos = nb < KN ? nb++ : KN - 1;
                while (pos > 0 && bd2[pos - 1] > d2) {
                    best[pos] = best[pos - 1]; bd2[pos] = bd2[pos - 1];
                    bvx[pos] = bvx[pos - 1]; bvy[pos] = bvy[pos - 1]; bvz[pos] = bvz[pos - 1];
                    pos--;
                }
                best[pos] = g; bd2[pos] = d2; bvx[pos] = vx; bvy[pos] = vy; bvz[pos] = vz;
            }
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
            bk.near(p, near);
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
            if (cand[a].w > 10.0 * m.cutoff) { keep++; sum += cand[a].w; }
        double ph[3] = {0, 0, 0};
        for (int a = 0; a < 6; a++) {
            if (a < keep) {
                const double v = cand[a].w / sum;
                ids[6 * n + a] = cand[a].id;
                phi[6 * n + a] = v;
                ph[cand[a].id / PF_MAXGRAIN_PER_PHASE - 1] += v;
            } else {
                ids[6 * n + a] = 0;
                phi[6 * n + a] = 0.0;
            }
        }
        for (int p = 0; p < 3; p++) phase[3 * n + p] = ph[p];
        for (long long q = 0; q < nsol; q++) {
            const double c = spec->C0[q] + spec->C_noise[q] * (2.0 * u01_at(seed, 1 + q, (uint64_t)n) - 1.0);
            C[q * N + n] = c;
            if (conc) {
                // solver.cpp:389-405
                for (int a = 1; a <= 3; a++) {
                    double t1 = 0., t2 = 0.;
                    for (int b = 1; b <= 3; b++) {
                        t1 += ph[b - 1] * P.k[q][e3(a, b)];
                        t2 += ph[b - 1] * P.c[q][e3(a, b)];
                    }
                    conc[q * 3 * N + 3 * n + a - 1] = (c - t2) / t1;
                }
            }
        }
    }
    }  // omp parallel
    return PF_OK;
}
