// pf_host.cpp -- host side of libpfstep: configuration and thermodynamic file
// parsers, per-step parameter evaluation and the reference output writers.
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

#include "pf_drag.h"
#endif
#include "pf_host.h"
#include "pf_init.h"

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
    m->thermo_model = 0;
    m->avg_carbon = 0;
    m->drag = 0;
    m->drag_binding = m->drag_vmax0 = m->drag_qsd = 0.;
    m->coherent = 0;
    m->coh_npp0 = 0;
    {
        std::string word;
        f >> word;
        if (word == "F90_POLYNOMIAL") {  // every coefficient is built in (pf_f90_thermo)
            m->thermo_model = 1;
            // Optional keywords on the following lines ('#' starts a comment line).
            std::string line;
            std::getline(f, line);
            while (std::getline(f, line)) {
                std::istringstream ls(line);
                std::string kw;
                if (!(ls >> kw) || kw[0] == '#') continue;
                if (kw == "AVERAGED_INTERFACE_CARBON") m->avg_carbon = 1;
                else if (kw == "SOLUTE_DRAG") {  // binding energy, v_max0, Q_sd (pre_process.f90:150-151)
                    if (!(ls >> m->drag_binding >> m->drag_vmax0 >> m->drag_qsd) || !(m->drag_vmax0 > 0.))
                        return pf_fail(PF_ERR_IO, "thermo file: SOLUTE_DRAG needs binding energy, v_max0 > 0, Q_sd");
                    m->drag = 1;
                } else if (kw == "COHERENT_MOBILITY") {  // last id of the initial ferrite class (Npp0)
                    if (!(ls >> m->coh_npp0) || m->coh_npp0 < 0)
                        return pf_fail(PF_ERR_IO, "thermo file: COHERENT_MOBILITY needs npp0 >= 0");
                    m->coherent = 1;
                } else return pf_fail(PF_ERR_IO, "thermo file: unknown keyword " + kw);
            }
            return PF_OK;
        }
        f.clear();
        f.seekg(0);
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

// The Fortran model's thermodynamics at temperature T (sparse.f90:797-923,
// Poly4/Diff_poly4 of util_func.f90:491-503), in the C++ model's terms: eq_ij
// = Ref_c_para(i,j), dcdT_ij = 1/Slope_para(i,j) (diagonal: eq 0, dcdT 1, the
// initial values of pre_process.f90:139-140), so the partition k_ij, c_ij that
// follows (thermo_data.cpp:34-40) equals the Fortran Partition_k_para(j,i),
// Partition_c_para(j,i); the driving force of an austenite pair is
// -Ratio_k_para(i,j) * (max(c_i, c_j) - Ref_c_para(2,1)) (sparse.f90:500-528,
// without the stored energy of deformed grains).  Evaluated in double (the
// Fortran source declares default REAL).
void pf_f90_thermo(double T, pf_step_params &p) {
    auto poly4 = [](double x, double a, double b, double c, double d) {
        return a * x + b * x * x + c * x * x * x + d * x * x * x * x;
    };
    auto dpoly4 = [](double x, double a, double b, double c, double d) {
        return a + 2 * b * x + 3 * c * x * x + 4 * d * x * x * x;
    };
    double ref12, ref21, dcdt12, dcdt21;
    if (T < 1086.52) {
        const double x = T - 273.15;
        ref12 = poly4(x, -8.309e-5, 0., 0., 0.) + 6.883e-2;
        ref21 = poly4(x, 2.607e-2, -6.58e-5, 3.984e-8, 0.) + 0.9115;
        dcdt12 = dpoly4(x, -8.309e-5, 0., 0., 0.);
        dcdt21 = dpoly4(x, 2.607e-2, -6.58e-5, 3.984e-8, 0.);
    } else {
        const double x = T - 1086.52;
        ref12 = poly4(x, -1.1428e-4, 0., 0., 0.);
        ref21 = poly4(x, -0.00325, 0., 0., 0.);
        dcdt12 = dpoly4(0., -1.1428e-4, -1.78883e-7, -3.66186e-10, 2.53049e-12);
        dcdt21 = dpoly4(0., -0.00325, 1.13712e-5, -2.88193e-8, 1.05482e-10);
    }
    for (int e = 0; e < 9; e++) {
        p.eq[e] = 0.;
        p.dcdT[e] = 1.;
        p.entropy[e] = 0.;
        p.df_ratio[e] = 0.;
    }
    // (1,2) and (1,3) take the ferrite line; (2,1), (3,1), (2,3), (3,2) the
    // austenite line (sparse.f90:882-889).
    p.eq[e3(1, 2)] = p.eq[e3(1, 3)] = ref12;
    p.dcdT[e3(1, 2)] = p.dcdT[e3(1, 3)] = dcdt12;
    p.eq[e3(2, 1)] = p.eq[e3(3, 1)] = p.eq[e3(2, 3)] = p.eq[e3(3, 2)] = ref21;
    p.dcdT[e3(2, 1)] = p.dcdT[e3(3, 1)] = p.dcdT[e3(2, 3)] = p.dcdT[e3(3, 2)] = dcdt21;
    const double x = T - 273.15;
    const double r12 = (0.000264 * x * x - 0.4466 * x + 243.4713) * 1.03e-12;  // sparse.f90:916-921
    p.df_ratio[e3(1, 2)] = r12;
    p.df_ratio[e3(2, 1)] = -r12;
    p.df_ratio[e3(3, 2)] = r12;
    p.df_ratio[e3(2, 3)] = -r12;
    p.df_ref = ref21;
    p.df_model = 1;
}

// PARAMETER_DRAG_PB (sparse.f90:958-1003) at temperature T, after
// pf_f90_thermo: v_max, E0, the heating / cooling segregation parameters of
// the three species (the bulk fractions Ux0 and the NPLE lines M_nple, N_nple
// of the Fortran), and the correction factors that make the zero-velocity
// drag equal the NPLE driving force |Ratio_k_para(2,1) (Ref_c_para(2,1) -
// Ref_c_nple(2,1))| (heating; Ref_c_nple_r for cooling, sparse.f90:870-880,
// zero below 1041.3 K where the Fortran leaves it at its initial value).
void pf_f90_drag(const pf_model &m, double T, pf_step_params &p) {
    const double x = T - 273.15;
    p.drag_vmax = m.drag_vmax0 * pf_exp(-m.drag_qsd / (8.314 * T));
    double M[3], Nn[3];
    M[0] = std::max(1.E-10, 3.9793e-5 * x - 2.3163e-2);
    M[1] = std::max(1.E-10, -2.928e-8 * (x * x) + 5.629e-5 * x - 2.35e-2);
    M[2] = std::max(1.E-10, 2.253e-8 * (x * x) - 4.255e-5 * x + 2.351e-2);
    Nn[0] = std::max(1.E-10, -3.818e-9 * (x * x * x) + 9.055e-6 * (x * x) - 7.408e-3 * x + 2.118);
    Nn[1] = std::max(1.E-10, -7.1227e-10 * (x * x * x) + 1.6307e-6 * (x * x) - 1.2584e-3 * x + 3.3166e-1);
    Nn[2] = 3.E-3;
    const double U[3] = {1.887e-2, 3.65e-3, 3.12e-3};
    double deh[3], dec[3];
    for (int i = 0; i < 3; i++) {
        deh[i] = -0.5 * pf_log(M[i] * (1. - U[i]) / (U[i] * (1. - M[i])));
        dec[i] = -0.5 * pf_log(Nn[i] * (1. - U[i]) / (U[i] * (1. - Nn[i])));
    }
    p.drag_ex0 = m.drag_binding / (8.314 * T);
    auto poly4 = [](double y, double a, double b, double c, double d) {
        return a * y + b * y * y + c * y * y * y + d * y * y * y * y;
    };
    const double nple21 = T < 1110.64 ? poly4(T - 1110.64, -3.3441e-3, 1.0406e-5, -5.6345e-8, 0.0)
                                      : poly4(T - 1110.64, -3.23154e-3, 0., 0., 0.);
    const double nple_r21 = T < 1041.3 ? 0. : -2.39e-3 * (T - 1041.3);
    const double ratio21 = p.df_ratio[e3(2, 1)], ref21 = p.eq[e3(2, 1)];
    const double driv_f[2] = {std::abs(ratio21 * (ref21 - nple21)), std::abs(ratio21 * (ref21 - nple_r21))};
    const double vmax = p.drag_vmax;
    double d0h = pf_solute_drag_pb(0., p.drag_ex0, deh[0], U[0], vmax, T) + pf_solute_drag_pb(0., 0., deh[1], U[1], vmax, T) +
                 pf_solute_drag_pb(0., 0., deh[2], U[2], vmax, T);
    double d0c = pf_solute_drag_pb(0., p.drag_ex0, dec[0], U[0], vmax, T) + pf_solute_drag_pb(0., 0., dec[1], U[1], vmax, T) +
                 pf_solute_drag_pb(0., 0., dec[2], U[2], vmax, T);
    p.drag_corr[0] = driv_f[0] / d0h;
    p.drag_corr[1] = driv_f[1] / d0c;
    p.drag_drag0[0] = pf_solute_drag_pb(0., p.drag_ex0, deh[0], U[0], vmax, T) * p.drag_corr[0];
    p.drag_drag0[1] = pf_solute_drag_pb(0., p.drag_ex0, dec[0], U[0], vmax, T) * p.drag_corr[1];
    p.drag_de_heat = deh[0];
    p.drag_de_cool = dec[0];
    p.drag_u0 = U[0];
    p.drag_model = 1;
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
    p.avg_range = (m.avg_carbon || m.coherent) ? m.i_intf + 1 : 0;  // sparse.f90:186
    p.avg_conc = m.avg_carbon ? 1 : 0;
    p.coh_model = m.coherent ? 1 : 0;
    p.coh_npp0 = m.coh_npp0;
    if (m.thermo_model == 1) {
        pf_f90_thermo(T, p);
        if (m.drag) pf_f90_drag(m, T, p);
    } else {
        // thermo_data.cpp:25-32 with linear_functor.h / quadratic_functor.h
        for (int j = 1; j <= 3; j++)
            for (int i = 1; i <= 3; i++) {
                const int e = e3(i, j);
                p.entropy[e] = m.ent_a[e] * T + m.ent_b[e];
                p.eq[e] = m.eq_a[e] * T * T + m.eq_b[e] * T + m.eq_c[e];
                p.dcdT[e] = (2 * m.eq_a[e]) * T + m.eq_b[e];
            }
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
    f.dfmax = p.df_model == 1 ? 1 : 0;
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            const int e = e3(i, j);
            const bool inter = std::abs(i - j) != 2;
            const double dm = p.pfm_dt * p.m[e];
            f.A[e] = inter ? (float)(dm * p.sigma[e] * p.factor1) : 0.f;
            f.B[e] = inter ? (float)(dm * p.sigma[e] * p.factor2) : 0.f;
            if (p.df_model == 1) {  // G * (max(c_i, c_j) - E)
                f.G[e] = (inter && i != j) ? (float)(-dm * p.factor3 * p.df_ratio[e]) : 0.f;
                f.E[e] = (float)p.df_ref;
            } else {                // G * (c_i - E)
                f.G[e] = (inter && i != j) ? (float)(dm * p.factor3 * p.entropy[e] / p.dcdT[e]) : 0.f;
                f.E[e] = (float)p.eq[e];
            }
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
// Seeded initial microstructure: the generator lives in pf_init.cpp (shared
// with the CPU baseline); here the partition at the start time is evaluated.
// ---------------------------------------------------------------------------
extern "C" int pf_init_microstructure(const pf_model *model, const pf_init_spec *spec, double time,
                                      int32_t *ids, double *phi, double *phase, double *conc, double *C) {
    if (!model || !spec || !ids || !phi || !phase || !C) return pf_fail(PF_ERR_ARG, "pf_init_microstructure: null argument");
    return pf_init_microstructure_box(model, spec, time, 0, model->iz, ids, phi, phase, conc, C);
}

extern "C" int pf_init_microstructure_box(const pf_model *model, const pf_init_spec *spec, double time, int z0,
                                          int nz, int32_t *ids, double *phi, double *phase, double *conc,
                                          double *C) {
    if (!model || !spec || !ids || !phi || !phase || !C)
        return pf_fail(PF_ERR_ARG, "pf_init_microstructure_box: null argument");
    pf_step_params P;
    pf_compute_params(*model, time, P);
    const char *msg = nullptr;
    const int st = pf_init_state(model->ix, model->iy, model->iz, model->nsol, model->cutoff, spec, &P.k[0][0],
                                 &P.c[0][0], z0, nz, ids, phi, phase, conc, C, &msg);
    return st == PF_OK ? PF_OK : pf_fail(st, std::string("pf_init_microstructure: ") + (msg ? msg : "failed"));
}

extern "C" int pf_init_coherent(const pf_model *model, const pf_init_spec *spec, int32_t *partners) {
    if (!model || !spec) return pf_fail(PF_ERR_ARG, "pf_init_coherent: null argument");
    const char *msg = nullptr;
    const int st = pf_init_coherent_table(model->ix, model->iy, model->iz, model->nsol, model->cutoff, spec, partners,
                                          &msg);
    return st == PF_OK ? PF_OK : pf_fail(st, std::string("pf_init_coherent: ") + (msg ? msg : "failed"));
}
