// pfm -- command-line driver over libpfstep, the counterpart of the reference's
// main (zhubq/PhaseField, C++-openmp-cuda/src/main.cpp:10-43):
//
//   pfm config.txt [--fp32] [--seed S] [--grains G] [--nuclei M] [--radius R]
//                  [--particles P] [--prad r] [--width W] [--noise A] [--steps K]
//
// Reads the reference configuration and thermodynamic files, builds a seeded
// initial microstructure (the reference's unseeded Voronoi + nucleation step is
// replaced), writes the initial statistics, then loops Update/Write_data until
// the end of the temperature path (or K steps) and prints the wall time.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>
#include "pfstep.h"

static int check(int st, const char *what) {
    if (st != PF_OK) {
        std::fprintf(stderr, "%s: %s (%s)\n", what, pf_status_string(st), pf_last_error());
        std::exit(1);
    }
    return st;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::printf("PROGRAM ARGUMENT IS NOT ENOUGH.\n");
        return 0;
    }
    pf_model m;
    check(pf_model_read(argv[1], &m), "read config");
    pf_init_spec spec;
    std::memset(&spec, 0, sizeof(spec));
    spec.seed = 0;
    spec.n_grains = m.num_grain[0] > 0 ? m.num_grain[0] : 20;
    spec.n_nuclei = (int)m.num_nuclei;
    spec.nucleus_radius = 3.0;
    spec.width = m.i_intf;
    spec.C0[0] = m.init_conc[0];
    spec.C0[1] = 1.5;
    spec.max_slots = 4;
    int prec = PF_PREC_FP64;
    long long max_steps = -1;
    for (int a = 2; a < argc; a++) {
        std::string s = argv[a];
        auto nxt = [&]() { return a + 1 < argc ? argv[++a] : (char *)"0"; };
        if (s == "--fp32") prec = PF_PREC_FP32C;
        else if (s == "--seed") spec.seed = std::strtoull(nxt(), nullptr, 10);
        else if (s == "--grains") spec.n_grains = std::atoi(nxt());
        else if (s == "--nuclei") spec.n_nuclei = std::atoi(nxt());
        else if (s == "--radius") spec.nucleus_radius = std::atof(nxt());
        else if (s == "--particles") spec.n_particles = std::atoi(nxt());
        else if (s == "--prad") spec.particle_radius = std::atof(nxt());
        else if (s == "--width") spec.width = std::atof(nxt());
        else if (s == "--noise") spec.C_noise[0] = std::atof(nxt());
        else if (s == "--steps") max_steps = std::atoll(nxt());
    }
    const long long N = (long long)m.ix * m.iy * m.iz;
    std::vector<int32_t> ids(6 * N);
    std::vector<double> phi(6 * N), phase(3 * N), conc(3 * N * m.nsol), C(N * m.nsol);
    double time = m.T_time[0];
    check(pf_init_microstructure(&m, &spec, time, ids.data(), phi.data(), phase.data(), conc.data(), C.data()),
          "initial microstructure");
    mkdir(m.directory, 0755);
    pf_ctx *ctx = nullptr;
    check(pf_create(&m, prec, &ctx), "create context");
    check(pf_upload_state(ctx, ids.data(), phi.data(), phase.data(), conc.data(), C.data(), time), "upload");
    if (m.coherent && spec.n_nuclei > 0) {  // the Fortran model's coherent partners, by its boundary-nucleation rule
        std::vector<int32_t> partners(2 * (size_t)spec.n_nuclei);
        check(pf_init_coherent(&m, &spec, partners.data()), "coherent partners");
        check(pf_set_coherent_grains(ctx, partners.data(), spec.n_nuclei), "coherent partners");
    }
    check(pf_use_graph(ctx, 0), "graph");
    int written = 0;
    check(pf_write_data(ctx, m.directory, 1, &written), "write data");
    const double end_time = m.T_time[m.nT - 1];
    auto t0 = std::chrono::steady_clock::now();
    long long steps = 0;
    while (time < end_time && (max_steps < 0 || steps < max_steps)) {
        check(pf_step(ctx, 1), "step");
        check(pf_get_time(ctx, &time), "time");
        check(pf_write_data(ctx, m.directory, 0, &written), "write data");
        steps++;
    }
    check(pf_synchronize(ctx), "synchronize");
    auto t1 = std::chrono::steady_clock::now();
    std::printf("SIMULATION IS FINISHED.\n\n");
    std::printf("steps: %lld  cells: %lld\n", steps, N);
    std::printf("Total Physical Time (s): %g\n", std::chrono::duration<double>(t1 - t0).count());
    pf_destroy(ctx);
    return 0;
}
