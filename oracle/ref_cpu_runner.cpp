// ref_cpu_runner.cpp -- C entry points around the reference's own CPU time step.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_oracle.py (build_ref_cpu) compiles
// this file together with the UNMODIFIED reference sources
// zhubq/PhaseField C++-openmp-cuda/src/{phase_field,solver,thermo_data,
// thermo_functor,write_data}.cpp against the minimal Blitz++ stand-in in
// oracle/blitz_shim/, into oracle/_ref/libpfref_cpu.so.  The library then runs
// the reference's phase_field::Read_data (phase_field.cpp:27-230),
// phase_field::Update (phase_field.cpp:243-305, CPU branch) and
// phase_field::Write_data (write_data.cpp:3-40) on a state the caller supplies,
// so the oracle's restatement (pf_oracle.c) and the product's FP64 path can be
// checked against the reference's own code.
//
// The initial microstructure is supplied by the caller (the reference's
// Construct / Nucleate1in2 draw from an unseeded generator and are not built).
// The reference's GPU plug-in is replaced by stubs that report "no GPU"
// (gpu_solver.h:18-23), so Update takes its CPU diffusion branch.
#include <cstring>

#include "phase_field.h"

// gpu_solver.h declares these with C++ linkage; GPU_Init returning 0 keeps
// the reference on its CPU path (phase_field.cpp:229).
int GPU_Init(const int, const int, const int) { return 0; }
void GPU_Diffusion_solver(real *, real *, real *, real *, real *, int, int, int, real, real) {}
void GPU_Cleanup() {}

// Linked with --wrap=system: the reference's mkdir command string is a
// dangling pointer (phase_field.cpp:47-49), so no shell is ever started.
extern "C" int __wrap_system(const char *) { return 0; }

namespace {
struct Ref {
    phase_field F;
    int ix = 0, iy = 0, iz = 0;
};
}  // namespace

extern "C" {

// Parse the configuration file (and the thermodynamic file it names, which
// Read_data opens relative to the working directory).  Returns a handle.
void *pfr_create(const char *config_path) {
    Ref *r = new Ref();
    r->F.Read_data(config_path);
    r->ix = r->F.index_grain1.extent(1);
    r->iy = r->F.index_grain1.extent(2);
    r->iz = r->F.index_grain1.extent(3);
    return r;
}

void pfr_destroy(void *h) { delete static_cast<Ref *>(h); }

void pfr_dims(void *h, int out[3]) {
    Ref *r = static_cast<Ref *>(h);
    out[0] = r->ix;
    out[1] = r->iy;
    out[2] = r->iz;
}

// State in the reference layout (slot / phase fastest, then x, y, z):
// ids[6N], phi[6N], phase[3N], conc[3N], C[N].
void pfr_set_state(void *h, const int *ids, const double *phi, const double *phase, const double *conc,
                   const double *C) {
    Ref *r = static_cast<Ref *>(h);
    const size_t N = (size_t)r->ix * r->iy * r->iz;
    std::memcpy(r->F.index_grain1.data(), ids, 6 * N * sizeof(int));
    std::memcpy(r->F.value_grain1.data(), phi, 6 * N * sizeof(double));
    std::memcpy(r->F.value_phase.data(), phase, 3 * N * sizeof(double));
    std::memcpy(r->F.value_conc1.data(), conc, 3 * N * sizeof(double));
    std::memcpy(r->F.total_conc.data(), C, N * sizeof(double));
}

void pfr_get_state(void *h, int *ids, double *phi, double *phase, double *conc, double *C) {
    Ref *r = static_cast<Ref *>(h);
    const size_t N = (size_t)r->ix * r->iy * r->iz;
    std::memcpy(ids, r->F.index_grain1.data(), 6 * N * sizeof(int));
    std::memcpy(phi, r->F.value_grain1.data(), 6 * N * sizeof(double));
    std::memcpy(phase, r->F.value_phase.data(), 3 * N * sizeof(double));
    std::memcpy(conc, r->F.value_conc1.data(), 3 * N * sizeof(double));
    std::memcpy(C, r->F.total_conc.data(), N * sizeof(double));
}

// nsteps calls of phase_field::Update(false) (main.cpp:29-32 without output).
void pfr_update(void *h, int nsteps) {
    Ref *r = static_cast<Ref *>(h);
    for (int s = 0; s < nsteps; s++) r->F.Update(false);
}

// Only the phase sweep and its buffer swap: Update(true) returns before the
// diffusion sub-steps (phase_field.cpp:262).
void pfr_phase_only(void *h) { static_cast<Ref *>(h)->F.Update(true); }

double pfr_time(void *h) { return static_cast<Ref *>(h)->F.Time(); }
double pfr_temperature(void *h) { return static_cast<Ref *>(h)->F.Temperature(); }

// phase_field::Write_data(forced): appends to <directory>/fraction_time.txt
// and writes a VTI file when the configuration asks for one.
void pfr_write_data(void *h, int forced) { static_cast<Ref *>(h)->F.Write_data(forced != 0); }

}  // extern "C"
