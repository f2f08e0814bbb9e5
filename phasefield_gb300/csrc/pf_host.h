// pf_host.h -- host-side helpers of libpfstep (internal).
#pragma once
#include <string>
#include "pf_types.h"

// Record an error message for pf_last_error() and return 'status'.
int pf_fail(int status, const std::string &msg);
// Per-step parameters (phase_field.cpp:307-315, thermo_data.cpp:24-41,
// phase_field.cpp:247-248); 'time' is the time at the start of the step.
void pf_compute_params(const pf_model &m, double time, pf_step_params &p);
// The Fortran model's thermodynamics (thermo_model 1) at temperature T:
// eq, dcdT, entropy, df_model, df_ratio, df_ref of p.
void pf_f90_thermo(double T, pf_step_params &p);
// Fold FP64 step parameters into the FP32 kernels' block.
struct pf_f32_map;
void pf_fold_f32(const pf_step_params &p, int b1, int b2, pf_f32_params &f);
// The kinetics line of write_data.cpp:9-18 for the given statistics.
std::string pf_format_fraction_line(double time, double temperature, const double frac3[3],
                                    double deformed);
// write_data.cpp:3-8 output condition.
bool pf_output_due(double time, double timestep_output, double pfm_dt, double temperature,
                   double last_temperature);
