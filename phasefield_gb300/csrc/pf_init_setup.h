// pf_init_setup.h -- host-side set-up of the seeded microstructure generator
// (internal C++; pf_init.cpp): seed coordinates and their bucket grids, kept
// in host vectors, and the pfinit::Setup that views them.
#pragma once
#include <vector>

#include "pf_init.h"
#include "pf_init_cell.h"

struct PfHostBuckets {
    int n[3] = {1, 1, 1};
    double edge[3] = {1, 1, 1};
    std::vector<int> start, items;  // CSR lists, ascending point index
    void build(const std::vector<double> &x, const std::vector<double> &y, const std::vector<double> &z,
               const int len[3], double target_edge);
    // A view whose lists live at start_ptr / items_ptr (host or device copies).
    pfinit::Buckets view(const int *start_ptr, const int *items_ptr) const;
};

struct PfInitHost {
    std::vector<double> gx, gy, gz, nx, ny, nz, px, py, pz;
    PfHostBuckets bgr, bnuc, bpar;
    pfinit::Setup S;  // views of the vectors above
};

// Draw the seeds of 'spec' for an ix x iy x iz domain and build their grids.
int pf_init_prepare(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec, PfInitHost &out,
                    const char **msg);
