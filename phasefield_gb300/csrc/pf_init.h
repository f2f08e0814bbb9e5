// pf_init.h -- the seeded synthetic microstructure generator (pf_init.cpp).
//
// Plain C interface on purpose: the same source is compiled into libpfstep
// (pf_init_microstructure*) and into the CPU oracle library, so the GPU
// product and the CPU baseline step exactly the same initial state.
#pragma once
#include <stdint.h>
#include "pfstep.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Planes [z0, z0 + nz) of the periodic ix x iy x iz domain described by spec
 * (cell (i, j, z0 + kk) stored at n = i + ix*(j + iy*kk)).  k and c are the
 * partition coefficients k[q][9], c[q][9] (3x3 column-major per solute) used to
 * fill conc (which may be NULL).  Every value depends only on the global cell,
 * so any slab equals the same planes of the whole domain.  Returns PF_OK or a
 * negative status with *msg set to a static description. */
int pf_init_state(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec, const double *k,
                  const double *c, int z0, int nz, int32_t *ids, double *phi, double *phase, double *conc,
                  double *C, const char **msg);

/* Coherent partners of the nuclei of spec (module_nucleation.f90:357-367,
 * nucleation in a grain boundary): at the cell nearest nucleus n, evaluated
 * without any nucleus, Or_num = min(2, ferrite grains there - 1) partners, the
 * largest ferrite ids first; partners[2n], partners[2n+1] (0: none). */
int pf_init_coherent_table(int ix, int iy, int iz, int nsol, double cutoff, const pf_init_spec *spec,
                           int32_t *partners, const char **msg);

#ifdef __cplusplus
}
#endif
