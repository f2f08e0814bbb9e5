// pf_output.h -- asynchronous microstructure writer of a context (pf_output.cu, internal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

struct pf_out;
pf_out *pf_out_create();
// Joins a write in flight and frees the buffers.
void pf_out_destroy(pf_out *o);
// Waits for the write in flight (if any); its status.
int pf_out_wait(pf_out *o);
// Form the fields on 'stream' from the reference layout (ids[6N], C[N]) or the
// compact layout (gid, sol, local-id phase bounds b1, b2), then copy and
// write the pieces asynchronously.  Waits for the previous write first.
int pf_out_write_fp64(pf_out *o, cudaStream_t stream, int ix, int iy, int iz, double dx, const int *ids,
                      const double *C, const char *directory, int index, int pieces);
int pf_out_write_fp32(pf_out *o, cudaStream_t stream, int ix, int iy, int iz, double dx, int nsol, int b1, int b2,
                      const ushort4 *gid, const float2 *sol, const char *directory, int index, int pieces);
