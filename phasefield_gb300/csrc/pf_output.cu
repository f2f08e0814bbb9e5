// pf_output.cu -- microstructure files written from device buffers (sm_103a + host).
//
// The reference writes its microstructure as ASCII VTK image data from host
// arrays (zhubq/PhaseField C++-openmp-cuda/src/write_data.cpp:42-82), and its
// MPI variant one piece per rank plus a .pvti index
// (C++-MPI/source/write_data.cpp:30-110).  Here the two point fields of those
// files -- "korn" (0 where a cell's second slot is occupied, else the phase of
// its first grain; write_data.cpp:58-64) and "conc" (total carbon as Float32)
// -- are formed on the GPU by one kernel, copied to pinned host memory on a
// stream of their own, and written by a host thread as z-slab pieces in
// appended raw binary (header_type UInt64) with a .pvti index, while the
// caller keeps stepping: the field buffer is separate from the state, so the
// next steps may overwrite the state as soon as the field kernel has run.
//
// Files: <directory>/<index:07d>_<piece>.vti and <directory>/<index:07d>.pvti
// (the MPI variant's names, write_data.cpp:35-40,58-66).  Pieces are z slabs
// that share their boundary plane, so the pieces together cover every cell of
// the image and ParaView draws no gap between them.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "pf_f32.cuh"
#include "pf_host.h"
#include "pf_output.h"

namespace {

int cuda_fail(cudaError_t e) { return pf_fail(PF_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e)); }

__global__ void __launch_bounds__(256) k_fields_f64(long long N, const int *__restrict__ ids,
                                                    const double *__restrict__ C, int *__restrict__ korn,
                                                    float *__restrict__ conc) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    korn[n] = ids[6 * n + 1] > 0 ? 0 : pf_phase_of_grain(ids[6 * n]);
    conc[n] = (float)C[n];
}

__global__ void __launch_bounds__(256) k_fields_f32(long long N, int nsol, int b1, int b2,
                                                    const ushort4 *__restrict__ gid, const float2 *__restrict__ sol,
                                                    int *__restrict__ korn, float *__restrict__ conc) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const ushort4 g = gid[n];
    korn[n] = g.y > 0 ? 0 : pf_lphase(g.x, b1, b2);
    const float2 s = sol[n * nsol];
    conc[n] = (float)((double)s.x - (double)s.y);  // the compensated total, as the FP64 download forms it
}

std::string file_name(const char *dir, int index, int piece) {
    char b[64];
    if (piece >= 0) std::snprintf(b, sizeof b, "%07d_%d.vti", index, piece);
    else std::snprintf(b, sizeof b, "%07d.pvti", index);
    return std::string(dir) + "/" + b;
}

// Planes [k0, k1] of piece p out of P (neighbouring pieces share a plane).
void piece_planes(int iz, int P, int p, int &k0, int &k1) {
    k0 = (int)((long long)p * iz / P);
    k1 = p + 1 == P ? iz - 1 : (int)((long long)(p + 1) * iz / P);
}

std::string extent(int ix, int iy, int k0, int k1) {
    std::ostringstream s;
    s << 1 << ' ' << ix << ' ' << 1 << ' ' << iy << ' ' << k0 + 1 << ' ' << k1 + 1;
    return s.str();
}

int write_piece(const std::string &path, int ix, int iy, int k0, int k1, double dx, const int32_t *korn,
                const float *conc) {
    std::ofstream f(path, std::ios::binary);
    if (!f.is_open()) return PF_ERR_IO;
    const unsigned long long n = (unsigned long long)ix * iy * (k1 - k0 + 1);
    const unsigned long long bytes = 4ull * n;
    const std::string ext = extent(ix, iy, k0, k1);
    f << "<?xml version=\"1.0\"?>\n"
      << "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "<ImageData WholeExtent=\"" << ext << "\" Origin=\"0 0 0\" Spacing=\"" << dx << ' ' << dx << ' ' << dx
      << "\">\n"
      << "<Piece Extent=\"" << ext << "\">\n"
      << "<PointData Scalars=\"energy\">\n"
      << "<DataArray type=\"Int32\" Name=\"korn\" format=\"appended\" offset=\"0\"/>\n"
      << "<DataArray type=\"Float32\" Name=\"conc\" format=\"appended\" offset=\"" << 8 + bytes << "\"/>\n"
      << "</PointData>\n</Piece>\n</ImageData>\n"
      << "<AppendedData encoding=\"raw\">\n_";
    const size_t off = (size_t)ix * iy * k0;
    f.write(reinterpret_cast<const char *>(&bytes), 8);
    f.write(reinterpret_cast<const char *>(korn + off), (std::streamsize)bytes);
    f.write(reinterpret_cast<const char *>(&bytes), 8);
    f.write(reinterpret_cast<const char *>(conc + off), (std::streamsize)bytes);
    f << "\n</AppendedData>\n</VTKFile>\n";
    return f ? PF_OK : PF_ERR_IO;
}

int write_index(const char *dir, int index, int ix, int iy, int iz, int P, double dx) {
    std::ofstream f(file_name(dir, index, -1));
    if (!f.is_open()) return PF_ERR_IO;
    f << "<?xml version=\"1.0\"?>\n"
      << "<VTKFile type=\"PImageData\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "<PImageData WholeExtent=\"" << extent(ix, iy, 0, iz - 1) << "\" GhostLevel=\"0\" Origin=\"0 0 0\" Spacing=\""
      << dx << ' ' << dx << ' ' << dx << "\">\n"
      << "<PPointData Scalars=\"energy\">\n"
      << "<PDataArray type=\"Int32\" Name=\"korn\"/>\n"
      << "<PDataArray type=\"Float32\" Name=\"conc\"/>\n"
      << "</PPointData>\n";
    for (int p = 0; p < P; p++) {
        int k0, k1;
        piece_planes(iz, P, p, k0, k1);
        char b[64];
        std::snprintf(b, sizeof b, "%07d_%d.vti", index, p);
        f << "<Piece Extent=\"" << extent(ix, iy, k0, k1) << "\" Source=\"" << b << "\"/>\n";
    }
    f << "</PImageData>\n</VTKFile>\n";
    return f ? PF_OK : PF_ERR_IO;
}

}  // namespace

// Every piece by its own host thread, then the index.
extern "C" int pf_write_vti_binary_host(const char *directory, int index, int pieces, int ix, int iy, int iz,
                                        double dx, const int32_t *korn, const float *conc) {
    if (!directory || !korn || !conc || ix < 1 || iy < 1 || iz < 1 || pieces < 1 || index < 0)
        return pf_fail(PF_ERR_ARG, "pf_write_vti_binary_host: bad argument");
    const int P = pieces < iz ? pieces : iz;
    std::vector<int> st(P, PF_OK);
    std::vector<std::thread> th;
    th.reserve(P);
    for (int p = 0; p < P; p++)
        th.emplace_back([&, p] {
            int k0, k1;
            piece_planes(iz, P, p, k0, k1);
            st[p] = write_piece(file_name(directory, index, p), ix, iy, k0, k1, dx, korn, conc);
        });
    for (auto &t : th) t.join();
    for (int p = 0; p < P; p++)
        if (st[p] != PF_OK) return pf_fail(st[p], "pf_write_vti_binary_host: cannot write " + file_name(directory, index, p));
    const int s = write_index(directory, index, ix, iy, iz, P, dx);
    return s == PF_OK ? PF_OK : pf_fail(s, "pf_write_vti_binary_host: cannot write " + file_name(directory, index, -1));
}

struct pf_out {
    long long N = 0;
    int *d_korn = nullptr;       // device fields: korn[N] then conc[N]
    int32_t *h_buf = nullptr;    // pinned copy of both
    cudaStream_t copy = nullptr;
    cudaEvent_t formed = nullptr, copied = nullptr;
    bool pending = false;        // a copy + write is in flight
    std::thread writer;
    int status = PF_OK;
    std::string message;
};

pf_out *pf_out_create() { return new pf_out(); }

int pf_out_wait(pf_out *o) {
    if (!o) return PF_OK;
    if (o->writer.joinable()) o->writer.join();
    o->pending = false;
    const int s = o->status;
    o->status = PF_OK;
    if (s != PF_OK) return pf_fail(s, o->message);
    return PF_OK;
}

void pf_out_destroy(pf_out *o) {
    if (!o) return;
    if (o->writer.joinable()) o->writer.join();
    cudaFree(o->d_korn);
    if (o->h_buf) cudaFreeHost(o->h_buf);
    if (o->copy) cudaStreamDestroy(o->copy);
    if (o->formed) cudaEventDestroy(o->formed);
    if (o->copied) cudaEventDestroy(o->copied);
    delete o;
}

namespace {

int ensure(pf_out *o, long long N) {
    if (o->N == N && o->d_korn) return PF_OK;
    if (o->writer.joinable()) o->writer.join();
    cudaFree(o->d_korn);
    o->d_korn = nullptr;
    if (o->h_buf) cudaFreeHost(o->h_buf);
    o->h_buf = nullptr;
    o->N = 0;
    if (!o->copy && cudaStreamCreateWithFlags(&o->copy, cudaStreamNonBlocking) != cudaSuccess) goto fail;
    if (!o->formed && cudaEventCreateWithFlags(&o->formed, cudaEventDisableTiming) != cudaSuccess) goto fail;
    if (!o->copied && cudaEventCreateWithFlags(&o->copied, cudaEventDisableTiming) != cudaSuccess) goto fail;
    if (cudaMalloc(&o->d_korn, 8ull * N) != cudaSuccess) goto fail;
    if (cudaMallocHost(&o->h_buf, 8ull * N) != cudaSuccess) goto fail;
    o->N = N;
    return PF_OK;
fail:
    cudaGetLastError();
    return pf_fail(PF_ERR_NOMEM, "pf_write_vti_binary: cannot allocate the output buffers");
}

// After the field kernel was enqueued on 'stream': copy on the output stream,
// then write on a host thread.
int start_copy_and_write(pf_out *o, cudaStream_t stream, const char *directory, int index, int pieces, int ix, int iy,
                         int iz, double dx) {
    cudaError_t e = cudaEventRecord(o->formed, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(o->copy, o->formed, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(o->h_buf, o->d_korn, 8ull * o->N, cudaMemcpyDeviceToHost, o->copy);
    if (e == cudaSuccess) e = cudaEventRecord(o->copied, o->copy);
    if (e != cudaSuccess) return cuda_fail(e);
    o->pending = true;
    o->status = PF_OK;
    const std::string dir(directory);
    o->writer = std::thread([o, dir, index, pieces, ix, iy, iz, dx] {
        cudaError_t w = cudaEventSynchronize(o->copied);
        if (w != cudaSuccess) {
            o->status = PF_ERR_CUDA;
            o->message = std::string("pf_write_vti_binary: ") + cudaGetErrorString(w);
            return;
        }
        const float *conc = reinterpret_cast<const float *>(o->h_buf + o->N);
        const int s = pf_write_vti_binary_host(dir.c_str(), index, pieces, ix, iy, iz, dx, o->h_buf, conc);
        if (s != PF_OK) {
            o->status = s;
            o->message = pf_last_error();
        }
    });
    return PF_OK;
}

inline unsigned blocks_of(long long N) { return (unsigned)((N + 255) / 256); }

}  // namespace

int pf_out_write_fp64(pf_out *o, cudaStream_t stream, int ix, int iy, int iz, double dx, const int *ids,
                      const double *C, const char *directory, int index, int pieces) {
    const long long N = (long long)ix * iy * iz;
    int s = pf_out_wait(o);  // the previous write owns the buffers until it has finished
    if (s != PF_OK) return s;
    s = ensure(o, N);
    if (s != PF_OK) return s;
    k_fields_f64<<<blocks_of(N), 256, 0, stream>>>(N, ids, C, o->d_korn, reinterpret_cast<float *>(o->d_korn + N));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e);
    return start_copy_and_write(o, stream, directory, index, pieces, ix, iy, iz, dx);
}

int pf_out_write_fp32(pf_out *o, cudaStream_t stream, int ix, int iy, int iz, double dx, int nsol, int b1, int b2,
                      const ushort4 *gid, const float2 *sol, const char *directory, int index, int pieces) {
    const long long N = (long long)ix * iy * iz;
    int s = pf_out_wait(o);
    if (s != PF_OK) return s;
    s = ensure(o, N);
    if (s != PF_OK) return s;
    k_fields_f32<<<blocks_of(N), 256, 0, stream>>>(N, nsol, b1, b2, gid, sol, o->d_korn,
                                                   reinterpret_cast<float *>(o->d_korn + N));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e);
    return start_copy_and_write(o, stream, directory, index, pieces, ix, iy, iz, dx);
}
