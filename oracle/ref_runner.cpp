// ref_runner.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own CUDA diffusion plug-in kernels, GPU_Partitioning
// and Diff3D (zhubq/PhaseField, C++-openmp-cuda/src/gpu_solver.cpp:131-188),
// compiled from that source file into a cubin by build_oracle.py, with a host
// loop that follows GPU_Diffusion_solver (gpu_solver.cpp:204-218): copy the
// coefficients to the module's __constant__ arrays and the fields to the device,
// num_loop = ceil(dt/del_t) times launch partition then flux on a
// (ceil(x/256), y, z) x (256,1,1) grid, copy the total concentration back.
// The CUDA driver API is used so the module can be loaded from the cubin file.
#include <cuda.h>
#include <cmath>
#include <cstring>
#include <string>

namespace {
std::string g_err;

int fail(const char *what, CUresult r) {
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "?");
    return -1;
}

// Itanium-mangled names of the two kernels (real = double).
const char *kPart = "_Z16GPU_PartitioningPKdS0_Pdiii";
const char *kDiff = "_Z6Diff3DPKdPdS0_iiidi";
}  // namespace

extern "C" const char *ref_last_error(void) { return g_err.c_str(); }

extern "C" int ref_gpu_diffusion_solver(const char *cubin, const double *D3, const double *k9, const double *c9,
                                        const double *phase, double *C, int x, int y, int z, double dt, double dx) {
    CUresult r = cuInit(0);
    if (r != CUDA_SUCCESS) return fail("cuInit", r);
    CUdevice dev;
    if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return fail("cuDeviceGet", r);
    CUcontext ctx;
    if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return fail("cuDevicePrimaryCtxRetain", r);
    cuCtxPushCurrent(ctx);
    int ret = -1;
    CUmodule mod = nullptr;
    CUdeviceptr dphase = 0, dC = 0, dconc = 0;
    do {
        if ((r = cuModuleLoad(&mod, cubin)) != CUDA_SUCCESS) { fail("cuModuleLoad", r); break; }
        CUfunction fpart, fdiff;
        if ((r = cuModuleGetFunction(&fpart, mod, kPart)) != CUDA_SUCCESS) { fail("GPU_Partitioning", r); break; }
        if ((r = cuModuleGetFunction(&fdiff, mod, kDiff)) != CUDA_SUCCESS) { fail("Diff3D", r); break; }
        CUdeviceptr pk, pc, pd;
        size_t sk, sc, sd;
        if ((r = cuModuleGetGlobal(&pk, &sk, mod, "dpara_partition_k")) != CUDA_SUCCESS) { fail("k", r); break; }
        if ((r = cuModuleGetGlobal(&pc, &sc, mod, "dpara_partition_c")) != CUDA_SUCCESS) { fail("c", r); break; }
        if ((r = cuModuleGetGlobal(&pd, &sd, mod, "ddiffusivity")) != CUDA_SUCCESS) { fail("D", r); break; }
        if (sk != 9 * sizeof(double) || sc != 9 * sizeof(double) || sd != 3 * sizeof(double)) {
            g_err = "unexpected constant sizes";
            break;
        }
        cuMemcpyHtoD(pk, k9, sk);
        cuMemcpyHtoD(pc, c9, sc);
        cuMemcpyHtoD(pd, D3, sd);
        const size_t N = (size_t)x * y * z;
        if ((r = cuMemAlloc(&dphase, 3 * N * sizeof(double))) != CUDA_SUCCESS) { fail("alloc", r); break; }
        if ((r = cuMemAlloc(&dC, N * sizeof(double))) != CUDA_SUCCESS) { fail("alloc", r); break; }
        if ((r = cuMemAlloc(&dconc, 3 * N * sizeof(double))) != CUDA_SUCCESS) { fail("alloc", r); break; }
        cuMemcpyHtoD(dphase, phase, 3 * N * sizeof(double));
        cuMemcpyHtoD(dC, C, N * sizeof(double));
        const int dims = z > 1 ? 3 : 2;
        double max_diff = D3[0];
        for (int p = 1; p < 3; p++)
            if (D3[p] > max_diff) max_diff = D3[p];
        const double del_t = dx * dx / max_diff / dims * 0.2f;
        int num_loop = (int)std::ceil(dt / del_t);
        double dt_dxdx = dt / num_loop / (dx * dx);
        const unsigned gx = (unsigned)((x + 255) / 256);
        int xx = x, yy = y, zz = z;
        bool ok = true;
        for (int n = 1; n <= num_loop && ok; n++) {
            void *a1[] = {&dphase, &dC, &dconc, &xx, &yy, &zz};
            r = cuLaunchKernel(fpart, gx, (unsigned)y, (unsigned)z, 256, 1, 1, 0, nullptr, a1, nullptr);
            if (r != CUDA_SUCCESS) { fail("launch GPU_Partitioning", r); ok = false; break; }
            void *a2[] = {&dphase, &dC, &dconc, &xx, &yy, &zz, &dt_dxdx, &num_loop};
            r = cuLaunchKernel(fdiff, gx, (unsigned)y, (unsigned)z, 256, 1, 1, 0, nullptr, a2, nullptr);
            if (r != CUDA_SUCCESS) { fail("launch Diff3D", r); ok = false; break; }
        }
        if (!ok) break;
        if ((r = cuMemcpyDtoH(C, dC, N * sizeof(double))) != CUDA_SUCCESS) { fail("copy back", r); break; }
        ret = num_loop;
    } while (0);
    if (dphase) cuMemFree(dphase);
    if (dC) cuMemFree(dC);
    if (dconc) cuMemFree(dconc);
    if (mod) cuModuleUnload(mod);
    CUcontext popped;
    cuCtxPopCurrent(&popped);
    cuDevicePrimaryCtxRelease(dev);
    return ret;
}
