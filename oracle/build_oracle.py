"""Build recipes for the oracle side (test infrastructure only).

* ``build_oracle()`` compiles the FP64 CPU oracle ``pf_oracle.c`` into
  ``oracle/_build/liboracle.so`` with ``-ffp-contract=off`` (no fused
  multiply-add, so its rounding matches the product's FP64 GPU path and the
  reference's host arithmetic) and OpenMP, together with the seeded input
  generator (``phasefield_gb300/csrc/pf_init.cpp``) so the CPU baseline can
  build its input state without loading the product library.
* ``build_ref()`` compiles the reference's own CUDA diffusion plug-in,
  ``C++-openmp-cuda/src/gpu_solver.cpp`` from the read-only reference checkout,
  into device-only cubins under ``oracle/_ref/`` (one with the default
  multiply-add contraction, one with ``-fmad=false``).  Its two kernels,
  ``GPU_Partitioning`` and ``Diff3D``, then run on the GPU as an independent
  check of the oracle's partition and diffusion sub-step.  The host part of that
  file and the rest of the reference (which needs Blitz++) are not built.  This
  step only runs where the reference checkout exists; the cubins travel with
  the repository copy.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
# The zhubq/PhaseField checkout: PF_REFERENCE_ROOT, else a "reference" folder
# beside the repository.  It is read only where it exists.
REF_ROOT = os.path.abspath(os.environ.get("PF_REFERENCE_ROOT",
                                          os.path.join(HERE, os.pardir, os.pardir, "reference")))
REF_SRC = os.path.join(REF_ROOT, "C++-openmp-cuda", "src")
REF_CUBIN = os.path.join(REF_OUT, "gpu_solver_ref.cubin")
REF_CUBIN_NOFMA = os.path.join(REF_OUT, "gpu_solver_ref_nofma.cubin")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


REPO = os.path.dirname(HERE)
# The seeded input generator is one source file shared with the product, so
# the CPU baseline steps exactly the state the GPU steps (it generates inputs;
# it is not part of what is checked).
INIT_SRC = os.path.join(REPO, "phasefield_gb300", "csrc", "pf_init.cpp")
INIT_HDRS = [os.path.join(REPO, "phasefield_gb300", "csrc", "pf_init.h"), os.path.join(REPO, "include", "pfstep.h"),
             os.path.join(REPO, "phasefield_gb300", "csrc", "pf_init_cell.h"),
             os.path.join(REPO, "phasefield_gb300", "csrc", "pf_init_setup.h"),
             # exp/log shared with the product so the solute-drag bisection rounds alike
             os.path.join(REPO, "phasefield_gb300", "csrc", "pf_math.h")]


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = [os.path.join(HERE, "pf_oracle.c"), os.path.join(HERE, "pf_oracle.h")]
    if force or _newer(LIB, src + [INIT_SRC] + INIT_HDRS + [__file__]):
        o1 = os.path.join(BUILD, "pf_oracle.o")
        o2 = os.path.join(BUILD, "pf_init.o")
        inc = ["-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "phasefield_gb300", "csrc")]
        cmds = [["gcc", "-O3", "-std=c99", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"] + inc +
                ["-c", src[0], "-o", o1],
                ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"] + inc +
                ["-c", INIT_SRC, "-o", o2],
                ["g++", "-shared", "-fopenmp", o1, o2, "-o", LIB, "-lm"]]
        for cmd in cmds:
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    return LIB


RUNNER = os.path.join(BUILD, "libref_runner.so")


def build_ref_runner(force: bool = False) -> str:
    """Driver-API host loop that launches the reference's kernels from a cubin."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_runner.cpp")
    if force or _newer(RUNNER, [src, __file__]):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", RUNNER,
               "-I", os.path.join(CUDA_HOME, "include"), "-L", os.path.join(CUDA_HOME, "lib64", "stubs"), "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference runner build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    return RUNNER


def build_ref(force: bool = False) -> list[str]:
    """Compile the reference's GPU plug-in kernels (where the checkout exists)."""
    src = os.path.join(REF_SRC, "gpu_solver.cpp")
    if not os.path.exists(src):
        return [p for p in (REF_CUBIN, REF_CUBIN_NOFMA) if os.path.exists(p)]
    os.makedirs(REF_OUT, exist_ok=True)
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc") or "nvcc"
    out = []
    for target, extra in ((REF_CUBIN, []), (REF_CUBIN_NOFMA, ["-fmad=false"])):
        if force or _newer(target, [src, __file__]):
            # cudaDeviceProp::deviceOverlap (read by the host-only GPU_Init
            # printout) no longer exists in CUDA 13; the macro maps it onto a
            # member that does.  Device code is unaffected.
            cmd = [nvcc, "-cubin", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                   "-DdeviceOverlap=asyncEngineCount", "-I", REF_SRC] + extra + [src, "-o", target]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("reference kernel build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
        out.append(target)
    return out


REF_CPU_LIB = os.path.join(REF_OUT, "libpfref_cpu.so")
REF_CPU_SOURCES = ["phase_field.cpp", "solver.cpp", "thermo_data.cpp", "thermo_functor.cpp", "write_data.cpp"]


def build_ref_cpu(force: bool = False) -> str | None:
    """Compile the reference's own CPU time step into oracle/_ref/libpfref_cpu.so.

    The unmodified sources C++-openmp-cuda/src/{phase_field,solver,thermo_data,
    thermo_functor,write_data}.cpp are compiled straight from the read-only
    checkout against oracle/blitz_shim (a minimal stand-in for the Blitz++
    Array API they use), together with ref_cpu_runner.cpp (C entry points and
    "no GPU" stubs for gpu_solver.h).  -ffp-contract=off keeps the reference's
    x86 build semantics (no fused multiply-add) on every host.  Returns None
    where the checkout is absent (the library is then used only if it exists).
    """
    srcs = [os.path.join(REF_SRC, f) for f in REF_CPU_SOURCES]
    if not all(os.path.exists(p) for p in srcs):
        return REF_CPU_LIB if os.path.exists(REF_CPU_LIB) else None
    os.makedirs(REF_OUT, exist_ok=True)
    shim = os.path.join(HERE, "blitz_shim")
    runner = os.path.join(HERE, "ref_cpu_runner.cpp")
    deps = srcs + [runner, os.path.join(shim, "blitz", "array.h"), __file__]
    if force or _newer(REF_CPU_LIB, deps):
        # phase_field::Read_data hands system() a pointer into a destroyed
        # temporary string (phase_field.cpp:47-49), so the shell runs whatever
        # that memory holds; the linker's --wrap sends the call to a no-op in
        # the runner (the caller creates the output directory itself).
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               "-w", "-Wl,--wrap=system", "-I", shim, "-I", REF_SRC] + srcs + [runner, "-o", REF_CPU_LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference CPU build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    return REF_CPU_LIB


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    print(build_ref_cpu())
