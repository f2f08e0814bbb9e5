"""Build libpfstep.so (CUDA for sm_103a + host C++) and the pfm driver in-tree.

Each translation unit is compiled in parallel with its own flags:

* ``pf_f64.cu``  ``-fmad=false``: the FP64 parity kernels must not contract
  multiply-adds, so they reproduce the CPU solver's rounding exactly.
* ``pf_f32.cu``  ``-prec-div=false -prec-sqrt=false``: approximate division and
  square root in the FP32 kernels (the solute update is compensated).
* ``pf_f32_diffuse.cu`` additionally ``-fmad=false``: every kernel variant of the
  diffusion sub-step rounds identically (their FMAs are explicit).
* ``pf_host.cpp`` ``-ffp-contract=off``: host-side per-step parameters must be
  bit-identical to the reference's host arithmetic on x86 and on Arm.

Outputs: ``phasefield_gb300/lib/libpfstep.so`` and ``phasefield_gb300/bin/pfm``
(both git-ignored; object files go to ``_build/``).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
OBJDIR = os.path.join(REPO, "_build", "pfstep")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libpfstep.so")
PFM = os.path.join(BINDIR, "pfm")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc() -> str:
    cand = os.path.join(CUDA_HOME, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", INCLUDE, "-I", CSRC,
]
PER_FILE = {
    "pf_f64.cu": ["-fmad=false"],
    "pf_f32.cu": ["-prec-div=false", "-prec-sqrt=false"],
    # no implicit contraction: every variant of the sub-step kernel must round
    # identically (every intended FMA is an explicit fmaf)
    "pf_f32_diffuse.cu": ["-fmad=false", "-prec-div=false", "-prec-sqrt=false"],
    "pf_batch.cu": ["-prec-div=false", "-prec-sqrt=false"],
    # no implicit contraction (forward and reverse must rebuild identical
    # decisions); approximate FP32 division/sqrt (same code path in both)
    "pf_adjoint.cu": ["-fmad=false", "-prec-div=false", "-prec-sqrt=false"],
    # the device generator rounds as the host generator does
    "pf_init_dev.cu": ["-fmad=false"],
}
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp",
             "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(CUDA_HOME, "include")]

CU_SOURCES = ["pf_f64.cu", "pf_f32.cu", "pf_f32_diffuse.cu", "pf_batch.cu", "pf_reduce.cu", "pf_api.cu",
              "pf_reduce_noalloc.cu", "pf_adjoint.cu", "pf_output.cu",
              "pf_init_dev.cu"]
CXX_SOURCES = ["pf_host.cpp", "pf_init.cpp"]
HEADERS = ["pf_types.h", "pf_dev.cuh", "pf_f32.cuh", "pf_kernels.h", "pf_host.h", "pf_init.h"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile every translation unit (in parallel) and link libpfstep.so."""
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "pfstep.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs + [__file__]):
            jobs.append([_nvcc()] + NVCC_FLAGS + PER_FILE.get(src, []) + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs + [__file__]):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _newer(LIB, objs):
        _run([_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    main = os.path.join(CSRC, "pfm_main.cpp")
    if force or _newer(PFM, [main, LIB, os.path.join(INCLUDE, "pfstep.h")]):
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, main, "-o", PFM, "-L", LIBDIR, "-lpfstep",
              "-Wl,-rpath,$ORIGIN/../lib"])
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


def ptxas_report() -> str:
    """Register / spill / shared-memory usage of every kernel (-Xptxas -v)."""
    out = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        cmd = [_nvcc()] + NVCC_FLAGS + PER_FILE.get(src, []) + ["-Xptxas", "-v", "-c", s, "-o", os.devnull]
        r = subprocess.run(cmd, capture_output=True, text=True)
        out.append(f"== {src}\n{r.stderr}")
    return "\n".join(out)


if __name__ == "__main__":
    build(verbose=True)
