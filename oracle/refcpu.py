"""ctypes binding of oracle/_ref/libpfref_cpu.so -- the reference's own CPU
time step (TEST INFRASTRUCTURE ONLY).

The library is zhubq/PhaseField C++-openmp-cuda/src/{phase_field,solver,
thermo_data,thermo_functor,write_data}.cpp compiled unmodified against the
minimal Blitz++ stand-in oracle/blitz_shim (build_oracle.build_ref_cpu).  It
exists only where the reference checkout does (it is built from there); the
golden fixture tests/golden/ref_cpu_steps.npz carries its outputs elsewhere.
"""
from __future__ import annotations

import ctypes
import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libpfref_cpu.so")
_lib = None
_P = ctypes.c_void_p


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        L.pfr_create.restype = _P
        L.pfr_create.argtypes = [ctypes.c_char_p]
        L.pfr_destroy.argtypes = [_P]
        L.pfr_dims.argtypes = [_P, _P]
        L.pfr_set_state.argtypes = [_P] * 6
        L.pfr_get_state.argtypes = [_P] * 6
        L.pfr_update.argtypes = [_P, ctypes.c_int]
        L.pfr_phase_only.argtypes = [_P]
        L.pfr_time.argtypes = [_P]
        L.pfr_time.restype = ctypes.c_double
        L.pfr_temperature.argtypes = [_P]
        L.pfr_temperature.restype = ctypes.c_double
        L.pfr_write_data.argtypes = [_P, ctypes.c_int]
        _lib = L
    return _lib


def rewrite_config(path: str, directory: str, micro_out: int) -> str:
    """Set the output folder (line 2) and the VTI flag of a configuration file
    written by phasefield_gb300.workloads.write_config, in place."""
    lines = open(path).read().splitlines()
    lines[1] = os.path.abspath(directory)
    for i, ln in enumerate(lines):
        if ln.startswith("write VTI"):
            lines[i + 1] = str(int(micro_out))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def run(config_path: str, state: dict, nsteps: int, write: bool = False, phase_only: bool = False) -> dict:
    """Read the configuration with phase_field::Read_data (thermo file resolved
    from the configuration's folder), load the carbon state (reference layout),
    optionally Write_data(true), run nsteps x Update(false) (or one
    Update(true) when phase_only), optionally Write_data(true) again, and
    return the state, time and written outputs."""
    L = lib()
    cfg = os.path.abspath(config_path)
    d = os.path.dirname(cfg)
    outdir = open(cfg).read().splitlines()[1].strip()
    os.makedirs(outdir if os.path.isabs(outdir) else os.path.join(d, outdir), exist_ok=True)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = L.pfr_create(cfg.encode())
        dims = np.zeros(3, np.int32)
        L.pfr_dims(h, _ptr(dims))
        N = int(dims[0]) * int(dims[1]) * int(dims[2])
        cur = {"ids": np.ascontiguousarray(state["ids"][: 6 * N], np.int32),
               "phi": np.ascontiguousarray(state["phi"][: 6 * N], np.float64),
               "phase": np.ascontiguousarray(state["phase"][: 3 * N], np.float64),
               "conc": np.ascontiguousarray(state["conc"][: 3 * N], np.float64),
               "C": np.ascontiguousarray(state["C"][:N], np.float64)}
        L.pfr_set_state(h, _ptr(cur["ids"]), _ptr(cur["phi"]), _ptr(cur["phase"]), _ptr(cur["conc"]), _ptr(cur["C"]))
        if write:
            L.pfr_write_data(h, 1)
        if phase_only:
            L.pfr_phase_only(h)
        else:
            L.pfr_update(h, int(nsteps))
        if write:
            L.pfr_write_data(h, 1)
        out = {k: np.zeros_like(v) for k, v in cur.items()}
        L.pfr_get_state(h, _ptr(out["ids"]), _ptr(out["phi"]), _ptr(out["phase"]), _ptr(out["conc"]), _ptr(out["C"]))
        out["time"] = float(L.pfr_time(h))
        L.pfr_destroy(h)  # closes fraction_time.txt
    finally:
        os.chdir(cwd)
    if write:
        base = outdir if os.path.isabs(outdir) else os.path.join(d, outdir)
        out["fraction"] = open(os.path.join(base, "fraction_time.txt")).read()
        # field%07d_%d.vti: the counter after "_" orders the writes
        vtis = sorted(glob.glob(os.path.join(base, "field*_*.vti")),
                      key=lambda p: int(os.path.basename(p)[:-4].rsplit("_", 1)[1]))
        out["vti"] = open(vtis[-1]).read() if vtis else ""
    return out
