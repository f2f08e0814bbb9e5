"""phasefield_gb300 -- GB300-native Steinbach multi-phase-field time step.

The product is ``lib/libpfstep.so`` (hand-written sm_103a CUDA kernels behind a
C ABI, ``include/pfstep.h``).  This module is a thin ctypes mirror of the
reference's ``phase_field`` class (zhubq/PhaseField,
C++-openmp-cuda/src/phase_field.h:20-120): ``read_data``, ``construct``,
``update``, ``write_data``.  It does no arithmetic of its own and has no CPU
fallback: if the library is missing every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libpfstep.so")
CONFIG_DIR = os.path.join(_HERE, "configs")

PF_OK = 0
PF_ERR_ARG = -1
PF_ERR_NOMEM = -2
PF_ERR_CUDA = -3
PF_ERR_TIMEOUT = -4
PF_ERR_NONFINITE = -5
PF_ERR_IO = -6
PF_ERR_NODEV = -7
PF_ERR_RANGE = -8
PF_ERR_DRIFT = -9
PF_PREC_FP64 = 0
PF_PREC_FP32C = 1
PF_MAXT = 64

_d9 = ctypes.c_double * 9
_d3 = ctypes.c_double * 3


class PfModel(ctypes.Structure):
    """Mirror of ``pf_model`` (pfstep.h)."""

    _fields_ = [
        ("directory", ctypes.c_char * 256),
        ("ix", ctypes.c_int), ("iy", ctypes.c_int), ("iz", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("i_intf", ctypes.c_int),
        ("cutoff", ctypes.c_double),
        ("num_grain", ctypes.c_int * 3),
        ("phase_fraction", _d3),
        ("init_conc", _d3),
        ("nT", ctypes.c_int),
        ("T_time", ctypes.c_double * PF_MAXT), ("T_temp", ctypes.c_double * PF_MAXT),
        ("reduction", ctypes.c_double),
        ("num_init_iteration", ctypes.c_int),
        ("timestep_output", ctypes.c_double),
        ("micro_out", ctypes.c_int),
        ("num_nuclei", ctypes.c_double),
        ("m0", _d9), ("mQ", _d9),
        ("sigma", _d9),
        ("D0", _d3 * 2), ("DQ", _d3 * 2),
        ("thermo_file", ctypes.c_char * 256),
        ("gpu_flag", ctypes.c_int),
        ("nsol", ctypes.c_int),
        ("mn_ratio", _d3),
        ("ent_a", _d9), ("ent_b", _d9),
        ("nple1_a", _d9), ("nple1_b", _d9), ("nple1_c", _d9),
        ("nple2_a", _d9), ("nple2_b", _d9), ("nple2_c", _d9),
        ("eq_a", _d9), ("eq_b", _d9), ("eq_c", _d9),
        ("thermo_model", ctypes.c_int),
        ("avg_carbon", ctypes.c_int),
        ("drag", ctypes.c_int),
        ("drag_binding", ctypes.c_double), ("drag_vmax0", ctypes.c_double), ("drag_qsd", ctypes.c_double),
        ("coherent", ctypes.c_int), ("coh_npp0", ctypes.c_int),
    ]


class PfStepParams(ctypes.Structure):
    """Mirror of ``pf_step_params`` (pfstep.h)."""

    _fields_ = [
        ("ix", ctypes.c_int), ("iy", ctypes.c_int), ("iz", ctypes.c_int),
        ("nnb", ctypes.c_int), ("nsol", ctypes.c_int), ("n_sub", ctypes.c_int),
        ("N", ctypes.c_longlong),
        ("T", ctypes.c_double), ("time", ctypes.c_double),
        ("dx", ctypes.c_double), ("cutoff", ctypes.c_double), ("eta", ctypes.c_double),
        ("pfm_dt", ctypes.c_double), ("diff_dt", ctypes.c_double), ("dt_sub", ctypes.c_double),
        ("factor1", ctypes.c_double), ("factor2", ctypes.c_double), ("factor3", ctypes.c_double),
        ("coef_diff", ctypes.c_double),
        ("m", _d9), ("sigma", _d9),
        ("entropy", _d9), ("eq", _d9), ("dcdT", _d9),
        ("D", _d3 * 2),
        ("k", _d9 * 2), ("c", _d9 * 2),
        ("df_model", ctypes.c_int),
        ("df_ratio", _d9), ("df_ref", ctypes.c_double),
        ("avg_range", ctypes.c_int), ("avg_conc", ctypes.c_int),
        ("drag_model", ctypes.c_int),
        ("drag_vmax", ctypes.c_double), ("drag_ex0", ctypes.c_double), ("drag_de_heat", ctypes.c_double),
        ("drag_de_cool", ctypes.c_double), ("drag_u0", ctypes.c_double),
        ("drag_corr", ctypes.c_double * 2), ("drag_drag0", ctypes.c_double * 2),
        ("coh_model", ctypes.c_int), ("coh_npp0", ctypes.c_int),
    ]


class PfInitSpec(ctypes.Structure):
    """Mirror of ``pf_init_spec`` (pfstep.h)."""

    _fields_ = [
        ("seed", ctypes.c_uint64),
        ("n_grains", ctypes.c_int),
        ("n_nuclei", ctypes.c_int),
        ("nucleus_radius", ctypes.c_double),
        ("n_particles", ctypes.c_int),
        ("particle_radius", ctypes.c_double),
        ("width", ctypes.c_double),
        ("C0", ctypes.c_double * 2),
        ("C_noise", ctypes.c_double * 2),
        ("max_slots", ctypes.c_int),
    ]


# Every symbol pfstep.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
SYMBOLS = {
    "GPU_Init": (_I, [_I, _I, _I]),
    "GPU_Diffusion_solver": (None, [_DP, _DP, _DP, _DP, _DP, _I, _I, _I, _D, _D]),
    "GPU_Cleanup": (None, []),
    "pf_status_string": (ctypes.c_char_p, [_I]),
    "pf_last_error": (ctypes.c_char_p, []),
    "pf_abi_sizes": (_I, [ctypes.POINTER(ctypes.c_longlong)]),
    "pf_model_read": (_I, [ctypes.c_char_p, ctypes.POINTER(PfModel)]),
    "pf_thermo_read": (_I, [ctypes.c_char_p, ctypes.POINTER(PfModel)]),
    "pf_params_at": (_I, [ctypes.POINTER(PfModel), _D, ctypes.POINTER(PfStepParams)]),
    "pf_init_microstructure": (_I, [ctypes.POINTER(PfModel), ctypes.POINTER(PfInitSpec), _D, _P, _P, _P, _P, _P]),
    "pf_init_microstructure_box": (_I, [ctypes.POINTER(PfModel), ctypes.POINTER(PfInitSpec), _D, _I, _I, _P, _P, _P,
                                        _P, _P]),
    "pf_create": (_I, [ctypes.POINTER(PfModel), _I, ctypes.POINTER(_P)]),
    "pf_destroy": (_I, [_P]),
    "pf_set_stream": (_I, [_P, _P]),
    "pf_upload_state": (_I, [_P, _P, _P, _P, _P, _P, _D]),
    "pf_download_state": (_I, [_P, _P, _P, _P, _P, _P, _DP]),
    "pf_step": (_I, [_P, _I]),
    "pf_diffuse": (_I, [_P, _I]),
    "pf_reduce": (_I, [_P, _DP]),
    "pf_synchronize": (_I, [_P]),
    "pf_check_state": (_I, [_P, _DP, _D, _DP]),
    "pf_get_time": (_I, [_P, _DP]),
    "pf_last_params": (_I, [_P, ctypes.POINTER(PfStepParams)]),
    "pf_truncated_cells": (_I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    "pf_enable_kernel_timing": (_I, [_P, _I]),
    "pf_kernel_times": (_I, [_P, _DP, ctypes.POINTER(ctypes.c_longlong)]),
    "pf_use_graph": (_I, [_P, _I]),
    "pf_autotune": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                         ctypes.POINTER(ctypes.c_float)]),
    "pf_set_diffusion_tile": (_I, [_P, _I, _I, _I]),
    "pf_diffusion_candidates": (_I, [_P, ctypes.POINTER(_I), _I]),
    "pf_write_data": (_I, [_P, ctypes.c_char_p, _I, ctypes.POINTER(_I)]),
    "pf_write_vti": (_I, [ctypes.c_char_p, _I, _I, _I, _D, _P, _P]),
    "pf_reduce_noalloc": (_I, [ctypes.c_longlong, _I, _P, _P, _P, _P, _P, _P]),
    "pf_write_vti_binary": (_I, [_P, ctypes.c_char_p, _I, _I]),
    "pf_write_wait": (_I, [_P]),
    "pf_init_device": (_I, [_P, _P, _D]),
    "pf_set_coherent_grains": (_I, [_P, _P, _I]),
    "pf_init_coherent": (_I, [ctypes.POINTER(PfModel), ctypes.POINTER(PfInitSpec), _P]),
    "pf_write_vti_binary_host": (_I, [ctypes.c_char_p, _I, _I, _I, _I, _I, _D, _P, _P]),
    "pf_batch_create": (_I, [ctypes.POINTER(PfModel), _I, ctypes.POINTER(_P)]),
    "pf_batch_upload": (_I, [_P, _I, _P, _P, _P, _P, _D]),
    "pf_batch_run": (_I, [_P, _I]),
    "pf_batch_download": (_I, [_P, _I, _P, _P, _P, _P, _P, _DP]),
    "pf_batch_reduce": (_I, [_P, _I, _DP]),
    "pf_batch_info": (_I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    "pf_batch_set_timeout": (_I, [_P, ctypes.c_ulonglong, _I]),
    "pf_batch_set_tile": (_I, [_P, _I, _I]),
    "pf_batch_autotune": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_float)]),
    "pf_batch_destroy": (_I, [_P]),
    "pf_adj_create": (_I, [ctypes.POINTER(PfModel), _I, _I, ctypes.POINTER(_P)]),
    "pf_adj_upload": (_I, [_P, _P, _P, _P, _P, _D]),
    "pf_adj_set_scales": (_I, [_P, _DP]),
    "pf_adj_forward": (_I, [_P, _I, _DP]),
    "pf_adj_gradient": (_I, [_P, _I, _DP]),
    "pf_adj_timings": (_I, [_P, _DP]),
    "pf_adj_final_state": (_I, [_P, _DP, _DP]),
    "pf_adj_destroy": (_I, [_P]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load libpfstep.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SYMBOLS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class PfError(RuntimeError):
    def __init__(self, status: int, what: str):
        L = lib()
        msg = f"{what}: {L.pf_status_string(status).decode()} ({L.pf_last_error().decode()})"
        super().__init__(msg)
        self.status = status


def check(status: int, what: str) -> None:
    if status != PF_OK:
        raise PfError(status, what)


def _ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def read_model(config_path: str) -> PfModel:
    m = PfModel()
    check(lib().pf_model_read(config_path.encode(), ctypes.byref(m)), f"pf_model_read({config_path})")
    return m


def params_at(model: PfModel, time: float) -> PfStepParams:
    p = PfStepParams()
    check(lib().pf_params_at(ctypes.byref(model), time, ctypes.byref(p)), "pf_params_at")
    return p


def empty_state(model: PfModel) -> dict:
    N = model.ix * model.iy * model.iz
    return {
        "ids": np.zeros(6 * N, np.int32),
        "phi": np.zeros(6 * N, np.float64),
        "phase": np.zeros(3 * N, np.float64),
        "conc": np.zeros(3 * N * model.nsol, np.float64),
        "C": np.zeros(N * model.nsol, np.float64),
    }


def init_microstructure(model: PfModel, spec: PfInitSpec, time: float) -> dict:
    """Seeded initial state in the reference layout (host arrays)."""
    st = empty_state(model)
    check(lib().pf_init_microstructure(ctypes.byref(model), ctypes.byref(spec), time, _ptr(st["ids"]),
                                       _ptr(st["phi"]), _ptr(st["phase"]), _ptr(st["conc"]), _ptr(st["C"])),
          "pf_init_microstructure")
    return st


def init_microstructure_box(model: PfModel, spec: PfInitSpec, time: float, z0: int, nz: int) -> dict:
    """Planes [z0, z0+nz) of the seeded initial state (equal to those planes of
    init_microstructure on the whole grid)."""
    N = model.ix * model.iy * nz
    st = {"ids": np.zeros(6 * N, np.int32), "phi": np.zeros(6 * N, np.float64), "phase": np.zeros(3 * N, np.float64),
          "conc": np.zeros(3 * N * model.nsol, np.float64), "C": np.zeros(N * model.nsol, np.float64)}
    check(lib().pf_init_microstructure_box(ctypes.byref(model), ctypes.byref(spec), time, z0, nz, _ptr(st["ids"]),
                                           _ptr(st["phi"]), _ptr(st["phase"]), _ptr(st["conc"]), _ptr(st["C"])),
          "pf_init_microstructure_box")
    return st


def init_coherent(model: PfModel, spec: PfInitSpec) -> np.ndarray:
    """Coherent ferrite partners of the nuclei of spec (pf_init_coherent):
    int32 [n_nuclei, 2], 0 = none."""
    out = np.zeros(2 * max(spec.n_nuclei, 0), np.int32)
    check(lib().pf_init_coherent(ctypes.byref(model), ctypes.byref(spec), _ptr(out)), "pf_init_coherent")
    return out.reshape(-1, 2)


class PhaseField:
    """Host-side mirror of the reference's ``phase_field`` object, running the
    whole time step on the GPU through libpfstep."""

    def __init__(self, model: PfModel, precision: int = PF_PREC_FP64):
        self.model = model
        self.precision = precision
        self._ctx = ctypes.c_void_p()
        check(lib().pf_create(ctypes.byref(model), precision, ctypes.byref(self._ctx)), "pf_create")

    @classmethod
    def read_data(cls, config_path: str, precision: int = PF_PREC_FP64) -> "PhaseField":
        """phase_field::Read_data (phase_field.cpp:166-366)."""
        return cls(read_model(config_path), precision)

    @property
    def N(self) -> int:
        return self.model.ix * self.model.iy * self.model.iz

    def close(self) -> None:
        if self._ctx:
            lib().pf_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, state: dict, time: float) -> None:
        check(lib().pf_upload_state(self._ctx, _ptr(state["ids"]), _ptr(state["phi"]), _ptr(state["phase"]),
                                    _ptr(state.get("conc")), _ptr(state["C"]), time), "pf_upload_state")

    def set_coherent_grains(self, partners: np.ndarray) -> None:
        """Coherent ferrite partners of austenite grains 200001, 200002, ...
        (int32 [n, 2], 0 = none) for the coherent-grain mobility."""
        p = np.ascontiguousarray(partners, dtype=np.int32).reshape(-1, 2)
        check(lib().pf_set_coherent_grains(self._ctx, _ptr(p), p.shape[0]), "pf_set_coherent_grains")

    def construct_on_device(self, spec: PfInitSpec, time: float | None = None) -> None:
        """The seeded initial state generated on the GPU, straight into the
        context (pf_init_device): no host arrays, no upload."""
        t = self.model.T_time[0] if time is None else time
        check(lib().pf_init_device(self._ctx, ctypes.byref(spec), t), "pf_init_device")

    def construct(self, spec: PfInitSpec, time: float | None = None) -> dict:
        """Seeded replacement of Construct + Nucleate1in2; uploads and returns the state."""
        t = self.model.T_time[0] if time is None else time
        st = init_microstructure(self.model, spec, t)
        self.upload(st, t)
        return st

    def update(self, nsteps: int = 1) -> None:
        """phase_field::Update(false) nsteps times (phase_field.cpp:243-305)."""
        check(lib().pf_step(self._ctx, nsteps), "pf_step")

    def diffuse(self, nsub: int) -> None:
        """Only the diffusion sub-cycle (phases fixed, time not advanced)."""
        check(lib().pf_diffuse(self._ctx, nsub), "pf_diffuse")

    def synchronize(self) -> None:
        check(lib().pf_synchronize(self._ctx), "pf_synchronize")

    def download(self, conc: bool = True) -> dict:
        st = empty_state(self.model)
        t = ctypes.c_double()
        check(lib().pf_download_state(self._ctx, _ptr(st["ids"]), _ptr(st["phi"]), _ptr(st["phase"]),
                                      _ptr(st["conc"]) if conc else None, _ptr(st["C"]), ctypes.byref(t)),
              "pf_download_state")
        st["time"] = t.value
        return st

    def reduce(self) -> np.ndarray:
        out = np.zeros(8, np.float64)
        check(lib().pf_reduce(self._ctx, out.ctypes.data_as(_DP)), "pf_reduce")
        return out

    def check_state(self, reference_totals=None, max_rel_drift: float = 0.0) -> int:
        """Status of pf_check_state (PF_OK, PF_ERR_NONFINITE or PF_ERR_DRIFT), without raising."""
        ref = None if reference_totals is None else np.ascontiguousarray(reference_totals, np.float64)
        return lib().pf_check_state(self._ctx, None if ref is None else ref.ctypes.data_as(_DP), max_rel_drift, None)

    def fractions(self) -> np.ndarray:
        """write_data.cpp:14-18: phase volume fractions and the deformed fraction."""
        r = self.reduce()
        return r[:4] / self.N

    @property
    def time(self) -> float:
        t = ctypes.c_double()
        check(lib().pf_get_time(self._ctx, ctypes.byref(t)), "pf_get_time")
        return t.value

    def last_params(self) -> PfStepParams:
        p = PfStepParams()
        check(lib().pf_last_params(self._ctx, ctypes.byref(p)), "pf_last_params")
        return p

    @property
    def temperature(self) -> float:
        return self.last_params().T

    @property
    def end_time(self) -> float:
        return self.model.T_time[self.model.nT - 1]

    def truncated_cells(self) -> int:
        v = ctypes.c_longlong()
        check(lib().pf_truncated_cells(self._ctx, ctypes.byref(v)), "pf_truncated_cells")
        return v.value

    def use_graph(self, on: bool = True) -> None:
        check(lib().pf_use_graph(self._ctx, int(on)), "pf_use_graph")

    def autotune(self) -> dict:
        """Pick the FP32C diffusion tile shape by timing the candidates on this state."""
        ty, zc, d, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        check(lib().pf_autotune(self._ctx, ctypes.byref(ty), ctypes.byref(zc), ctypes.byref(d), ctypes.byref(ms)),
              "pf_autotune")
        return {"tile_y": ty.value, "zchunk": zc.value, "variant": d.value, "ms": ms.value}

    def set_diffusion_tile(self, tile_y: int, zchunk: int, variant: int) -> None:
        check(lib().pf_set_diffusion_tile(self._ctx, tile_y, zchunk, variant), "pf_set_diffusion_tile")

    def diffusion_candidates(self) -> list:
        buf = (ctypes.c_int * 192)()
        n = lib().pf_diffusion_candidates(self._ctx, buf, 64)
        if n < 0:
            check(n, "pf_diffusion_candidates")
        return [(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]) for i in range(n)]

    def set_stream(self, stream_handle: int | None) -> None:
        check(lib().pf_set_stream(self._ctx, ctypes.c_void_p(stream_handle) if stream_handle else None),
              "pf_set_stream")

    def enable_kernel_timing(self, on: bool = True) -> None:
        check(lib().pf_enable_kernel_timing(self._ctx, int(on)), "pf_enable_kernel_timing")

    def kernel_times(self):
        t = (ctypes.c_double * 2)()
        n = (ctypes.c_longlong * 2)()
        check(lib().pf_kernel_times(self._ctx, t, n), "pf_kernel_times")
        return {"phase": (t[0], n[0]), "diffusion": (t[1], n[1])}

    def write_vti_binary(self, directory: str, index: int, pieces: int = 1) -> None:
        """Binary microstructure files of the current state, written by a host
        thread from device buffers while stepping continues (pf_write_vti_binary)."""
        check(lib().pf_write_vti_binary(self._ctx, directory.encode(), index, pieces), "pf_write_vti_binary")

    def write_wait(self) -> None:
        check(lib().pf_write_wait(self._ctx), "pf_write_wait")

    def write_data(self, directory: str | None = None, forced: bool = False) -> bool:  # noqa: D401
        """phase_field::Write_data (write_data.cpp:3-40)."""
        d = directory if directory is not None else self.model.directory.decode()
        w = ctypes.c_int()
        check(lib().pf_write_data(self._ctx, d.encode(), int(forced), ctypes.byref(w)), "pf_write_data")
        return bool(w.value)


class Batch:
    """Many independent 2D domains advanced by one persistent launch (pf_batch_*)."""

    def __init__(self, models: list):
        arr = (PfModel * len(models))(*models)
        self.models = list(models)
        self._b = ctypes.c_void_p()
        check(lib().pf_batch_create(arr, len(models), ctypes.byref(self._b)), "pf_batch_create")

    def close(self) -> None:
        if self._b:
            lib().pf_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, d: int, state: dict, time: float) -> None:
        check(lib().pf_batch_upload(self._b, d, _ptr(state["ids"]), _ptr(state["phi"]), _ptr(state["phase"]),
                                    _ptr(state["C"]), time), "pf_batch_upload")

    def run(self, nsteps: int) -> int:
        """Returns the status (PF_OK or PF_ERR_TIMEOUT) instead of raising on a timeout."""
        st = lib().pf_batch_run(self._b, nsteps)
        if st not in (PF_OK, PF_ERR_TIMEOUT):
            check(st, "pf_batch_run")
        return st

    def download(self, d: int) -> dict:
        st = empty_state(self.models[d])
        t = ctypes.c_double()
        check(lib().pf_batch_download(self._b, d, _ptr(st["ids"]), _ptr(st["phi"]), _ptr(st["phase"]),
                                      _ptr(st["conc"]), _ptr(st["C"]), ctypes.byref(t)), "pf_batch_download")
        st["time"] = t.value
        return st

    def reduce(self, d: int) -> np.ndarray:
        out = np.zeros(8, np.float64)
        check(lib().pf_batch_reduce(self._b, d, out.ctypes.data_as(_DP)), "pf_batch_reduce")
        return out

    def info(self) -> dict:
        v = (ctypes.c_longlong * 4)()
        check(lib().pf_batch_info(self._b, v), "pf_batch_info")
        return {"cells": v[0], "blocks": v[1], "domains": v[2], "n_sub_max": v[3]}

    def set_timeout(self, timeout_ns: int, unreachable_barrier: bool = False) -> None:
        check(lib().pf_batch_set_timeout(self._b, timeout_ns, int(unreachable_barrier)), "pf_batch_set_timeout")

    def set_tile(self, tile_y: int, occupancy_divisor: int = 1) -> None:
        check(lib().pf_batch_set_tile(self._b, tile_y, occupancy_divisor), "pf_batch_set_tile")

    def autotune(self, nsteps: int) -> dict:
        """Pick the persistent kernel's tile shape by timing each on nsteps (states restored)."""
        ty, dv, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        check(lib().pf_batch_autotune(self._b, nsteps, ctypes.byref(ty), ctypes.byref(dv), ctypes.byref(ms)),
              "pf_batch_autotune")
        return {"tile_y": ty.value, "occupancy_divisor": dv.value, "ms": ms.value}


class Adjoint:
    """Forward + hand-written adjoint of the compact step (pf_adj_*).
    checkpoint_every = 0: record mode (every step kept by the forward, the
    gradient without recomputation)."""

    def __init__(self, model: PfModel, precision: int = PF_PREC_FP64, checkpoint_every: int = 100):
        self.model = model
        self._a = ctypes.c_void_p()
        check(lib().pf_adj_create(ctypes.byref(model), precision, checkpoint_every, ctypes.byref(self._a)),
              "pf_adj_create")

    def close(self) -> None:
        if self._a:
            lib().pf_adj_destroy(self._a)
            self._a = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, state: dict, time: float) -> None:
        check(lib().pf_adj_upload(self._a, _ptr(state["ids"]), _ptr(state["phi"]), _ptr(state["phase"]),
                                  _ptr(state["C"]), time), "pf_adj_upload")

    def set_scales(self, scales) -> None:
        s = np.ascontiguousarray(scales, np.float64)
        check(lib().pf_adj_set_scales(self._a, s.ctypes.data_as(_DP)), "pf_adj_set_scales")

    def forward(self, nsteps: int) -> np.ndarray:
        J = np.zeros(2, np.float64)
        check(lib().pf_adj_forward(self._a, nsteps, J.ctypes.data_as(_DP)), "pf_adj_forward")
        return J

    def gradient(self, objective: int) -> np.ndarray:
        g = np.zeros(4, np.float64)
        check(lib().pf_adj_gradient(self._a, objective, g.ctypes.data_as(_DP)), "pf_adj_gradient")
        return g

    def final_state(self) -> dict:
        N = self.model.ix * self.model.iy * self.model.iz
        ph, C = np.zeros(3 * N), np.zeros(N)
        check(lib().pf_adj_final_state(self._a, ph.ctypes.data_as(_DP), C.ctypes.data_as(_DP)), "pf_adj_final_state")
        return {"phase": ph, "C": C}

    def timings(self) -> dict:
        t = np.zeros(2, np.float64)
        check(lib().pf_adj_timings(self._a, t.ctypes.data_as(_DP)), "pf_adj_timings")
        return {"forward_ms": float(t[0]), "gradient_ms": float(t[1])}
