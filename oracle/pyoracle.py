"""ctypes binding of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU legs.  It
also carries an independent restatement of the reference's positional
configuration / thermodynamic readers (phase_field.cpp:166-330,
thermo_functor.cpp:11-53) so the oracle never depends on the product's parser.

Pinned against the reference's own code: full time steps of its CPU path
(built unmodified against the minimal Blitz++ stand-in, oracle/blitz_shim) and
its CUDA partition + diffusion kernels, through the golden files of
tests/golden (see build_oracle.py).
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
MAXT = 64
_d9 = ctypes.c_double * 9
_d3 = ctypes.c_double * 3


class OModel(ctypes.Structure):
    _fields_ = [
        ("ix", ctypes.c_int), ("iy", ctypes.c_int), ("iz", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("i_intf", ctypes.c_int),
        ("cutoff", ctypes.c_double),
        ("nT", ctypes.c_int),
        ("T_time", ctypes.c_double * MAXT), ("T_temp", ctypes.c_double * MAXT),
        ("m0", _d9), ("mQ", _d9), ("sigma", _d9),
        ("nsol", ctypes.c_int),
        ("D0", _d3 * 2), ("DQ", _d3 * 2),
        ("ent_a", _d9), ("ent_b", _d9),
        ("eq_a", _d9), ("eq_b", _d9), ("eq_c", _d9),
        ("mn_ratio", _d3),
        ("thermo_model", ctypes.c_int),
        ("avg_carbon", ctypes.c_int),
        ("drag", ctypes.c_int),
        ("drag_binding", ctypes.c_double), ("drag_vmax0", ctypes.c_double), ("drag_qsd", ctypes.c_double),
        ("coherent", ctypes.c_int), ("coh_npp0", ctypes.c_int),
    ]


class OParams(ctypes.Structure):
    _fields_ = [
        ("T", ctypes.c_double),
        ("m", _d9),
        ("D", _d3 * 2),
        ("pfm_dt", ctypes.c_double), ("diff_dt", ctypes.c_double),
        ("n_sub", ctypes.c_int),
        ("dt_sub", ctypes.c_double),
        ("entropy", _d9), ("eq", _d9), ("dcdT", _d9),
        ("k", _d9 * 2), ("c", _d9 * 2),
        ("dims", ctypes.c_double), ("eta", ctypes.c_double),
        ("df_model", ctypes.c_int),
        ("df_ratio", _d9), ("df_ref", ctypes.c_double),
        ("avg_range", ctypes.c_int), ("avg_conc", ctypes.c_int),
        ("drag_model", ctypes.c_int),
        ("drag_vmax", ctypes.c_double), ("drag_ex0", ctypes.c_double), ("drag_de_heat", ctypes.c_double),
        ("drag_de_cool", ctypes.c_double), ("drag_u0", ctypes.c_double),
        ("drag_corr", ctypes.c_double * 2), ("drag_drag0", ctypes.c_double * 2),
        ("coh_model", ctypes.c_int), ("coh_npp0", ctypes.c_int),
    ]


class OInitSpec(ctypes.Structure):
    """Layout of pf_init_spec (include/pfstep.h): the seeded input generator's spec."""
    _fields_ = [
        ("seed", ctypes.c_uint64), ("n_grains", ctypes.c_int), ("n_nuclei", ctypes.c_int),
        ("nucleus_radius", ctypes.c_double), ("n_particles", ctypes.c_int), ("particle_radius", ctypes.c_double),
        ("width", ctypes.c_double), ("C0", ctypes.c_double * 2), ("C_noise", ctypes.c_double * 2),
        ("max_slots", ctypes.c_int),
    ]


class OState(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("ids1", "ids2", "phi1", "phi2", "phase", "conc1", "conc2", "C")]


_lib = None
_P = ctypes.c_void_p
_D = ctypes.c_double


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run oracle/build_oracle.py (or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        M, PP = ctypes.POINTER(OModel), ctypes.POINTER(OParams)
        L.pfo_params_at.argtypes = [M, _D, PP]
        L.pfo_params_at.restype = None
        L.pfo_partition_all.argtypes = [M, PP, _P, _P, _P]
        L.pfo_phase_sweep.argtypes = [M, PP, _P, _P, _P, _P, _P, _P, _P]
        L.pfo_avg_conc.argtypes = [M, PP, _P, _P, _P, _P, _P]
        L.pfo_set_coherent.argtypes = [_P, ctypes.c_int]
        L.pfo_set_coherent.restype = None
        L.pfo_diffusion_substep.argtypes = [M, PP, _D, _P, _P, _P, _P]
        L.pfo_run.argtypes = [M, ctypes.POINTER(OState), ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.pfo_gpu_diffusion_solver.argtypes = [_P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                               _D, _D, _P]
        L.pfo_gpu_diffusion_solver.restype = ctypes.c_int
        L.pfo_fractions.argtypes = [M, _P, _P, _P, _P]
        L.pfo_temperature.argtypes = [M, _D]
        L.pfo_temperature.restype = _D
        L.pf_init_state.argtypes = [ctypes.c_int] * 4 + [_D, ctypes.POINTER(OInitSpec), _P, _P, ctypes.c_int,
                                                          ctypes.c_int, _P, _P, _P, _P, _P,
                                                          ctypes.POINTER(ctypes.c_char_p)]
        L.pf_init_state.restype = ctypes.c_int
        L.pfo_num_threads.restype = ctypes.c_int
        L.pfo_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# Positional readers, restated from the reference's iostream usage.
# --------------------------------------------------------------------------
_FLOAT = re.compile(r"[+-]?(?:\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)")
_INT = re.compile(r"[+-]?\d+")


class _Stream:
    """Minimal istream: ignore(1000,'\\n'), getline, operator>> for int/double."""

    def __init__(self, text: str):
        self.t = text
        self.p = 0

    def ignore(self, n: int = 1) -> None:
        for _ in range(n):
            j = self.t.find("\n", self.p)
            self.p = len(self.t) if j < 0 else j + 1

    def getline(self) -> str:
        j = self.t.find("\n", self.p)
        if j < 0:
            s, self.p = self.t[self.p:], len(self.t)
        else:
            s, self.p = self.t[self.p:j], j + 1
        return s

    def _skipws(self) -> None:
        while self.p < len(self.t) and self.t[self.p].isspace():
            self.p += 1

    def read(self, kind=float):
        self._skipws()
        m = (_INT if kind is int else _FLOAT).match(self.t, self.p)
        if not m:
            raise ValueError(f"cannot read {kind.__name__} at offset {self.p}")
        self.p = m.end()
        return kind(m.group(0))


def _e(i: int, j: int) -> int:
    return (i - 1) + 3 * (j - 1)


def parse_thermo(path: str, out: dict) -> None:
    text = open(path).read()
    for k in ("ent_a", "ent_b", "eq_a", "eq_b", "eq_c"):
        out[k] = [0.0] * 9
    out["thermo_model"] = 0
    out["avg_carbon"] = 0
    out["drag"] = 0
    out["coherent"] = 0
    if text.split()[:1] == ["F90_POLYNOMIAL"]:  # the Fortran model's built-in polynomials
        out["thermo_model"] = 1
        for line in text.splitlines()[1:]:
            words = line.split()
            if not words or words[0].startswith("#"):
                continue
            if words[0] == "AVERAGED_INTERFACE_CARBON":
                out["avg_carbon"] = 1
            elif words[0] == "SOLUTE_DRAG":
                out["drag"] = 1
                out["drag_binding"], out["drag_vmax0"], out["drag_qsd"] = (float(w) for w in words[1:4])
            elif words[0] == "COHERENT_MOBILITY":
                out["coherent"] = 1
                out["coh_npp0"] = int(words[1])
            else:
                raise ValueError(f"thermo file: unknown keyword {words[0]}")
        return
    s = _Stream(text)
    s.ignore(3)
    for _ in range(3):
        i, j = s.read(int), s.read(int)
        a, b = s.read(), s.read()
        out["ent_a"][_e(i, j)], out["ent_b"][_e(i, j)] = a, b
        out["ent_a"][_e(j, i)], out["ent_b"][_e(j, i)] = -a, -b
    s.ignore(4)
    for _ in range(6):
        [s.read(int), s.read(int), s.read(), s.read(), s.read()]
    s.ignore(2)
    for _ in range(6):
        [s.read(int), s.read(int), s.read(), s.read(), s.read()]
    s.ignore(2)
    for _ in range(6):
        i, j = s.read(int), s.read(int)
        out["eq_a"][_e(i, j)], out["eq_b"][_e(i, j)], out["eq_c"][_e(i, j)] = s.read(), s.read(), s.read()


def parse_config(path: str) -> dict:
    s = _Stream(open(path).read())
    d: dict = {}
    s.ignore(1)
    d["directory"] = s.getline()
    s.ignore(3)
    d["ix"], d["iy"], d["iz"] = s.read(int), s.read(int), s.read(int)
    s.ignore(2); d["dx"] = s.read()
    s.ignore(2); d["i_intf"] = s.read(int)
    s.ignore(2); d["cutoff"] = s.read()
    s.ignore(2); d["num_grain"] = [s.read(int) for _ in range(3)]
    s.ignore(2); d["phase_fraction"] = [s.read() for _ in range(3)]
    s.ignore(2); d["init_conc"] = [s.read() for _ in range(3)]
    s.ignore(2); nT = s.read(int)
    d["T_path"] = [(s.read(), s.read()) for _ in range(nT)]
    s.ignore(2); d["reduction"] = s.read()
    s.ignore(2); d["num_init_iteration"] = s.read(int)
    s.ignore(2); d["timestep_output"] = s.read()
    s.ignore(2); d["micro_out"] = s.read(int)
    s.ignore(2); d["num_nuclei"] = s.read()
    m0, mQ, sig = [0.0] * 9, [0.0] * 9, [0.0] * 9
    for i in range(1, 4):
        for j in range(i, 4):
            s.ignore(2)
            m0[_e(i, j)], mQ[_e(i, j)] = s.read(), s.read()
            m0[_e(j, i)], mQ[_e(j, i)] = m0[_e(i, j)], mQ[_e(i, j)]
    for i in range(1, 4):
        for j in range(i, 4):
            s.ignore(2)
            sig[_e(i, j)] = s.read()
            sig[_e(j, i)] = sig[_e(i, j)]
    d["m0"], d["mQ"], d["sigma"] = m0, mQ, sig
    D0, DQ = [[0.0] * 3, [0.0] * 3], [[0.0] * 3, [0.0] * 3]
    for i in range(3):
        s.ignore(2)
        D0[0][i], DQ[0][i] = s.read(), s.read()
    s.ignore(2)
    d["thermo_file"] = s.getline()
    s.ignore(1)
    d["gpu_flag"] = s.read(int)
    d["nsol"], d["mn_ratio"] = 1, [1.0, 1.0, 1.0]
    try:  # optional Mn extension
        dm, qm = [0.0] * 3, [0.0] * 3
        for i in range(3):
            s.ignore(2)
            dm[i], qm[i] = s.read(), s.read()
        s.ignore(2)
        r = [s.read() for _ in range(3)]
        D0[1], DQ[1], d["mn_ratio"], d["nsol"] = dm, qm, r, 2
    except ValueError:
        pass
    d["D0"], d["DQ"] = D0, DQ
    tf = d["thermo_file"]
    if not os.path.exists(tf):
        tf = os.path.join(os.path.dirname(os.path.abspath(path)), tf)
    parse_thermo(tf, d)
    return d


def model_from_dict(d: dict) -> OModel:
    m = OModel()
    m.ix, m.iy, m.iz = d["ix"], d["iy"], d["iz"]
    m.dx, m.i_intf, m.cutoff = d["dx"], d["i_intf"], d["cutoff"]
    m.nT = len(d["T_path"])
    for k, (t, T) in enumerate(d["T_path"]):
        m.T_time[k], m.T_temp[k] = t, T
    for k in ("m0", "mQ", "sigma", "ent_a", "ent_b", "eq_a", "eq_b", "eq_c", "mn_ratio"):
        arr = getattr(m, k)
        for e, v in enumerate(d[k]):
            arr[e] = v
    m.nsol = d["nsol"]
    m.thermo_model = d.get("thermo_model", 0)
    m.avg_carbon = d.get("avg_carbon", 0)
    m.drag = d.get("drag", 0)
    if m.drag:
        m.drag_binding, m.drag_vmax0, m.drag_qsd = d["drag_binding"], d["drag_vmax0"], d["drag_qsd"]
    m.coherent = d.get("coherent", 0)
    m.coh_npp0 = d.get("coh_npp0", 0)
    for q in range(2):
        for p in range(3):
            m.D0[q][p], m.DQ[q][p] = d["D0"][q][p], d["DQ"][q][p]
    return m


def load_model(config_path: str, grid=None) -> OModel:
    d = parse_config(config_path)
    if grid is not None:
        d["ix"], d["iy"], d["iz"] = grid
    return model_from_dict(d)


def params_at(m: OModel, time: float) -> OParams:
    p = OParams()
    lib().pfo_params_at(ctypes.byref(m), time, ctypes.byref(p))
    return p


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def run(m: OModel, state: dict, time: float, nsteps: int) -> float:
    """phase_field::Update(false) x nsteps on copies of the reference-layout arrays.
    Mutates ``state`` in place (ids, phi, phase, conc, C); returns the new time."""
    st = OState()
    scratch_ids = np.zeros_like(state["ids"])
    scratch_phi = np.zeros_like(state["phi"])
    scratch_conc = np.zeros_like(state["conc"])
    st.ids1, st.ids2 = state["ids"].ctypes.data, scratch_ids.ctypes.data
    st.phi1, st.phi2 = state["phi"].ctypes.data, scratch_phi.ctypes.data
    st.phase = state["phase"].ctypes.data
    st.conc1, st.conc2 = state["conc"].ctypes.data, scratch_conc.ctypes.data
    st.C = state["C"].ctypes.data
    t = ctypes.c_double(time)
    lib().pfo_run(ctypes.byref(m), ctypes.byref(st), ctypes.byref(t), nsteps)
    return t.value


def partition_all(m: OModel, p: OParams, phase, C, conc) -> None:
    lib().pfo_partition_all(ctypes.byref(m), ctypes.byref(p), _ptr(phase), _ptr(C), _ptr(conc))


def phase_sweep(m: OModel, p: OParams, ids1, phi1, ids2, phi2, phase, conc1, C) -> None:
    lib().pfo_phase_sweep(ctypes.byref(m), ctypes.byref(p), _ptr(ids1), _ptr(phi1), _ptr(ids2), _ptr(phi2),
                          _ptr(phase), _ptr(conc1), _ptr(C))


def exp_log(x: np.ndarray):
    """The shared pf_exp/pf_log of the drag solve, element-wise."""
    L = lib()
    L.pfo_exp.restype = L.pfo_log.restype = ctypes.c_double
    L.pfo_exp.argtypes = L.pfo_log.argtypes = [ctypes.c_double]
    x = np.asarray(x, dtype=np.float64).ravel()
    return np.array([L.pfo_exp(float(v)) for v in x]), np.array([L.pfo_log(float(v)) for v in x])


def dissipation(p: OParams, unchanged: float, driv: float, drag: float, norm: float, heating: int) -> float:
    """The oracle's DISSIPATION_ITERATION (heating = 1) / _R (0) for one entry."""
    L = lib()
    L.pfo_dissipation.restype = ctypes.c_double
    L.pfo_dissipation.argtypes = [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.POINTER(OParams)]
    return L.pfo_dissipation(unchanged, driv, drag, norm, heating, ctypes.byref(p))


def drag_failures(clear: bool = True) -> int:
    """Whether a solute-drag iteration found no root since the last call."""
    v = ctypes.c_int.in_dll(lib(), "pfo_drag_failures")
    out = v.value
    if clear:
        v.value = 0
    return out


def avg_conc(m: OModel, p: OParams, phase, conc1, ids=None, with_flags: bool = False):
    """The interface-averaged phase concentrations of every cell (sparse.f90:184-255);
    with_flags (needs ids): also the scan's Has_ferrite (bit 0) / Rex_intf (bit 1) bytes."""
    N = m.ix * m.iy * m.iz
    out = np.zeros_like(conc1[: 3 * N])
    flags = np.zeros(N, np.uint8) if with_flags else None
    ids = np.zeros(6 * N, np.int32) if ids is None else ids
    lib().pfo_avg_conc(ctypes.byref(m), ctypes.byref(p), _ptr(ids), _ptr(phase), _ptr(conc1), _ptr(out),
                       _ptr(flags))
    return (out, flags) if with_flags else out


def set_coherent(partners) -> None:
    """Coherent_grain of the oracle: partners[n] = the two ferrite ids coherent
    with austenite grain 200001 + n (None clears)."""
    if partners is None:
        lib().pfo_set_coherent(None, 0)
        return
    p = np.ascontiguousarray(partners, dtype=np.int32).reshape(-1, 2)
    lib().pfo_set_coherent(_ptr(p), p.shape[0])


def diffusion_substep(m: OModel, p: OParams, dt_sub, phase, conc1, conc2, C) -> None:
    lib().pfo_diffusion_substep(ctypes.byref(m), ctypes.byref(p), dt_sub, _ptr(phase), _ptr(conc1), _ptr(conc2),
                                _ptr(C))


def gpu_diffusion_solver(D3, k9, c9, phase, C, x, y, z, dt, dx, conc_out=None) -> int:
    """Restatement of the reference plug-in's GPU_Diffusion_solver; C updated in place."""
    D3 = np.ascontiguousarray(D3, np.float64)
    k9 = np.ascontiguousarray(k9, np.float64)
    c9 = np.ascontiguousarray(c9, np.float64)
    return lib().pfo_gpu_diffusion_solver(_ptr(D3), _ptr(k9), _ptr(c9), _ptr(phase), _ptr(C), x, y, z, dt, dx,
                                          _ptr(conc_out))


def fractions(m: OModel, ids, phi, phase) -> np.ndarray:
    out = np.zeros(4, np.float64)
    lib().pfo_fractions(ctypes.byref(m), _ptr(ids), _ptr(phi), _ptr(phase), _ptr(out))
    return out


RUNNER_PATH = os.path.join(HERE, "_build", "libref_runner.so")
REF_CUBINS = {"fma": os.path.join(HERE, "_ref", "gpu_solver_ref.cubin"),
              "nofma": os.path.join(HERE, "_ref", "gpu_solver_ref_nofma.cubin")}
_runner = None


def ref_kernels_available() -> bool:
    return all(os.path.exists(p) for p in REF_CUBINS.values())


def ref_gpu_diffusion_solver(variant, D3, k9, c9, phase, C, x, y, z, dt, dx) -> int:
    """Run the reference's own GPU_Partitioning/Diff3D kernels (cubin built from
    gpu_solver.cpp) under the host loop of GPU_Diffusion_solver; C in place."""
    global _runner
    if _runner is None:
        import build_oracle

        build_oracle.build_ref_runner()
        R = ctypes.CDLL(RUNNER_PATH)
        R.ref_gpu_diffusion_solver.argtypes = [ctypes.c_char_p, _P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, _D, _D]
        R.ref_gpu_diffusion_solver.restype = ctypes.c_int
        R.ref_last_error.restype = ctypes.c_char_p
        _runner = R
    D3 = np.ascontiguousarray(D3, np.float64)
    k9 = np.ascontiguousarray(k9, np.float64)
    c9 = np.ascontiguousarray(c9, np.float64)
    n = _runner.ref_gpu_diffusion_solver(REF_CUBINS[variant].encode(), _ptr(D3), _ptr(k9), _ptr(c9), _ptr(phase),
                                         _ptr(C), x, y, z, dt, dx)
    if n < 0:
        raise RuntimeError("reference kernels: " + _runner.ref_last_error().decode())
    return n


def init_state(m: OModel, spec, time: float, grid=None, z0: int = 0, nz: int | None = None) -> dict:
    """The seeded input state (reference layout) of planes [z0, z0+nz) of the
    periodic domain 'grid' (default: the model's grid), generated by the same
    source as the product's pf_init_microstructure.  'spec' is any object with
    the fields of pf_init_spec.  conc is partitioned with the model's
    parameters at 'time'."""
    ix, iy, iz = grid if grid is not None else (m.ix, m.iy, m.iz)
    nz = iz - z0 if nz is None else nz
    s = OInitSpec()
    for f, _ in OInitSpec._fields_:
        v = getattr(spec, f)
        if f in ("C0", "C_noise"):
            for q in range(2):
                getattr(s, f)[q] = v[q]
        else:
            setattr(s, f, v)
    p = params_at(m, time)
    k = np.array([[p.k[q][e] for e in range(9)] for q in range(2)], np.float64)
    c = np.array([[p.c[q][e] for e in range(9)] for q in range(2)], np.float64)
    N = ix * iy * nz
    st = {"ids": np.zeros(6 * N, np.int32), "phi": np.zeros(6 * N, np.float64), "phase": np.zeros(3 * N, np.float64),
          "conc": np.zeros(3 * N * m.nsol, np.float64), "C": np.zeros(N * m.nsol, np.float64)}
    msg = ctypes.c_char_p()
    rc = lib().pf_init_state(ix, iy, iz, m.nsol, m.cutoff, ctypes.byref(s), _ptr(k), _ptr(c), z0, nz,
                             _ptr(st["ids"]), _ptr(st["phi"]), _ptr(st["phase"]), _ptr(st["conc"]), _ptr(st["C"]),
                             ctypes.byref(msg))
    if rc != 0:
        raise RuntimeError("pf_init_state: " + (msg.value or b"failed").decode())
    return st


def set_threads(n: int) -> None:
    lib().pfo_set_num_threads(n)


def num_threads() -> int:
    return lib().pfo_num_threads()
