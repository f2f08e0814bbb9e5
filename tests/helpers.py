"""Shared helpers for the tests: small workloads built from the packaged
configs, and comparisons between the product's GPU state and the oracle's."""
from __future__ import annotations

import os

import numpy as np

import phasefield_gb300 as pf
import pyoracle as po
from phasefield_gb300 import workloads as W


def small_case(tmpdir: str, name: str, grid, *, T=None, n_grains=None, n_nuclei=None, radius=None,
               n_particles=None, noise=None, seed=0, max_slots=4, mn=True, C0=None):
    """A reduced copy of a packaged workload: returns (pf_model, oracle_model, spec)."""
    wl = W.WORKLOADS[name]
    os.makedirs(tmpdir, exist_ok=True)
    W.write_thermo(os.path.join(tmpdir, "thermo_steel.txt"))
    cfg = W.write_config(os.path.join(tmpdir, f"{name}_small.txt"), grid=grid, dx=wl.dx,
                         T=wl.T if T is None else T, mn=mn, directory=os.path.join(tmpdir, "out"))
    m = pf.read_model(cfg)
    om = po.load_model(cfg)
    spec = wl.spec()
    if n_grains is not None:
        spec.n_grains = n_grains
    if n_nuclei is not None:
        spec.n_nuclei = n_nuclei
    if radius is not None:
        spec.nucleus_radius = radius
    if n_particles is not None:
        spec.n_particles = n_particles
    if noise is not None:
        spec.C_noise[0], spec.C_noise[1] = noise
    if C0 is not None:
        spec.C0[0], spec.C0[1] = C0
    spec.seed = seed
    spec.max_slots = max_slots
    return m, om, spec


def copy_state(st: dict) -> dict:
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}


def rel_maxnorm(a: np.ndarray, b: np.ndarray) -> float:
    """max|a-b| / max(max|b|, tiny): the relative max-norm used for parity."""
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


REF_CPU_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cpu_steps.npz")
REF_CPU_CASES = ("2d", "ragged6", "3d", "cem", "line")


def ref_cpu_case(tmpdir: str, golden, name: str):
    """One case of tests/golden/ref_cpu_steps.npz (outputs of the reference's own
    CPU code): writes its configuration (output folder moved under tmpdir) and
    thermodynamic file, and returns (config path, initial state, expected)."""
    os.makedirs(tmpdir, exist_ok=True)
    lines = str(golden[f"{name}_config"]).splitlines()
    lines[1] = os.path.join(tmpdir, "out")
    os.makedirs(lines[1], exist_ok=True)
    cfg = os.path.join(tmpdir, f"{name}.txt")
    with open(cfg, "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(tmpdir, "thermo_steel.txt"), "w") as f:
        f.write(str(golden[f"{name}_thermo"]))
    st0 = {k: golden[f"{name}_{k}0"].copy() for k in ("ids", "phi", "phase", "conc", "C")}
    exp = {k: golden[f"{name}_{k}"] for k in ("ids", "phi", "phase", "conc", "C")}
    exp["time"] = float(golden[f"{name}_time"])
    exp["steps"] = int(golden[f"{name}_steps"])
    exp["fraction"] = str(golden[f"{name}_fraction"])
    exp["vti"] = str(golden[f"{name}_vti"]) if f"{name}_vti" in golden.files else None
    return cfg, st0, exp


def adjacent_partners(ids, phi, n_nuclei, cutoff):
    """A coherent-partner table that makes every nucleus coherent with the
    (up to two largest) ferrite grains it shares a cell with in 'ids' -- a
    table under which the coherent mobility acts on most interfaces."""
    I = ids.reshape(-1, 6)
    V = phi.reshape(-1, 6)
    sets = [set() for _ in range(n_nuclei)]
    for row, val in zip(I, V):
        live = [int(g) for g, v in zip(row, val) if v > cutoff]
        fer = [g for g in live if g // 100000 == 1]
        for g in live:
            if g // 100000 == 2 and g - 200001 < n_nuclei:
                sets[g - 200001].update(fer)
    out = np.zeros((n_nuclei, 2), np.int32)
    for n, s_ in enumerate(sets):
        top = sorted(s_, reverse=True)[:2]
        out[n, : len(top)] = top
    return out
