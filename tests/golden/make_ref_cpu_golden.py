"""Generate tests/golden/ref_cpu_steps.npz: full time steps computed by the
reference's OWN CPU code.

oracle/build_oracle.py (build_ref_cpu) compiles zhubq/PhaseField
C++-openmp-cuda/src/{phase_field,solver,thermo_data,thermo_functor,write_data}.cpp
unmodified against a minimal Blitz++ stand-in (oracle/blitz_shim) into
oracle/_ref/libpfref_cpu.so.  This script drives that library through
oracle/refcpu.py: for each case it writes a configuration in the reference's
format (carbon only, as the reference has no Mn), seeds an initial
microstructure, runs phase_field::Write_data(true), nsteps x
phase_field::Update(false), and Write_data(true) again, and stores

  <case>_config    the configuration text (its directory line is rewritten by
                   the tests), <case>_thermo the thermodynamic file text;
  <case>_ids0 ... <case>_C0   the initial state (reference layout);
  <case>_ids ... <case>_C     the state after nsteps;
  <case>_time      the reference's time after nsteps;
  <case>_fraction  the two fraction_time.txt rows it wrote;
  <case>_vti       the VTI file of the second write (cases with micro_out).

Run here, where the reference checkout exists:
    python tests/golden/make_ref_cpu_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

OUT = os.path.join(HERE, "ref_cpu_steps.npz")

# name, workload, grid, steps, micro_out, init overrides
CASES = [
    ("2d", "2d256", (40, 32, 1), 12, 1, dict(n_grains=5, n_nuclei=4)),
    ("ragged6", "2d256", (29, 21, 1), 10, 0, dict(n_grains=4, n_nuclei=3, max_slots=6)),
    ("3d", "3d256", (16, 12, 10), 6, 1, dict(n_grains=5, n_nuclei=6, radius=2.0, noise=(0.02, 0.0))),
    ("cem", "2d512cem", (48, 48, 1), 10, 0, dict(n_grains=5, n_nuclei=4, n_particles=6)),
    ("line", "2d256", (96, 1, 1), 15, 0, dict(n_grains=3, n_nuclei=2)),
]


def make() -> str:
    import build_oracle
    import refcpu

    import phasefield_gb300 as pf
    from helpers import small_case

    if build_oracle.build_ref_cpu() is None:
        raise SystemExit("the reference checkout is needed to build oracle/_ref/libpfref_cpu.so")
    out = {}
    for name, wl, grid, steps, micro, kw in CASES:
        with tempfile.TemporaryDirectory() as tmp:
            m, _, spec = small_case(tmp, wl, grid, mn=False, **kw)
            cfg = refcpu.rewrite_config(os.path.join(tmp, f"{wl}_small.txt"), os.path.join(tmp, "out"), micro)
            st0 = pf.init_microstructure(m, spec, 0.0)
            res = refcpu.run(cfg, st0, steps, write=True)
            out[f"{name}_config"] = np.array(open(cfg).read())
            out[f"{name}_thermo"] = np.array(open(os.path.join(tmp, "thermo_steel.txt")).read())
            out[f"{name}_steps"] = np.array(steps)
            for k in ("ids", "phi", "phase", "conc", "C"):
                out[f"{name}_{k}0"] = st0[k][: res[k].size].copy()
                out[f"{name}_{k}"] = res[k]
            out[f"{name}_time"] = np.array(res["time"])
            out[f"{name}_fraction"] = np.array(res["fraction"])
            if micro:
                out[f"{name}_vti"] = np.array(res["vti"])
    np.savez_compressed(OUT, **out)
    return OUT


if __name__ == "__main__":
    print(make())
