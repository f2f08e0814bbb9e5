"""Generate tests/golden/ref_gpu_diffusion.npz from the reference itself.

Runs the reference's own CUDA diffusion plug-in kernels (GPU_Partitioning and
Diff3D from zhubq/PhaseField C++-openmp-cuda/src/gpu_solver.cpp, compiled
into oracle/_ref/*.cubin by oracle/build_oracle.py) on small seeded states and
stores inputs and outputs.  Needs a GPU and the cubins:

    python tests/golden/make_ref_golden.py

Two outputs per case: the kernels built with nvcc's default multiply-add
contraction ("fma", how the reference builds them) and with -fmad=false
("nofma", the same arithmetic as the reference's CPU solver).
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import phasefield_gb300 as pf  # noqa: E402
import pyoracle as po  # noqa: E402
from phasefield_gb300 import workloads as W  # noqa: E402

CASES = [("2d", (32, 24, 1), 7), ("3d", (12, 10, 8), 11)]


def make_inputs(grid, seed):
    with tempfile.TemporaryDirectory() as d:
        W.write_thermo(os.path.join(d, "thermo_steel.txt"))
        cfg = W.write_config(os.path.join(d, "g.txt"), grid=grid, T=1013.0)
        m = pf.read_model(cfg)
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.seed = 4, 3, seed
    spec.nucleus_radius = 2.0
    st = pf.init_microstructure(m, spec, 0.0)
    P = pf.params_at(m, 0.0)
    N = grid[0] * grid[1] * grid[2]
    return {
        "phase": st["phase"], "C": st["C"][:N].copy(),
        "D": np.array([P.D[0][p] for p in range(3)]), "k": np.array(list(P.k[0])), "c": np.array(list(P.c[0])),
        "dt": np.float64(P.pfm_dt), "dx": np.float64(m.dx), "grid": np.array(grid, np.int64),
    }


def main():
    out = {}
    for tag, grid, seed in CASES:
        inp = make_inputs(grid, seed)
        for k, v in inp.items():
            out[f"{tag}_{k}"] = v
        x, y, z = grid
        for variant in ("fma", "nofma"):
            C = inp["C"].copy()
            n = po.ref_gpu_diffusion_solver(variant, inp["D"], inp["k"], inp["c"], inp["phase"], C, x, y, z,
                                            float(inp["dt"]), float(inp["dx"]))
            out[f"{tag}_C_{variant}"] = C
            out[f"{tag}_num_loop"] = np.int64(n)
    path = os.path.join(HERE, "ref_gpu_diffusion.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
