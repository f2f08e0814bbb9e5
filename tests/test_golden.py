"""Golden vectors from the reference's own code, reproduced by the oracle on
the CPU.

* tests/golden/ref_gpu_diffusion.npz -- the reference's CUDA diffusion kernels
  (tests/golden/make_ref_golden.py, run on a GB300): the oracle's restatement of
  GPU_Diffusion_solver matches bit-for-bit against the kernels built without
  multiply-add contraction, within 1e-12 (relative max-norm) against the
  kernels built as the reference builds them.
* tests/golden/ref_cpu_steps.npz -- full time steps of the reference's own CPU
  code (phase_field::Update, solver.cpp, thermo_data.cpp compiled unmodified
  against a minimal Blitz++ stand-in; tests/golden/make_ref_cpu_golden.py): the
  oracle's restatement matches every field bit-for-bit, on 2D, ragged six-slot,
  3D, three-phase and 1D cases.  Where the reference checkout exists, a live run
  of that library on further seeded cases is compared as well."""
import os

import numpy as np
import pytest

import pyoracle as po
from helpers import REF_CPU_CASES, REF_CPU_GOLDEN, copy_state, ref_cpu_case, rel_maxnorm, small_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_diffusion.npz")


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("golden vectors not generated yet (tests/golden/make_ref_golden.py needs a GPU)")
    return np.load(GOLDEN)


@pytest.mark.parametrize("tag", ["2d", "3d"])
def test_oracle_reproduces_reference_kernels(golden, tag):
    g = {k[len(tag) + 1:]: golden[k] for k in golden.files if k.startswith(tag + "_")}
    x, y, z = (int(v) for v in g["grid"])
    C = g["C"].copy()
    n = po.gpu_diffusion_solver(g["D"], g["k"], g["c"], g["phase"].copy(), C, x, y, z, float(g["dt"]), float(g["dx"]))
    assert n == int(g["num_loop"])
    assert np.array_equal(C, g["C_nofma"])
    assert rel_maxnorm(C, g["C_fma"]) <= 1e-12
    assert not np.array_equal(C, g["C"])  # the step did something


@pytest.fixture(scope="module")
def ref_cpu_golden():
    if not os.path.exists(REF_CPU_GOLDEN):
        pytest.fail("tests/golden/ref_cpu_steps.npz missing (tests/golden/make_ref_cpu_golden.py)")
    return np.load(REF_CPU_GOLDEN)


@pytest.mark.parametrize("name", REF_CPU_CASES)
def test_oracle_reproduces_reference_cpu_steps(ref_cpu_golden, tmp_path, name):
    cfg, st, exp = ref_cpu_case(str(tmp_path), ref_cpu_golden, name)
    om = po.load_model(cfg)
    t = po.run(om, st, 0.0, exp["steps"])
    assert t == exp["time"]
    for k in ("ids", "phi", "phase", "conc", "C"):
        assert np.array_equal(st[k], exp[k]), k
    assert not np.array_equal(st["phi"], ref_cpu_golden[f"{name}_phi0"])  # the steps did something


@pytest.mark.parametrize(
    "name,grid,steps,kw",
    [
        ("3d256", (14, 12, 9), 5, dict(n_grains=4, n_nuclei=5, radius=2.0, seed=7)),
        ("2d512cem", (40, 36, 1), 8, dict(n_grains=4, n_nuclei=3, n_particles=8, seed=3)),
        ("2d256", (33, 27, 1), 8, dict(n_grains=3, n_nuclei=4, max_slots=6, seed=11)),
    ],
)
def test_oracle_matches_reference_cpu_live(tmp_path, name, grid, steps, kw):
    """Further seeded cases against a live build of the reference's CPU code
    (only where the reference checkout exists to build it)."""
    import build_oracle
    import refcpu

    if build_oracle.build_ref_cpu() is None or not refcpu.available():
        pytest.skip("the reference checkout is not present: the golden fixture covers this")
    import phasefield_gb300 as pf

    m, om, spec = small_case(str(tmp_path), name, grid, mn=False, **kw)
    cfg = refcpu.rewrite_config(os.path.join(str(tmp_path), f"{name}_small.txt"), str(tmp_path / "out"), 0)
    st0 = pf.init_microstructure(m, spec, 0.0)
    got = refcpu.run(cfg, st0, steps)
    ref = copy_state(st0)
    t = po.run(po.load_model(cfg), ref, 0.0, steps)
    assert t == got["time"]
    for k in ("ids", "phi", "phase", "conc", "C"):
        assert np.array_equal(ref[k], got[k]), k
