"""The product's FP64 path on the GPU against full time steps of the
reference's OWN CPU code (tests/golden/ref_cpu_steps.npz: phase_field::Update,
solver.cpp and thermo_data.cpp compiled unmodified against a minimal Blitz++
stand-in, see tests/golden/make_ref_cpu_golden.py).

Tolerance: bit-identical -- every grain id, phase-field value, phase
fraction, phase concentration and total concentration, and the time, after
the recorded number of steps (the FP64 kernels are built without multiply-add
contraction).  The fraction_time.txt rows and the VTI file written through
pf_write_data are compared as text with the reference's Write_data output."""
import glob
import os

import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import REF_CPU_CASES, REF_CPU_GOLDEN, ref_cpu_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(REF_CPU_GOLDEN):
        pytest.fail("tests/golden/ref_cpu_steps.npz missing")
    return np.load(REF_CPU_GOLDEN)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", REF_CPU_CASES)
def test_fp64_step_matches_reference_cpu(gpu, golden, tmp_path, name, graph):
    cfg, st0, exp = ref_cpu_case(str(tmp_path), golden, name)
    m = pf.read_model(cfg)
    assert m.nsol == 1
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.use_graph(graph)
    F.upload(st0, 0.0)
    F.update(exp["steps"])
    got = F.download()
    F.close()
    assert got["time"] == exp["time"]
    for k in ("ids", "phi", "phase", "conc", "C"):
        assert np.array_equal(got[k], exp[k]), k


@pytest.mark.parametrize("name", [n for n in REF_CPU_CASES])
def test_write_data_matches_reference_text(gpu, golden, tmp_path, name):
    cfg, st0, exp = ref_cpu_case(str(tmp_path), golden, name)
    m = pf.read_model(cfg)
    out = os.path.join(str(tmp_path), "out")
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    assert F.write_data(out, forced=True)
    F.update(exp["steps"])
    assert F.write_data(out, forced=True)
    F.close()
    assert open(os.path.join(out, "fraction_time.txt")).read() == exp["fraction"]
    if exp["vti"] is not None:
        vtis = sorted(glob.glob(os.path.join(out, "field*_*.vti")),
                      key=lambda p: int(os.path.basename(p)[:-4].rsplit("_", 1)[1]))
        assert len(vtis) == 2
        assert open(vtis[-1]).read() == exp["vti"]
