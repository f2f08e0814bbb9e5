"""Golden vectors produced by the reference's own CUDA diffusion kernels
(tests/golden/make_ref_golden.py, run on a GB300): the oracle's restatement of
GPU_Diffusion_solver must reproduce them on the CPU -- bit-for-bit against the
kernels built without multiply-add contraction, within 1e-12 (relative
max-norm) against the kernels built as the reference builds them."""
import os

import numpy as np
import pytest

import pyoracle as po
from helpers import rel_maxnorm

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
