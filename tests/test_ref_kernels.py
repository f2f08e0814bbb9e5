"""The reference's own CUDA diffusion kernels (GPU_Partitioning + Diff3D from
gpu_solver.cpp, built into oracle/_ref/*.cubin) against the oracle's
restatement and against this library's drop-in GPU_Diffusion_solver.

* kernels built with -fmad=false: bit-identical to the oracle and the drop-in
  (same IEEE operations in the same order);
* kernels built as the reference builds them (multiply-add contraction on):
  relative max-norm <= 1e-12 on the total carbon."""
import ctypes

import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from helpers import rel_maxnorm, small_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_kernels():
    import build_oracle

    build_oracle.build_ref()
    if not po.ref_kernels_available():
        pytest.fail("reference kernels (oracle/_ref/*.cubin) missing: build them where the reference checkout is")
    return True


@pytest.mark.parametrize("grid", [(64, 48, 1), (300, 7, 1), (20, 18, 12), (33, 17, 9)])
def test_reference_kernels_pin_oracle_and_dropin(gpu, ref_kernels, tmp_path, grid):
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=6, n_nuclei=6, radius=2.0, noise=(0.02, 0.02))
    st0 = pf.init_microstructure(m, spec, 0.0)
    P = pf.params_at(m, 0.0)
    x, y, z = grid
    N = x * y * z
    D = np.array([P.D[0][p] for p in range(3)])
    k = np.array(list(P.k[0]))
    c = np.array(list(P.c[0]))
    phase = st0["phase"].copy()
    C0 = st0["C"][:N].copy()

    C_oracle = C0.copy()
    n_o = po.gpu_diffusion_solver(D, k, c, phase, C_oracle, x, y, z, P.pfm_dt, m.dx)
    C_nofma = C0.copy()
    n_r = po.ref_gpu_diffusion_solver("nofma", D, k, c, phase, C_nofma, x, y, z, P.pfm_dt, m.dx)
    C_fma = C0.copy()
    po.ref_gpu_diffusion_solver("fma", D, k, c, phase, C_fma, x, y, z, P.pfm_dt, m.dx)
    assert n_o == n_r
    assert np.array_equal(C_nofma, C_oracle), f"max diff {np.max(np.abs(C_nofma - C_oracle))}"
    assert rel_maxnorm(C_fma, C_oracle) <= 1e-12

    L = pf.lib()
    assert L.GPU_Init(x, y, z) == 1
    C_ours = C0.copy()
    dp = ctypes.POINTER(ctypes.c_double)
    L.GPU_Diffusion_solver(D.ctypes.data_as(dp), k.ctypes.data_as(dp), c.ctypes.data_as(dp),
                           phase.ctypes.data_as(dp), C_ours.ctypes.data_as(dp), x, y, z, P.pfm_dt, m.dx)
    L.GPU_Cleanup()
    assert np.array_equal(C_ours, C_nofma)
