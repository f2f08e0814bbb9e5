"""The seeded initial state generated on the GPU (pf_init_device) against the
host generator (pf_init_microstructure): the same per-cell code, so the grain
ids and solutes agree exactly and the phase values to a few ulp (the device's
tanh); a few FP64 steps from either start agree to the parity tolerance."""
import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import rel_maxnorm, small_case

pytestmark = pytest.mark.gpu

CASES = {
    "3d": ("3d256", (40, 36, 28), dict(n_grains=9, n_nuclei=30, radius=2.0, noise=(0.02, 0.02))),
    "2d": ("3d256", (96, 80, 1), dict(n_grains=7, n_nuclei=12, radius=3.0)),
    "cem": ("2d512cem", (64, 64, 1), dict(n_grains=5, n_nuclei=6, radius=3.0, n_particles=20)),
    "line": ("3d256", (150, 1, 1), dict(n_grains=4, n_nuclei=3, radius=2.0)),
    "slab": ("3d512", (64, 64, 16), dict(n_grains=3, n_nuclei=40, radius=2.0)),
}


@pytest.mark.parametrize("prec", [pf.PF_PREC_FP64, pf.PF_PREC_FP32C])
@pytest.mark.parametrize("case", sorted(CASES))
def test_device_init_matches_host_generator(gpu, tmp_path, prec, case):
    name, grid, kw = CASES[case]
    m, om, spec = small_case(str(tmp_path), name, grid, **kw)
    host = pf.init_microstructure(m, spec, 0.0)
    A = pf.PhaseField(m, prec)
    A.construct_on_device(spec, 0.0)
    B = pf.PhaseField(m, prec)
    B.upload(host, 0.0)
    a, b = A.download(), B.download()
    assert np.array_equal(a["ids"], b["ids"])
    tol = 1e-14 if prec == pf.PF_PREC_FP64 else 1.2e-7  # one float rounding of a value that moved by ulps
    assert float(np.max(np.abs(a["phi"] - b["phi"]))) <= tol
    assert float(np.max(np.abs(a["phase"] - b["phase"]))) <= 2 * tol
    assert np.array_equal(a["C"], b["C"])
    if prec == pf.PF_PREC_FP64:
        assert np.array_equal(a["ids"], host["ids"])
        assert rel_maxnorm(a["conc"], host["conc"]) <= 1e-13
        A.update(3)
        B.update(3)
        a, b = A.download(), B.download()
        for k in ("phi", "phase", "C"):
            assert rel_maxnorm(a[k], b[k]) <= 1e-10, k
    A.close()
    B.close()


def test_device_init_rejects_crowded_neighbourhoods(gpu, tmp_path):
    """More nuclei near one cell than the generator's per-cell list holds is
    reported (PF_ERR_RANGE), not truncated."""
    m, om, spec = small_case(str(tmp_path), "3d256", (16, 16, 16), n_grains=2, n_nuclei=400, radius=1.0)
    A = pf.PhaseField(m, pf.PF_PREC_FP64)
    assert pf.lib().pf_init_device(A._ctx, pf.ctypes.byref(spec), pf.ctypes.c_double(0.0)) == pf.PF_ERR_RANGE
    A.close()
