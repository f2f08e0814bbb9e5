"""Failure detection without any device fault: non-finite values planted in
the HOST input are reported by the statistics check, a solute drift beyond a
tolerance is reported, bad arguments are refused before anything launches."""
import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [pf.PF_PREC_FP64, pf.PF_PREC_FP32C])
def test_nonfinite_and_drift_are_reported(gpu, tmp_path, prec):
    m, _, spec = small_case(str(tmp_path), "2d256", (40, 32, 1), n_grains=4, n_nuclei=3)
    st = pf.init_microstructure(m, spec, 0.0)
    N = 40 * 32
    F = pf.PhaseField(m, prec)
    F.upload(st, 0.0)
    F.update(3)
    totals = [st["C"][:N].sum(), st["C"][N:].sum()]
    assert F.check_state(totals, 1e-6) == pf.PF_OK
    assert F.check_state([totals[0] * 1.01, totals[1]], 1e-6) == pf.PF_ERR_DRIFT  # drift beyond tolerance
    assert b"drifted" in pf.lib().pf_last_error()
    bad = {k: v.copy() for k, v in st.items()}
    bad["C"][17] = np.nan
    F.upload(bad, 0.0)
    assert F.check_state() == pf.PF_ERR_NONFINITE
    assert b"non-finite" in pf.lib().pf_last_error()


def test_bad_arguments_are_refused(gpu, tmp_path):
    m, _, _ = small_case(str(tmp_path), "2d256", (16, 16, 1))
    F = pf.PhaseField(m, pf.PF_PREC_FP32C)
    assert pf.lib().pf_step(F._ctx, 1) == pf.PF_ERR_ARG          # no state uploaded
    assert pf.lib().pf_step(F._ctx, -1) == pf.PF_ERR_ARG
    assert pf.lib().pf_set_diffusion_tile(F._ctx, 5, 8, 0) == pf.PF_ERR_ARG
    assert pf.lib().pf_set_diffusion_tile(F._ctx, 8, 8, 7) == pf.PF_ERR_ARG      # unknown kernel variant
    bad = pf.PfModel()
    bad.ix = 0
    h = pf.ctypes.c_void_p()
    assert pf.lib().pf_create(pf.ctypes.byref(bad), pf.PF_PREC_FP64, pf.ctypes.byref(h)) == pf.PF_ERR_ARG
