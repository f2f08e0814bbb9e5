"""Diffusion sub-cycle alone (phases fixed): the FP64 kernel against the
oracle's Diffusion_solver (solver.cpp:343-372), bit-for-bit, and the tiled FP32
compensated kernel against the FP64 kernel.  The FP32 tolerance is written in
the test: relative max-norm of the total concentration <= 2e-6 after 20
sub-steps (FP32 rounding of the partitioned concentrations; no discrete
decisions are involved)."""
import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from helpers import copy_state, rel_maxnorm, small_case

pytestmark = pytest.mark.gpu

GRIDS = [
    (64, 48, 1),     # 2D, tile multiple in x
    (37, 23, 1),     # 2D ragged
    (20, 18, 12),    # 3D ragged
    (64, 40, 33),    # 3D, z not a chunk multiple
    (40, 36, 2),     # 3D with iz = 2 (z neighbours coincide)
    (200, 1, 1),     # 1D
    (48, 1, 20),     # iy = 1 with iz > 1: two dimensions x, y (y wraps to itself)
]


def _oracle_diffuse(om, st, time, nsub):
    p = po.params_at(om, time)
    conc_a, conc_b = st["conc"], np.zeros_like(st["conc"])
    for _ in range(nsub):
        po.diffusion_substep(om, p, p.dt_sub, st["phase"], conc_a, conc_b, st["C"])
        conc_a, conc_b = conc_b, conc_a
    st["conc"] = conc_a
    return st


@pytest.mark.parametrize("grid", GRIDS)
def test_diffusion_fp64_matches_oracle(gpu, tmp_path, grid):
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=5, n_nuclei=6, radius=2.0, noise=(0.02, 0.02))
    st0 = pf.init_microstructure(m, spec, 0.0)
    ref = _oracle_diffuse(om, copy_state(st0), 0.0, 13)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.diffuse(13)
    got = F.download()
    assert np.array_equal(got["C"], ref["C"])
    assert np.array_equal(got["conc"], ref["conc"])


@pytest.mark.parametrize("grid", [(64, 40, 33), (37, 23, 1), (48, 1, 20), (128, 32, 24)])
def test_every_tile_candidate_gives_the_same_answer(gpu, tmp_path, grid):
    """Each tile shape / kernel variant the autotuner may pick, against FP64."""
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=5, n_nuclei=6, radius=2.0, noise=(0.02, 0.02))
    st0 = pf.init_microstructure(m, spec, 0.0)
    F64 = pf.PhaseField(m, pf.PF_PREC_FP64)
    F64.upload(st0, 0.0)
    F64.diffuse(6)
    ref = F64.download()
    N = m.ix * m.iy * m.iz
    F = pf.PhaseField(m, pf.PF_PREC_FP32C)
    F.upload(st0, 0.0)
    cands = F.diffusion_candidates()
    assert len(cands) >= 3 and {c[2] for c in cands} <= {0, 1}
    first = {}
    for ty, zc, var in cands:
        F.upload(st0, 0.0)
        F.set_diffusion_tile(ty, zc, var)
        F.diffuse(6)
        got = F.download()
        err = rel_maxnorm(got["C"][:N], ref["C"][:N])
        assert err <= 2e-6, (ty, zc, var, err)
        # the TMA-staged variant does the same arithmetic: bit-identical to variant 0
        if (ty, zc) in first:
            assert np.array_equal(got["C"], first[(ty, zc)]), (ty, zc, var)
        else:
            first[(ty, zc)] = got["C"]


@pytest.mark.parametrize("grid", GRIDS)
def test_diffusion_fp32_tracks_fp64(gpu, tmp_path, grid):
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=5, n_nuclei=6, radius=2.0, noise=(0.02, 0.02))
    st0 = pf.init_microstructure(m, spec, 0.0)
    F64 = pf.PhaseField(m, pf.PF_PREC_FP64)
    F64.upload(st0, 0.0)
    F32 = pf.PhaseField(m, pf.PF_PREC_FP32C)
    F32.upload(st0, 0.0)
    F64.diffuse(20)
    F32.diffuse(20)
    a, b = F64.download(), F32.download()
    N = m.ix * m.iy * m.iz
    err_c = rel_maxnorm(b["C"][:N], a["C"][:N])
    err_mn = rel_maxnorm(b["C"][N:], a["C"][N:])
    moved = float(np.max(np.abs(a["C"][:N] - st0["C"][:N])))
    print(f"grid {grid}: fp32 diffusion rel err C {err_c:.3e} Mn {err_mn:.3e}; max change {moved:.3e}")
    assert moved > 1e-4
    assert err_c <= 2e-6 and err_mn <= 2e-6
    r32 = F32.reduce()
    assert abs(r32[4] - st0["C"][:N].sum()) / st0["C"][:N].sum() < 1e-7
