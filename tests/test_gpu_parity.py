"""GPU parity: the product's sm_103a kernels, called through the C ABI, against
the FP64 CPU oracle on the same seeded inputs.

Tolerances (stated per test):
* FP64 plain path: bit-identical ids, and relative max-norm <= 1e-10 on every
  phase field, phase fraction and concentration (the kernels are built without
  multiply-add contraction, so in practice the difference is exactly 0).
* FP32 compensated path: compared with the FP64 path on the same input.
"""
import ctypes

import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from helpers import copy_state, rel_maxnorm, small_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _run_both(tmp_path, name, grid, steps, **kw):
    m, om, spec = small_case(str(tmp_path), name, grid, **kw)
    st0 = pf.init_microstructure(m, spec, 0.0)
    ref = copy_state(st0)
    t_ref = po.run(om, ref, 0.0, steps)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(steps)
    got = F.download()
    F.close()
    return ref, t_ref, got


def _assert_fp64_parity(ref, t_ref, got):
    assert got["time"] == t_ref
    assert np.array_equal(got["ids"], ref["ids"]), "grain ids differ"
    for k in ("phi", "phase", "conc", "C"):
        err = rel_maxnorm(got[k], ref[k])
        assert err <= FP64_TOL, f"{k}: relative max-norm {err:.3e} > {FP64_TOL}"


@pytest.mark.parametrize(
    "name,grid,steps,kw",
    [
        ("2d256", (64, 64, 1), 30, dict(n_grains=6, n_nuclei=4)),
        ("2d256", (37, 23, 1), 20, dict(n_grains=4, n_nuclei=3)),       # ragged, not a block multiple
        ("3d256", (24, 20, 16), 10, dict(n_grains=8, n_nuclei=12, noise=(0.02, 0.02))),
        ("2d256", (200, 1, 1), 40, dict(n_grains=3, n_nuclei=2)),       # 1D: two neighbours
        ("2d512cem", (64, 64, 1), 20, dict(n_grains=5, n_nuclei=4, n_particles=6)),  # three phases
    ],
)
def test_fp64_step_matches_oracle(gpu, tmp_path, name, grid, steps, kw):
    ref, t_ref, got = _run_both(tmp_path, name, grid, steps, **kw)
    _assert_fp64_parity(ref, t_ref, got)


def test_fp64_single_solute_reference_config(gpu, tmp_path):
    """Carbon only (no Mn extension): exactly the reference's state arrays."""
    ref, t_ref, got = _run_both(tmp_path, "2d256", (48, 40, 1), 25, n_grains=5, n_nuclei=4, mn=False)
    assert got["C"].size == 48 * 40
    _assert_fp64_parity(ref, t_ref, got)


def test_fp64_deformed_grain_ids(gpu, tmp_path):
    """Grain ids below 100000 are phase 1 (phase_field.h:25-29)."""
    m, om, spec = small_case(str(tmp_path), "2d256", (40, 40, 1), n_grains=5, n_nuclei=3)
    st0 = pf.init_microstructure(m, spec, 0.0)
    ids = st0["ids"]
    ferrite = (ids >= 100000) & (ids < 200000)
    ids[ferrite] -= 100000  # 1..5: deformed ferrite grains
    ref = copy_state(st0)
    t_ref = po.run(om, ref, 0.0, 15)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(15)
    got = F.download()
    _assert_fp64_parity(ref, t_ref, got)
    fr = F.fractions()
    ofr = po.fractions(om, ref["ids"], ref["phi"], ref["phase"])
    assert fr[3] > 0.1
    np.testing.assert_allclose(fr, ofr / 1.0, rtol=1e-12, atol=1e-15)


def test_fp64_graph_replay_matches(gpu, tmp_path):
    """CUDA-graph replay of constant-temperature steps gives the same state."""
    m, om, spec = small_case(str(tmp_path), "2d256", (64, 48, 1), n_grains=6, n_nuclei=5)
    st0 = pf.init_microstructure(m, spec, 0.0)
    ref = copy_state(st0)
    t_ref = po.run(om, ref, 0.0, 11)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.use_graph(True)
    F.upload(st0, 0.0)
    F.update(4)
    F.update(7)
    got = F.download()
    _assert_fp64_parity(ref, t_ref, got)


def test_reduce_matches_oracle(gpu, tmp_path):
    m, om, spec = small_case(str(tmp_path), "3d256", (32, 24, 20), n_grains=8, n_nuclei=10, noise=(0.02, 0.02))
    st0 = pf.init_microstructure(m, spec, 0.0)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(5)
    got = F.download()
    r = F.reduce()
    N = m.ix * m.iy * m.iz
    ofr = po.fractions(om, got["ids"], got["phi"], got["phase"])
    np.testing.assert_allclose(r[:4] / N, ofr, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(r[4], got["C"][:N].sum(), rtol=1e-12)
    np.testing.assert_allclose(r[5], got["C"][N:].sum(), rtol=1e-12)
    assert r[7] == 0


def test_dropin_gpu_diffusion_solver(gpu, tmp_path):
    """GPU_Diffusion_solver (gpu_solver.h:19) against the oracle's restatement of
    gpu_solver.cpp:204-218, 2D and 3D, bit-identical."""
    L = pf.lib()
    for grid in ((64, 48, 1), (20, 18, 12)):
        m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=6, n_nuclei=6, noise=(0.02, 0.02))
        st0 = pf.init_microstructure(m, spec, 0.0)
        P = pf.params_at(m, 0.0)
        x, y, z = grid
        N = x * y * z
        D = np.array([P.D[0][p] for p in range(3)])
        k = np.array(list(P.k[0]))
        c = np.array(list(P.c[0]))
        phase = st0["phase"].copy()
        C_ref = st0["C"][:N].copy()
        nloop = po.gpu_diffusion_solver(D, k, c, phase, C_ref, x, y, z, P.pfm_dt, m.dx)
        assert nloop >= 1
        assert L.GPU_Init(x, y, z) == 1
        C_gpu = st0["C"][:N].copy()
        dp = ctypes.POINTER(ctypes.c_double)
        L.GPU_Diffusion_solver(D.ctypes.data_as(dp), k.ctypes.data_as(dp), c.ctypes.data_as(dp),
                               phase.ctypes.data_as(dp), C_gpu.ctypes.data_as(dp), x, y, z, P.pfm_dt, m.dx)
        L.GPU_Cleanup()
        assert np.array_equal(C_gpu, C_ref), f"max diff {np.max(np.abs(C_gpu - C_ref))}"
        assert not np.array_equal(C_ref, st0["C"][:N])


def _fp32_vs_fp64(tmp_path, steps, **kw):
    m, om, spec = small_case(str(tmp_path), "3d256", (48, 40, 32), n_grains=10, n_nuclei=30, radius=2.0, **kw)
    st0 = pf.init_microstructure(m, spec, 0.0)
    F64 = pf.PhaseField(m, pf.PF_PREC_FP64)
    F64.upload(st0, 0.0)
    F32 = pf.PhaseField(m, pf.PF_PREC_FP32C)
    F32.upload(st0, 0.0)
    assert F32.truncated_cells() == 0
    F64.update(steps)
    F32.update(steps)
    a, b = F64.download(), F32.download()
    N = m.ix * m.iy * m.iz
    dphase = np.abs(a["phase"] - b["phase"])
    dphi = np.abs(a["phi"] - b["phi"])
    dC = np.abs(a["C"] - b["C"])
    fa, fb = F64.fractions(), F32.fractions()
    r64, r32 = F64.reduce(), F32.reduce()
    out = dict(dphase=float(dphase.max()), dphase_mean=float(dphase.mean()),
               n_bad=int((dphase > 1e-3).sum()), dphi=float(dphi.max()), dC=float(dC.max()),
               dC_mean=float(dC.mean()), dfrac=float(np.max(np.abs(fa[:3] - fb[:3]))),
               mass64=abs(r64[4] - st0["C"][:N].sum()) / st0["C"][:N].sum(),
               mass32=abs(r32[4] - st0["C"][:N].sum()) / st0["C"][:N].sum(),
               mn32=abs(r32[5] - st0["C"][N:].sum()) / st0["C"][N:].sum())
    print(f"fp32c vs fp64 after {steps} steps {kw}: {out}")
    return out


def test_fp32c_tracks_fp64_gentle(gpu, tmp_path):
    """Near-equilibrium carbon (weak driving force): the compact FP32 path
    follows the six-slot FP64 path in the mean; single cells differ where the
    FP64 path holds a fifth or sixth grain that the four-slot layout drops."""
    e = _fp32_vs_fp64(tmp_path, 40, C0=(0.0090, 1.5))
    assert e["dphase_mean"] < 2e-4
    assert e["dfrac"] < 1e-4
    assert e["mass32"] < 1e-6 and e["mass64"] < 1e-12 and e["mn32"] < 1e-6


def test_fp32c_tracks_fp64_stiff(gpu, tmp_path):
    """Supersaturated carbon (the workload's driving force moves interfaces by
    ~0.5 in phi per step): pointwise differences appear where fronts cross a
    cell one step apart; the phase fractions stay close and solute is conserved."""
    e = _fp32_vs_fp64(tmp_path, 40, noise=(0.02, 0.02))
    assert e["dfrac"] < 1e-2
    assert e["mass32"] < 1e-6 and e["mass64"] < 1e-12 and e["mn32"] < 1e-6
