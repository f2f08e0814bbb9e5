"""The Fortran model's thermodynamics on the GPU: the FP64 path matches the
oracle bit for bit (tolerance written: 1e-10 relative max-norm, met exactly),
and the compact FP32 path tracks it: phase fractions within 1e-3 after one
step from the same state (beyond that the four-slot model and FP32 rounding
put a few fronts of these small boxes one step apart; the Fortran driving
force moves fronts across a cell every few steps)."""
import os

import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from helpers import adjacent_partners, copy_state, rel_maxnorm
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _case(tmp, grid, T=1023.0):
    W.write_thermo(os.path.join(tmp, "thermo_f90.txt"), "f90")
    cfg = W.write_config(os.path.join(tmp, "f90.txt"), grid=grid, T=T, thermo_file="thermo_f90.txt",
                         directory=os.path.join(tmp, "out"))
    return pf.read_model(cfg), po.load_model(cfg)


@pytest.mark.parametrize("grid,T", [((64, 48, 1), 1023.0), ((20, 18, 12), 1013.0), ((48, 40, 1), 1100.0)])
def test_f90_fp64_matches_oracle(gpu, tmp_path, grid, T):
    m, om = _case(str(tmp_path), grid, T)
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.nucleus_radius = 5, 6, 3.0
    st0 = pf.init_microstructure(m, spec, 0.0)
    ref = copy_state(st0)
    t_ref = po.run(om, ref, 0.0, 6)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(6)
    got = F.download()
    assert got["time"] == t_ref
    assert np.array_equal(got["ids"], ref["ids"])
    for k in ("phi", "phase", "conc", "C"):
        assert rel_maxnorm(got[k], ref[k]) <= 1e-10, k
        assert np.array_equal(got[k], ref[k]), k
    F.upload(st0, 0.0)
    F.update(1)
    G = pf.PhaseField(m, pf.PF_PREC_FP32C)
    G.upload(st0, 0.0)
    G.update(1)
    np.testing.assert_allclose(G.fractions()[:3], F.fractions()[:3], atol=1e-3)


@pytest.mark.parametrize("grid", [(48, 40, 1), (16, 14, 12)])
def test_f90_averaged_carbon_fp64_matches_oracle(gpu, tmp_path, grid):
    """The interface-averaged carbon (sparse.f90:184-255) on the FP64 path:
    every field bit for bit equal to the oracle after six steps."""
    W.write_thermo(str(tmp_path / "thermo_avg.txt"), "f90avg")
    cfg = W.write_config(str(tmp_path / "avg.txt"), grid=grid, T=1023.0, thermo_file="thermo_avg.txt",
                         directory=str(tmp_path / "out"))
    m, om = pf.read_model(cfg), po.load_model(cfg)
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.nucleus_radius = 4, 5, 3.0
    st0 = pf.init_microstructure(m, spec, 0.0)
    ref = copy_state(st0)
    t_ref = po.run(om, ref, 0.0, 6)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(6)
    got = F.download()
    F.close()
    assert got["time"] == t_ref
    assert np.array_equal(got["ids"], ref["ids"])
    for k in ("phi", "phase", "conc", "C"):
        assert np.array_equal(got[k], ref[k]), k
    # the averaging is in effect: the same steps without it end elsewhere
    plain = copy_state(st0)
    W.write_thermo(str(tmp_path / "thermo_f90.txt"), "f90")
    cfg2 = W.write_config(str(tmp_path / "f90.txt"), grid=grid, T=1023.0, thermo_file="thermo_f90.txt",
                          directory=str(tmp_path / "out"))
    po.run(po.load_model(cfg2), plain, 0.0, 6)
    assert not np.array_equal(plain["phi"], ref["phi"])


@pytest.mark.parametrize("grid,T", [((48, 40, 1), 1023.0), ((16, 14, 12), 1023.0), ((40, 36, 1), 1060.0)])
def test_f90_solute_drag_fp64_matches_oracle(gpu, tmp_path, grid, T):
    """The Purdy-Brechet solute drag (sparse.f90:958-1185, 1587-1641) on the
    FP64 path: every field bit for bit equal to the oracle after six steps,
    the velocity solves all converged (no error from synchronize), and the
    drag is in effect (the same steps without it end elsewhere)."""
    W.write_thermo(str(tmp_path / "thermo_drag.txt"), "f90drag")
    cfg = W.write_config(str(tmp_path / "drag.txt"), grid=grid, T=T, thermo_file="thermo_drag.txt",
                         directory=str(tmp_path / "out"))
    m, om = pf.read_model(cfg), po.load_model(cfg)
    assert m.drag == 1
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.nucleus_radius = 4, 5, 3.0
    st0 = pf.init_microstructure(m, spec, 0.0)
    ref = copy_state(st0)
    po.drag_failures()
    t_ref = po.run(om, ref, 0.0, 6)
    assert po.drag_failures() == 0
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(6)
    F.synchronize()
    got = F.download()
    F.close()
    assert got["time"] == t_ref
    assert np.array_equal(got["ids"], ref["ids"])
    for k in ("phi", "phase", "conc", "C"):
        assert np.array_equal(got[k], ref[k]), k
    plain = copy_state(st0)
    W.write_thermo(str(tmp_path / "thermo_f90.txt"), "f90")
    cfg2 = W.write_config(str(tmp_path / "f90.txt"), grid=grid, T=T, thermo_file="thermo_f90.txt",
                          directory=str(tmp_path / "out"))
    po.run(po.load_model(cfg2), plain, 0.0, 6)
    assert not np.array_equal(plain["phi"], ref["phi"])


@pytest.mark.parametrize("grid,model,npp0", [((48, 40, 1), "f90", 0), ((16, 14, 12), "f90drag", 0),
                                             ((40, 36, 1), "f90avg", 100002)])
def test_f90_coherent_mobility_fp64_matches_oracle(gpu, tmp_path, grid, model, npp0):
    """The coherent-grain mobility (sparse.f90:298-315) on the FP64 path, alone,
    with the solute drag and with the averaged carbon plus a recrystallisation
    class split: every field bit for bit equal to the oracle after six steps
    under a table that makes each nucleus coherent with its neighbouring
    ferrite grains, and different from the same steps without the table."""
    W.write_thermo(str(tmp_path / "thermo_coh.txt"), model, coherent_npp0=npp0)
    cfg = W.write_config(str(tmp_path / "coh.txt"), grid=grid, T=1023.0, thermo_file="thermo_coh.txt",
                         directory=str(tmp_path / "out"))
    m, om = pf.read_model(cfg), po.load_model(cfg)
    assert m.coherent == 1
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.nucleus_radius = 4, 5, 3.0
    st0 = pf.init_microstructure(m, spec, 0.0)
    table = adjacent_partners(st0["ids"], st0["phi"], spec.n_nuclei, m.cutoff)
    assert (table > 0).any()
    ref = copy_state(st0)
    po.set_coherent(table)
    po.drag_failures()
    t_ref = po.run(om, ref, 0.0, 6)
    po.set_coherent(None)
    assert po.drag_failures() == 0
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.set_coherent_grains(table)
    F.upload(st0, 0.0)
    F.update(6)
    F.synchronize()
    got = F.download()
    # the same steps without the table
    F.set_coherent_grains(np.zeros((0, 2), np.int32))
    F.upload(st0, 0.0)
    F.update(6)
    plain = F.download()
    F.close()
    assert got["time"] == t_ref
    assert np.array_equal(got["ids"], ref["ids"])
    for k in ("phi", "phase", "conc", "C"):
        assert np.array_equal(got[k], ref[k]), k
    assert not np.array_equal(plain["phi"], got["phi"])

