"""Configuration / thermodynamic file readers: the product's C++ parser against
the oracle's independent restatement, known values of the reference's own
sample inputs, malformed inputs, and the per-step parameters (host FP64,
bit-identical between product and oracle)."""
import os

import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from phasefield_gb300 import workloads as W

from build_oracle import REF_ROOT

REF_BUILD = os.path.join(REF_ROOT, "C++-openmp-cuda", "build")


def _same(m: pf.PfModel, d: dict):
    assert (m.ix, m.iy, m.iz) == (d["ix"], d["iy"], d["iz"])
    assert m.dx == d["dx"] and m.i_intf == d["i_intf"] and m.cutoff == d["cutoff"]
    assert m.nT == len(d["T_path"])
    for k, (t, T) in enumerate(d["T_path"]):
        assert (m.T_time[k], m.T_temp[k]) == (t, T)
    for k in ("m0", "mQ", "sigma", "ent_a", "ent_b", "eq_a", "eq_b", "eq_c"):
        assert list(getattr(m, k)) == d[k], k
    assert m.nsol == d["nsol"]
    for q in range(m.nsol):
        assert list(m.D0[q]) == d["D0"][q] and list(m.DQ[q]) == d["DQ"][q]
    assert m.thermo_file.decode() == d["thermo_file"]
    assert m.gpu_flag == d["gpu_flag"]


@pytest.mark.parametrize("name", sorted(W.WORKLOADS))
def test_packaged_configs_parse_identically(name):
    cfg = W.packaged_config(name)
    _same(pf.read_model(cfg), po.parse_config(cfg))


@pytest.mark.skipif(not os.path.exists(REF_BUILD), reason="reference checkout not mounted")
def test_reference_sample_input(monkeypatch):
    """The reference's own sample config + thermo file (C++-openmp-cuda/build)."""
    monkeypatch.chdir(REF_BUILD)
    cfg = os.path.join(REF_BUILD, "log_file.txt")
    m = pf.read_model(cfg)
    d = po.parse_config(cfg)
    _same(m, d)
    # Known values read off the sample file.
    assert (m.ix, m.iy, m.iz) == (500, 500, 1)
    assert m.dx == 0.15 and m.i_intf == 5 and m.cutoff == 1e-5
    assert list(m.num_grain) == [8, 1, 0]
    assert m.nT == 2 and (m.T_time[1], m.T_temp[1]) == (4.6, 1003.0)
    assert m.num_nuclei == 1.0
    assert m.m0[0] == 24e29 and m.mQ[0] == 360000.0          # (1,1)
    assert m.m0[3] == 200.e16 and m.m0[1] == 200.e16          # (1,2) and (2,1)
    assert m.sigma[4] == 0.76e-12 and m.sigma[7] == 0.94e-12  # (2,2), (2,3)
    assert list(m.D0[0]) == [0.1e8, 0.15e8, 0.0]
    assert m.thermo_file == b"thermo_data.txt" and m.gpu_flag == 1 and m.nsol == 1
    assert m.ent_b[3] == 0.2e-12 and m.ent_b[1] == -0.2e-12   # (1,2) and (2,1)
    assert (m.eq_a[3], m.eq_b[3], m.eq_c[3]) == (0.0, -1e-4, 0.11)    # PARA (1,2)
    assert (m.eq_b[1], m.eq_c[1]) == (-5e-3, 5.395)                   # PARA (2,1)
    om = po.model_from_dict(d)
    for t in (0.0, 2.3):
        a, b = pf.params_at(m, t), po.params_at(om, t)
        assert a.T == b.T == 1003.0
        assert a.pfm_dt == b.pfm_dt and a.diff_dt == b.diff_dt and a.n_sub == b.n_sub


@pytest.mark.parametrize("name", sorted(W.WORKLOADS))
def test_step_parameters_bit_identical(name):
    cfg = W.packaged_config(name)
    m, om = pf.read_model(cfg), po.load_model(cfg)
    for t in (0.0, 0.5, 123.25):
        a, b = pf.params_at(m, t), po.params_at(om, t)
        assert a.T == b.T
        assert a.pfm_dt == b.pfm_dt and a.diff_dt == b.diff_dt
        assert a.n_sub == b.n_sub and a.dt_sub == b.dt_sub
        assert list(a.m) == list(b.m)
        for q in range(m.nsol):
            assert list(a.D[q]) == list(b.D[q])
            assert list(a.k[q]) == list(b.k[q]) and list(a.c[q]) == list(b.c[q])
        assert list(a.entropy) == list(b.entropy) and list(a.eq) == list(b.eq) and list(a.dcdT) == list(b.dcdT)


def test_parameters_known_answer():
    """pfm_dt = 0.2*dx^2/(dim*max m*sigma), diff_dt = 0.2*dx^2/(dim*max D) and the
    linear partition coefficients k_ij = dcdT_ji/dcdT_ij (phase_field.cpp:307-315,
    thermo_data.cpp:34-40), evaluated independently in numpy."""
    m = pf.read_model(W.packaged_config("2d256"))
    p = pf.params_at(m, 0.0)
    T, R = 1023.0, 8.314
    mob = np.array(m.m0) * np.exp(-np.array(m.mQ) / (R * T))
    assert np.isclose(p.pfm_dt, 0.5 ** 2 / 2 * 0.2 / np.max(mob * np.array(m.sigma)), rtol=1e-14)
    Dc = np.array(m.D0[0]) * np.exp(-np.array(m.DQ[0]) / (R * T))
    assert np.isclose(p.diff_dt, 0.5 ** 2 / Dc.max() / 2 * 0.2, rtol=1e-14)
    assert p.n_sub == int(np.ceil(p.pfm_dt / p.diff_dt)) == 8
    dcdT12, dcdT21 = -1e-4, -5e-3
    assert np.isclose(p.k[0][3], dcdT21 / dcdT12)            # k(1,2)
    eq12, eq21 = -1e-4 * T + 0.11, -5e-3 * T + 5.395
    assert np.isclose(p.c[0][3], eq21 - (dcdT21 / dcdT12) * eq12)
    assert p.k[1][1] == 0.5 and p.k[1][3] == 2.0             # Mn: k(2,1) = r1/r2, k(1,2) = r2/r1
    assert p.nnb == 4


def test_malformed_config_reports_io_error(tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("output?\nout\n\n\n\n12 x 1\n")
    m = pf.PfModel()
    st = pf.lib().pf_model_read(str(bad).encode(), m)
    assert st == pf.PF_ERR_IO
    assert b"domain size" in pf.lib().pf_last_error()
    assert pf.lib().pf_model_read(str(tmp_path / "missing.txt").encode(), m) == pf.PF_ERR_IO


def test_truncated_config_and_missing_thermo(tmp_path):
    cfg = W.write_config(str(tmp_path / "c.txt"), grid=(8, 8, 1), thermo_file="nope.txt")
    m = pf.PfModel()
    assert pf.lib().pf_model_read(cfg.encode(), m) == pf.PF_ERR_IO
    text = open(W.packaged_config("2d256")).read().splitlines()
    (tmp_path / "t.txt").write_text("\n".join(text[:30]) + "\n")
    assert pf.lib().pf_model_read(str(tmp_path / "t.txt").encode(), m) == pf.PF_ERR_IO


def test_config_without_mn_extension_is_single_solute(tmp_path):
    W.write_thermo(str(tmp_path / "thermo_steel.txt"))
    cfg = W.write_config(str(tmp_path / "c.txt"), grid=(16, 16, 1), mn=False)
    assert pf.read_model(cfg).nsol == 1
    assert po.parse_config(cfg)["nsol"] == 1
