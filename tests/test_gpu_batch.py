"""Batched ensemble: one persistent launch over many 2D domains against the
same domains advanced one by one through the single-domain FP32C path, and
the bounded group-barrier wait (the failure path is exercised by a test knob
that makes a barrier unreachable -- no device fault is involved)."""
import numpy as np
import pytest

import phasefield_gb300 as pf
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _domains(tmp_path, gentle=True):
    doms = [W.EnsembleDomain((64, 64, 1), 993.0, 0.0095, 5, 3, 11),
            W.EnsembleDomain((96, 64, 1), 1023.0, 0.0080, 6, 4, 12),
            W.EnsembleDomain((128, 32, 1), 1053.0, 0.0070, 4, 2, 13),
            W.EnsembleDomain((37, 45, 1), 1010.0, 0.0090, 3, 2, 14)]
    if not gentle:
        for d in doms:
            d.C0 = 0.12
    paths = W.ensemble_inputs(str(tmp_path), doms)
    models = [pf.read_model(p) for p in paths]
    states = [pf.init_microstructure(m, W.ensemble_spec(d), 0.0) for m, d in zip(models, doms)]
    return models, states


def test_batch_matches_single_domain_runs(gpu, tmp_path):
    models, states = _domains(tmp_path)
    B = pf.Batch(models)
    for d, st in enumerate(states):
        B.upload(d, st, 0.0)
    steps = 12
    assert B.run(5) == pf.PF_OK
    assert B.run(steps - 5) == pf.PF_OK  # two launches: buffer roles carry over
    info = B.info()
    assert info["domains"] == 4 and info["cells"] == sum(m.ix * m.iy for m in models)
    for d, (m, st) in enumerate(zip(models, states)):
        F = pf.PhaseField(m, pf.PF_PREC_FP32C)
        F.upload(st, 0.0)
        F.update(steps)
        a, b = F.download(), B.download(d)
        assert a["time"] == b["time"]
        N = m.ix * m.iy
        fa, fb = F.fractions(), B.reduce(d)[:4] / N
        print(f"domain {d}: fractions {fa[:2]} vs {fb[:2]}; max|dphase| {np.max(np.abs(a['phase'] - b['phase'])):.2e}")
        np.testing.assert_allclose(fb[:3], fa[:3], atol=1e-5)
        np.testing.assert_allclose(b["C"], a["C"], rtol=1e-5, atol=1e-7)
        tot0 = st["C"][:N].sum()
        assert abs(B.reduce(d)[4] - tot0) / tot0 < 1e-6


def test_batch_barrier_timeout_is_reported_and_recoverable(gpu, tmp_path):
    models, states = _domains(tmp_path)
    B = pf.Batch(models)
    for d, st in enumerate(states):
        B.upload(d, st, 0.0)
    B.set_timeout(20_000_000, unreachable_barrier=True)  # 20 ms, and a barrier no block can satisfy
    assert B.run(3) == pf.PF_ERR_TIMEOUT
    B.set_timeout(2_000_000_000, unreachable_barrier=False)
    for d, st in enumerate(states):
        B.upload(d, st, 0.0)
    assert B.run(3) == pf.PF_OK
    for d in range(len(models)):
        assert np.all(np.isfinite(B.reduce(d)))


def test_batch_rejects_3d_and_mixed_solutes(gpu, tmp_path):
    models, _ = _domains(tmp_path)
    m3 = pf.read_model(W.write_config(str(tmp_path / "c3.txt"), grid=(16, 16, 8)))
    with pytest.raises(pf.PfError):
        pf.Batch([models[0], m3])
    m1 = pf.read_model(W.write_config(str(tmp_path / "c1.txt"), grid=(32, 32, 1), mn=False))
    with pytest.raises(pf.PfError):
        pf.Batch([models[0], m1])


def test_batch_matches_oracle(gpu, tmp_path):
    """Two domains of one persistent launch against the FP64 CPU oracle (the
    six-slot reference algorithm) on the same inputs: the tolerances of the
    single-domain FP32C-vs-FP64 test (near-equilibrium carbon): mean |dphase|
    <= 2e-4, phase fractions within 1e-4, total carbon within 1e-4 relative
    max-norm."""
    import os

    import pyoracle as po
    from helpers import copy_state, rel_maxnorm

    models, states = _domains(tmp_path)
    B = pf.Batch(models)
    for d, st in enumerate(states):
        B.upload(d, st, 0.0)
    steps = 12
    assert B.run(steps) == pf.PF_OK
    paths = sorted(p for p in os.listdir(tmp_path) if p.startswith("ens") and p.endswith(".txt"))
    for d in (0, 2):
        m = models[d]
        N = m.ix * m.iy
        om = po.load_model(os.path.join(str(tmp_path), paths[d]))
        ref = copy_state(states[d])
        t = po.run(om, ref, 0.0, steps)
        got = B.download(d)
        assert got["time"] == t
        dphase = np.abs(got["phase"] - ref["phase"])
        fr_b = got["phase"].reshape(N, 3).mean(0)
        fr_o = ref["phase"].reshape(N, 3).mean(0)
        print(f"domain {d}: mean|dphase| {dphase.mean():.2e}, fractions {fr_b[:2]} vs {fr_o[:2]}")
        assert dphase.mean() <= 2e-4
        np.testing.assert_allclose(fr_b, fr_o, atol=1e-4)
        assert rel_maxnorm(got["C"][:N], ref["C"][:N]) <= 1e-4


def test_batch_tile_shapes_agree_and_autotune_restores(gpu, tmp_path):
    """Every tile shape gives bit-identical states; the autotuner leaves the
    ensemble exactly where it found it."""
    models, states = _domains(tmp_path, gentle=False)
    out = {}
    for ty, div in ((8, 1), (4, 1), (4, 2)):
        B = pf.Batch(models)
        for d, st in enumerate(states):
            B.upload(d, st, 0.0)
        B.set_tile(ty, div)
        assert B.run(6) == pf.PF_OK
        out[(ty, div)] = [B.download(d) for d in range(len(models))]
        B.close()
    for key, res in out.items():
        for d in range(len(models)):
            for k in ("ids", "phi", "phase", "C"):
                assert np.array_equal(res[d][k], out[(8, 1)][d][k]), (key, d, k)
    B = pf.Batch(models)
    for d, st in enumerate(states):
        B.upload(d, st, 0.0)
    best = B.autotune(3)
    assert best["tile_y"] in (4, 8) and best["ms"] > 0
    assert B.run(6) == pf.PF_OK
    for d in range(len(models)):
        got = B.download(d)
        for k in ("ids", "phi", "phase", "C"):
            assert np.array_equal(got[k], out[(8, 1)][d][k]), (d, k)
