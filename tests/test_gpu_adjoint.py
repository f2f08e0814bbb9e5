"""Hand-written adjoint of the explicit step against central finite differences
of the FP64 forward step (relative step 1e-4), on a small three-phase 2D case.

Tolerance written here: relative error <= 2e-3 per gradient component (the
finite-difference truncation is O(h^2) ~ 1e-8; the rest is the few cells whose
discrete decisions -- clamps, the cutoff, the top-four choice -- the +-h
perturbation flips, which the adjoint holds fixed by construction)."""
import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import small_case

pytestmark = pytest.mark.gpu

REL_H = 1e-4


def _setup(tmp_path, prec=pf.PF_PREC_FP64, K=7, grid=(48, 40, 1)):
    m, _, spec = small_case(str(tmp_path), "2d512cem", grid, n_grains=5, n_nuclei=4, radius=3.0, n_particles=5,
                            C0=(0.02, 1.5))
    st = pf.init_microstructure(m, spec, 0.0)
    A = pf.Adjoint(m, prec, K)
    A.upload(st, 0.0)
    return A


def _fd(A, steps, obj, i):
    s = np.ones(4)
    s[i] = 1 + REL_H
    A.set_scales(s)
    jp = A.forward(steps)[obj]
    s[i] = 1 - REL_H
    A.set_scales(s)
    jm = A.forward(steps)[obj]
    A.set_scales(np.ones(4))
    return (jp - jm) / (2 * REL_H)


@pytest.mark.parametrize("obj", [0, 1])
def test_adjoint_matches_central_differences(gpu, tmp_path, obj):
    steps = 20
    A = _setup(tmp_path)
    J = A.forward(steps)
    g = A.gradient(obj)
    fd = [_fd(A, steps, obj, i) for i in range(3)]
    print(f"objective {obj}: J = {J[obj]:.6g}, adjoint {g[:3]}, central differences {fd}")
    for i in range(3):
        scale = max(abs(fd[i]), 1e-3 * max(abs(x) for x in fd))
        assert abs(g[i] - fd[i]) <= 2e-3 * scale, (i, g[i], fd[i])
    assert g[3] == 0.0  # Mn does not feed back into the phase update or the carbon field


def test_gradient_independent_of_checkpoint_interval(gpu, tmp_path):
    """Checkpoint intervals 3, 4 and 50 and the record mode (0: every step
    kept by the forward, no recomputation) give the same objective and
    gradient; in record mode a repeated forward/gradient (graph replays)
    gives them again."""
    steps = 15
    out, Js = [], []
    for K in (3, 4, 50, 0):
        A = _setup(tmp_path, K=K)
        Js.append(A.forward(steps))
        out.append(A.gradient(1))
        if K == 0:
            # J sums per-block FP64 partials with atomics: equal to rounding
            np.testing.assert_allclose(A.forward(steps), Js[-1], rtol=1e-13)
            np.testing.assert_allclose(A.gradient(1), out[-1], rtol=1e-12, atol=1e-300)
            A.gradient(0)
            np.testing.assert_allclose(A.gradient(1), out[-1], rtol=1e-12, atol=1e-300)
        A.close()
    for J in Js[1:]:
        np.testing.assert_allclose(J, Js[0], rtol=1e-13)
    for g in out[1:]:
        np.testing.assert_allclose(g, out[0], rtol=1e-10, atol=1e-300)


def test_record_mode_matches_central_differences(gpu, tmp_path):
    """Record mode against central differences of the FP64 forward (the
    checkpointed gradient's tolerance)."""
    steps = 20
    A = _setup(tmp_path, K=0)
    A.forward(steps)
    g = A.gradient(0)
    fd = [_fd(A, steps, 0, i) for i in range(3)]
    for i in range(3):
        scale = max(abs(fd[i]), 1e-3 * max(abs(x) for x in fd))
        assert abs(g[i] - fd[i]) <= 2e-3 * scale, (i, g[i], fd[i])


def test_record_mode_fp32_equals_checkpointed(gpu, tmp_path):
    """FP32 calibration: record mode and checkpoint interval 7 agree."""
    steps = 30
    res = []
    for K in (7, 0):
        A = _setup(tmp_path, prec=pf.PF_PREC_FP32C, K=K)
        J = A.forward(steps)
        res.append((J, A.gradient(0), A.gradient(1)))
        A.close()
    np.testing.assert_allclose(res[1][0], res[0][0], rtol=1e-12)
    np.testing.assert_allclose(res[1][1], res[0][1], rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(res[1][2], res[0][2], rtol=1e-9, atol=1e-300)


def test_torch_autograd_wrapper(gpu, tmp_path):
    import torch

    from phasefield_gb300 import calibration

    A = _setup(tmp_path)
    s = torch.ones(4, dtype=torch.float64, requires_grad=True)
    J = calibration.objective(s, A, 10, 1)
    J.backward()
    g = A.gradient(1)
    np.testing.assert_allclose(s.grad.numpy(), g, rtol=1e-12)
    assert J.item() == pytest.approx(A.forward(10)[1], rel=1e-12)


def test_fp32_gradient_tracks_fp64(gpu, tmp_path):
    steps = 12
    g64 = _setup(tmp_path, pf.PF_PREC_FP64)
    g64.forward(steps)
    a = g64.gradient(0)
    g32 = _setup(tmp_path, pf.PF_PREC_FP32C)
    g32.forward(steps)
    b = g32.gradient(0)
    print(f"fp64 {a[:3]} fp32 {b[:3]}")
    np.testing.assert_allclose(b[:3], a[:3], rtol=2e-2, atol=1e-3 * np.max(np.abs(a[:3])))


@pytest.mark.parametrize("K", [4, 0])
def test_adjoint_3d_matches_central_differences(gpu, tmp_path, K):
    """A 3D box (the phase kernels' 3D cell patches), checkpointed and record
    mode, against central differences of the FP64 forward."""
    steps = 10
    A = _setup(tmp_path, K=K, grid=(16, 16, 8))
    A.forward(steps)
    g = A.gradient(0)
    fd = [_fd(A, steps, 0, i) for i in range(3)]
    for i in range(3):
        scale = max(abs(fd[i]), 1e-3 * max(abs(x) for x in fd))
        assert abs(g[i] - fd[i]) <= 2e-3 * scale, (i, g[i], fd[i])
