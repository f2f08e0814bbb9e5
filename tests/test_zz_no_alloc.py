"""pf_reduce_noalloc: the grid statistics without any allocation by the library.

It exists for callers that cannot call cudaMalloc (an application pool that
owns all device memory, a framework caching allocator, a loop that cannot take
cudaMalloc's implicit synchronisation); its scratch is a fixed __device__ array
inside the library.  The caller owns every input and output buffer -- here
torch allocates them.  Two calls in a row, on states of different sizes, must
agree with pf_reduce (the allocating entry point) within the tolerance the
reduction tests use (rtol 1e-12); a third request beyond the scratch capacity
must be refused before anything is launched.

Collected last on purpose (file name): a failure here cannot hide the others.
"""
import ctypes

import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import small_case

pytestmark = pytest.mark.gpu


def _state_and_expected(tmp_path, grid, steps, seed):
    m, _, spec = small_case(str(tmp_path), "3d256", grid, n_grains=6, n_nuclei=8, radius=2.0,
                            noise=(0.02, 0.02), seed=seed)
    st0 = pf.init_microstructure(m, spec, 0.0)
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.upload(st0, 0.0)
    F.update(steps)
    st = F.download()
    expected = F.reduce()
    F.close()
    return m, st, expected


def test_reduce_noalloc_matches_pf_reduce(gpu, tmp_path):
    import torch

    L = pf.lib()
    stream = torch.cuda.current_stream()
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    cases = [((40, 36, 30), 3, 1), ((17, 13, 5), 2, 2)]  # 43200 cells (11 chunks), then 1105 cells (1 chunk)
    for grid, steps, seed in cases:
        m, st, expected = _state_and_expected(tmp_path, grid, steps, seed)
        N = m.ix * m.iy * m.iz
        d = {k: torch.from_numpy(st[k]).cuda() for k in ("ids", "phi", "phase", "C")}
        out.fill_(-1.0)
        rc = L.pf_reduce_noalloc(N, m.nsol, d["ids"].data_ptr(), d["phi"].data_ptr(), d["phase"].data_ptr(),
                                 d["C"].data_ptr(), out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == pf.PF_OK, L.pf_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, expected, rtol=1e-12, atol=1e-12)
        assert got[7] == 0.0


def test_reduce_noalloc_allocates_nothing(gpu, tmp_path):
    """After a first call on the device (which loads the library's module and
    looks up the scratch address), repeated calls leave the device's free
    memory exactly unchanged: the entry point allocates nothing."""
    import torch

    L = pf.lib()
    m, st, expected = _state_and_expected(tmp_path, (24, 20, 10), 2, 3)
    N = m.ix * m.iy * m.iz
    d = {k: torch.from_numpy(st[k]).cuda() for k in ("ids", "phi", "phase", "C")}
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()

    def call():
        return L.pf_reduce_noalloc(N, m.nsol, d["ids"].data_ptr(), d["phi"].data_ptr(), d["phase"].data_ptr(),
                                   d["C"].data_ptr(), out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))

    assert call() == pf.PF_OK, L.pf_last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        assert call() == pf.PF_OK, L.pf_last_error()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    np.testing.assert_allclose(out.cpu().numpy(), expected, rtol=1e-12, atol=1e-12)


def test_reduce_noalloc_rejects_oversize(gpu):
    import torch

    L = pf.lib()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    rc = L.pf_reduce_noalloc(16777217, 1, p, p, p, p, p, None)
    assert rc == pf.PF_ERR_RANGE
    assert b"PF_NOALLOC_MAX_CELLS" in L.pf_last_error()
    assert L.pf_reduce_noalloc(0, 1, p, p, p, p, p, None) == pf.PF_ERR_RANGE
