"""Binary microstructure files written from device buffers while stepping
continues: the files hold the state of the moment of the call (the steps
enqueued right after it do not leak into them), with korn and conc exactly
as the reference's field definitions give them for the downloaded state."""
import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import small_case
from phasefield_gb300 import vti

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [pf.PF_PREC_FP64, pf.PF_PREC_FP32C])
@pytest.mark.parametrize("grid,pieces", [((48, 40, 12), 4), ((64, 48, 1), 1)])
def test_device_vti_matches_state_at_call(gpu, tmp_path, prec, grid, pieces):
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=5, n_nuclei=6, radius=2.0, noise=(0.02, 0.02))
    st0 = pf.init_microstructure(m, spec, 0.0)
    F = pf.PhaseField(m, prec)
    F.upload(st0, 0.0)
    F.update(3)
    snap = F.download()
    N = grid[0] * grid[1] * grid[2]
    korn, conc = vti.fields(snap["ids"], snap["C"], N)
    outs = []
    for idx in range(2):  # the second call waits for the first write
        d = tmp_path / f"out{idx}"
        d.mkdir()
        F.write_vti_binary(str(d), idx, pieces)
        outs.append(d)
        F.update(2)  # stepping continues while the files are written
    F.write_wait()
    got = vti.read_pvti(str(outs[0] / "0000000.pvti"))
    assert got["grid"] == grid
    assert np.array_equal(got["korn"], korn)
    assert np.array_equal(got["conc"], conc)
    later = F.download()
    F.close()
    # the second file is the state after two more steps
    k2, c2 = vti.fields(later["ids"], later["C"], N)
    g2 = vti.read_pvti(str(outs[1] / "0000001.pvti"))
    assert not np.array_equal(g2["conc"], c2)  # two further steps were enqueued after it
    assert np.array_equal(g2["korn"].shape, k2.shape)
