"""Binary microstructure files (no GPU): the piece/index writer from host
arrays against the reference's field definitions (write_data.cpp:42-82) and
against the ASCII writer's values; the z-slab pieces share their boundary
plane and together cover the image."""
import numpy as np
import pytest

import phasefield_gb300 as pf
from helpers import small_case
from phasefield_gb300 import vti


@pytest.mark.parametrize("grid,pieces", [((24, 20, 9), 4), ((31, 17, 1), 3), ((16, 12, 5), 1), ((8, 8, 3), 7)])
def test_binary_pieces_round_trip(tmp_path, grid, pieces):
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=4, n_nuclei=5, radius=2.0, noise=(0.02, 0.02))
    st = pf.init_microstructure(m, spec, 0.0)
    N = grid[0] * grid[1] * grid[2]
    korn, conc = vti.fields(st["ids"], st["C"], N)
    assert set(np.unique(korn)) <= {0, 1, 2}
    d = tmp_path / "out"
    d.mkdir()
    vti.write_host(str(d), 3, pieces, grid, 0.5, korn, conc)
    got = vti.read_pvti(str(d / "0000003.pvti"))
    assert got["whole_extent"] == [1, grid[0], 1, grid[1], 1, grid[2]]
    assert np.array_equal(got["korn"], korn)
    assert np.array_equal(got["conc"], conc)
    npieces = len(list(d.glob("0000003_*.vti")))
    assert npieces == min(pieces, grid[2])


def test_binary_fields_match_the_ascii_writer(tmp_path):
    """korn and conc of the binary files equal the values the ASCII writer
    (the reference's Vti_write layout) prints for the same state."""
    grid = (20, 16, 3)
    m, om, spec = small_case(str(tmp_path), "3d256", grid, n_grains=4, n_nuclei=4, radius=2.0)
    st = pf.init_microstructure(m, spec, 0.0)
    N = grid[0] * grid[1] * grid[2]
    path = str(tmp_path / "a.vti")
    pf.check(pf.lib().pf_write_vti(path.encode(), *grid, 0.5, pf._ptr(st["ids"]), pf._ptr(st["C"])), "pf_write_vti")
    text = open(path).read()
    blocks = text.split('format="ascii">')
    ascii_korn = np.array(blocks[1].split("</DataArray>")[0].split(), np.int32)
    ascii_conc = np.array(blocks[2].split("</DataArray>")[0].split(), np.float64)
    korn, conc = vti.fields(st["ids"], st["C"], N)
    assert np.array_equal(korn, ascii_korn)
    # the ASCII file prints 3 significant digits
    assert np.allclose(conc, ascii_conc, rtol=5e-3)


def test_binary_writer_rejects_bad_arguments(tmp_path):
    k = np.zeros(8, np.int32)
    c = np.zeros(8, np.float32)
    assert pf.lib().pf_write_vti_binary_host(str(tmp_path).encode(), 0, 0, 2, 2, 2, 0.5, pf._ptr(k), pf._ptr(c)) == pf.PF_ERR_ARG
    assert pf.lib().pf_write_vti_binary_host(str(tmp_path / "missing").encode(), 0, 1, 2, 2, 2, 0.5, pf._ptr(k),
                                             pf._ptr(c)) == pf.PF_ERR_IO
