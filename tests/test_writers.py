"""Output writers (write_data.cpp:3-82): the ASCII VTI layout on the CPU; the
fraction_time.txt rows and the pfm driver on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import phasefield_gb300 as pf
from phasefield_gb300 import workloads as W


def test_vti_layout(tmp_path):
    ix, iy, iz = 4, 3, 2
    N = ix * iy * iz
    ids = np.zeros(6 * N, np.int32)
    ids[0::6] = 100001
    ids[6 * 5 + 0], ids[6 * 5 + 1] = 200003, 100001       # interface cell -> korn 0
    ids[6 * 7 + 0] = 200002                                # austenite -> 2
    ids[6 * 8 + 0] = 42                                    # deformed ferrite id -> 1
    C = np.linspace(0.01, 0.24, N)
    path = str(tmp_path / "f.vti")
    assert pf.lib().pf_write_vti(path.encode(), ix, iy, iz, 0.5, ids.ctypes.data, C.ctypes.data) == pf.PF_OK
    text = open(path).read().splitlines()
    assert text[0] == '<?xml version="1.0"?>'
    assert text[2] == '<ImageData WholeExtent="1 4 1 3 1 2" Origin="0 0 0" Spacing="0.5 0.5 0.5">'
    assert text[3] == '<Piece Extent="1 4 1 3 1 2">'
    korn = [int(v) for v in text[6].split()]
    assert len(korn) == N and korn[5] == 0 and korn[7] == 2 and korn[8] == 1 and korn[0] == 1
    conc = text[9].split()
    # write_data.cpp:74-77: the closing tag follows the last value on the same line
    assert conc[-1] == "</DataArray>"
    conc = conc[:-1]
    assert len(conc) == N and conc[0] == "0.01" and conc[-1] == "0.24"
    assert text[-1] == "</VTKFile>"


@pytest.mark.gpu
def test_fraction_time_rows(gpu, tmp_path):
    W.write_thermo(str(tmp_path / "thermo_steel.txt"))
    cfg = W.write_config(str(tmp_path / "c.txt"), grid=(40, 32, 1), directory=str(tmp_path), timestep_output=0.1)
    m = pf.read_model(cfg)
    spec = W.WORKLOADS["2d256"].spec()
    spec.n_grains, spec.n_nuclei = 4, 3
    F = pf.PhaseField(m, pf.PF_PREC_FP64)
    F.construct(spec)
    assert F.write_data(str(tmp_path), forced=True)
    rows = 1
    for _ in range(12):
        F.update(1)
        rows += F.write_data(str(tmp_path))
    lines = open(tmp_path / "fraction_time.txt").read().splitlines()
    assert len(lines) == rows >= 2
    first = lines[0].split()
    assert len(first) == 6 and float(first[1]) == 1023.0
    fr = F.fractions()
    last = [float(v) for v in lines[-1].split()]
    assert abs(sum(last[2:5]) - 1.0) < 2e-3
    np.testing.assert_allclose(last[2:5], fr[:3], atol=5e-4)


@pytest.mark.gpu
def test_pfm_driver(gpu, tmp_path):
    W.write_thermo(str(tmp_path / "thermo_steel.txt"))
    out = tmp_path / "out"
    cfg = W.write_config(str(tmp_path / "c.txt"), grid=(48, 40, 1), directory=str(out), timestep_output=0.1,
                         num_nuclei=3, num_grain=(4, 0, 0))
    exe = os.path.join(os.path.dirname(pf.LIB_PATH), "..", "bin", "pfm")
    r = subprocess.run([exe, cfg, "--steps", "20"], capture_output=True, text=True, cwd=str(tmp_path), timeout=120)
    assert r.returncode == 0, r.stderr
    assert "SIMULATION IS FINISHED" in r.stdout and "steps: 20" in r.stdout
    assert (out / "fraction_time.txt").exists()


@pytest.mark.gpu
def test_pfm_driver_fortran_options(gpu, tmp_path):
    """The driver with the Fortran model's thermodynamics, solute drag and
    coherent-grain mobility (it builds the coherent-partner table of its seeded
    state): runs to completion on the FP64 path."""
    W.write_thermo(str(tmp_path / "thermo_steel.txt"), "f90drag", coherent_npp0=0)
    out = tmp_path / "out"
    cfg = W.write_config(str(tmp_path / "c.txt"), grid=(48, 40, 1), directory=str(out), timestep_output=0.1,
                         num_nuclei=3, num_grain=(4, 0, 0))
    exe = os.path.join(os.path.dirname(pf.LIB_PATH), "..", "bin", "pfm")
    r = subprocess.run([exe, cfg, "--steps", "10"], capture_output=True, text=True, cwd=str(tmp_path), timeout=120)
    assert r.returncode == 0, r.stderr
    assert "steps: 10" in r.stdout
