"""Known-answer tests of the FP64 CPU oracle (no GPU).  The reference ships no
tests or golden outputs for the phase sweep, so these pin the restatement by
the properties the reference's equations guarantee:

* every diffusion flux is antisymmetric -> total solute is conserved;
* partitioning satisfies sum_p phi_p c_p = C (solver.cpp:389-405);
* a single-grain domain is a fixed point (solver.cpp:207-216);
* after a sweep the kept slots of every interface cell sum to 1 (:292-296);
* single-phase diffusion is the discrete heat equation: a Fourier mode decays
  by 1 - 4 D dt/dx^2 sin^2(pi k/N) per sub-step (one dimension);
* with no driving force, the Steinbach sine profile phi = 1/2 - 1/2 sin(pi x/eta)
  of a planar two-grain interface is (nearly) stationary (model PDF Eq. 4.3).
"""
import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from helpers import copy_state, small_case


def test_solute_conservation_and_partition_identity(tmp_path):
    m, om, spec = small_case(str(tmp_path), "3d256", (20, 18, 12), n_grains=6, n_nuclei=8, radius=2.0,
                             noise=(0.02, 0.02))
    st = pf.init_microstructure(m, spec, 0.0)
    N = 20 * 18 * 12
    tot0 = st["C"].reshape(2, N).sum(1)
    s = copy_state(st)
    po.run(om, s, 0.0, 15)
    tot1 = s["C"].reshape(2, N).sum(1)
    np.testing.assert_allclose(tot1, tot0, rtol=1e-13)
    phase = s["phase"].reshape(N, 3)
    for q in range(2):
        conc = s["conc"][q * 3 * N:(q + 1) * 3 * N].reshape(N, 3)
        np.testing.assert_allclose((phase * conc).sum(1), s["C"][q * N:(q + 1) * N], rtol=1e-12, atol=1e-14)


def test_single_grain_domain_is_fixed_point(tmp_path):
    m, om, spec = small_case(str(tmp_path), "2d256", (16, 12, 1), n_grains=1, n_nuclei=0, noise=(0.0, 0.0))
    st = pf.init_microstructure(m, spec, 0.0)
    assert np.all(st["ids"].reshape(-1, 6)[:, 1] == 0)
    s = copy_state(st)
    po.run(om, s, 0.0, 5)
    for k in ("ids", "phi", "phase", "C"):
        np.testing.assert_array_equal(s[k], st[k])


def test_kept_slots_sum_to_one(tmp_path):
    m, om, spec = small_case(str(tmp_path), "2d256", (48, 40, 1), n_grains=6, n_nuclei=5)
    s = pf.init_microstructure(m, spec, 0.0)
    po.run(om, s, 0.0, 10)
    phi = s["phi"].reshape(-1, 6)
    np.testing.assert_allclose(phi.sum(1), 1.0, rtol=0, atol=5e-15)
    np.testing.assert_allclose(s["phase"].reshape(-1, 3).sum(1), 1.0, rtol=0, atol=5e-15)


def test_heat_equation_fourier_mode(tmp_path):
    """One phase, no interfaces: C' = C + D dt/dx^2 (C_{i-1} - 2C_i + C_{i+1})."""
    L = 64
    m, om, spec = small_case(str(tmp_path), "2d256", (L, 1, 1), n_grains=1, n_nuclei=0, mn=False)
    st = pf.init_microstructure(m, spec, 0.0)
    k = 3
    x = np.arange(L)
    amp = 1e-3
    st["C"][:] = 0.1 + amp * np.cos(2 * np.pi * k * x / L)
    p = po.params_at(om, 0.0)
    phase = st["phase"].copy()
    conc = np.zeros(3 * L)
    po.partition_all(om, p, phase, st["C"], conc)
    C = st["C"].copy()
    conc2 = np.zeros_like(conc)
    nsub = 7
    for _ in range(nsub):
        po.diffusion_substep(om, p, p.dt_sub, phase, conc, conc2, C)
        conc, conc2 = conc2, conc
    # ferrite only: c_1 = C, flux D_1 (C_nb - C)
    r = p.D[0][0] * p.dt_sub / (m.dx * m.dx)
    g = 1 - 4 * r * np.sin(np.pi * k / L) ** 2
    expect = 0.1 + amp * g ** nsub * np.cos(2 * np.pi * k * x / L)
    np.testing.assert_allclose(C, expect, rtol=0, atol=1e-15)


def test_planar_sine_interface_without_driving_force(tmp_path):
    """Two ferrite grains (same phase: no driving force) separated by the
    Steinbach profile; explicit steps leave it nearly unchanged."""
    L = 80
    m, om, spec = small_case(str(tmp_path), "2d256", (L, 4, 1), n_grains=2, n_nuclei=0, mn=False)
    st = pf.init_microstructure(m, spec, 0.0)
    eta_cells = m.i_intf
    x = np.arange(L) + 0.5
    ids = np.zeros((L * 4, 6), np.int32)
    phi = np.zeros((L * 4, 6))
    for j in range(4):
        for i in range(L):
            n = i + L * j
            # interfaces at L/4 and 3L/4 (periodic): grain A in the middle
            d = min(abs(x[i] - L / 4), abs(x[i] - 3 * L / 4))
            inside = L / 4 < x[i] < 3 * L / 4
            s = d if inside else -d
            a = 0.5 + 0.5 * np.sin(np.pi * np.clip(s / eta_cells, -0.5, 0.5))
            vals = sorted([(a, 100001), (1 - a, 100002)], reverse=True)
            k = 0
            for v, g in vals:
                if v > 1e-12:
                    ids[n, k], phi[n, k] = g, v
                    k += 1
    st["ids"][:] = ids.ravel()
    st["phi"][:] = phi.ravel()
    s = copy_state(st)
    po.run(om, s, 0.0, 30)
    frac_a = lambda S: np.where(S["ids"].reshape(-1, 6) == 100001, S["phi"].reshape(-1, 6), 0).sum() / (L * 4)
    assert abs(frac_a(s) - frac_a(st)) < 2e-3
