"""The Fortran model's thermodynamics as a selectable model (thermo file
F90_POLYNOMIAL): piecewise polynomial para lines, their slopes and the linear
austenite driving force of Fortran_openmp_phase_field/PFM/src/sparse.f90:
500-528 and 797-923.  The product's parameters equal the oracle's bit for bit,
and both agree with a literal restatement of the Fortran route (slopes
1/diff_poly4, Partition_k = transpose(Slope)/Slope, Partition_c = Ref -
Partition_k * transpose(Ref)) written out here."""
import os

import numpy as np
import pytest

import phasefield_gb300 as pf
import pyoracle as po
from helpers import adjacent_partners
from phasefield_gb300 import workloads as W


def _case(tmp, grid=(64, 48, 1), T=1023.0):
    W.write_thermo(os.path.join(tmp, "thermo_f90.txt"), "f90")
    cfg = W.write_config(os.path.join(tmp, "f90.txt"), grid=grid, T=T, thermo_file="thermo_f90.txt",
                         directory=os.path.join(tmp, "out"))
    return cfg, pf.read_model(cfg), po.load_model(cfg)


def _fortran_route(T):
    """sparse.f90:797-923 literally (Ref_c_para, Slope_para, Partition_k_para,
    Partition_c_para, Ratio_k_para), 0-based 3x3 arrays [i][j]."""
    poly4 = lambda x, a, b, c, d: a * x + b * x * x + c * x * x * x + d * x * x * x * x
    dpoly4 = lambda x, a, b, c, d: a + 2 * b * x + 3 * c * x * x + 4 * d * x * x * x
    ref = np.zeros((3, 3))
    slope = np.ones((3, 3))
    if T < 1086.52:
        ref[0, 1] = poly4(T - 273.15, -8.309e-5, 0, 0, 0) + 6.883e-2
        ref[1, 0] = poly4(T - 273.15, 2.607e-2, -6.58e-5, 3.984e-8, 0) + 0.9115
        slope[0, 1] = 1.0 / dpoly4(T - 273.15, -8.309e-5, 0, 0, 0)
        slope[1, 0] = 1.0 / dpoly4(T - 273.15, 2.607e-2, -6.58e-5, 3.984e-8, 0)
    else:
        ref[0, 1] = poly4(T - 1086.52, -1.1428e-4, 0, 0, 0)
        ref[1, 0] = poly4(T - 1086.52, -0.00325, 0, 0, 0)
        slope[0, 1] = 1.0 / dpoly4(0, -1.1428e-4, -1.78883e-7, -3.66186e-10, 2.53049e-12)
        slope[1, 0] = 1.0 / dpoly4(0, -0.00325, 1.13712e-5, -2.88193e-8, 1.05482e-10)
    ref[0, 2], ref[2, 0] = ref[0, 1], ref[1, 0]
    slope[0, 2], slope[2, 0] = slope[0, 1], slope[1, 0]
    ref[1, 2] = ref[2, 1] = ref[1, 0]
    slope[1, 2] = slope[2, 1] = slope[1, 0]
    pk = slope.T / slope
    pc = ref - pk * ref.T
    x = T - 273.15
    ratio = np.zeros((3, 3))
    ratio[0, 1] = (0.000264 * x * x - 0.4466 * x + 243.4713) * 1.03e-12
    ratio[1, 0] = -ratio[0, 1]
    ratio[2, 1] = ratio[0, 1]
    ratio[1, 2] = -ratio[2, 1]
    return ref, pk, pc, ratio


def _m3(arr):
    """Column-major 3x3 (i,j) at (i-1)+3(j-1) -> [i][j]."""
    return np.array([[arr[i + 3 * j] for j in range(3)] for i in range(3)])


@pytest.mark.parametrize("T", [900.0, 1013.0, 1023.0, 1086.0, 1090.0, 1150.0])
def test_f90_parameters_product_oracle_and_fortran_route(tmp_path, T):
    cfg, m, om = _case(str(tmp_path), T=T)
    assert m.thermo_model == 1 and om.thermo_model == 1
    p, q = pf.params_at(m, 0.0), po.params_at(om, 0.0)
    assert p.T == T and q.T == T
    assert p.df_model == 1 and q.df_model == 1 and p.df_ref == q.df_ref
    for name in ("eq", "dcdT", "df_ratio"):
        assert list(getattr(p, name)) == list(getattr(q, name)), name
    assert list(p.k[0]) == list(q.k[0]) and list(p.c[0]) == list(q.c[0])
    ref, pk, pc, ratio = _fortran_route(T)
    # the C++ model's k_ij, c_ij are the Fortran Partition_k(j,i), Partition_c(j,i)
    np.testing.assert_allclose(_m3(p.k[0]), pk.T, rtol=1e-13, atol=0)
    np.testing.assert_allclose(_m3(p.c[0]), pc.T, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(_m3(p.df_ratio), ratio, rtol=1e-15, atol=0)
    assert p.df_ref == pytest.approx(ref[1, 0], rel=1e-15)
    np.testing.assert_allclose(_m3(p.eq), ref, rtol=1e-15, atol=0)


def test_f90_model_steps_differ_from_linear_model(tmp_path):
    """The oracle advances the same state differently under the two models
    (the Fortran driving force is in effect), and conserves carbon."""
    grid = (48, 40, 1)
    cfg, m, om = _case(str(tmp_path), grid=grid)
    W.write_thermo(str(tmp_path / "thermo_steel.txt"))
    cfg_lin = W.write_config(str(tmp_path / "lin.txt"), grid=grid, T=1023.0, directory=str(tmp_path / "out"))
    om_lin = po.load_model(cfg_lin)
    spec = W.WORKLOADS["2d256"].spec()
    spec.n_grains, spec.n_nuclei = 5, 4
    st = po.init_state(om, spec, 0.0)
    st_lin = {k: v.copy() for k, v in st.items()}
    tot0 = st["C"][: 48 * 40].sum()
    po.run(om, st, 0.0, 20)
    po.run(om_lin, st_lin, 0.0, 20)
    assert not np.array_equal(st["phi"], st_lin["phi"])
    assert np.all(np.isfinite(st["phi"]))
    assert abs(st["C"][: 48 * 40].sum() - tot0) / tot0 < 1e-12


def test_adjoint_rejects_f90_thermodynamics(tmp_path):
    cfg, m, om = _case(str(tmp_path))
    h = pf.ctypes.c_void_p()
    assert pf.lib().pf_adj_create(pf.ctypes.byref(m), pf.PF_PREC_FP64, 10, pf.ctypes.byref(h)) == pf.PF_ERR_ARG


def _avg_fortran_literal(phase, conc, grid, cutoff, i_intf, ids=None, npp0=0):
    """sparse.f90:141-146 and 184-255 written out literally (1-based indices,
    MYNGB of util_func.f90:33-47), on the values of the start of the sweep.
    With ids: also Has_ferrite (bit 0) and Rex_intf (bit 1) of every cell
    (sparse.f90:137-139, 214-222; PHASE_INDEX of util_func.f90:50-60 on this
    model's ids: ferrite 1000xx, austenite 2000xx, cementite 3000xx)."""
    ix, iy, iz = grid
    ph = phase.reshape(iz, iy, ix, 3)
    cc = conc.reshape(iz, iy, ix, 3)
    out = cc.copy()
    flags = np.zeros((iz, iy, ix), np.uint8)
    ind = None if ids is None else ids.reshape(iz, iy, ix, 6)

    def phase_index(g):
        return -10000 if g <= 0 else g // 100000

    def myngb(coord, lcoord, n):
        nn = n % lcoord
        r = coord + nn
        return r - lcoord if r > lcoord else (r + lcoord if r < 1 else r)

    def vp(p, i, j, k):  # Val_phase(p, i, j, k), 1-based
        return ph[k - 1, j - 1, i - 1, p - 1]

    rng_ = i_intf + 1
    for K in range(1, iz + 1):
        for J in range(1, iy + 1):
            for I in range(1, ix + 1):
                if not (vp(1, I, J, K) > cutoff and vp(2, I, J, K) > cutoff):
                    continue
                grad = [vp(1, myngb(I, ix, 1), J, K) - vp(1, myngb(I, ix, -1), J, K),
                        vp(1, I, myngb(J, iy, 1), K) - vp(1, I, myngb(J, iy, -1), K),
                        vp(1, I, J, myngb(K, iz, 1)) - vp(1, I, J, myngb(K, iz, -1))]
                grad = [g / 2. for g in grad]
                g2 = 0.
                for g in grad:
                    g2 += g * g
                num, acc = 0., [0., 0., 0.]
                has_ferrite = rex_intf = False
                for Kk in range(-min((iz - 1) // 2, rng_), min((iz - 1) // 2, rng_) + 1):
                    Iiz = myngb(K, iz, Kk)
                    for Jj in range(-min((iy - 1) // 2, rng_), min((iy - 1) // 2, rng_) + 1):
                        Iiy = myngb(J, iy, Jj)
                        for Ii in range(-min((ix - 1) // 2, rng_), min((ix - 1) // 2, rng_) + 1):
                            Iix = myngb(I, ix, Ii)
                            a = Jj * grad[2] - Kk * grad[1]
                            b = Kk * grad[0] - Ii * grad[2]
                            c = Ii * grad[1] - Jj * grad[0]
                            if a * a + b * b + c * c > g2 * 1.0:
                                continue
                            if vp(1, Iix, Iiy, Iiz) > 1. - cutoff:
                                has_ferrite = True
                            if vp(1, Iix, Iiy, Iiz) < cutoff or vp(2, Iix, Iiy, Iiz) < cutoff:
                                continue
                            if ind is not None:
                                lst = [int(g) for g in ind[Iiz - 1, Iiy - 1, Iix - 1]]
                                rex_intf = rex_intf or (any(phase_index(g) == 1 and g <= npp0 for g in lst) and
                                                        any(phase_index(g) == 1 and g > npp0 for g in lst))
                            h = [vp(1, myngb(Iix, ix, 1), Iiy, Iiz) - vp(1, myngb(Iix, ix, -1), Iiy, Iiz),
                                 vp(1, Iix, myngb(Iiy, iy, 1), Iiz) - vp(1, Iix, myngb(Iiy, iy, -1), Iiz),
                                 vp(1, Iix, Iiy, myngb(Iiz, iz, 1)) - vp(1, Iix, Iiy, myngb(Iiz, iz, -1))]
                            dot = 0.
                            for d in range(3):
                                dot += grad[d] * h[d]
                            if dot < 0.:
                                continue
                            p1, p2 = vp(1, Iix, Iiy, Iiz), vp(2, Iix, Iiy, Iiz)
                            if p1 < 0.4 * p2 or p1 > 2.5 * p2:
                                continue
                            for d in range(3):
                                acc[d] += cc[Iiz - 1, Iiy - 1, Iix - 1, d]
                            num += 1.
                if num > 0.:
                    out[K - 1, J - 1, I - 1] = [a_ / num for a_ in acc]
                flags[K - 1, J - 1, I - 1] = int(has_ferrite) | (int(rex_intf) << 1)
    return out.ravel() if ids is None else (out.ravel(), flags.ravel())


@pytest.mark.parametrize("grid", [(24, 20, 1), (10, 9, 8)])
def test_averaged_interface_carbon_oracle_equals_fortran_literal(tmp_path, grid):
    W.write_thermo(str(tmp_path / "thermo_avg.txt"), "f90avg")
    cfg = W.write_config(str(tmp_path / "avg.txt"), grid=grid, T=1023.0, thermo_file="thermo_avg.txt",
                         directory=str(tmp_path / "out"))
    m, om = pf.read_model(cfg), po.load_model(cfg)
    assert m.avg_carbon == 1 and om.avg_carbon == 1
    assert pf.params_at(m, 0.0).avg_range == m.i_intf + 1 == po.params_at(om, 0.0).avg_range
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.nucleus_radius = 3, 4, 2.5
    st = po.init_state(om, spec, 0.0)
    p = po.params_at(om, 0.0)
    N = grid[0] * grid[1] * grid[2]
    conc = np.zeros(3 * N * om.nsol)
    po.partition_all(om, p, st["phase"], st["C"], conc)
    conc = conc[: 3 * N] + 1e-3 * np.sin(np.arange(3 * N))  # distinct values per cell
    got = po.avg_conc(om, p, st["phase"], conc)
    want = _avg_fortran_literal(st["phase"], conc, grid, om.cutoff, om.i_intf)
    assert np.array_equal(got, want)
    assert not np.array_equal(got, conc)  # the averaging changed some cells


def test_averaged_carbon_keyword_and_precision_checks(tmp_path):
    with open(tmp_path / "bad.txt", "w") as f:
        f.write("F90_POLYNOMIAL\nNO_SUCH_OPTION\n")
    cfg = W.write_config(str(tmp_path / "bad_cfg.txt"), grid=(8, 8, 1), thermo_file="bad.txt",
                         directory=str(tmp_path / "out"))
    with pytest.raises(pf.PfError):
        pf.read_model(cfg)
    W.write_thermo(str(tmp_path / "thermo_avg.txt"), "f90avg")
    cfg = W.write_config(str(tmp_path / "avg.txt"), grid=(8, 8, 1), thermo_file="thermo_avg.txt",
                         directory=str(tmp_path / "out"))
    m = pf.read_model(cfg)
    h = pf.ctypes.c_void_p()
    assert pf.lib().pf_create(pf.ctypes.byref(m), pf.PF_PREC_FP32C, pf.ctypes.byref(h)) == pf.PF_ERR_ARG


def _drag_case(tmp_path, grid=(48, 40, 1), T=1023.0, model="f90drag"):
    W.write_thermo(str(tmp_path / "thermo_drag.txt"), model)
    cfg = W.write_config(str(tmp_path / "drag.txt"), grid=grid, T=T, thermo_file="thermo_drag.txt",
                         directory=str(tmp_path / "out"))
    return pf.read_model(cfg), po.load_model(cfg)


def _sd_literal(V0, E0, De, U0, V_max, T):
    """SOLUTE_DRAG_PB (sparse.f90:1005-1037) in Python floats."""
    import math
    V = V0 / V_max
    A = (De - E0) + V
    B = (De + E0) + V
    D0 = 1. - U0
    Vu0 = V * U0
    D1_d0 = (A - Vu0) / (A * D0 + (A - V) * U0 * math.exp(-(A - Vu0)))
    D1 = D0 * D1_d0
    U1 = 1. - D1
    D2_d1 = (B - Vu0) / (B * D1 + (B * U1 - Vu0) * math.exp(-(B - Vu0)))
    return (2. * De * U0 - ((A - V) / A * (Vu0 + math.log(D1_d0)) + (B - V) / B * (Vu0 + math.log(D2_d1)))) * 8.314 * T / 7.2e12


@pytest.mark.parametrize("T", [1000.0, 1023.0, 1050.0, 1120.0])
def test_drag_parameters_product_oracle_and_fortran_literal(tmp_path, T):
    """PARAMETER_DRAG_PB: the product's values equal the oracle's bit for bit;
    both agree with a literal Python restatement (Python's exp/log) to 1e-13."""
    import math
    m, om = _drag_case(tmp_path, T=T)
    assert m.drag == 1 and om.drag == 1 and m.drag_vmax0 == 1.0e11
    p, q = pf.params_at(m, 0.0), po.params_at(om, 0.0)
    assert p.drag_model == 1 and q.drag_model == 1
    for name in ("drag_vmax", "drag_ex0", "drag_de_heat", "drag_de_cool", "drag_u0"):
        assert getattr(p, name) == getattr(q, name), name
    assert list(p.drag_corr) == list(q.drag_corr) and list(p.drag_drag0) == list(q.drag_drag0)
    # sparse.f90:958-1003 literally
    x = T - 273.15
    vmax = 1.0e11 * math.exp(-247650. / (8.314 * T))
    Mn = [max(1e-10, 3.9793e-5 * x - 2.3163e-2), max(1e-10, -2.928e-8 * x ** 2 + 5.629e-5 * x - 2.35e-2),
          max(1e-10, 2.253e-8 * x ** 2 - 4.255e-5 * x + 2.351e-2)]
    Nn = [max(1e-10, -3.818e-9 * x ** 3 + 9.055e-6 * x ** 2 - 7.408e-3 * x + 2.118),
          max(1e-10, -7.1227e-10 * x ** 3 + 1.6307e-6 * x ** 2 - 1.2584e-3 * x + 3.3166e-1), 3e-3]
    U = [1.887e-2, 3.65e-3, 3.12e-3]
    deh = [-0.5 * math.log(Mn[i] * (1 - U[i]) / (U[i] * (1 - Mn[i]))) for i in range(3)]
    dec = [-0.5 * math.log(Nn[i] * (1 - U[i]) / (U[i] * (1 - Nn[i]))) for i in range(3)]
    ex0 = 10000. / (8.314 * T)
    y = T - 1110.64
    nple = (-3.3441e-3 * y + 1.0406e-5 * y * y - 5.6345e-8 * y ** 3) if T < 1110.64 else -3.23154e-3 * y
    nple_r = 0.0 if T < 1041.3 else -2.39e-3 * (T - 1041.3)
    r21, ref21 = p.df_ratio[1], p.eq[1]  # (2,1) at (2-1)+3*(1-1)
    drivf = [abs(r21 * (ref21 - nple)), abs(r21 * (ref21 - nple_r))]
    d0 = [sum(_sd_literal(0., ex0 if i == 0 else 0., de[i], U[i], vmax, T) for i in range(3)) for de in (deh, dec)]
    corr = [drivf[0] / d0[0], drivf[1] / d0[1]]
    drag0 = [_sd_literal(0., ex0, deh[0], U[0], vmax, T) * corr[0], _sd_literal(0., ex0, dec[0], U[0], vmax, T) * corr[1]]
    np.testing.assert_allclose([p.drag_vmax, p.drag_ex0, p.drag_de_heat, p.drag_de_cool],
                               [vmax, ex0, deh[0], dec[0]], rtol=1e-13)
    np.testing.assert_allclose(list(p.drag_corr) + list(p.drag_drag0), corr + drag0, rtol=1e-12)


def test_drag_changes_the_oracle_step(tmp_path):
    """With the solute drag the oracle advances the ferrite/austenite
    interfaces differently, finds a velocity root wherever it solves, and
    keeps carbon."""
    grid = (48, 40, 1)
    _, om = _drag_case(tmp_path, grid=grid)
    (tmp_path / "plain").mkdir()
    _, om2 = _drag_case(tmp_path / "plain", grid=grid, model="f90")
    spec = W.WORKLOADS["2d256"].spec()
    spec.n_grains, spec.n_nuclei = 4, 5
    st = po.init_state(om, spec, 0.0)
    st2 = {k: v.copy() for k, v in st.items()}
    N = grid[0] * grid[1]
    tot0 = st["C"][:N].sum()
    po.drag_failures()
    po.run(om, st, 0.0, 10)
    po.run(om2, st2, 0.0, 10)
    assert po.drag_failures() == 0
    assert not np.array_equal(st["phi"], st2["phi"])
    assert abs(st["C"][:N].sum() - tot0) / tot0 < 1e-12


def test_shared_exp_log_against_c_library():
    """pf_exp/pf_log (the drag solve's own exp and log) stay within 4 ulp of
    the C library over the arguments the drag model meets and well beyond."""
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-700, 700, 4000), rng.uniform(-2, 2, 4000), [0.0, -0.0, 1e-300, -1e-300]])
    e, _ = po.exp_log(x)
    ref = np.exp(x)
    assert np.all(np.abs(e - ref) <= 4 * np.spacing(ref))
    y = np.concatenate([10.0 ** rng.uniform(-300, 300, 4000), rng.uniform(0.5, 2.0, 4000), [1.0, 2.0, 0.5]])
    _, lg = po.exp_log(y)
    ref = np.log(y)
    assert np.all(np.abs(lg - ref) <= 4 * np.spacing(np.abs(ref)) + 1e-300)
    assert lg[-3] == 0.0


def test_solute_drag_keyword_and_precision(tmp_path):
    """`SOLUTE_DRAG b v q` sets the model's drag fields; a line with missing
    values is an input error; compact FP32 contexts refuse the option."""
    m, om = _drag_case(tmp_path)
    assert (m.drag_binding, m.drag_vmax0, m.drag_qsd) == (10000.0, 1.0e11, 247650.0)
    assert (om.drag_binding, om.drag_vmax0, om.drag_qsd) == (10000.0, 1.0e11, 247650.0)
    (tmp_path / "bad.txt").write_text("F90_POLYNOMIAL\nSOLUTE_DRAG 10000. 1.0e11\n")
    cfg = W.write_config(str(tmp_path / "c_bad.txt"), grid=(8, 8, 1), thermo_file="bad.txt",
                         directory=str(tmp_path / "out"))
    with pytest.raises(pf.PfError):
        pf.read_model(cfg)
    h = pf.ctypes.c_void_p()
    assert pf.lib().pf_create(pf.ctypes.byref(m), pf.PF_PREC_FP32C, pf.ctypes.byref(h)) == pf.PF_ERR_ARG


def _coh_case(tmp_path, grid, model="f90", npp0=0, T=1023.0):
    W.write_thermo(str(tmp_path / "thermo_coh.txt"), model, coherent_npp0=npp0)
    cfg = W.write_config(str(tmp_path / "coh.txt"), grid=grid, T=T, thermo_file="thermo_coh.txt",
                         directory=str(tmp_path / "out"))
    return pf.read_model(cfg), po.load_model(cfg)


@pytest.mark.parametrize("grid,npp0", [((24, 20, 1), 0), ((24, 20, 1), 100002), ((10, 9, 8), 100001)])
def test_coherent_flags_oracle_equal_fortran_literal(tmp_path, grid, npp0):
    """The scan's Has_ferrite / Rex_intf flags and the averaged carbon of the
    oracle equal a literal 1-based restatement of sparse.f90:137-139, 184-255."""
    m, om = _coh_case(tmp_path, grid, npp0=npp0)
    assert m.coherent == 1 and om.coherent == 1 and m.coh_npp0 == npp0
    p, q = pf.params_at(m, 0.0), po.params_at(om, 0.0)
    assert (p.avg_range, p.avg_conc, p.coh_model, p.coh_npp0) == (m.i_intf + 1, 0, 1, npp0)
    assert (q.avg_range, q.avg_conc, q.coh_model, q.coh_npp0) == (p.avg_range, 0, 1, npp0)
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.nucleus_radius = 4, 4, 2.5
    st = po.init_state(om, spec, 0.0)
    N = grid[0] * grid[1] * grid[2]
    conc = np.zeros(3 * N * om.nsol)
    po.partition_all(om, q, st["phase"], st["C"], conc)
    conc = conc[: 3 * N]
    got, fl = po.avg_conc(om, q, st["phase"], conc, ids=st["ids"], with_flags=True)
    want, wfl = _avg_fortran_literal(st["phase"], conc, grid, om.cutoff, om.i_intf, ids=st["ids"], npp0=npp0)
    assert np.array_equal(got, want)
    assert np.array_equal(fl, wfl)
    assert (fl & 1).any()
    if npp0:
        assert (fl & 2).any()


def _splitmix64(s):
    M = (1 << 64) - 1
    s = (s + 0x9E3779B97F4A7C15) & M
    z = s
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return s, z ^ (z >> 31)


@pytest.mark.parametrize("grid", [(40, 36, 1), (16, 14, 12)])
def test_init_coherent_follows_boundary_nucleation_rule(tmp_path, grid):
    """pf_init_coherent: at the cell nearest each nucleus of the matrix
    without nuclei, Or_num = min(2, ferrite grains - 1) partners, the largest
    ferrite ids (module_nucleation.f90:357-367).  Nucleus positions are
    re-drawn here from the generator's seed stream (grains first, then
    nuclei, three uniforms each)."""
    m, _ = _coh_case(tmp_path, grid)
    spec = W.WORKLOADS["3d256"].spec()
    spec.n_grains, spec.n_nuclei, spec.n_particles, spec.nucleus_radius = 6, 40, 0, 2.0
    got = pf.init_coherent(m, spec)
    assert got.shape == (40, 2)
    spec0 = W.WORKLOADS["3d256"].spec()
    spec0.n_grains, spec0.n_nuclei, spec0.n_particles, spec0.nucleus_radius = 6, 0, 0, 2.0
    matrix = pf.init_microstructure(m, spec0, 0.0)
    ix, iy, iz = grid
    I = matrix["ids"].reshape(iz, iy, ix, 6)
    s = spec.seed
    draws = []
    for _ in range(3 * (spec.n_grains + spec.n_nuclei)):
        s, z = _splitmix64(s)
        draws.append((z >> 11) * (1.0 / 9007199254740992.0))
    nuc = np.array(draws[3 * spec.n_grains:]).reshape(-1, 3) * [ix, iy, iz]
    n_two = n_one = 0
    for n, (x, y, z) in enumerate(nuc):
        i = int(np.floor(x + 0.5)) % ix
        j = 0 if iy == 1 else int(np.floor(y + 0.5)) % iy
        k = 0 if iz == 1 else int(np.floor(z + 0.5)) % iz
        fer = sorted((int(g) for g in I[k, j, i] if g // 100000 == 1), reverse=True)
        or_num = min(2, len(fer) - 1)
        want = [fer[0] if or_num >= 1 else 0, fer[1] if or_num >= 2 else 0]
        assert list(got[n]) == want, n
        n_two += or_num >= 2
        n_one += or_num == 1
    assert n_one + n_two > 0


def test_coherent_keyword_and_precision(tmp_path):
    (tmp_path / "bad.txt").write_text("F90_POLYNOMIAL\nCOHERENT_MOBILITY\n")
    cfg = W.write_config(str(tmp_path / "c_bad.txt"), grid=(8, 8, 1), thermo_file="bad.txt",
                         directory=str(tmp_path / "out"))
    with pytest.raises(pf.PfError):
        pf.read_model(cfg)
    with pytest.raises(ValueError):
        W.write_thermo(str(tmp_path / "t.txt"), "linear", coherent_npp0=0)
    m, _ = _coh_case(tmp_path, (8, 8, 1))
    h = pf.ctypes.c_void_p()
    assert pf.lib().pf_create(pf.ctypes.byref(m), pf.PF_PREC_FP32C, pf.ctypes.byref(h)) == pf.PF_ERR_ARG
    ms = (pf.PfModel * 1)(m)
    assert pf.lib().pf_batch_create(ms, 1, pf.ctypes.byref(h)) == pf.PF_ERR_ARG


def test_coherent_mobility_changes_the_oracle_step(tmp_path):
    """With every nucleus coherent with its neighbouring ferrite grains the
    oracle slows those interfaces: the state differs from the same steps
    without the table, and with a recrystallisation front everywhere
    (every ferrite grain of the other class) it differs again."""
    grid = (48, 40, 1)
    m, om = _coh_case(tmp_path, grid)
    spec = W.WORKLOADS["2d256"].spec()
    spec.n_grains, spec.n_nuclei = 4, 5
    st0 = po.init_state(om, spec, 0.0)
    table = adjacent_partners(st0["ids"], st0["phi"], spec.n_nuclei, om.cutoff)
    assert (table > 0).any()
    runs = []
    for tab in (table, None):
        po.set_coherent(tab)
        st = {k: v.copy() for k, v in st0.items()}
        po.run(om, st, 0.0, 8)
        runs.append(st)
    po.set_coherent(None)
    assert not np.array_equal(runs[0]["phi"], runs[1]["phi"])


def _dissipation_literal(solution, driv, drag, norm, heating, p, T, exp, log):
    """DISSIPATION_ITERATION (heating) / DISSIPATION_ITERATION_R (cooling),
    sparse.f90:538-655, written out literally (with the drag pressure of
    SOLUTE_DRAG_PB, sparse.f90:1005-1037); exp/log are passed in.  Returns
    (solution, stopped): the _R form stops the Fortran program when no bracket
    is found."""
    f = np.float64  # IEEE arithmetic as in the C code (x / 0 is +-inf, not an exception)
    drag0 = f(p.drag_drag0[0] if heating else p.drag_drag0[1])
    de = f(p.drag_de_heat if heating else p.drag_de_cool)
    corr = f(p.drag_corr[0] if heating else p.drag_corr[1])
    ex0, u0, vmax = f(p.drag_ex0), f(p.drag_u0), f(p.drag_vmax)
    driv, drag, norm = f(driv), f(drag), f(norm)

    def sdpb(V0, E0, De, U0):
        V = V0 / vmax
        A = (De - E0) + V
        B = (De + E0) + V
        D0 = 1. - U0
        Vu0 = V * U0
        D1_d0 = (A - Vu0) / (A * D0 + (A - V) * U0 * exp(-(A - Vu0)))
        D1 = D0 * D1_d0
        U1 = 1. - D1
        D2_d1 = (B - Vu0) / (B * D1 + (B * U1 - Vu0) * exp(-(B - Vu0)))
        return (2. * De * U0 - ((A - V) / A * (Vu0 + log(D1_d0)) + (B - V) / B * (Vu0 + log(D2_d1)))) * 8.314 * T / 7.2e12

    with np.errstate(all="ignore"):
        return _dissipation_loops(solution, driv, drag, norm, heating, drag0, de, corr, ex0, u0, vmax, sdpb)


def _dissipation_loops(solution, driv, drag, norm, heating, drag0, de, corr, ex0, u0, vmax, sdpb):
    err2 = driv - drag * drag0
    if err2 < 0.:
        return 0., False
    dv = 0.1 * vmax
    v = np.float64(0.)
    for _ in range(2):
        for _ in range(40):
            err1 = err2
            v = v + dv
            err2 = driv - v * norm - drag * (sdpb(v, ex0, de, u0) * corr)
            if err1 * err2 <= 0.:
                x1, x2 = v - dv, v
                n = 0
                while (x2 - x1) > 0.01 * x2:
                    n += 1
                    assert n < 10000
                    tv = 0.5 * (x1 + x2)
                    te = driv - tv * norm - drag * (sdpb(tv, ex0, de, u0) * corr)
                    if err1 * te <= 0.:
                        x2, err2 = tv, te
                    else:
                        x1, err1 = tv, te
                return float(0.5 * (x1 + x2) * norm), False
        v = driv / norm
        dv = -0.2 * v
        err2 = np.float64(-1.)
    return solution, not heating


@pytest.mark.parametrize("T", [1023.0, 1060.0])
def test_drag_velocity_solve_oracle_equals_fortran_literal(tmp_path, T):
    """The oracle's velocity solve equals the literal Fortran bit for bit (same
    exp/log) over rates, drag weights and interface norms spanning the
    no-drag, bracketed and no-bracket cases of both branches; a cooling solve
    without a bracket is flagged where the Fortran stops."""
    _, om = _drag_case(tmp_path, T=T)
    p = po.params_at(om, 0.0)
    exp = lambda x: np.float64(po.exp_log(np.array([x]))[0][0])
    log = lambda x: np.float64(po.exp_log(np.array([x]))[1][0])
    rng = np.random.default_rng(11)
    seen = {"zero": 0, "root": 0, "none": 0}
    # drag weights m_ij f3 sqrt(phi_i phi_j) and rates of the sweep's magnitudes
    for t in range(320):
        driv = float(10.0 ** rng.uniform(-1, 3.5))
        drag = float(10.0 ** rng.uniform(10, 13))
        # norm = f3 sqrt(phi (1 - phi)) is 0 for phi = 1: the second pass then
        # starts at an infinite velocity and finds no bracket
        norm = float(rng.uniform(0.05, 1.0)) if t < 300 else 0.0
        heating = int(rng.integers(0, 2)) if t < 300 else t % 2
        po.drag_failures()
        got = po.dissipation(p, driv, driv, drag, norm, heating)
        failed = po.drag_failures()
        want, stopped = _dissipation_literal(driv, driv, drag, norm, heating, p, T, exp, log)
        assert got == want, (driv, drag, norm, heating, got, want)
        assert bool(failed) == stopped
        seen["zero" if want == 0. else ("none" if want == driv or stopped else "root")] += 1
    assert min(seen.values()) > 0, seen
