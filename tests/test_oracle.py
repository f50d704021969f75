"""CPU tests of the oracle: its published-method pieces (cubature, DFT), its
restatement of the reference (bit-for-bit against the reference compiled from
its own sources, where present) and the committed golden fixtures."""
import ctypes
import math
import os

import numpy as np
import pytest

from conftest import golden, rel_err


# ---- cubature (published Gauss-Kronrod / Genz-Malik rules) ------------------------

CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_uint, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                      ctypes.c_uint, ctypes.POINTER(ctypes.c_double))


def hcub(port, f, dim, fdim, max_eval, abs_tol, rel_tol, norm=0):
    fn = port.lib.hcubature
    fn.argtypes = [ctypes.c_uint, CB, ctypes.c_void_p, ctypes.c_uint, ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_double), ctypes.c_size_t, ctypes.c_double, ctypes.c_double,
                   ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    calls = [0]

    def cb(ndim, x, data, fd, fval):
        calls[0] += 1
        vals = f([x[i] for i in range(ndim)])
        for j in range(fd):
            fval[j] = vals[j]
        return 0

    lo = (ctypes.c_double * dim)(*([0.0] * dim))
    hi = (ctypes.c_double * dim)(*([1.0] * dim))
    val = (ctypes.c_double * fdim)()
    err = (ctypes.c_double * fdim)()
    code = fn(fdim, CB(cb), None, dim, lo, hi, max_eval, abs_tol, rel_tol, norm, val, err)
    return code, list(val), list(err), calls[0]


def test_gk15_exact_to_degree_22(port):
    for k in (0, 1, 5, 13, 22):
        code, val, err, n = hcub(port, lambda x, k=k: [x[0] ** k], 1, 1, 15, 0.0, 0.0)
        assert code == 0 and n == 15
        assert abs(val[0] - 1.0 / (k + 1)) < 1e-14


def test_genz_malik_exact_to_degree_7(port):
    for a, b in ((0, 0), (3, 4), (7, 0), (2, 5), (1, 1)):
        code, val, err, n = hcub(port, lambda x, a=a, b=b: [x[0] ** a * x[1] ** b], 2, 1, 17, 0.0, 0.0)
        assert code == 0 and n == 17
        assert abs(val[0] - 1.0 / ((a + 1) * (b + 1))) < 1e-14
        if a + b <= 5:
            assert err[0] < 1e-14   # embedded degree-5 rule is exact too


def test_adaptive_singular_corner(port):
    # int_0^1 int_0^1 (x + y)^(-1/2) = (4/3)(2 sqrt 2 - 2)
    exact = 4.0 / 3.0 * (2.0 * math.sqrt(2.0) - 2.0)
    code, val, err, n = hcub(port, lambda x: [1.0 / math.sqrt(x[0] + x[1]), 0.0], 2, 2, 0, 0.0, 1e-10, 1)
    assert code == 0
    assert abs(val[0] - exact) < 1e-9 * exact
    code, val2, err2, n2 = hcub(port, lambda x: [1.0 / math.sqrt(x[0] + x[1]), 0.0], 2, 2, 200, 0.0, 1e-12, 1)
    assert n2 <= 200 + 34   # max_eval stops the refinement (checked after each split)


def test_dft_matches_numpy(port):
    rng = np.random.default_rng(3)
    for nt in (16, 17, 4094, 255):
        x = rng.standard_normal(nt)
        g, s = port.laplace_trans(x, 1.0)
        c = math.log(float(nt) ** 2) / 1.0
        dt = 1.0 / (nt - 1)
        w = x * dt * np.exp(-c * np.arange(nt) * dt)
        assert rel_err(g, np.fft.rfft(w)) < 1e-12
        y = port.inv_laplace_trans(g, s, 1.0, nt, 0)
        # the inverse re-applies e^{c t}, up to nt^2 at t_max: eps * nt^2
        assert rel_err(y, x) < 1e-15 * nt * nt + 1e-12


# ---- restatement pinned against the reference build ------------------------------

def _grid_geom(pkg):
    e, nd = pkg.electrode_grid(4, 3, 9.0, 6.0, 3, 2, 6e-3, -0.4)
    return e, nd


def test_port_equals_reference_fill(pkg, port, ref, orc_mod):
    O = orc_mod
    e, nd = _grid_geom(pkg)
    img = O.images(e)
    for s in (2j * np.pi * 60.0, 1.3e5 + 2j * np.pi * 3e6):
        kappa = 1 / 300.0 + s * 15 * O.EPS0
        for it in (O.INTG_DOUBLE, O.INTG_MHEM, O.INTG_SINGLE, O.INTG_NONE):
            a = port.hem_impedances(e, img, s, kappa, 1.0, 0, 1e-6, 1e-6, it)
            b = ref.hem_impedances(e, img, s, kappa, 1.0, 0, 1e-6, 1e-6, it)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), it


def test_port_equals_reference_integral_and_self(port, ref, pkg):
    e, _ = _grid_geom(pkg)
    for i, k in ((0, 1), (0, 5), (2, 9), (7, 3)):
        for it in (1, 2, 3, 4):
            a = port.integral(e[i], e[k], 0.3 + 0.4j, 0, 1e-7, 1e-7, it)
            b = ref.integral(e[i], e[k], 0.3 + 0.4j, 0, 1e-7, 1e-7, it)
            assert a == b
    assert port.self_integral(e[0]) == ref.self_integral(e[0])
    assert port.integral(e[0], e[1], 0.1, 0, 1e-6, 1e-6, 7)[2] == -10


def test_port_equals_reference_linalg(pkg, port, ref, orc_mod):
    O = orc_mod
    e, nd = _grid_geom(pkg)
    m, n = e.shape[0], nd.shape[0]
    N = n + 2 * m
    img = O.images(e)
    s = 2e5 + 2j * np.pi * 1e6
    kappa = 0.01 + s * 10 * O.EPS0
    zl, zt = ref.hem_impedances(e, img, s, kappa)
    zlf = np.ascontiguousarray(zl.T).reshape(-1)
    ztf = np.ascontiguousarray(zt.T).reshape(-1)
    out = []
    for lib in (port, ref):
        wg = np.zeros(N * N, dtype=np.complex128)
        assert lib.fill_incidence_imm(wg, e, nd) == 0
        lib.fill_impedance_imm(wg, zlf, ztf, m, n)
        w0 = wg.copy()
        ie = np.zeros(N, dtype=np.complex128)
        ie[0] = 1.0
        assert lib.solve_immittance(wg, ie, m, n) == 0
        out.append((w0, ie))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    # incidence checksums of the reference (src/linalg.c:77-84)
    W = out[0][0].reshape(N, N).T
    A = W[n:n + m, :n]
    B = W[n + m:, :n]
    assert A.sum() == 0 and B.sum() == m


def test_port_equals_reference_nlt_soil_heidler(port, ref):
    f = np.sin(np.linspace(0, 7, 300)) ** 2
    g1, s1 = port.laplace_trans(f, 2e-4)
    g2, s2 = ref.laplace_trans(f, 2e-4)
    assert np.array_equal(g1, g2) and np.array_equal(s1, s2)
    for filt in range(5):
        a = port.inv_laplace_trans(g1, s1, 2e-4, 300, filt)
        b = ref.inv_laplace_trans(g1, s1, 2e-4, 300, filt)
        assert np.array_equal(a, b, equal_nan=True)
    for s in (2j * np.pi * 10.0, 3e4 + 2j * np.pi * 1e6):
        assert port.alipio_soil(1e-3, s, 1.26, 0.54, 12) == ref.alipio_soil(1e-3, s, 1.26, 0.54, 12)
    assert port.heidler(1e-6, 1e3, 1.8e-6, 95e-6, 2.0) == ref.heidler(1e-6, 1e3, 1.8e-6, 95e-6, 2.0)


def test_port_sweep_matches_reference_calls(pkg, port, ref, orc_mod):
    O = orc_mod
    e, nd = pkg.segment_electrode([0, 0, 0], [0, 0, -3], 10, 7e-3)
    img = O.images(e)
    s = 2j * np.pi * np.array([1e3, 1e6])
    kappa = 0.01 + s * 10 * O.EPS0
    sol, info = port.hem_sweep(e, img, nd, s, kappa, 0, np.ones(2), req_abs=1e-6, req_rel=1e-6, threads=2)
    assert np.all(info == 0)
    m, n = e.shape[0], nd.shape[0]
    N = n + 2 * m
    for k in range(2):
        zl, zt = ref.hem_impedances(e, img, s[k], kappa[k])
        wg = np.zeros(N * N, dtype=np.complex128)
        ref.fill_incidence_imm(wg, e, nd)
        ref.fill_impedance_imm(wg, np.ascontiguousarray(zl.T).reshape(-1), np.ascontiguousarray(zt.T).reshape(-1), m, n)
        ie = np.zeros(N, dtype=np.complex128)
        ie[0] = 1.0
        ref.solve_immittance(wg, ie, m, n)
        assert np.array_equal(ie, sol[k])


def _mhem_potentials(lib, e, img):
    m = e.shape[0]
    pot = [np.zeros(m * m, dtype=np.complex128) for _ in range(4)]
    assert lib.calculate_impedances(pot[0], pot[1], e, 0.0, 0.0, 0.0, 0.0, itype=4) == 0
    assert lib.impedances_images(pot[2], pot[3], e, img, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, itype=4) == 0
    return pot


def test_port_equals_reference_admittance(pkg, port, ref, orc_mod):
    """Nodal admittance formulation (src/linalg.c:142-350): incidence, yla /
    ytb (inverses overwrite ZL, ZT), YN in one and in two calls, zsysv on YN;
    restatement and reference agree bit for bit."""
    O = orc_mod
    e, nd = _grid_geom(pkg)
    m, n = e.shape[0], nd.shape[0]
    img = O.images(e)
    s = 2e5 + 2j * np.pi * 1e6
    kappa = 0.01 + s * 10 * O.EPS0
    zl, zt = ref.hem_impedances(e, img, s, kappa)
    zlf = np.ascontiguousarray(zl.T).reshape(-1)
    ztf = np.ascontiguousarray(zt.T).reshape(-1)
    out = []
    for lib in (port, ref):
        a = np.zeros(m * n, dtype=np.complex128)
        b = np.zeros(m * n, dtype=np.complex128)
        assert lib.fill_incidence_adm(a, b, e, nd) == 0
        zl1, zt1 = zlf.copy(), ztf.copy()
        yla = np.zeros(m * n, dtype=np.complex128)
        ytb = np.zeros(m * n, dtype=np.complex128)
        assert lib.calculate_yla_ytb(yla, ytb, zl1, zt1, a, b, m, n) == 0
        yn2 = np.zeros(n * n, dtype=np.complex128)
        lib.fill_impedance_adm2(yn2, yla, ytb, a, b, m, n)
        yn1 = np.zeros(n * n, dtype=np.complex128)
        assert lib.fill_impedance_adm(yn1, zlf.copy(), ztf.copy(), a, b, m, n) == 0
        ic = np.zeros(n, dtype=np.complex128)
        ic[0] = 1.0
        assert lib.solve_admittance(yn1.copy(), ic, n) == 0
        out.append((a, b, zl1, zt1, yla, ytb, yn2, yn1, ic))
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
    # the admittance potentials are the immittance ones (YN is W_G's node Schur complement)
    N = n + 2 * m
    wg = np.zeros(N * N, dtype=np.complex128)
    ref.fill_incidence_imm(wg, e, nd)
    ref.fill_impedance_imm(wg, zlf, ztf, m, n)
    ie = np.zeros(N, dtype=np.complex128)
    ie[0] = 1.0
    ref.solve_immittance(wg, ie, m, n)
    assert np.max(np.abs(out[0][8] - ie[:n])) < 1e-10 * np.max(np.abs(ie[:n]))


def test_mhem_sweep_follows_the_example_loop(pkg, port, ref, orc_mod):
    """The mHEM sample loop (examples/three_grids.c:270-392): per-sample
    impedances from the static potentials (numpy restatement of the loop's
    rescale), then the reference's yla/ytb, YN and zsysv; the restated sweep
    gives the same node potentials bit for bit."""
    O = orc_mod
    e, nd = _grid_geom(pkg)
    m, n = e.shape[0], nd.shape[0]
    img = O.images(e)
    s = np.array([3e4 + 2j * np.pi * 1e3, 3e4 + 2j * np.pi * 2e6])
    kappa = 0.01 + s * 10 * O.EPS0
    inj = np.array([1.0 + 0.5j, 2.0])
    sol, info = port.mhem_sweep(e, img, nd, s, kappa, 3, inj, threads=2)
    assert np.all(info == 0)
    pl, pt, pli, pti = (np.ascontiguousarray(x) for x in _mhem_potentials(ref, e, img))
    a = np.zeros(m * n, dtype=np.complex128)
    b = np.zeros(m * n, dtype=np.complex128)
    ref.fill_incidence_adm(a, b, e, nd)
    for k in range(2):
        gamma, ref_t = O.medium(s[k], kappa[k])
        iwu = s[k] * O.MU0 / (4 * np.pi)
        one_4pik = 1.0 / (4 * np.pi * kappa[k])
        zl = np.zeros(m * m, dtype=np.complex128)
        zt = np.zeros(m * m, dtype=np.complex128)
        for i in range(m):
            for j in range(i, m):
                rb = np.linalg.norm(e[j, 6:9] - e[i, 6:9])
                eg = np.exp(-gamma * rb)
                zl[i * m + j] = eg * pl[i * m + j]
                zt[i * m + j] = eg * pt[i * m + j]
                rb = np.linalg.norm(e[j, 6:9] - img[i, 6:9])
                eg = np.exp(-gamma * rb)
                zl[i * m + j] += 1.0 * eg * pli[i * m + j]
                zt[i * m + j] += ref_t * eg * pti[i * m + j]
                zl[i * m + j] *= iwu
                zt[i * m + j] *= one_4pik
        yla = np.zeros(m * n, dtype=np.complex128)
        ytb = np.zeros(m * n, dtype=np.complex128)
        assert ref.calculate_yla_ytb(yla, ytb, zl, zt, a.copy(), b.copy(), m, n) == 0
        yn = np.zeros(n * n, dtype=np.complex128)
        ref.fill_impedance_adm2(yn, yla, ytb, a.copy(), b.copy(), m, n)
        ic = np.zeros(n, dtype=np.complex128)
        ic[3] = inj[k]
        assert ref.solve_admittance(yn, ic, n) == 0
        assert np.max(np.abs(ic - sol[k])) <= 1e-12 * np.max(np.abs(ic))


# ---- golden fixtures (made by the reference) against the restatement ----------------

def test_golden_rod_zf(port, orc_mod):
    gd = golden("rod_zf.npz")
    e, nd = gd["elec"], gd["nodes"]
    img = orc_mod.images(e)
    idx = [0, 37, 99]
    sol, info = port.hem_sweep(e, img, nd, gd["s"][idx], gd["kappa"][idx], 0, np.ones(3), req_abs=0.0,
                               req_rel=1e-11, threads=2)
    assert np.all(info == 0)
    assert rel_err(sol[:, 0], gd["sol"][idx, 0]) < 1e-12


def test_golden_nlt(port):
    gd = golden("nlt.npz")
    for nt in (256, 255):
        g, s = port.laplace_trans(gd[f"f_{nt}"], 1e-4)
        assert rel_err(g, gd[f"g_{nt}"]) < 1e-13
        for filt in (0, 1, 2, 4):
            assert rel_err(port.inv_laplace_trans(g, s, 1e-4, nt, filt), gd[f"inv_{nt}_{filt}"]) < 1e-12
        # the reference's Lanczos window divides 0/0 at w = 0 (NaN everywhere)
        assert np.all(np.isnan(gd[f"inv_{nt}_3"])) == np.all(np.isnan(port.inv_laplace_trans(g, s, 1e-4, nt, 3)))


def test_golden_incidence_codes(port):
    gd = golden("incidence.npz")
    e = gd["elec"]
    for name in ("ok", "disconnected", "duplicate"):
        nd = gd[f"{name}_nodes"]
        N = nd.shape[0] + 2 * e.shape[0]
        wg = np.full(N * N, 7.0 + 7.0j, dtype=np.complex128)
        assert port.fill_incidence_imm(wg, e, nd) == int(gd[f"{name}_code"])
        assert np.array_equal(wg, gd[f"{name}_wg"])


# ---- known answers from the reference's closed forms ------------------------------

def test_self_integral_is_static_reduced_kernel(port, pkg):
    from scipy import integrate
    e = pkg.populate_electrode([0, 0, 0], [1.3, 0, 0], 4e-3)
    L, a = 1.3, 4e-3
    # \int_0^L \int_0^L dx dy / sqrt((x-y)^2 + a^2) = 2 \int_0^L (L-u)/sqrt(u^2+a^2) du
    val, _ = integrate.quad(lambda u: 2 * (L - u) / math.sqrt(u * u + a * a), 0, L, epsabs=0, epsrel=1e-13,
                            limit=200, points=[a, 10 * a])
    assert abs(port.self_integral(e) - val) < 1e-12 * val


def test_mhem_kernel_is_exact_static_integral(port, pkg):
    # logNf is the exact inner integral of 1/r: INTG_MHEM equals the 2-D static integral
    from scipy import integrate
    s_ = pkg.populate_electrode([0, 0, 0], [1.0, 0, 0], 5e-3)
    r_ = pkg.populate_electrode([0.3, 0.7, 0.2], [0.9, 1.5, -0.4], 5e-3)
    val, _, code = port.integral(s_, r_, 0.0, 0, 0.0, 1e-13, 4)
    L0, L1 = r_[9], s_[9]

    def f(t1, t0):
        pr = r_[0:3] + t0 * (r_[3:6] - r_[0:3])
        ps = s_[0:3] + t1 * (s_[3:6] - s_[0:3])
        return 1.0 / np.linalg.norm(pr - ps)
    num, _ = integrate.dblquad(f, 0, 1, 0, 1, epsabs=0, epsrel=1e-12)
    assert code == 0
    assert abs(val.real - num * L0 * L1) < 1e-10 * abs(val.real)


@pytest.mark.parametrize("grid,mn", [((5, 5, 10.0, 10.0, 3, 3), (120, 105)),
                                     ((13, 13, 60.0, 60.0, 5, 5), (1560, 1417)),
                                     ((25, 25, 120.0, 120.0, 5, 5), (6000, 5425))])
def test_grid_counts(pkg, grid, mn):
    vx, vy, lx, ly, nx, ny = grid
    assert (pkg.number_segments(vx, vy, nx, ny), pkg.number_nodes(vx, vy, nx, ny)) == mn


# ---- post-processing: potentials, fields, path voltage -----------------------

def test_port_equals_reference_fields(port, ref):
    """The restatement of src/electrode.c:434-668 against the reference's own
    functions (same cubature, same expression order: equal to rounding)."""
    d = golden("fields.npz")
    e = d["elec"]
    for k in (0, 2):
        for p in (0, 5, 6):
            pt = d["points"][p]
            a = port.electric_potential(pt, e, d["it"][k, 0], d["gamma"][k], d["kappa"][k], 0, 1e-13, 1e-11)
            b = ref.electric_potential(pt, e, d["it"][k, 0], d["gamma"][k], d["kappa"][k], 0, 1e-13, 1e-11)
            assert a == b
            va = port.magnetic_potential(pt, e, d["il"][k, 1], d["gamma"][k], 1.0, 0, 1e-13, 1e-11)
            vb = ref.magnetic_potential(pt, e, d["il"][k, 1], d["gamma"][k], 1.0, 0, 1e-13, 1e-11)
            assert np.array_equal(va, vb)
            for sv, ve in ((d["s"][k], None), (0.0, d["ve0"])):
                fa, ca = port.electric_field(pt, e, d["il"][k, 1], d["it"][k, 1], d["gamma"][k], sv, d["kappa"][k],
                                             1.0, 0, 1e-13, 1e-11, ve=ve)
                fb, cb = ref.electric_field(pt, e, d["il"][k, 1], d["it"][k, 1], d["gamma"][k], sv, d["kappa"][k],
                                            1.0, 0, 1e-13, 1e-11, ve=ve)
                assert ca == cb and np.array_equal(fa, fb)
        pa = d["paths"][0]
        a = port.voltage(pa[:3], pa[3:], e, d["il"][k, 0], d["it"][k, 0], d["gamma"][k], d["s"][k], d["kappa"][k],
                         1.0, 0, 1e-11, 1e-9)
        b = ref.voltage(pa[:3], pa[3:], e, d["il"][k, 0], d["it"][k, 0], d["gamma"][k], d["s"][k], d["kappa"][k],
                        1.0, 0, 1e-11, 1e-9)
        assert a == b


def test_golden_fields(port):
    """The restatement reproduces the reference's fixture (tests/golden/fields.npz)."""
    d = golden("fields.npz")
    e = d["elec"]
    for k in range(3):
        for r in range(2):
            for p in range(d["points"].shape[0]):
                u = port.electric_potential(d["points"][p], e, d["it"][k, r], d["gamma"][k], d["kappa"][k], 0, 1e-13,
                                            1e-11)
                assert abs(u - d["pot"][k, p, r]) <= 1e-12 * abs(d["pot"][k, p, r])
            l = 1
            v = port.voltage(d["paths"][l, :3], d["paths"][l, 3:], e, d["il"][k, r], d["it"][k, r], d["gamma"][k],
                             d["s"][k], d["kappa"][k], 1.0, 0, 1e-11, 1e-10)
            assert abs(v - d["voltage"][k, l, r]) <= 1e-12 * abs(d["voltage"][k, l, r])


def test_voltage_closed_form_equals_nested_cubature(port, orc_mod):
    """The identity the GPU path voltage rests on: the reference's nested
    integral of E . dl / |dl| over t equals (u(p1) - u(p2)) / |p2 - p1| (u the
    field-convention potential) minus s mu / 4pi sum_m il_m (D_m . t_hat)
    JJ_m, JJ_m the double integral of e^{-gamma r}/r between the path and
    electrode m (the INTG_DOUBLE pair integral)."""
    O = orc_mod
    d = golden("fields.npz")
    e = d["elec"]
    for k in (1, 2):
        for l in range(d["paths"].shape[0]):
            p1, p2 = d["paths"][l, :3], d["paths"][l, 3:]
            lp = float(np.linalg.norm(p2 - p1))
            th = (p2 - p1) / lp
            line = np.zeros(11)
            line[0:3], line[3:6], line[6:9], line[9] = p1, p2, (p1 + p2) / 2, lp
            it = d["it"][k, 1].copy()
            it[np.abs(it) < np.finfo(float).eps] = 0.0        # the field skips these
            u1 = port.electric_potential(p1, e, it, d["gamma"][k], d["kappa"][k], 0, 1e-14, 1e-12)
            u2 = port.electric_potential(p2, e, it, d["gamma"][k], d["kappa"][k], 0, 1e-14, 1e-12)
            acc = 0.0
            for q in range(e.shape[0]):
                il = d["il"][k, 1, q]
                if abs(il) < np.finfo(float).eps:
                    continue
                jj, _, code = port.integral(e[q], line, d["gamma"][k], 0, 1e-14, 1e-12, O.INTG_DOUBLE)
                assert code == 0
                acc += il * np.dot(e[q, 3:6] - e[q, 0:3], th) * jj / (lp * e[q, 9])
            v = (u1 - u2) / lp - d["s"][k] * O.MU0 / (4 * np.pi) * acc
            assert abs(v - d["voltage"][k, l, 1]) <= 1e-9 * abs(d["voltage"][k, l, 1])


def test_gpd_mhem_restates_the_example_loop(port, orc_mod):
    """examples/visacro57emc01.c:406-430 written out in numpy against the
    oracle's C restatement, and the mHEM closed form close to the full
    potential far from the grid."""
    O = orc_mod
    d = golden("fields.npz")
    e = d["elec"]
    pts = np.array([[1.0, 1.0, 0.0], [30.0, 20.0, 0.0]])
    k = 1
    it = d["it"][k].T                                          # (m, nrhs)
    want = np.zeros((2, 2), np.complex128)
    for p in range(2):
        for q in range(e.shape[0]):
            rbar = np.sqrt(np.sum((pts[p] - e[q, 6:9]) ** 2))
            r1 = np.sqrt(np.sum((pts[p] - e[q, 0:3]) ** 2))
            r2 = np.sqrt(np.sum((pts[p] - e[q, 3:6]) ** 2))
            r0 = (r1 + r2 + e[q, 9]) / (r1 + r2 - e[q, 9])
            want[p] += it[q] * np.exp(-d["gamma"][k] * rbar) * np.log(r0) / e[q, 9] / (O.FOUR_PI * d["kappa"][k])
    got = port.gpd_mhem(pts, e, it, d["gamma"][k], d["kappa"][k])
    assert np.max(np.abs(got - want) / np.abs(want)) <= 1e-13
    full = port.electric_potential(pts[1], e, it[:, 0], d["gamma"][k], d["kappa"][k], 0, 1e-13, 1e-11)
    assert abs(got[1, 0] - full) <= 2e-3 * abs(full)
