"""GPU parity of the nodal admittance formulation the reference's mHEM
examples use (src/linalg.c:142-350, examples/three_grids.c:270-392): the five
drop-ins against the oracle (itself equal to the reference bit for bit), and
the plans' mHEM impedance model against the oracle's admittance sweep."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_fill_incidence_adm_bit_exact(gpu_pkg, port):
    pkg = gpu_pkg
    gd = golden("incidence.npz")
    e = gd["elec"]
    m = e.shape[0]
    pkg.lib().tags_gpu_set_quiet(1)
    try:
        for name in ("ok", "disconnected", "duplicate"):
            nd = gd[f"{name}_nodes"]
            n = nd.shape[0]
            res = []
            for lib in (pkg, port):
                a = np.full(m * n, 7.0 + 7.0j)
                b = np.full(m * n, 7.0 + 7.0j)
                code = lib.fill_incidence_adm(a, b, e, nd)
                same = np.full(m * n, 7.0 + 7.0j)          # a == b: the reference leaves A there
                code2 = lib.fill_incidence_adm(same, same, e, nd)
                res.append((code, a, b, code2, same))
            for x, y in zip(res[0], res[1]):
                assert np.array_equal(x, y), name
    finally:
        pkg.lib().tags_gpu_set_quiet(0)


def test_admittance_dropins_match_oracle(gpu_pkg, port):
    """yla / ytb (and the inverses left in ZL, ZT), YN in one and in two
    calls, and the YN solve: within 1e-10 of the oracle (LAPACK's symmetric
    factorisation there, LU with partial pivoting here)."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nd = gd["elec"], gd["nodes"]
    img = pkg.images(e)
    m, n = e.shape[0], nd.shape[0]
    s = 3e4 + 2j * np.pi * 5e5
    kappa = 0.01 + s * 10 * pkg.EPS0
    zl, zt = port.hem_impedances(e, img, s, kappa)
    zlf = np.ascontiguousarray(zl.T).reshape(-1)
    ztf = np.ascontiguousarray(zt.T).reshape(-1)
    a = np.zeros(m * n, np.complex128)
    b = np.zeros(m * n, np.complex128)
    assert port.fill_incidence_adm(a, b, e, nd) == 0
    out = {}
    for name, lib in (("gpu", pkg), ("cpu", port)):
        zl1, zt1 = zlf.copy(), ztf.copy()
        yla = np.zeros(m * n, np.complex128)
        ytb = np.zeros(m * n, np.complex128)
        assert lib.calculate_yla_ytb(yla, ytb, zl1, zt1, a, b, m, n) == 0
        yn2 = np.zeros(n * n, np.complex128)
        lib.fill_impedance_adm2(yn2, yla, ytb, a, b, m, n)
        yn1 = np.zeros(n * n, np.complex128)
        assert lib.fill_impedance_adm(yn1, zlf.copy(), ztf.copy(), a, b, m, n) == 0
        ic = np.zeros(n, np.complex128)
        ic[0] = 1.0
        yn_in = yn1.copy()
        assert lib.solve_admittance(yn_in, ic, n) == 0
        out[name] = (zl1, zt1, yla, ytb, yn2, yn1, ic, yn_in)
    g, c = out["gpu"], out["cpu"]
    lower = np.tril(np.ones((m, m), bool)).T.reshape(-1)       # element (k, i), k >= i, at k + m i
    assert _rel(g[0][lower], c[0][lower]) < 1e-10 and _rel(g[1][lower], c[1][lower]) < 1e-10
    for x, y in zip(g[2:7], c[2:7]):
        assert _rel(x, y) < 1e-10
    assert np.array_equal(g[7], g[5])                          # the GPU solve leaves YN unchanged


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_mhem_plan_matches_admittance_sweep(gpu_pkg, port, precision):
    """Config-2 grid, 16 samples of the 1024-sample set: the plan with the
    mHEM impedance model (immittance solve) gives the node potentials of the
    oracle's mHEM + nodal-admittance sweep: 1e-8 plain FP64, 1e-6 mixed."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nd = gd["elec"], gd["nodes"]
    img = pkg.images(e)
    n = nd.shape[0]
    idx = np.linspace(0, len(gd["s"]) - 1, 16).astype(int)
    s, kappa = gd["s"][idx], gd["kappa"][idx]
    ref, info = port.mhem_sweep(e, img, nd, s, kappa, 0, np.ones(len(s)), req_abs=1e-13, req_rel=1e-13)
    assert np.all(info == 0)
    prec = pkg.PLAIN_FP64 if precision == "plain" else pkg.MIXED
    sol, info, st = pkg.hem_sweep(e, img, nd, s, kappa, inj_node=0, precision=prec, fill=pkg.INTG_MHEM)
    assert np.all(info == 0) and st.fallbacks == 0
    tol = 1e-8 if precision == "plain" else 1e-6
    assert _rel(sol[:, :n], ref) < tol
