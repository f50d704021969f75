"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own C sources (compiled by ``make -C oracle ref`` into
oracle/_ref/libtags_ref.so, with the project-written stand-ins for its absent
third-party code: adaptive cubature, FFTW-compatible DFT, scipy's OpenBLAS for
zsysv) on the synthetic workloads the tests use, at tight cubature tolerance so
that the quadrature method does not limit the comparison. Needs the reference
sources at build time; the fixtures it writes are what travels.

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py fields     # one of them
"""
from __future__ import annotations

import math
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# 1.2/50 us double exponential, i(t) = I0 k (e^{-a t} - e^{-b t}) (the form of
# examples/three_grids.c:956-960 with the standard 1.2/50 constants)
I0, K12, ALPHA, BETA = 1000.0, 1.037, 1.0 / 68.2e-6, 1.0 / 0.405e-6
TIGHT = 1e-11
FABS = 1e-13


def ref():
    from oracle import oracle
    return oracle.get("ref")


def solve_sample(R, elec, img, nodes, s, kappa, inj_node, inj, rel):
    """One sample through the reference's own immittance path."""
    from oracle import oracle as O
    m, n = elec.shape[0], nodes.shape[0]
    N = n + 2 * m
    zl, zt = R.hem_impedances(elec, img, s, kappa, 1.0, 0, 0.0, rel)
    zl_flat = np.ascontiguousarray(zl.T).reshape(-1)
    zt_flat = np.ascontiguousarray(zt.T).reshape(-1)
    wg = np.zeros(N * N, dtype=np.complex128)
    code = R.fill_incidence_imm(wg, elec, nodes)
    assert code == 0, code
    R.fill_impedance_imm(wg, zl_flat, zt_flat, m, n)
    ie = np.zeros(N, dtype=np.complex128)
    ie[inj_node] = inj
    info = R.solve_immittance(wg, ie, m, n)
    assert info == 0, info
    return ie, zl, zt


def _worker(args):
    idx, elec, img, nodes, s, kappa, inj_node, inj, rel = args
    R = ref()
    out = []
    for k in idx:
        x, _, _ = solve_sample(R, elec, img, nodes, s[k], kappa[k], inj_node, inj[k], rel)
        out.append((k, x))
    return out


def sweep_parallel(elec, img, nodes, s, kappa, inj_node, inj, rel, procs=None):
    procs = procs or os.cpu_count() or 4
    chunks = [list(range(i, len(s), procs)) for i in range(procs)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_worker, [(c, elec, img, nodes, s, kappa, inj_node, inj, rel) for c in chunks])
    N = nodes.shape[0] + 2 * elec.shape[0]
    sol = np.zeros((len(s), N), dtype=np.complex128)
    for part in res:
        for k, x in part:
            sol[k] = x
    return sol


def lower_pack(z):
    m = z.shape[0]
    r, c = np.tril_indices(m)
    return z[r, c]


def make_rod():
    R = ref()
    elec, nodes = R.segment_electrode([0.0, 0.0, 0.0], [0.0, 0.0, -3.0], 10, 7e-3)
    from oracle import oracle as O
    img = O.images(elec)
    freq = np.array([10.0 ** (2 + i * (5.0 / 99)) for i in range(99)] + [1e7])
    s = 2j * np.pi * freq
    kappa = 1.0 / 100.0 + s * 10.0 * O.EPS0
    N = nodes.shape[0] + 2 * elec.shape[0]
    sols = np.zeros((len(s), N), dtype=np.complex128)
    zls, zts = [], []
    for k in range(len(s)):
        x, zl, zt = solve_sample(R, elec, img, nodes, s[k], kappa[k], 0, 1.0, TIGHT)
        sols[k] = x
        if k in (0, 50, 99):
            zls.append(lower_pack(zl))
            zts.append(lower_pack(zt))
    # the other integration types (no scaling) at one frequency, images included
    types = {}
    for name, it in (("mhem", O.INTG_MHEM), ("single", O.INTG_SINGLE), ("none", O.INTG_NONE)):
        zl, zt = R.hem_impedances(elec, img, s[60], kappa[60], 1.0, 0, 0.0, TIGHT, it)
        types[name + "_zl"] = lower_pack(zl)
        types[name + "_zt"] = lower_pack(zt)
    np.savez_compressed(os.path.join(HERE, "rod_zf.npz"), elec=elec, nodes=nodes, freq=freq, s=s, kappa=kappa,
                        sol=sols, zl=np.array(zls), zt=np.array(zts), z_idx=np.array([0, 50, 99]),
                        type_s=s[60], type_kappa=kappa[60], **types)


def make_grid2():
    R = ref()
    from oracle import oracle as O
    import __graft_entry__ as g
    pkg = g.load_package()
    elec, nodes = pkg.electrode_grid(5, 5, 10.0, 10.0, 3, 3, 7e-3, -0.5)
    img = O.images(elec)
    nt, tmax = 2046, 1023 / 10e6
    dt = tmax / (nt - 1)
    t = np.arange(nt) * dt
    i_t = I0 * K12 * (np.exp(-ALPHA * t) - np.exp(-BETA * t))
    inj_s, s = R.laplace_trans(i_t, tmax)
    kappa = 1.0 / 100.0 + s * 10.0 * O.EPS0
    t0 = time.time()
    sol = sweep_parallel(elec, img, nodes, s, kappa, 0, inj_s, 1e-10)
    print(f"grid2 sweep: {time.time() - t0:.1f} s")
    gpr = R.inv_laplace_trans(sol[:, 0], s, tmax, nt, O.FILTER_NONE)
    gpr_hann = R.inv_laplace_trans(sol[:, 0], s, tmax, nt, O.FILTER_HANNING)
    zl0, zt0 = R.hem_impedances(elec, img, s[0], kappa[0], 1.0, 0, 0.0, TIGHT)
    zl1, zt1 = R.hem_impedances(elec, img, s[700], kappa[700], 1.0, 0, 0.0, TIGHT)
    np.savez_compressed(os.path.join(HERE, "grid2.npz"), elec=elec, nodes=nodes, nt=nt, tmax=tmax, i_t=i_t,
                        inj_s=inj_s, s=s, kappa=kappa, u0=sol[:, 0], u_nodes_s0=sol[0, :nodes.shape[0]],
                        gpr=gpr, gpr_hann=gpr_hann, z_idx=np.array([0, 700]),
                        zl=np.array([lower_pack(zl0), lower_pack(zl1)]),
                        zt=np.array([lower_pack(zt0), lower_pack(zt1)]),
                        injection=np.array([I0, K12, ALPHA, BETA]))


def make_nlt():
    R = ref()
    out = {}
    for nt in (256, 255):
        tmax = 1e-4
        dt = tmax / (nt - 1)
        t = np.arange(nt) * dt
        f = np.exp(-t / 2e-5) * np.sin(2 * np.pi * t / 3e-5) + 0.3
        g, s = R.laplace_trans(f, tmax)
        out[f"f_{nt}"] = f
        out[f"g_{nt}"] = g
        out[f"s_{nt}"] = s
        for filt in range(5):
            out[f"inv_{nt}_{filt}"] = R.inv_laplace_trans(g, s, tmax, nt, filt)
    np.savez_compressed(os.path.join(HERE, "nlt.npz"), **out)


def make_incidence():
    """Return codes of fill_incidence_imm on valid and broken node sets."""
    R = ref()
    import __graft_entry__ as g
    pkg = g.load_package()
    elec, nodes = pkg.electrode_grid(3, 3, 4.0, 4.0, 2, 2, 5e-3, -0.6)
    m, n = elec.shape[0], nodes.shape[0]
    cases = {"ok": nodes.copy()}
    bad = nodes.copy()
    bad[4] = [50.0, 50.0, 50.0]
    cases["disconnected"] = bad
    dup = nodes.copy()
    dup[3] = dup[2]
    cases["duplicate"] = dup
    out = {"elec": elec}
    for name, nd in cases.items():
        N = n + 2 * m
        wg = np.full(N * N, 7.0 + 7.0j, dtype=np.complex128)
        code = R.fill_incidence_imm(wg, elec, nd)
        out[f"{name}_nodes"] = nd
        out[f"{name}_code"] = np.array(code)
        out[f"{name}_wg"] = wg
    np.savez_compressed(os.path.join(HERE, "incidence.npz"), **out)


def field_case():
    """Geometry, currents and observation points of the post-processing
    fixture: a 2 x 2-mesh grid at 0.5 m depth with a 3-segment rod at one
    corner, seeded complex currents for two injections and three samples, and
    points from far away to 1 cm off an electrode (and on a rod's axis below
    its tip)."""
    import __graft_entry__ as g
    from oracle import oracle as O
    pkg = g.load_package()
    grid, _ = pkg.electrode_grid(3, 3, 4.0, 4.0, 2, 2, 6e-3, -0.5)
    rod, _ = pkg.segment_electrode([0.0, 0.0, -0.5], [0.0, 0.0, -2.0], 3, 8e-3)
    elec = np.vstack([grid, rod])
    m = elec.shape[0]
    rng = np.random.default_rng(11)
    freq = np.array([60.0, 2.0e5, 8.0e6])
    s = 2j * np.pi * freq + np.array([0.0, 3.0e3, 4.0e4])
    kappa = 1.0 / 300.0 + s * 12.0 * O.EPS0
    gamma = np.array([O.medium(sk, kk)[0] for sk, kk in zip(s, kappa)])
    nrhs = 2
    il = rng.normal(size=(3, nrhs, m)) + 1j * rng.normal(size=(3, nrhs, m))
    it = rng.normal(size=(3, nrhs, m)) + 1j * rng.normal(size=(3, nrhs, m))
    il[:, 1, 5] = 0.0          # skipped electrodes (|I| < DBL_EPSILON)
    it[:, 1, 7] = 1e-17
    points = np.array([[1.0, 1.0, 0.0], [2.0, 0.5, 0.0], [-3.0, 7.0, 0.0], [25.0, -10.0, 0.0],
                       [0.7, 2.0, -0.49], [1.0, 0.01, -0.5], [0.0, 0.0, -2.6], [4.3, 4.1, -0.3]])
    paths = np.array([[-1.0, -1.0, 0.0, 1.0, 1.0, 0.0], [2.0, 2.0, 0.0, 6.0, 2.0, 0.0],
                      [0.5, 3.5, 0.0, 0.5, 3.5, -0.3]])
    return elec, s, kappa, gamma, il, it, points, paths


def make_fields():
    """electric_potential, magnetic_potential, electric_field (|s| > 0 and
    s = 0 with a nonzero ve to add to) and voltage from the reference itself.
    A small absolute tolerance (1e-13 on integrals of order one, 1e-11 on the
    nested voltage) ends the subdivision of field components that vanish by
    symmetry, which a purely relative request never satisfies."""
    R = ref()
    elec, s, kappa, gamma, il, it, points, paths = field_case()
    ns, nrhs = il.shape[0], il.shape[1]
    P, NL = points.shape[0], paths.shape[0]
    pot = np.zeros((ns, P, nrhs), np.complex128)
    vec = np.zeros((ns, P, nrhs, 3), np.complex128)
    ef = np.zeros((ns, P, nrhs, 3), np.complex128)
    ef0 = np.zeros((ns, P, nrhs, 3), np.complex128)
    ve0 = np.array([1.0 + 2.0j, -3.0, 0.5j])
    volt = np.zeros((ns, NL, nrhs), np.complex128)
    for k in range(ns):
        for r in range(nrhs):
            for p in range(P):
                pot[k, p, r] = R.electric_potential(points[p], elec, it[k, r], gamma[k], kappa[k], 0, FABS, TIGHT)
                vec[k, p, r] = R.magnetic_potential(points[p], elec, il[k, r], gamma[k], 1.0, 0, FABS, TIGHT)
                ef[k, p, r], _ = R.electric_field(points[p], elec, il[k, r], it[k, r], gamma[k], s[k], kappa[k],
                                                  1.0, 0, FABS, TIGHT)
                ef0[k, p, r], _ = R.electric_field(points[p], elec, il[k, r], it[k, r], gamma[k], 0.0, kappa[k],
                                                   1.0, 0, FABS, TIGHT, ve=ve0)
            for l in range(NL):
                volt[k, l, r] = R.voltage(paths[l, :3], paths[l, 3:], elec, il[k, r], it[k, r], gamma[k], s[k],
                                          kappa[k], 1.0, 0, 1e-11, 1e-10)
    np.savez_compressed(os.path.join(HERE, "fields.npz"), elec=elec, s=s, kappa=kappa, gamma=gamma, il=il, it=it,
                        points=points, paths=paths, pot=pot, vecpot=vec, efield=ef, efield_s0=ef0, ve0=ve0,
                        voltage=volt)


if __name__ == "__main__":
    from oracle import oracle as O
    O.build(ref=True)
    if len(sys.argv) > 1:
        for name in sys.argv[1:]:
            globals()["make_" + name]()
        sys.exit(0)
    make_nlt()
    make_incidence()
    make_fields()
    make_rod()
    make_grid2()
    print("fixtures written to", HERE)
