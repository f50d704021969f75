"""GPU checks of the other grid workloads: many uneven grids solved at once
(one plan per grid, plans in flight together) and the 120 x 120 m grid with
50 rods (N = 17875). The mixed form is held to 1e-6 against the plain FP64
form on the same samples; each test prints the figures it measured."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_uneven_grids_batched(gpu_pkg):
    """Eight of the 64 uneven grids (sizes spread from the smallest to the
    largest), 16 of each grid's 256 Laplace samples (nt = 510, 10 MHz), unit
    current at node 0: every grid's mixed-form node potentials within 1e-6 of
    the plain FP64 form's, no FP64 fallback."""
    pkg = gpu_pkg
    grids = pkg.uneven_grids(64, seed=0)
    order = np.argsort([len(g["electrodes"]) for g in grids])
    pick = [int(order[k]) for k in np.linspace(0, 63, 8).astype(int)]
    s = pkg.laplace_samples(510, 255 / 10e6)[::16]
    jobs = []
    for gi in pick:
        g = grids[gi]
        jobs.append({"electrodes": g["electrodes"], "images": pkg.images(g["electrodes"]), "nodes": g["nodes"],
                     "s": s, "kappa": 1.0 / g["rho"] + s * g["epsr"] * pkg.EPS0, "inj_node": 0})
    t0 = time.perf_counter()
    mixed = pkg.hem_sweep_grids(jobs, pkg.MIXED, workers=4)
    t_mixed = time.perf_counter() - t0
    plain = pkg.hem_sweep_grids(jobs, pkg.PLAIN_FP64, workers=4)
    errs = []
    for gi, job, (xm, im, sm), (xp, ip, _) in zip(pick, jobs, mixed, plain):
        n = len(job["nodes"])
        assert np.all(im == 0) and np.all(ip == 0)
        assert sm.fallbacks == 0
        errs.append(_rel(xm[:, :n], xp[:, :n]))
    print(f"\nuneven grids: m = {[len(grids[gi]['electrodes']) for gi in pick]}, "
          f"max rel err vs FP64 per grid = {['%.1e' % e for e in errs]}, "
          f"mixed {len(pick) * len(s) / t_mixed:.0f} solves/s (wall, incl. plan set-up)")
    assert max(errs) < 1e-6


def test_grid_with_rods_n17875(gpu_pkg):
    """The 120 x 120 m grid (24 x 24 meshes, 1 m segments) with 50 rods of
    3 m: m = 6150, n = 5575, N = 17875. Eight samples spread over a
    512-sample set (nt = 1022, 10 MHz), one at a time in the mixed form (its
    refinement steps per sample) and all in the plain FP64 form: node
    potentials within 1e-8 of FP64 (the mixed form's fill is FP64-accurate),
    no fallback."""
    pkg = gpu_pkg
    e, nodes = pkg.grid_with_rods()
    m, n = e.shape[0], nodes.shape[0]
    assert (m, n) == (6150, 5575)
    img = pkg.images(e)
    s_all = pkg.laplace_samples(1022, 511 / 10e6)
    idx = np.linspace(0, len(s_all) - 1, 8).astype(int)
    s = s_all[idx]
    kappa = 1.0 / 100.0 + s * 10.0 * pkg.EPS0
    centre = int(np.argmin(np.linalg.norm(nodes - [60.0, 60.0, -0.5], axis=1)))
    plan = pkg.Plan(e, img, nodes, pkg.MIXED, max_batch=1)
    xm, steps = [], []
    t0 = time.perf_counter()
    try:
        for k in range(len(s)):
            x, info, st = plan.run(s[k:k + 1], kappa[k:k + 1], 1.0, None, centre)
            assert np.all(info == 0) and st.fallbacks == 0
            xm.append(x[0])
            steps.append(st.max_iterations)
    finally:
        plan.close()
    t_mixed = time.perf_counter() - t0
    t0 = time.perf_counter()
    xp, ip, _ = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=centre, precision=pkg.PLAIN_FP64, max_batch=4)
    t_plain = time.perf_counter() - t0
    assert np.all(ip == 0)
    errs = [_rel(xm[k][:n], xp[k, :n]) for k in range(len(s))]
    print(f"\nN = 17875, samples {list(idx)} of 512: refinement steps {steps}, rel err vs FP64 "
          f"{['%.1e' % x for x in errs]}; mixed {t_mixed:.1f} s (one sample per run, incl. plan set-up), "
          f"plain FP64 {t_plain:.1f} s")
    assert max(errs) < 1e-8


def test_solve_batch_many_grids_matches_plans(gpu_pkg):
    """tags_gpu_solve_batch (many grids x many samples in one C call) gives the
    per-grid plans' solutions: three uneven grids, 12 samples each, plain FP64
    to rounding and the mixed form within 1e-6 of it."""
    pkg = gpu_pkg
    from oracle import oracle as O
    jobs = []
    for k, (nv, L, seg) in enumerate([(3, 10.0, 2), (4, 12.0, 1), (2, 6.0, 3)]):
        e, nd = pkg.electrode_grid(nv, nv, L, L, seg, seg, 7e-3, -0.5)
        f = np.logspace(2, 6.5, 12)
        s = 2j * np.pi * f + 1e3
        kappa = 1.0 / (100.0 * (k + 1)) + s * 10.0 * O.EPS0
        jobs.append({"electrodes": e, "images": pkg.images(e), "nodes": nd, "s": s, "kappa": kappa,
                     "inj_node": k})
    for precision, tol in ((pkg.PLAIN_FP64, 1e-13), (pkg.MIXED, 1e-6)):
        got = pkg.solve_batch(jobs, precision=precision, workers=3)
        ref = pkg.hem_sweep_grids(jobs, precision=pkg.PLAIN_FP64, workers=1)
        for (sol, info), (rsol, rinfo, _) in zip(got, ref):
            assert not np.any(info) and not np.any(rinfo)
            err = np.max(np.abs(sol - rsol)) / np.max(np.abs(rsol))
            assert err <= tol, (precision, err)


@pytest.mark.parametrize("sigma", [1e-3, 0.05])
def test_bent_wire_long_segments(gpu_pkg, sigma):
    """A bent wire of 4 m segments (a 40 m horizontal run and a 20 m rod
    down from its end): every neighbouring pair shares an endpoint, collinear
    along each leg and at a right angle at the bend. From 1 kHz to 20 MHz
    |gamma| L reaches ~5 (sigma = 1 mS/m) and ~12 (sigma = 50 mS/m), so the
    touching-pair rule runs from its series branch to its reduced exponential
    with up to 22 nodes per half. Mixed-form node potentials within 1e-6 of
    the plain FP64 form's, and the longitudinal currents as well."""
    pkg = gpu_pkg
    eh, nh = pkg.segment_electrode([0.0, 0.0, -0.5], [40.0, 0.0, -0.5], 10, 7e-3)
    ev, nv = pkg.segment_electrode([40.0, 0.0, -0.5], [40.0, 0.0, -20.5], 5, 7e-3)
    e = np.vstack([eh, ev])
    nodes = np.vstack([nh, nv[1:]])
    img = pkg.images(e)
    m, n = e.shape[0], nodes.shape[0]
    f = np.array([1e3, 1e5, 1e6, 5e6, 1e7, 2e7])
    s = 2e4 + 2j * np.pi * f
    kappa = sigma + s * 10.0 * pkg.EPS0
    xm, im, sm = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=0, precision=pkg.MIXED)
    xp, ip, _ = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=0, precision=pkg.PLAIN_FP64)
    assert np.all(im == 0) and np.all(ip == 0) and sm.fallbacks == 0
    for k in range(len(s)):
        assert _rel(xm[k, :n], xp[k, :n]) < 1e-6, (f[k], _rel(xm[k, :n], xp[k, :n]))
        assert _rel(xm[k, n:n + m], xp[k, n:n + m]) < 1e-6, (f[k], _rel(xm[k, n:n + m], xp[k, n:n + m]))


def test_near_dc_refinement_extrapolated(gpu_pkg):
    """The benchmark grid (60 x 60 m, N = 4537) at its four lowest Laplace
    samples (nt = 4094, 10 MHz; Alipio soil, sigma0 = 1 mS/m), where one slow
    mode makes plain refinement contract by up to ~0.5 per step (21 steps):
    with the extrapolated steps the mixed form needs at most 8, without
    fallback, and its node potentials stay within 1e-6 of the plain FP64
    form's."""
    pkg = gpu_pkg
    e, nodes = pkg.electrode_grid(13, 13, 60.0, 60.0, 5, 5, 7e-3, -0.5)
    img = pkg.images(e)
    n = nodes.shape[0]
    s = pkg.laplace_samples(4094, 2047 / 10e6)[:4]
    kappa = np.empty_like(s)
    for k, sk in enumerate(s):
        sig, epsr = pkg.alipio_soil(1e-3, sk, 1.26, 0.54, 12.0)
        kappa[k] = sig + sk * epsr * pkg.EPS0
    centre = int(np.argmin(np.linalg.norm(nodes - [30.0, 30.0, -0.5], axis=1)))
    xm, im, sm = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=centre, precision=pkg.MIXED)
    xp, ip, _ = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=centre, precision=pkg.PLAIN_FP64)
    assert np.all(im == 0) and np.all(ip == 0) and sm.fallbacks == 0
    print(f"\nnear DC: refinement steps <= {sm.max_iterations}, rel err {_rel(xm[:, :n], xp[:, :n]):.1e}")
    assert sm.max_iterations <= 8
    for k in range(len(s)):
        assert _rel(xm[k, :n], xp[k, :n]) < 1e-6
