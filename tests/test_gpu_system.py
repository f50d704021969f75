"""GPU parity of the immittance assembly, the solve, the Laplace pair and the
batched plans (plain FP64 and mixed) against golden fixtures and the oracle."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def test_incidence_bit_exact(gpu_pkg, port):
    pkg = gpu_pkg
    gd = golden("incidence.npz")
    e = gd["elec"]
    pkg.lib().tags_gpu_set_quiet(1)
    for name in ("ok", "disconnected", "duplicate"):
        nd = gd[f"{name}_nodes"]
        N = nd.shape[0] + 2 * e.shape[0]
        wg = np.full(N * N, 7.0 + 7.0j, dtype=np.complex128)
        assert pkg.fill_incidence_imm(wg, e, nd) == int(gd[f"{name}_code"])
        assert np.array_equal(wg, gd[f"{name}_wg"])
    pkg.lib().tags_gpu_set_quiet(0)


def test_fill_impedance_bit_exact(gpu_pkg, port):
    pkg = gpu_pkg
    rng = np.random.default_rng(2)
    m, n = 17, 13
    N = n + 2 * m
    zl = rng.standard_normal(m * m) + 1j * rng.standard_normal(m * m)
    zt = rng.standard_normal(m * m) + 1j * rng.standard_normal(m * m)
    w1 = rng.standard_normal(N * N) + 1j * rng.standard_normal(N * N)
    w2 = w1.copy()
    assert pkg.fill_impedance_imm(w1, zl, zt, m, n) == 0
    port.fill_impedance_imm(w2, zl, zt, m, n)
    assert np.array_equal(w1, w2)


def _assemble_host(pkg, e, img, nodes, s, kappa):
    m, n = e.shape[0], nodes.shape[0]
    N = n + 2 * m
    gamma, ref_t = pkg.medium(s, kappa)
    zl = np.zeros(m * m, np.complex128)
    zt = np.zeros(m * m, np.complex128)
    pkg.calculate_impedances(zl, zt, e, gamma, s, 1.0, kappa)
    pkg.impedances_images(zl, zt, e, img, gamma, s, 1.0, kappa, 1.0, ref_t)
    wg = np.zeros(N * N, np.complex128)
    assert pkg.fill_incidence_imm(wg, e, nodes) == 0
    pkg.fill_impedance_imm(wg, zl, zt, m, n)
    return wg, zl, zt


def test_solve_matches_zsysv(gpu_pkg, port):
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    img = pkg.images(e)
    m, n = e.shape[0], nodes.shape[0]
    N = n + 2 * m
    for k in (0, 300, 1023):
        wg, _, _ = _assemble_host(pkg, e, img, nodes, gd["s"][k], gd["kappa"][k])
        w2 = wg.copy()
        x1 = np.zeros(N, np.complex128)
        x1[0] = gd["inj_s"][k]
        x2 = x1.copy()
        assert pkg.solve_immittance(wg, x1, m, n) == 0
        assert port.solve_immittance(w2, x2, m, n) == 0
        assert rel_err(x1, x2) < 1e-10
    # singular system: a disconnected node makes a zero column
    z = np.zeros(9, np.complex128)
    w = np.zeros(9, np.complex128)
    w[0] = 1.0
    pkg.lib().tags_gpu_set_quiet(1)
    assert pkg.solve_immittance(w, z[:3].copy(), 1, 1) > 0
    pkg.lib().tags_gpu_set_quiet(0)


def test_laplace_pair_matches_golden(gpu_pkg):
    pkg = gpu_pkg
    gd = golden("nlt.npz")
    for nt in (256, 255):
        g, s = pkg.laplace_trans(gd[f"f_{nt}"], 1e-4)
        assert rel_err(g, gd[f"g_{nt}"]) < 1e-12 and rel_err(s, gd[f"s_{nt}"]) < 1e-15
        for filt in (0, 1, 2, 4):
            # fed the reference's spectrum, the inverse matches to rounding times e^{c t_max} = nt^2
            want = gd[f"inv_{nt}_{filt}"]
            assert rel_err(pkg.inv_laplace_trans(gd[f"g_{nt}"], s, 1e-4, nt, filt), want) < 4e-16 * nt * nt
            assert rel_err(pkg.inv_laplace_trans(g, s, 1e-4, nt, filt), want) < 2e-15 * nt * nt
        assert np.all(np.isnan(pkg.inv_laplace_trans(g, s, 1e-4, nt, 3)))   # reference's 0/0 at w = 0


def test_plain_plan_rod_harmonic_impedance(gpu_pkg):
    """Config 1: Z(f) of the 3 m rod, 100 frequencies, plain FP64 <= 1e-8."""
    pkg = gpu_pkg
    gd = golden("rod_zf.npz")
    e, nodes = gd["elec"], gd["nodes"]
    sol, info, _ = pkg.hem_sweep(e, pkg.images(e), nodes, gd["s"], gd["kappa"], inj_node=0)
    assert np.all(info == 0)
    z = sol[:, 0]
    assert np.max(np.abs(z - gd["sol"][:, 0]) / np.abs(gd["sol"][:, 0])) < 1e-8


def _grid2_gpr(pkg, precision, split=None):
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    n = nodes.shape[0]
    ie = np.zeros((len(gd["s"]), n), np.complex128)
    ie[:, 0] = gd["inj_s"]
    sol, info, st = pkg.hem_sweep(e, pkg.images(e), nodes, gd["s"], gd["kappa"], ie=ie, precision=precision,
                                  split=split)
    gpr = pkg.inv_laplace_trans(sol[:, 0], gd["s"], float(gd["tmax"]), int(gd["nt"]))
    return gd, sol, info, st, gpr


def test_plain_plan_grid_gpr(gpu_pkg):
    """Config 2: GPR at the corner node, 1024 samples, plain FP64 <= 1e-8."""
    gd, sol, info, _, gpr = _grid2_gpr(gpu_pkg, gpu_pkg.PLAIN_FP64)
    assert np.all(info == 0)
    assert np.max(np.abs(sol[:, 0] - gd["u0"]) / np.abs(gd["u0"])) < 1e-8
    assert rel_err(gpr, gd["gpr"]) < 1e-8


@pytest.mark.parametrize("split", [3, 16])
def test_mixed_plan_grid_gpr(gpu_pkg, split):
    """Config 2, mixed form (bf16 x3 and fp16 x2 products): impedance and GPR
    <= 1e-6 against the reference, no FP64 fallback."""
    gd, sol, info, st, gpr = _grid2_gpr(gpu_pkg, gpu_pkg.MIXED, split)
    assert np.all(info == 0)
    assert st.fallbacks == 0 and st.split == split
    assert np.max(np.abs(sol[:, 0] - gd["u0"]) / np.abs(gd["u0"])) < 1e-6
    assert rel_err(gpr, gd["gpr"]) < 1e-6
    assert st.max_iterations >= 1


def test_full_size_properties(gpu_pkg):
    """60 x 60 m grid (N = 4537): the plain and mixed plans agree with the
    drop-in solve, the drop-in solution has an FP64 backward error, and the
    transfer impedances are reciprocal (W_G symmetric)."""
    pkg = gpu_pkg
    e, nodes = pkg.electrode_grid(13, 13, 60.0, 60.0, 5, 5, 7e-3, -0.5)
    img = pkg.images(e)
    m, n = e.shape[0], nodes.shape[0]
    N = n + 2 * m
    c = np.log(4094.0 ** 2) / 204.7e-6
    s = np.array([c + 2j * np.pi * 2e4, c + 2j * np.pi * 7e6])
    kap = []
    for sk in s:
        sig, epsr = pkg.alipio_soil(1e-3, sk, 1.26 * (1e-3 * 1e3) ** -0.73, 0.54, 12)
        kap.append(sig + sk * epsr * pkg.EPS0)
    kappa = np.array(kap)
    centre = int(np.argmin(np.linalg.norm(nodes - [30.0, 30.0, -0.5], axis=1)))
    wg, _, _ = _assemble_host(pkg, e, img, nodes, s[0], kappa[0])
    W = wg.reshape(N, N).T.copy()
    Wsym = np.tril(W) + np.tril(W, -1).T
    x = np.zeros(N, np.complex128)
    x[centre] = 1.0
    assert pkg.solve_immittance(wg, x, m, n) == 0
    b = np.zeros(N, np.complex128)
    b[centre] = 1.0
    berr = np.linalg.norm(Wsym @ x - b, np.inf) / (np.linalg.norm(Wsym, np.inf) * np.linalg.norm(x, np.inf))
    assert berr < 1e-13
    plain, _, _ = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=centre, precision=pkg.PLAIN_FP64)
    assert rel_err(plain[0], x) < 1e-9
    for split in (3, 16):
        mixed, info, st = pkg.hem_sweep(e, img, nodes, s, kappa, inj_node=centre, precision=pkg.MIXED, split=split)
        assert np.all(info == 0) and st.fallbacks == 0 and st.split == split
        assert np.max(np.abs(mixed[:, :n] - plain[:, :n])) / np.max(np.abs(plain[:, :n])) < 1e-6
    # reciprocity: potential at node 0 for a current at the centre equals the reverse
    other, _, _ = pkg.hem_sweep(e, img, nodes, s[:1], kappa[:1], inj_node=0, precision=pkg.PLAIN_FP64)
    assert abs(other[0, centre] - plain[0, 0]) < 1e-11 * abs(plain[0, 0])


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_graph_passes_match_direct_launches(gpu_pkg, precision):
    """Config 2 grid, 40 samples in passes of 16 (two full passes and a
    ragged one of 8): each pass as one CUDA-graph launch (the mixed form's
    refinement as a conditional while-node) gives the same solutions and
    iteration counts as launching the kernels one by one."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    img = pkg.images(e)
    idx = np.linspace(0, len(gd["s"]) - 1, 40).astype(int)
    s, kappa = gd["s"][idx], gd["kappa"][idx]
    ie = np.zeros((len(idx), nodes.shape[0]), np.complex128)
    ie[:, 0] = gd["inj_s"][idx]
    prec = pkg.PLAIN_FP64 if precision == "plain" else pkg.MIXED
    out = {}
    for graphs in (False, True):
        launches0 = pkg.lib().tags_gpu_launch_count()
        sol, info, st = pkg.hem_sweep(e, img, nodes, s, kappa, ie=ie, precision=prec, max_batch=16,
                                      graphs=graphs)
        out[graphs] = (sol, info, st.max_iterations, st.fallbacks,
                       pkg.lib().tags_gpu_launch_count() - launches0)
        assert np.all(info == 0)
    (sd, _, itd, fbd, nd), (sg, _, itg, fbg, ng) = out[False], out[True]
    assert itd == itg and fbd == fbg == 0
    assert np.max(np.abs(sg - sd)) <= 1e-12 * np.max(np.abs(sd))
    assert np.max(np.abs(sg[:, 0] - gd["u0"][idx]) / np.abs(gd["u0"][idx])) < (1e-8 if precision == "plain" else 1e-6)
    # the graph path counts the kernels its launches ran: same order as direct
    assert ng > 0 and abs(ng - nd) <= 0.1 * nd


def test_autotuner_keeps_a_valid_configuration(gpu_pkg):
    """tags_plan_tune times the candidate configurations on 64 samples of the
    config-2 grid and keeps the fastest; solutions after tuning stay within
    1e-6 of the reference."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=64)
    try:
        res = plan.tune(gd["s"][:64], gd["kappa"][:64], inj_node=0)
        assert res.candidates >= 12
        assert res.samples_per_pass in (16, 32, 64) and res.panels_per_update in (1, 2, 4, 6) and res.split in (3, 16)
        assert res.solves_per_second > 0
        ie = np.zeros((len(gd["s"]), nodes.shape[0]), np.complex128)
        ie[:, 0] = gd["inj_s"]
        sol, info, st = plan.run(gd["s"], gd["kappa"], ie=ie)
        assert np.all(info == 0) and st.fallbacks == 0
        assert np.max(np.abs(sol[:, 0] - gd["u0"]) / np.abs(gd["u0"])) < 1e-6
    finally:
        plan.close()


def test_panels_per_update_give_the_same_solution(gpu_pkg):
    """tags_plan_set_panels: 1, 3, 5 and 6 panels per trailing update solve the
    config-2 grid's samples within 1e-6 of the reference and within 1e-9 of
    each other (refinement to the same FP64 tolerance); 7 is an argument
    error."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    s, kappa = gd["s"][::16], gd["kappa"][::16]
    ie = np.zeros((len(s), nodes.shape[0]), np.complex128)
    ie[:, 0] = gd["inj_s"][::16]
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=64)
    try:
        with pytest.raises(RuntimeError, match=f"failed \\({pkg.E_ARG}\\)"):
            plan.set_panels(7)
        u = {}
        for panels in (1, 3, 5, 6):
            plan.set_panels(panels)
            sol, info, st = plan.run(s, kappa, ie=ie)
            assert np.all(info == 0) and st.fallbacks == 0
            u[panels] = sol[:, 0]
            assert np.max(np.abs(u[panels] - gd["u0"][::16]) / np.abs(gd["u0"][::16])) < 1e-6
        for panels in (1, 3, 5):
            assert np.max(np.abs(u[panels] - u[6]) / np.abs(u[6])) < 1e-9
    finally:
        plan.close()


def test_tune_cache_applies_a_stored_configuration(gpu_pkg, tmp_path):
    """With a tune cache the first tune of a shape times the candidates and
    appends one line; another plan of the same shape applies that line without
    timing and solves within 1e-6 of the reference; TAGS_TUNE_REFRESH times
    again and appends a second line."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    s, kappa = gd["s"][:32], gd["kappa"][:32]
    path = tmp_path / "tune.txt"
    pkg.set_tune_cache(str(path))
    try:
        plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=32)
        try:
            first = plan.tune(s, kappa, inj_node=0)
        finally:
            plan.close()
        assert first.candidates >= 8
        lines = path.read_text().splitlines()
        N = nodes.shape[0] + 2 * e.shape[0]
        assert len(lines) == 1 and f" N={N} m={e.shape[0]} prec={pkg.MIXED} " in lines[0] and " cap=32 " in lines[0]
        plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=32)
        try:
            hit = plan.tune(s, kappa, inj_node=0)
            assert hit.candidates == 0
            assert (hit.samples_per_pass, hit.panels_per_update, hit.split) == \
                (first.samples_per_pass, first.panels_per_update, first.split)
            ie = np.zeros((len(gd["s"]), nodes.shape[0]), np.complex128)
            ie[:, 0] = gd["inj_s"]
            sol, info, st = plan.run(gd["s"], gd["kappa"], ie=ie)
            assert np.all(info == 0) and st.fallbacks == 0
            assert np.max(np.abs(sol[:, 0] - gd["u0"]) / np.abs(gd["u0"])) < 1e-6
            again = plan.tune(s, kappa, inj_node=0, refresh=True)
            assert again.candidates >= 8
        finally:
            plan.close()
        assert len(path.read_text().splitlines()) == 2
    finally:
        pkg.set_tune_cache(None)


def test_resumable_sweep_matches_one_run(gpu_pkg, tmp_path):
    """Plan.run_resumable over chunks of 128 samples (the injection node's
    potential kept) equals one run of the same plan within 1e-12; called again
    it loads every chunk and launches no kernel."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    s, kappa = gd["s"][:300], gd["kappa"][:300]
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=64)
    try:
        whole, info, _ = plan.run(s, kappa, inj_node=0)
        assert np.all(info == 0)
        d = str(tmp_path / "sweep")
        u, info_r, st = plan.run_resumable(s, kappa, d, inj_node=0, chunk=128, columns=[0])
        assert st["chunks_run"] == 3 and st["fallbacks"] == 0 and np.all(info_r == 0)
        assert u.shape == (300, 1)
        assert np.max(np.abs(u[:, 0] - whole[:, 0]) / np.abs(whole[:, 0])) <= 1e-12
        before = pkg.launch_count()
        u2, _, st2 = plan.run_resumable(s, kappa, d, inj_node=0, chunk=128, columns=[0])
        assert st2["chunks_run"] == 0 and pkg.launch_count() == before and np.array_equal(u2, u)
    finally:
        plan.close()


def test_batched_inverse_laplace_matches_single_series(gpu_pkg):
    """The batched inverse (examples' layout: sample-major series, scaled
    output) equals the single-series drop-in for every column and window, bit
    for bit (same sums in the same order), and the reference's golden inverse
    within the single-series bound."""
    pkg = gpu_pkg
    gd = golden("nlt.npz")
    rng = np.random.default_rng(5)
    for nt in (256, 255):
        g0, s = gd[f"g_{nt}"], gd[f"s_{nt}"]
        ns = nt // 2 + 1
        G = np.stack([g0, 2.0 * g0, rng.standard_normal(ns) + 1j * rng.standard_normal(ns)], axis=1)
        G[0, 2] = G[0, 2].real
        for filt in (0, 1, 2, 4):
            F = pkg.inv_laplace_batch(G, s, 1e-4, nt, filt)
            for q in range(G.shape[1]):
                assert np.array_equal(F[:, q], pkg.inv_laplace_trans(G[:, q].copy(), s, 1e-4, nt, filt))
            assert rel_err(F[:, 0], gd[f"inv_{nt}_{filt}"]) < 4e-16 * nt * nt


@pytest.mark.parametrize("pipes", [2, 3])
@pytest.mark.parametrize("graphs", [True, False])
def test_two_pipelines_match_one(gpu_pkg, graphs, pipes):
    """A plan with two or three passes in flight (twin plans take passes as
    they free up, each on its own stream from its own host thread) gives the
    single-pipeline solutions and statistics: config 2 grid, 72 samples in
    passes of 16 (five passes, the last ragged), with graphs and kernel by
    kernel, host buffers."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    img = pkg.images(e)
    idx = np.linspace(0, len(gd["s"]) - 1, 72).astype(int)
    s, kappa = gd["s"][idx], gd["kappa"][idx]
    ie = np.zeros((len(idx), nodes.shape[0]), np.complex128)
    ie[:, 0] = gd["inj_s"][idx]
    plan = pkg.Plan(e, img, nodes, pkg.MIXED, max_batch=16, graphs=graphs)
    count = pkg.lib().tags_gpu_launch_count
    try:
        c0 = count()
        one, info1, st1 = plan.run(s, kappa, 1.0, ie)
        c1 = count()
        plan.set_pipelines(pipes)
        two, info2, st2 = plan.run(s, kappa, 1.0, ie)      # the twins capture their graphs here
        c2 = count()
        again, _, _ = plan.run(s, kappa, 1.0, ie)
        c3 = count()
        plan.set_split(3)                       # settings follow to the twins
        three, info3, _ = plan.run(s, kappa, 1.0, ie)
    finally:
        plan.close()
    # the same passes launch the same kernels whichever pipeline runs them,
    # and captures made on concurrent host threads are not counted (a few
    # percent allowed for a refinement step more or less)
    n1, n2, n3 = c1 - c0, c2 - c1, c3 - c2
    assert n1 > 0 and abs(n2 - n1) <= 0.05 * n1 and abs(n3 - n1) <= 0.05 * n1
    assert np.max(np.abs(again - two)) <= 1e-12 * np.max(np.abs(two))
    assert np.all(info1 == 0) and np.all(info2 == 0) and np.all(info3 == 0)
    assert st1.max_iterations == st2.max_iterations and st1.fallbacks == st2.fallbacks == 0
    assert np.max(np.abs(two - one)) <= 1e-12 * np.max(np.abs(one))
    assert np.max(np.abs(three[:, 0] - gd["u0"][idx]) / np.abs(gd["u0"][idx])) < 1e-6
    assert st2.seconds > 0


def test_two_sm_updates_match_single_sm(gpu_pkg):
    """The trailing updates on two-SM clusters (tcgen05 cta_group::2, 256 x
    128 complex products, or real-form products of N = 256) give the
    single-SM results: config 2 grid, 40 samples, and two samples of the
    60 x 60 m grid (N = 4537)."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    idx = np.linspace(0, len(gd["s"]) - 1, 40).astype(int)
    cases = [(e, nodes, gd["s"][idx], gd["kappa"][idx], 0)]
    e4, n4 = pkg.electrode_grid(13, 13, 60.0, 60.0, 5, 5, 7e-3, -0.5)
    c = np.log(4094.0 ** 2) / 204.7e-6
    s4 = np.array([c + 2j * np.pi * 2e4, c + 2j * np.pi * 7e6])
    k4 = np.array([1e-3 + sk * 12 * pkg.EPS0 for sk in s4])
    cases.append((e4, n4, s4, k4, int(np.argmin(np.linalg.norm(n4 - [30.0, 30.0, -0.5], axis=1)))))
    for elec, nd, s, kappa, inj in cases:
        out = []
        for pairs in (0, 1, 2):
            plan = pkg.Plan(elec, pkg.images(elec), nd, pkg.MIXED, max_batch=len(s))
            try:
                plan.set_tc_pairs(pairs)
                sol, info, st = plan.run(s, kappa, 1.0, None, inj)
            finally:
                plan.close()
            assert np.all(info == 0) and st.fallbacks == 0
            out.append(sol)
        for o in out[1:]:
            assert rel_err(o, out[0]) < 1e-12


@pytest.mark.parametrize("count,per_pass", [(40, 16), (200, 100)])
def test_solve_paths_match_in_plans(gpu_pkg, count, per_pass):
    """The mixed form's refinement with its triangular solves chosen by pass
    size (the default: clusters of four CTAs per sample for passes of 16; for
    passes of 100 one CTA per sample, and clusters of four per sample in the
    steps with at most SMs / 4 samples left), on clusters of four, one CTA per
    sample, and block by block: identical solutions and refinement counts
    (config 2 grid, CUDA graphs; the first solve of each pass starts at the
    node rows in all)."""
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    idx = np.linspace(0, len(gd["s"]) - 1, count).astype(int)
    s, kappa = gd["s"][idx], gd["kappa"][idx]
    ie = np.zeros((len(idx), nodes.shape[0]), np.complex128)
    ie[:, 0] = gd["inj_s"][idx]
    out = []
    for path in (-1, 4, 1, 0):
        assert pkg.lib().tags_debug_solve_path(path) == 0
        try:
            sol, info, st = pkg.hem_sweep(e, pkg.images(e), nodes, s, kappa, ie=ie, precision=pkg.MIXED,
                                          max_batch=per_pass)
        finally:
            pkg.lib().tags_debug_solve_path(-1)
        assert np.all(info == 0) and st.fallbacks == 0
        out.append((sol, st.max_iterations))
    for sol, it in out[1:]:
        assert np.array_equal(sol, out[0][0]) and it == out[0][1]
    assert np.max(np.abs(out[0][0][:, 0] - gd["u0"][idx]) / np.abs(gd["u0"][idx])) < 1e-6
