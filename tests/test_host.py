"""CPU tests of the host side: geometry/soil helpers against the reference
(bit for bit), and the C-ABI library's exported symbols (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_electrode_grid_matches_reference(pkg, ref):
    class Grid(ctypes.Structure):
        _fields_ = [("vx", ctypes.c_uint), ("vy", ctypes.c_uint), ("lx", ctypes.c_double), ("ly", ctypes.c_double),
                    ("nx", ctypes.c_uint), ("ny", ctypes.c_uint), ("r", ctypes.c_double), ("z", ctypes.c_double)]
    ref.lib.electrode_grid.argtypes = [Grid, ctypes.c_void_p, ctypes.c_void_p]
    for g in ((5, 5, 10.0, 10.0, 3, 3, 7e-3, -0.5), (13, 13, 60.0, 60.0, 5, 5, 7e-3, -0.5),
              (4, 7, 17.3, 29.1, 3, 5, 9e-3, -0.73), (2, 2, 1.0, 1.0, 1, 1, 1e-3, 0.0)):
        m = ref.lib.number_segments(Grid(*g))
        n = ref.lib.number_nodes(Grid(*g))
        e = np.zeros((m, 11))
        nd = np.zeros((n, 3))
        ref.lib.electrode_grid(Grid(*g), e.ctypes.data, nd.ctypes.data)
        pe, pn = pkg.electrode_grid(*g)
        assert (m, n) == (pkg.number_segments(g[0], g[1], g[4], g[5]), pkg.number_nodes(g[0], g[1], g[4], g[5]))
        assert np.array_equal(pe, e) and np.array_equal(pn, nd)


def test_segment_electrode_and_images_match_reference(pkg, ref, orc_mod):
    for a, b, k in (([0, 0, 0], [0, 0, -3], 10), ([1.5, -2, -0.5], [7.25, 3.1, -4.0], 7)):
        e1, n1 = ref.segment_electrode(a, b, k, 7e-3)
        e2, n2 = pkg.segment_electrode(a, b, k, 7e-3)
        assert np.array_equal(e1, e2) and np.array_equal(n1, n2)
        assert np.array_equal(pkg.images(e2), orc_mod.images(e1))


def test_soil_and_samples_match_reference(pkg, ref):
    for s in (2j * np.pi * 10.0, 3e4 + 2j * np.pi * 1e6, 8.1e4 + 0j):
        a = pkg.alipio_soil(1e-3, s, 1.26, 0.54, 12)
        b = ref.alipio_soil(1e-3, s, 1.26, 0.54, 12)
        assert abs(a[0] - b[0]) <= 1e-14 * abs(b[0]) and abs(a[1] - b[1]) <= 1e-14 * abs(b[1])
    g, s = ref.laplace_trans(np.ones(4094), 204.7e-6)
    assert np.array_equal(pkg.laplace_samples(4094, 204.7e-6), s)


def test_heidler_matches_reference(pkg, ref):
    for t in (0.0, 1e-7, 1.9e-6, 2e-5, 1e-4):
        for tau1, tau2, n in ((1.8e-6, 95e-6, 2.0), (0.454e-6, 143e-6, 10.0), (1.9e-6, 485e-6, 2.0)):
            a, b = pkg.heidler(t, 1e3, tau1, tau2, n), ref.heidler(t, 1e3, tau1, tau2, n)
            assert abs(a - b) <= 1e-14 * max(abs(b), 1e-300)


def test_logspace_linspace_match_reference(pkg):
    f = pkg.logspace(2, 7, 100)
    assert f[-1] == 1e7 and f[0] == 100.0 and len(f) == 100
    u = pkg.linspace(0.0, -3.0, 11)
    assert u[-1] == -3.0 and u[1] == 0.0 + 1 * (-3.0 / 10)


def _header_functions():
    text = open(os.path.join(ROOT, "include", "tags_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\s*\*?\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, re.M)
    return sorted(set(n for n in names if n not in ("if", "sizeof")))


def test_library_exports_every_declared_symbol(pkg):
    pkg.build()
    lib = ctypes.CDLL(pkg.LIB_PATH)
    declared = _header_functions()
    assert len(declared) >= 13
    for name in declared:
        assert hasattr(lib, name), name
    assert set(pkg.EXPORTS) <= set(declared)


def test_electrode_record_layout(pkg):
    # the C-ABI passes the reference's 88-byte Electrode unchanged
    class Electrode(ctypes.Structure):
        _fields_ = [("start", ctypes.c_double * 3), ("end", ctypes.c_double * 3), ("mid", ctypes.c_double * 3),
                    ("length", ctypes.c_double), ("radius", ctypes.c_double)]
    assert ctypes.sizeof(Electrode) == 88
    e = pkg.populate_electrode([0, 0, -0.5], [1, 0, -0.5], 7e-3)
    assert e.dtype == np.float64 and e.shape == (11,)


def test_compute_calls_fail_loudly_without_library(pkg, monkeypatch, tmp_path):
    monkeypatch.setattr(pkg, "_lib", None)
    monkeypatch.setattr(pkg, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="missing"):
        pkg.solve_immittance(np.zeros(9, np.complex128), np.zeros(3, np.complex128), 1, 1)


def _ref_lib(orc_mod):
    if not orc_mod.available("ref"):
        pytest.skip("reference build (oracle/_ref) not present here")
    # A private handle: argtypes set here must not leak into the shared
    # oracle object's function table.
    return ctypes.CDLL(orc_mod.get("ref").lib._name)


def test_geometry_files_match_reference(pkg, orc_mod, tmp_path):
    """electrodes_file / nodes_file (src/electrode.c:45-101): the library's
    host readers give the reference's arrays and return codes, bad lines and
    degenerate segments included."""
    ref = _ref_lib(orc_mod)
    for name in ("electrodes_file", "nodes_file"):
        getattr(ref, name).argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]
        getattr(ref, name).restype = ctypes.c_int
    rng = np.random.default_rng(4)
    good = tmp_path / "elec.csv"
    rows = np.round(rng.uniform(-5, 5, (6, 7)), 6)
    rows[:, 6] = np.abs(rows[:, 6]) + 1e-3
    good.write_text("\n".join(", ".join(f"{v:.6f}" for v in r) for r in rows) + "\n")
    short = tmp_path / "short.csv"
    short.write_text("0, 0, 0, 1, 0, 0, 0.01\n1, 0, 0, 2, 0\n")
    degen = tmp_path / "degen.csv"
    degen.write_text("0, 0, 0, 1, 0, 0, 0.01\n3, 3, 3, 3, 3, 3, 0.01\n")
    for path, m in ((good, 6), (short, 2), (degen, 2), (tmp_path / "missing.csv", 1)):
        pkg.lib().tags_gpu_set_quiet(1)
        code, e = pkg.electrodes_file(str(path), m)
        pkg.lib().tags_gpu_set_quiet(0)
        e_ref = np.zeros((m, 11))
        code_ref = ref.electrodes_file(str(path).encode(), e_ref.ctypes.data, m)
        assert code == code_ref and np.array_equal(e, e_ref), path.name
    nodes = tmp_path / "nodes.csv"
    nodes.write_text("1.5, -2, 0.25\n3, 4, 5\n7, 8\n")
    for n in (2, 3):
        pkg.lib().tags_gpu_set_quiet(1)
        code, nd = pkg.nodes_file(str(nodes), n)
        pkg.lib().tags_gpu_set_quiet(0)
        nd_ref = np.zeros((n, 3))
        code_ref = ref.nodes_file(str(nodes).encode(), nd_ref.ctypes.data, n)
        assert code == code_ref and np.array_equal(nd, nd_ref)


def test_soil_models_match_reference(pkg, orc_mod):
    """alipio_soil / smith_longmire_soil (src/auxiliary.c:60-93) exported by
    the library: within 1e-13 of the reference (C++ complex pow against C's
    cpow)."""
    ref = _ref_lib(orc_mod)
    C = pkg.c_complex
    ref.smith_longmire_soil.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, C, ctypes.c_double]
    ref.alipio_soil.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, C, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double]
    for s in (2j * np.pi * 50.0, 1e4 + 2j * np.pi * 3e5, 8e4 + 2j * np.pi * 1e7):
        want = np.zeros(2, np.complex128)
        ref.smith_longmire_soil(want[:1].ctypes.data, want[1:].ctypes.data, 1e-3, C.of(s), 10.0)
        got = pkg.smith_longmire_soil(1e-3, s, 10.0)
        assert abs(got[0] - want[0]) <= 1e-13 * abs(want[0]) and abs(got[1] - want[1]) <= 1e-13 * abs(want[1])
        ref.alipio_soil(want[:1].ctypes.data, want[1:].ctypes.data, 1e-3, C.of(s), 1.26, 0.54, 12.0)
        out = np.zeros(2, np.complex128)
        pkg.lib().alipio_soil(out[:1].ctypes.data, out[1:].ctypes.data, 1e-3, C.of(s), 1.26, 0.54, 12.0)
        assert np.max(np.abs(out - want) / np.abs(want)) <= 1e-13


def test_solve_batch_rejects_bad_jobs(pkg):
    """tags_gpu_solve_batch checks its jobs before touching the GPU: a job
    without electrodes, or an injection node beyond the grid, is TAGS_E_ARG."""
    import ctypes
    L = pkg.lib()
    e, nd = pkg.segment_electrode([0.0, 0.0, 0.0], [0.0, 0.0, -2.0], 4, 7e-3)
    s = np.array([2j * np.pi * 1e3])
    k = np.array([0.01 + 0j])
    good = pkg.GridJob(e.ctypes.data, None, e.shape[0], nd.ctypes.data, nd.shape[0], s.ctypes.data, k.ctypes.data,
                       1, None, 0, None, None)
    bad_node = pkg.GridJob(e.ctypes.data, None, e.shape[0], nd.ctypes.data, nd.shape[0], s.ctypes.data,
                           k.ctypes.data, 1, None, nd.shape[0], None, None)
    no_elec = pkg.GridJob(None, None, 0, nd.ctypes.data, nd.shape[0], s.ctypes.data, k.ctypes.data, 1, None, 0,
                          None, None)
    for job in (bad_node, no_elec):
        arr = (pkg.GridJob * 2)(good, job)
        assert L.tags_gpu_solve_batch(arr, 2, pkg.MIXED, 1.0, 0, 2) == pkg.E_ARG
    assert L.tags_gpu_solve_batch(None, 0, pkg.MIXED, 1.0, 0, 2) == 0


def test_tune_cache_setter_checks_its_file(pkg, tmp_path):
    """tags_gpu_set_tune_cache opens the file for appending (creating it) and
    keeps what is there; a path that cannot be opened is TAGS_E_ARG; None
    switches the cache off. No GPU is touched."""
    path = tmp_path / "tune.txt"
    pkg.set_tune_cache(str(path))
    assert path.exists() and path.read_text() == ""
    path.write_text("tags-tune 1 N=1 m=1 prec=1 fill=2 cap=1 pipes=1 pairs=0 gpu=x/1/sm103 | 1 6 16 1\n")
    pkg.set_tune_cache(str(path))
    assert path.read_text().count("\n") == 1
    with pytest.raises(RuntimeError, match=str(pkg.E_ARG)):
        pkg.set_tune_cache(str(tmp_path))          # a directory
    pkg.set_tune_cache(None)


def test_resumable_sweep_resumes_after_an_interruption(pkg, tmp_path):
    """A sweep interrupted inside a chunk keeps the chunks finished before it;
    the next call with the same fingerprint runs only the rest and returns the
    whole result; a finished sweep runs nothing; another sweep's fingerprint
    is refused."""
    calls = []

    def runner(fail_at):
        def run_chunk(k0, k1):
            if k0 == fail_at:
                raise RuntimeError("interrupted")
            calls.append(k0)
            x = np.arange(k0, k1, dtype=np.float64)
            return ({"sol": np.stack([x, 2.0 * x], axis=1), "info": np.zeros(k1 - k0, np.int32)},
                    {"fallbacks": k0, "seconds": 0.5})
        return run_chunk

    d = str(tmp_path / "sweep")
    fp = pkg.sweep_fingerprint([np.arange(10.0), 1.0, None])
    with pytest.raises(RuntimeError, match="interrupted"):
        pkg.resumable_sweep(runner(6), 10, d, 3, fp)
    assert calls == [0, 3]
    calls.clear()
    out, stats, ran = pkg.resumable_sweep(runner(-1), 10, d, 3, fp)
    assert calls == [6, 9] and ran == 2
    assert [t["fallbacks"] for t in stats] == [0, 3, 6, 9]
    assert np.array_equal(out["sol"][:, 0], np.arange(10.0)) and np.array_equal(out["sol"][:, 1], 2 * np.arange(10.0))
    assert out["info"].shape == (10,)
    calls.clear()
    out2, _, ran = pkg.resumable_sweep(runner(-1), 10, d, 3, fp)
    assert calls == [] and ran == 0 and np.array_equal(out2["sol"], out["sol"])
    with pytest.raises(ValueError, match="another sweep"):
        pkg.resumable_sweep(runner(-1), 10, d, 3, pkg.sweep_fingerprint([np.arange(11.0), 1.0, None]))
    with pytest.raises(ValueError, match="another sweep"):
        pkg.resumable_sweep(runner(-1), 10, d, 4, fp)


def _tri_tiles_full(M, zlo, zhi, planes, planes_band):
    """The lower-triangle tiles of an update of M rows, row by row, that do
    work or only write the next panel's planes: tiles wholly inside the zero
    band's rows (or columns) are skipped, and a skipped first-column tile below
    the first writes planes when planes is set (in the band's rows only with
    planes_band)."""
    T = -(-M // 128)
    out = []
    for I in range(T):
        for J in range(I + 1):
            rz = zhi > zlo and 128 * I >= zlo and 128 * I + 128 <= zhi
            cz = zhi > zlo and 128 * J >= zlo and 128 * J + 128 <= zhi
            if not (rz or cz):
                out.append((I, J, 0))
            elif planes and J == 0 and I >= 1 and (planes_band or not rz):
                out.append((I, J, 1))
    return out


def test_trailing_tile_list_leaves_out_the_zero_band(pkg):
    """The persistent GEMM's tile list of a trailing update (the closed form
    the kernel uses for the compacted list, run on the host) equals the full
    triangle filtered to the tiles that do work, in the same order, for update
    sizes and zero bands of every alignment, with and without the next panel's
    planes (and their band rows)."""
    fn = pkg.lib().tags_debug_tri_tiles
    fn.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p, ctypes.c_int]
    fn.restype = ctypes.c_int
    cases = 0
    for M in [1, 100, 128, 129, 700, 1500, 3769, 2977, 4537 - 128, 17875 - 768]:
        for zlo in sorted({0, 1, 24, 127, 128, 129, 300, 792, M // 3, M // 2}):
            for width in (0, 100, 128, 256, 1559, 1560, 1561, 3000):
                zhi = zlo + width
                if zhi > M:
                    continue
                for planes, planes_band in ((0, 0), (1, 1), (1, 0), (0, 1)):
                    want = _tri_tiles_full(M, zlo, zhi, planes, planes_band)
                    n = fn(M, zlo, zhi, planes, planes_band, None, 0)
                    assert n >= 0
                    out = np.zeros(3 * max(n, 1), np.int32)
                    assert fn(M, zlo, zhi, planes, planes_band, out.ctypes.data, n) == n
                    got = [tuple(int(v) for v in out[3 * l:3 * l + 3]) for l in range(n)]
                    assert got == want, (M, zlo, zhi, planes, planes_band)
                    cases += 1
    assert cases > 200
    assert fn(-1, 0, 0, 0, 0, None, 0) == pkg.E_ARG


def test_bench_reference_arm_contract():
    """`bench.py --impl reference` (the CPU implementation of the path on the
    host cores) prints one JSON line carrying the bench contract's keys, with
    its own cpu_baseline and an e2e object without host-device traffic."""
    import json
    import subprocess
    import sys
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["metric"].startswith("Laplace-sample solves/s")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
