"""Benchmark of the HEM hot path: Laplace-sample solves/s on the 60 x 60 m,
12 x 12-mesh grid (1560 segments, 1417 nodes, N = n + 2m = 4537 unknowns),
Alipio soil (sigma0 = 1 mS/m), lightning current injected at the centre node,
2048 Laplace samples (nt = 4094, omega_max = 2 pi 10 MHz).

One step = one pass of the whole per-sample path (fill ZL/ZT with images,
immittance assembly, factorisation, solve/refinement) over one batch of
samples, cycling through the 2048-sample set. Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|plain]
  python bench.py --impl reference      # the reference's CPU path on the host cores
  python bench.py --workload fields     # post-processing: potentials and field along a line
  python bench.py --workload grids      # 64 grids of uneven size x 256 samples in one call
  python bench.py --workload mhem       # the examples' mHEM impedance model, same grid and samples
  python bench.py --workload rods       # 120 x 120 m grid with 50 rods (N = 17875), 512 samples
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = dict(vertices_x=13, vertices_y=13, length_x=60.0, length_y=60.0, edge_segments_x=5, edge_segments_y=5,
            radius=7e-3, depth=-0.5)
NT = 4094
TMAX = 2047 / 10e6          # omega_max = 2 pi 10 MHz
SIGMA0 = 1e-3
H_SOIL = 1.26 * (SIGMA0 * 1e3) ** -0.73
G_SOIL = 0.54
EPS_RATIO = 12.0
# 1.2/50 us double exponential, 1 kA
I0, K12, ALPHA, BETA = 1000.0, 1.037, 1.0 / 68.2e-6, 1.0 / 0.405e-6


def workload(pkg):
    """Geometry, Laplace samples, soil and injection of the benchmark."""
    elec, nodes = pkg.electrode_grid(**GRID)
    img = pkg.images(elec)
    s = pkg.laplace_samples(NT, TMAX)
    kappa = np.empty_like(s)
    for k, sk in enumerate(s):
        sig, epsr = pkg.alipio_soil(SIGMA0, sk, H_SOIL, G_SOIL, EPS_RATIO)
        kappa[k] = sig + sk * epsr * pkg.EPS0
    dt = TMAX / (NT - 1)
    t = np.arange(NT) * dt
    i_t = I0 * K12 * (np.exp(-ALPHA * t) - np.exp(-BETA * t))
    c = math.log(float(NT) ** 2) / TMAX
    inj = np.fft.rfft(i_t * dt * np.exp(-c * t))   # same transform as laplace_trans (host copy for inputs)
    centre = int(np.argmin(np.linalg.norm(nodes - [30.0, 30.0, GRID["depth"]], axis=1)))
    return elec, img, nodes, s, kappa, inj, centre


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[0]) for r in self.rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in self.rows for j in range(4) if r[3 + j].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        # the tensor-core kernels run inside seconds-long steps: the sustained
        # (power-capped) bf16 figure is their ceiling
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops_sustained", d["bf16_tflops"]),
                "bf16_kind": "sustained" if "bf16_tflops_sustained" in d else "burst", "src": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1700.0, "bf16_kind": "sustained", "src": "fallback"}


PROFILE_FAMILIES = 11
TENSOR_FAMILIES = {"ldl_trailing_gemm", "ldl_panel_gemm"}
FP64_FAMILIES = {"lu_fp64_gemm"}


def fp64_peak(pkg):
    """FP64 throughput of this GPU, measured here (tags_probe_fp64): DFMA on
    the CUDA cores and DMMA (mma.sync m8n8k4 f64) on the FP64 tensor path.
    The plain form's FP64 kernels run on DFMA."""
    dfma, dmma = pkg.probe_fp64()
    return {"dfma_tflops": dfma, "dmma_tflops": dmma, "peak": max(dfma, dmma),
            "note": "measured in this run by tags_probe_fp64 (8 FMA chains per thread; 4 m8n8k4 f64 "
                    "accumulators per warp), best of three launches each"}


def read_profile(pkg):
    import ctypes
    fn = pkg.lib().tags_gpu_profile_read
    fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_char_p, ctypes.c_int]
    out = {}
    for fam in range(PROFILE_FAMILIES):
        n = ctypes.c_longlong()
        ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        name = ctypes.create_string_buffer(64)
        if fn(fam, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(by), name, 64) == 0 and n.value:
            out[name.value.decode()] = {"launches": n.value, "ms": ms.value, "flops": fl.value, "bytes": by.value}
    return out


# DRAM bytes of the trailing-update family (k_gemm_tc<2, 0>), one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum, 1 pass) of all 35 launches of
# one 128-sample pass of this workload (groups of six panels, bench.py --steps 1
# --warmup 1 --pipelines 1 --no-graphs --batch 128, launches -k k_gemm_tc<2, 0>
# -c 35): 63.15 GB, i.e. 14.1 MB per launch per sample. The traffic grows in
# proportion to the samples in the pass.
TRAILING_DRAM_BYTES_PER_LAUNCH_SAMPLE = 63.15e9 / 35 / 128
# Pipe use of the mixed form's fill kernel (k_fill_moment), from an ncu
# --set full capture of its first launch in a 16-sample bench run.
FILL_PIPES = {"kernel": "k_fill_moment", "issue_active": 0.818, "fma_pipe": 0.627, "alu_pipe": 0.184,
              "fp64_pipe": 0.025, "xu_pipe": 0.016, "dram_frac": 0.117,
              "source": "ncu --set full, first k_fill_moment launch of a 16-sample pass (profiles/)",
              "note": "FP32 ALU-bound (float-pair series); the log-singular entries run on the FP64 pipe in "
                      "k_fill_special64 (84 % of its pipe)"}


def roofline(prof, peaks, pieces=3, fp64=None, samples_per_pass=None):
    """Roofline of the family with the largest device time.

    Tensor families: `achieved` counts the algorithmic complex flops of the
    update outside the structural zero band (8 per complex multiply-add);
    the split-bf16 execution runs `products` real bf16 products per real
    product (6 for three pieces, 3 for two), which `executed_tflops` gives."""
    if not prof:
        return None, None
    name, f = max(prof.items(), key=lambda kv: kv[1]["ms"])
    sec = f["ms"] * 1e-3
    if name in TENSOR_FAMILIES:
        ach = f["flops"] / sec / 1e12
        products = 6 if pieces == 3 else 3
        form = {3: "three bf16 pieces", 2: "two bf16 pieces", 16: "two fp16 pieces of 2^8 x"}.get(pieces, str(pieces))
        traffic = (TRAILING_DRAM_BYTES_PER_LAUNCH_SAMPLE * samples_per_pass
                   if name == "ldl_trailing_gemm" and samples_per_pass else None)
        roof = {"bound": "tensor", "achieved": ach, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["bf16_tflops"], "traffic": traffic,
                "traffic_note": "DRAM bytes per average launch (ncu capture of one pass, scaled by samples per "
                                "pass); algorithmic C traffic is 16 B per updated element per group of panels",
                "kernel": name, "launches": f["launches"], "avg_launch_ms": f["ms"] / f["launches"],
                "executed_tflops": ach * products, "executed_frac": ach * products / peaks["bf16_tflops"],
                "note": f"achieved = algorithmic complex LDL^T flops outside the zero ZL/ZT band; the "
                        f"split into {form} runs {products} tensor products per real product "
                        f"(executed_*); peak = {peaks['src']} dense bf16, {peaks['bf16_kind']}"}
    elif name in FP64_FAMILIES:
        ach = f["flops"] / sec / 1e12
        pk = fp64["peak"] if fp64 else None
        roof = {"bound": "fp64", "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                "frac": ach / pk if pk else None, "traffic": None, "kernel": name, "launches": f["launches"],
                "avg_launch_ms": f["ms"] / f["launches"],
                "note": "FP64 pipe; peak = the faster of DFMA and DMMA measured in this run (tags_probe_fp64)"}
    else:
        ach = f["bytes"] / sec / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": ach / peaks["hbm_gbs"], "traffic": None, "kernel": name, "launches": f["launches"],
                "avg_launch_ms": f["ms"] / f["launches"], "note": f"peak = {peaks['src']} HBM copy"}
    fams = {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                "share": round(v["ms"] / sum(x["ms"] for x in prof.values()), 4)} for k, v in prof.items()}
    return roof, fams


def cpu_baseline(args, elec, img, nodes, s, kappa, inj, centre, nsamp):
    """The oracle (restatement of the reference's path A) on the host cores:
    OpenMP over samples, OpenBLAS on 1 thread, the reference's tolerances."""
    from oracle import oracle as O
    port = O.get("port")
    cores = os.cpu_count() or 1
    idx = np.linspace(0, len(s) - 1, nsamp).astype(int)
    t0 = time.perf_counter()
    sol, info = port.hem_sweep(elec, img, nodes, s[idx], kappa[idx], centre, inj[idx], req_abs=1e-6, req_rel=1e-6,
                               threads=min(cores, nsamp))
    dt = time.perf_counter() - t0
    return {"value": nsamp / dt, "unit": "solves/s", "cores": min(cores, nsamp), "kind": "port",
            "sample": f"{nsamp} strided Laplace samples of the 2048-sample set, path A "
                      f"(INTG_DOUBLE cubature at req_abs=req_rel=1e-6, zsysv with lwork<=100), "
                      f"one sample per OpenMP thread, {dt:.1f} s"}, sol, info, idx


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__ as entry
    pkg = entry.load_package()
    elec, img, nodes, s, kappa, inj, centre = workload(pkg)
    cores = os.cpu_count() or 1
    nsamp = cores          # one Laplace sample per core per step
    from oracle import oracle as O
    port = O.get("port")
    times = []
    # each step is ~10-15 s of all host cores
    steps = args.ref_steps if args.steps <= 0 else max(1, min(args.steps, args.ref_steps))
    for step in range(steps):
        idx = (np.arange(nsamp) * 127 + step * 61) % len(s)
        t0 = time.perf_counter()
        port.hem_sweep(elec, img, nodes, s[idx], kappa[idx], centre, inj[idx], req_abs=1e-6, req_rel=1e-6,
                       threads=cores)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = nsamp * steps / tot
    line = {"impl": "reference", "metric": "Laplace-sample solves/s (1560-segment grid, 2048 samples)",
            "value": value, "unit": "solves/s", "n_gpus": 0, "steps": steps, "warmup": 0,
            "ms_per_step": 1e3 * tot / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic",
            "config": {"workload": "grid 60x60 m, 12x12 meshes, 1560 segments, N=4537, Alipio soil, "
                                   "2048 Laplace samples", "samples_per_step": nsamp, "path": "A (traditional HEM)"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"{nsamp} Laplace samples per step (one per core), {steps} step(s); the "
                                       "reference's path A restated in C (oracle/), cubature tolerance 1e-6, "
                                       "zsysv with lwork<=100; warm-up skipped (no device state)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---- post-processing workload -------------------------------------------------
# The field line of examples/visacro57emc01.c:229-247 (direction atan(5/4),
# starting 6 m outside the grid, four injections), here 251 points 0.3 m apart
# across the benchmark grid at ground level; every Laplace sample of the set.
FIELD_POINTS, FIELD_RHS, FIELD_STEP = 251, 4, 0.3
# FP64 pipe operations one rule-node evaluation executes in k_fields
# (potential, vector potential and field for four injections): (DFMA x 2 + DADD
# + DMUL) per evaluation, from an ncu count of the kernel (see profiles/).
FIELD_FP64_FLOPS_PER_EVAL = 196.9


def field_points():
    hyp = math.hypot(4.0, 5.0)
    d = np.arange(FIELD_POINTS) * FIELD_STEP
    return np.column_stack([-6.0 + d * 4.0 / hyp, -6.0 + d * 5.0 / hyp, np.zeros(FIELD_POINTS)])


def field_currents(step, nb, m):
    """Seeded synthetic currents of one step ([sample][injection][electrode]);
    the cost of the kernels does not depend on their values."""
    rng = np.random.default_rng(1000 + step)
    il = rng.standard_normal((nb, FIELD_RHS, m)) + 1j * rng.standard_normal((nb, FIELD_RHS, m))
    it = rng.standard_normal((nb, FIELD_RHS, m)) + 1j * rng.standard_normal((nb, FIELD_RHS, m))
    return il, it


def field_cpu_baseline(pkg, elec, pts, s, kappa, gamma, budget_s=12.0):
    """The reference's per-point loop (examples/visacro57emc01.c:436-458:
    electric_field with s = 0, then magnetic_potential, per injection) on the
    oracle, at the example's tolerances (1e-6), on all host cores (ctypes
    releases the GIL), for about budget_s seconds of wall time."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    port = O.get("port")
    cores = os.cpu_count() or 1
    m = elec.shape[0]
    il, it = field_currents(0, 1, m)

    def one(job):
        k, p = job
        for r in range(FIELD_RHS):
            port.electric_field(pts[p], elec, il[0, r], it[0, r], gamma[k], 0.0, kappa[k], 1.0, 0, 1e-6, 1e-6)
            port.magnetic_potential(pts[p], elec, il[0, r], gamma[k], 1.0, 0, 1e-6, 1e-6)
        return 1

    jobs = [(k, p) for k in np.linspace(0, len(s) - 1, 64).astype(int) for p in range(0, FIELD_POINTS, 10)]
    done, t0 = 0, time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        for q in range(0, len(jobs), cores):
            done += sum(ex.map(one, jobs[q:q + cores]))
            if time.perf_counter() - t0 > budget_s:
                break
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "point-samples/s", "cores": cores, "kind": "port",
            "sample": f"{done} (sample, point) pairs of the workload, 4 injections each, the example's loop "
                      f"(electric_field at s=0 + magnetic_potential per injection, cubature 1e-6) in {dt:.1f} s"}


def run_fields(args):
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    if args.steps <= 0:
        args.steps = 8
    import __graft_entry__ as entry
    pkg = entry.load_package()
    pkg.build()
    elec, img, nodes, s, kappa, inj, centre = workload(pkg)
    gamma = np.sqrt(s * pkg.MU0 * kappa)
    m = elec.shape[0]
    pts = field_points()
    B = args.batch or 128
    ns_total = len(s)
    dev = torch.device("cuda", local)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)   # > L2

    def batch(step):
        k0 = (step * B) % ns_total
        nb = min(B, ns_total - k0)
        il, it = field_currents(step, nb, m)
        return k0, nb, il, it

    for w in range(args.warmup):
        k0, nb, il, it = batch(w)
        pkg.fields_batch(pts, elec, il, it, gamma[k0:k0 + nb], kappa[k0:k0 + nb])
    steps = [batch(args.warmup + q) for q in range(args.steps)]     # host inputs made before the timed region
    torch.cuda.synchronize()
    pkg.fields_evaluations(reset=True)
    launches0 = pkg.launch_count()
    fp64 = fp64_peak(pkg)
    pkg.lib().tags_gpu_profile(1)
    wall, ps = 0.0, 0
    with ClockSampler(local) as clk:
        for k0, nb, il, it in steps:
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = pkg.fields_batch(pts, elec, il, it, gamma[k0:k0 + nb], kappa[k0:k0 + nb])
            wall += time.perf_counter() - t0
            ps += nb * FIELD_POINTS
            if out["status"] != 0:
                raise RuntimeError("field evaluation flagged a point on an electrode")
    prof = read_profile(pkg)
    pkg.lib().tags_gpu_profile(0)
    launches = pkg.launch_count() - launches0
    evals = pkg.fields_evaluations()
    f = prof.get("fields")
    dev_s = f["ms"] * 1e-3
    value = ps / dev_s
    roof = {"bound": "fp64", "kernel": "fields", "launches": f["launches"], "avg_launch_ms": f["ms"] / f["launches"],
            "evaluations_per_launch": evals / f["launches"], "evaluations_per_s": evals / dev_s,
            "unit": "TFLOP/s", "peak": fp64["peak"], "traffic": None}
    if FIELD_FP64_FLOPS_PER_EVAL:
        ach = evals * FIELD_FP64_FLOPS_PER_EVAL / dev_s / 1e12
        roof.update({"achieved": ach, "frac": ach / fp64["peak"],
                     "note": "executed FP64 flops (ncu count per rule-node evaluation x evaluations counted on "
                             "the device) over the measured DFMA throughput of this pool's GB300"})
    else:
        roof.update({"achieved": None, "frac": None, "note": "FP64 operations per evaluation not yet counted"})
    B_h2d = sum(2 * nb * FIELD_RHS * m * 16 + 2 * nb * 16 for _, nb, _, _ in steps) / len(steps)
    B_d2h = sum(7 * nb * FIELD_POINTS * FIELD_RHS * 16 for _, nb, _, _ in steps) / len(steps)
    line = {"metric": "field point-samples/s (1560-segment grid, 251-point line, 4 injections, 2048 samples)",
            "value": value, "unit": "point-samples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (reference grid generator, Alipio soil; "
                                                          "seeded currents)",
            "config": {"workload": "grid 60x60 m, 1560 segments; 251 ground-level points 0.3 m apart on the line "
                                   "atan(5/4) from (-6, -6); potential, vector potential and field for 4 "
                                   "injections; 2048 Laplace samples of the solve benchmark",
                       "samples_per_step": B, "l2": "flushed between steps (256 MB write)"},
            "roofline": roof, "gpu_launches": launches, "clocks": clk.summary(),
            "e2e": {"value": ps / wall, "unit": "point-samples/s", "h2d_bytes_per_step": int(B_h2d),
                    "d2h_bytes_per_step": int(B_d2h)}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = field_cpu_baseline(pkg, elec, pts, s, kappa, gamma)
    print(json.dumps(line))
    return 0


# ---- mHEM + nodal admittance: what the reference's examples run ---------------------
# The same grid, soil, current and samples; the impedances from the mHEM model
# (static potentials once per geometry, rescaled per sample by e^{-gamma r}
# of the midpoint distances, examples/three_grids.c:270-350) and the node
# potentials of the nodal-admittance system (src/linalg.c:142-350), which is
# the node-block Schur complement of the immittance system the plan solves.

def mhem_cpu_baseline(elec, img, nodes, s, kappa, inj, centre, cores):
    """Path B on the host cores: the oracle's restatement of the examples'
    loop (INTG_MHEM potentials once, then per sample the rescale,
    calculate_yla_ytb, fill_impedance_adm2 and zsysv on n x n; OpenMP over
    samples, OpenBLAS on one thread). Two runs separate the once-per-geometry
    potentials from the per-sample cost; the value is the whole 2048-sample
    job's rate with the potentials amortised over it."""
    from oracle import oracle as O
    port = O.get("port")
    idx1 = np.linspace(0, len(s) - 1, cores).astype(int)
    idx2 = np.linspace(0, len(s) - 1, 2 * cores).astype(int)
    t0 = time.perf_counter()
    port.mhem_sweep(elec, img, nodes, s[idx1], kappa[idx1], centre, inj[idx1], threads=cores)
    t1 = time.perf_counter()
    port.mhem_sweep(elec, img, nodes, s[idx2], kappa[idx2], centre, inj[idx2], threads=cores)
    t2 = time.perf_counter()
    per_sample = max((t2 - t1) - (t1 - t0), 1e-9) / cores          # wall s per sample at `cores` threads
    setup = max((t1 - t0) - cores * per_sample, 0.0)
    ns = len(s)
    return {"value": ns / (setup + ns * per_sample), "unit": "solves/s", "cores": cores, "kind": "port",
            "per_sample_rate": 1.0 / per_sample, "potentials_s": setup,
            "sample": f"path B (mHEM potentials at cubature 1e-6, per-sample rescale + calculate_yla_ytb + "
                      f"fill_impedance_adm2 + zsysv n x n), {cores} and {2 * cores} strided samples in "
                      f"{t1 - t0:.1f} s and {t2 - t1:.1f} s; value = 2048 samples with the once-per-geometry "
                      f"potentials amortised"}


def run_mhem(args):
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    pkg.build()
    elec, img, nodes, s, kappa, inj, centre = workload(pkg)
    m, n = elec.shape[0], nodes.shape[0]
    N = n + 2 * m
    B = args.batch or 128
    P = args.pipelines or 2
    SB = B * (args.step_passes or P)
    plan = pkg.Plan(elec, img, nodes, pkg.MIXED, max_batch=B)
    plan.set_fill(pkg.INTG_MHEM)
    if P > 1:
        plan.set_pipelines(P)
    ns_total = len(s)
    steps = args.steps if args.steps > 0 else -(-ns_total // SB)
    dev = torch.device("cuda", local)
    s_d = torch.from_numpy(s).to(dev)
    k_d = torch.from_numpy(kappa).to(dev)
    ie_full = np.zeros((ns_total, n), np.complex128)
    ie_full[:, centre] = inj
    ie_d = torch.from_numpy(ie_full).to(dev)
    sol_d = torch.empty((SB, N), dtype=torch.complex128, device=dev)
    info_d = torch.empty((SB,), dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def batch_index(step):
        start = (step * SB) % ns_total
        return start, min(SB, ns_total - start)

    def run_step(step):
        k0, nb = batch_index(step)
        return plan.run_device(s_d[k0:].data_ptr(), k_d[k0:].data_ptr(), nb, 1.0, ie_d[k0:].data_ptr(), centre,
                               sol_d.data_ptr(), info_d.data_ptr())

    for w in range(args.warmup):
        run_step(w)
    torch.cuda.synchronize()
    launches0 = pkg.launch_count()
    dev_time, it_max, fb, step_ms = 0.0, 0, 0, []
    with ClockSampler(local) as clk:
        for st_i in range(steps):
            flush.zero_()
            st = run_step(st_i)
            dev_time += st.seconds
            step_ms.append(round(st.seconds * 1e3, 3))
            it_max, fb = max(it_max, st.max_iterations), fb + st.fallbacks
        torch.cuda.synchronize()
    launches = pkg.launch_count() - launches0
    samples = sum(batch_index(q)[1] for q in range(steps))
    value = samples / dev_time
    # kernel families, one pass in flight, kernel by kernel
    plan.set_graphs(False)
    plan.set_pipelines(1)
    pkg.lib().tags_gpu_profile(1)
    for st_i in range(steps):
        flush.zero_()
        run_step(st_i)
    torch.cuda.synchronize()
    prof = read_profile(pkg)
    pkg.lib().tags_gpu_profile(0)
    plan.set_graphs(True)
    plan.set_pipelines(P)
    # end to end through tags_plan_run with pinned host buffers
    s_h = torch.from_numpy(s).pin_memory()
    k_h = torch.from_numpy(kappa).pin_memory()
    ie_h = torch.from_numpy(ie_full).pin_memory()
    sol_h = torch.empty((SB, N), dtype=torch.complex128).pin_memory()
    info_h = torch.empty((SB,), dtype=torch.int32).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for st_i in range(steps):
        k0, nb = batch_index(st_i)
        code = pkg.lib().tags_plan_run(plan.handle, s_h[k0:].data_ptr(), k_h[k0:].data_ptr(), 1.0, nb,
                                       ie_h[k0:].data_ptr(), centre, sol_h.data_ptr(), info_h.data_ptr(), 0, None)
        if code != 0:
            raise RuntimeError(pkg.last_error())
    e2e_t = time.perf_counter() - t0
    # accuracy: mixed mHEM against plain-FP64 mHEM, 8 strided samples
    idx = np.linspace(0, ns_total - 1, 8).astype(int)
    um, _, _ = plan.run(s[idx], kappa[idx], 1.0, ie_full[idx])
    ref = pkg.Plan(elec, img, nodes, pkg.PLAIN_FP64, max_batch=8)
    try:
        ref.set_fill(pkg.INTG_MHEM)
        up, _, _ = ref.run(s[idx], kappa[idx], 1.0, ie_full[idx])
    finally:
        ref.close()
    plan.close()
    peaks = measured_peaks()
    roof, fams = roofline(prof, peaks, 16)
    line = {"metric": "Laplace-sample solves/s, mHEM model (1560-segment grid, 2048 samples)", "value": value,
            "unit": "solves/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_time / steps, "step_ms": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64+c128",
            "data": "synthetic (reference grid generator, Alipio soil, 1.2/50 us current)",
            "config": {"workload": "grid 60x60 m, 12x12 meshes, 1560 segments, N=4537, 2048 Laplace samples, mHEM "
                                   "impedances (tags_plan_set_fill(INTG_MHEM)), mixed-precision solve",
                       "samples_per_step": SB, "samples_per_pass": B, "passes_in_flight": P,
                       "l2": "flushed between steps (256 MB write)"},
            "roofline": roof, "kernel_families": fams, "gpu_launches": launches, "clocks": clk.summary(),
            "e2e": {"value": samples / e2e_t, "unit": "solves/s", "h2d_bytes_per_step": SB * 16 * (2 + n),
                    "d2h_bytes_per_step": SB * (16 * N + 4)},
            "refinement": {"max_iterations": it_max, "fallbacks": fb},
            "accuracy": {"samples": int(len(idx)), "reference": "plain FP64 form of this library, mHEM fill",
                         "max_rel_err_u_inj": float(np.max(np.abs(um[:, centre] - up[:, centre]) /
                                                           np.abs(up[:, centre]))),
                         "max_rel_err_u_all": float(np.max(np.abs(um[:, :n] - up[:, :n])) / np.max(np.abs(up[:, :n])))}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = mhem_cpu_baseline(elec, img, nodes, s, kappa, inj, centre, os.cpu_count() or 1)
    print(json.dumps(line))
    return 0


# ---- the 120 x 120 m grid with 50 rods (N = 17875) ------------------------------------
# 24 x 24 meshes, 1 m segmentation (m = 6000) plus 50 vertical rods of 3 m (3
# segments each) at seeded grid vertices: m = 6150, n = 5575, N = 17875;
# soil 100 ohm m, eps_r 10; unit current at the centre; 512 Laplace samples
# (nt = 1022, 10 MHz), streamed through the plan's memory-admitted passes.
RODS_NT = 1022
RODS_TMAX = 511 / 10e6


def run_rods(args):
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    pkg.build()
    elec, nodes = pkg.grid_with_rods()
    img = pkg.images(elec)
    m, n = elec.shape[0], nodes.shape[0]
    N = n + 2 * m
    s = pkg.laplace_samples(RODS_NT, RODS_TMAX)
    kappa = 1.0 / 100.0 + s * 10.0 * pkg.EPS0
    centre = int(np.argmin(np.linalg.norm(nodes - [60.0, 60.0, -0.5], axis=1)))
    t0 = time.perf_counter()
    plan = pkg.Plan(elec, img, nodes, pkg.MIXED, max_batch=args.batch or 0)
    setup_s = time.perf_counter() - t0
    ns = len(s)
    dev = torch.device("cuda", local)
    s_d = torch.from_numpy(s).to(dev)
    k_d = torch.from_numpy(kappa).to(dev)
    sol_d = torch.empty((ns, N), dtype=torch.complex128, device=dev)
    info_d = torch.empty((ns,), dtype=torch.int32, device=dev)
    # warm-up: one small run (graph capture of the first pass shape, tables)
    plan.run_device(s_d.data_ptr(), k_d.data_ptr(), 2, 1.0, None, centre, sol_d.data_ptr(), info_d.data_ptr())
    torch.cuda.synchronize()
    launches0 = pkg.launch_count()
    with ClockSampler(local) as clk:
        st = plan.run_device(s_d.data_ptr(), k_d.data_ptr(), ns, 1.0, None, centre, sol_d.data_ptr(),
                             info_d.data_ptr())
        torch.cuda.synchronize()
    launches = pkg.launch_count() - launches0
    if int(info_d.abs().max().item()) != 0:
        raise RuntimeError("a sample reported a failed solve")
    # end to end: host buffers through tags_plan_run
    t0 = time.perf_counter()
    sol_h, info_h, st_h = plan.run(s, kappa, 1.0, None, centre)
    e2e_t = time.perf_counter() - t0
    # accuracy against the plain FP64 form on two samples (lowest and 6 MHz)
    idx = np.array([0, 306])
    xp, ip, _ = pkg.hem_sweep(elec, img, nodes, s[idx], kappa[idx], inj_node=centre, precision=pkg.PLAIN_FP64,
                              max_batch=2)
    err = float(max(np.max(np.abs(sol_h[k, :n] - xp[j, :n])) / np.max(np.abs(xp[j, :n])) for j, k in enumerate(idx)))
    plan.close()
    line = {"metric": "Laplace-sample solves/s, 120 x 120 m grid with 50 rods (N = 17875), 512 samples",
            "value": ns / st.seconds, "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * st.seconds, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64+c128", "data": "synthetic (reference grid generator plus seeded rods)",
            "config": {"workload": "grid 120x120 m, 24x24 meshes, 1 m segments, 50 rods of 3 m; m=6150, n=5575, "
                                   "N=17875; 512 Laplace samples (nt=1022, 10 MHz); soil 100 ohm m, eps_r 10",
                       "samples": ns, "plan_setup_s": setup_s,
                       "passes": "memory-admitted: the plan's samples per pass are sized from free device memory"},
            "gpu_launches": launches, "clocks": clk.summary(),
            "e2e": {"value": ns / e2e_t, "unit": "solves/s", "h2d_bytes_per_step": ns * 32,
                    "d2h_bytes_per_step": ns * (16 * N + 4)},
            "refinement": {"max_iterations": st.max_iterations, "fallbacks": st.fallbacks,
                           "max_backward_error": st.max_backward_error},
            "accuracy": {"samples": len(idx), "reference": "plain FP64 form of this library",
                         "max_rel_err_u_all": err}}
    print(json.dumps(line))
    return 0


# ---- many uneven grids ---------------------------------------------------------------
# 64 square grids of uneven size (side 5-40 m, 2-10 meshes, 1 m segmentation,
# m = 36..880), each with its own soil, 256 Laplace samples each (nt = 510,
# 10 MHz), unit current at the first node: all through one
# tags_gpu_solve_batch call (a plan per grid, plans in flight together).
GRIDS_COUNT, GRIDS_NT = 64, 510
GRIDS_TMAX = (GRIDS_NT // 2) / 10e6


def grid_jobs(pkg, count=GRIDS_COUNT):
    s = pkg.laplace_samples(GRIDS_NT, GRIDS_TMAX)
    jobs = []
    for g in pkg.uneven_grids(count, seed=0):
        kappa = 1.0 / g["rho"] + s * g["epsr"] * pkg.EPS0
        jobs.append({"electrodes": g["electrodes"], "images": pkg.images(g["electrodes"]), "nodes": g["nodes"],
                     "s": s, "kappa": kappa, "inj_node": 0})
    return jobs


def run_grids(args):
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    pkg.build()
    jobs = grid_jobs(pkg)
    ms = [j["electrodes"].shape[0] for j in jobs]
    ns = len(jobs[0]["s"])
    steps = args.steps if args.steps > 0 else 3
    # the grid batch: a plan per grid and one CUDA graph over all of them,
    # built once (outside the timed region, like a plan)
    t0 = time.perf_counter()
    batch = pkg.GridBatch(jobs, precision=pkg.MIXED)
    setup_s = time.perf_counter() - t0
    for _ in range(max(1, args.warmup)):
        batch.run(jobs)
    torch.cuda.synchronize()
    launches0 = pkg.launch_count()
    dev_s, wall, it_max, fb = 0.0, 0.0, 0, 0
    with ClockSampler(local) as clk:
        for _ in range(steps):
            t0 = time.perf_counter()
            out, st = batch.run(jobs)
            wall += time.perf_counter() - t0
            dev_s += st.seconds
            it_max, fb = max(it_max, st.max_iterations), fb + st.fallbacks
            if any(np.any(info) for _, info in out):
                raise RuntimeError("a grid reported a failed sample")
    launches = pkg.launch_count() - launches0
    batch.close()
    solves = len(jobs) * ns * steps
    # accuracy: mixed against plain FP64 on every grid, 8 strided samples each
    idx = np.linspace(0, ns - 1, 8).astype(int)
    sub = [dict(j, s=j["s"][idx], kappa=j["kappa"][idx]) for j in jobs]
    mx = pkg.solve_batch(sub, precision=pkg.MIXED)
    pl = pkg.solve_batch(sub, precision=pkg.PLAIN_FP64)
    per_grid = [float(np.max(np.abs(a[0][:, :j["nodes"].shape[0]] - b[0][:, :j["nodes"].shape[0]])) /
                      np.max(np.abs(b[0][:, :j["nodes"].shape[0]]))) for a, b, j in zip(mx, pl, jobs)]
    line = {"metric": "Laplace-sample solves/s over 64 uneven grids (m = %d..%d), 256 samples each" % (min(ms), max(ms)),
            "value": solves / dev_s, "unit": "solves/s", "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup),
            "ms_per_step": 1e3 * dev_s / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64+c128", "data": "synthetic (reference grid generator; per-grid soil)",
            "config": {"workload": "64 square grids, side 5-40 m, 2-10 meshes, 1 m segmentation, depth 0.3-1 m, "
                                   "rho 50-5000 ohm m, eps_r 5-40; 256 Laplace samples each (nt = 510, 10 MHz); "
                                   "one grid batch (tags_batch_*): every grid a branch of one CUDA graph, one "
                                   "graph launch per step",
                       "grids": len(jobs), "segments": [min(ms), max(ms)], "setup_s": setup_s},
            "roofline": None, "gpu_launches": launches, "clocks": clk.summary(),
            "e2e": {"value": solves / wall, "unit": "solves/s",
                    "h2d_bytes_per_step": int(sum(16 * ns * 2 for _ in jobs)),
                    "d2h_bytes_per_step": int(sum(ns * (16 * (j["nodes"].shape[0] + 2 * j["electrodes"].shape[0]) + 4)
                                                  for j in jobs))},
            "refinement": {"max_iterations": it_max, "fallbacks": fb},
            "accuracy": {"grids": len(jobs), "samples": len(idx),
                         "reference": "plain FP64 form of this library (node potentials)",
                         "max_rel_err": max(per_grid), "per_grid_max_rel_err": [float("%.3g" % e) for e in per_grid]},
            "note": "value = samples / device time of the graph launches (tags_batch_run stats); e2e = the same "
                    "runs' wall time with the host copies; setup_s = building the 64 plans and capturing the graph "
                    "once; the kernels are those of the solves workload, whose line carries their roofline"}
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        port = O.get("port")
        cores = os.cpu_count() or 1
        sidx = np.linspace(0, ns - 1, cores).astype(int)
        picked = (0, 21, 42, 63)
        t0 = time.perf_counter()
        for q in picked:
            j = jobs[q]
            port.hem_sweep(j["electrodes"], j["images"], j["nodes"], j["s"][sidx], j["kappa"][sidx], 0,
                           np.ones(len(sidx)), req_abs=1e-6, req_rel=1e-6, threads=cores)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(picked) * len(sidx) / dt, "unit": "solves/s", "cores": cores,
                                "kind": "port",
                                "sample": f"grids {picked} (m = {[ms[q] for q in picked]}), {len(sidx)} strided samples "
                                          f"each, path A at the reference's tolerances, {dt:.1f} s"}
    print(json.dumps(line))
    return 0


GPR_FIXTURE = os.path.join(ROOT, "tests", "golden", "gpr4.npz")


def plain_fp64_record(pkg, elec, img, nodes, s_d, k_d, ie_d, centre, local, flush, steps=3, batch=8):
    """The plain FP64 form (FP64 fill, LU with partial pivoting) timed the way
    the mixed form is: device time from the plan's CUDA events, inputs in
    HBM, L2 flushed between steps; `steps` steps of `batch` samples spread
    over the band after one warm-up step (its cost does not depend on the
    sample: no refinement)."""
    import torch
    n = nodes.shape[0]
    N = n + 2 * elec.shape[0]
    ns = s_d.shape[0]
    plan = pkg.Plan(elec, img, nodes, pkg.PLAIN_FP64, max_batch=batch)
    sol = torch.empty((batch, N), dtype=torch.complex128, device=s_d.device)
    info = torch.empty((batch,), dtype=torch.int32, device=s_d.device)
    starts = np.linspace(0, ns - batch, steps).astype(int)

    def one(k0):
        return plan.run_device(s_d[k0:].data_ptr(), k_d[k0:].data_ptr(), batch, 1.0, ie_d[k0:].data_ptr(), centre,
                               sol.data_ptr(), info.data_ptr())
    try:
        one(int(starts[-1]))
        torch.cuda.synchronize()
        dt, step_ms = 0.0, []
        with ClockSampler(local) as clk:
            for k0 in starts:
                flush.zero_()
                st = one(int(k0))
                dt += st.seconds
                step_ms.append(round(st.seconds * 1e3, 1))
            torch.cuda.synchronize()
        if int(info.abs().max().item()) != 0:
            raise RuntimeError("plain FP64 solve reported a singular pivot")
        # one more step kernel by kernel with per-family events: where the time goes
        plan.set_graphs(False)
        pkg.lib().tags_gpu_profile(1)
        one(int(starts[0]))
        torch.cuda.synchronize()
        prof = read_profile(pkg)
        pkg.lib().tags_gpu_profile(0)
    finally:
        plan.close()
    fp64 = fp64_peak(pkg)
    roof, fams = roofline(prof, measured_peaks(), fp64=fp64)
    return {"value": steps * batch / dt, "unit": "solves/s", "steps": steps, "samples_per_step": batch,
            "ms_per_step": 1e3 * dt / steps, "step_ms": step_ms, "clocks": clk.summary(),
            "roofline": roof, "kernel_families": fams, "fp64_peak": fp64,
            "note": "plain FP64 form of this library on the same workload: FP64 fill, FP64 LU with partial "
                    "pivoting, device time from the plan's events, L2 flushed between steps; roofline and "
                    "kernel_families from one more step launched kernel by kernel"}


def gpr_accuracy(pkg, plan, s_d, k_d, ie_d, centre, n, SB, sol_d, info_d, s, tmax, nt):
    """The mixed form over every sample of the workload (outside the timed
    region): U at the injection node per sample, its GPR through the
    inverse Laplace transform, and both against the plain FP64 form's
    (tests/golden/gpr4.npz, made by tests/golden/make_gpr4.py, its 16
    strided samples pinned to the reference's own C code)."""
    if not os.path.exists(GPR_FIXTURE):
        return None
    fx = np.load(GPR_FIXTURE)
    if not np.array_equal(fx["s"], s):
        return None
    ns = len(s)
    u = np.zeros(ns, np.complex128)
    pin = {int(k): j for j, k in enumerate(fx["pin_idx"])}
    u_nodes = np.zeros((len(pin), n), np.complex128)
    for k0 in range(0, ns, SB):
        nb = min(SB, ns - k0)
        plan.run_device(s_d[k0:].data_ptr(), k_d[k0:].data_ptr(), nb, 1.0, ie_d[k0:].data_ptr(), centre,
                        sol_d.data_ptr(), info_d.data_ptr())
        u[k0:k0 + nb] = sol_d[:nb, centre].cpu().numpy()
        for k in range(k0, k0 + nb):
            if k in pin:
                u_nodes[pin[k]] = sol_d[k - k0, :n].cpu().numpy()
    gpr = pkg.inv_laplace_trans(u, s, tmax, nt)
    per = np.abs(u - fx["u_centre"]) / np.abs(fx["u_centre"])
    out = {"samples": ns, "reference": "plain FP64 form of this library over all samples (tests/golden/gpr4.npz)",
           "gpr_rel_err": float(np.max(np.abs(gpr - fx["gpr"])) / np.max(np.abs(fx["gpr"]))),
           "max_rel_err_u_inj": float(per.max()),
           "max_rel_err_u_all": float(np.max(np.abs(u_nodes - fx["u_nodes"])) / np.max(np.abs(fx["u_nodes"]))),
           "gpr_peak_v": float(np.max(np.abs(fx["gpr"])))}
    if "ref_u_nodes" in fx:
        ref = fx["ref_u_nodes"]
        out["plain_vs_reference_build"] = float(np.max(np.abs(fx["u_nodes"] - ref)) / np.max(np.abs(ref)))
        out["mixed_vs_reference_build"] = float(np.max(np.abs(u_nodes - ref)) / np.max(np.abs(ref)))
        out["reference_samples"] = int(ref.shape[0])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="timed steps (0: the whole 2048-sample job once, 8 steps of 2 x 128 samples)")
    ap.add_argument("--pipelines", type=int, default=0, help="passes in flight (0: 2 mixed, 1 plain)")
    ap.add_argument("--step-passes", type=int, default=0,
                    help="passes per step, taken by the pipelines as they free up (0 = pipelines)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "plain"])
    ap.add_argument("--batch", type=int, default=0, help="samples per step (0 = 128 mixed / 8 plain)")
    ap.add_argument("--cpu-samples", type=int, default=0, help="CPU-baseline samples (0 = host cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graphs", action="store_true", help="launch kernel by kernel in the measured pass")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the all-sample GPR check against plain FP64")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 sub-record")
    ap.add_argument("--tc-pairs", type=int, default=-1,
                    help="trailing updates: 0 one SM per tile, 1 two-SM clusters, 2 two-SM real-form N=256 "
                         "(-1 = the plan's default)")
    ap.add_argument("--panels", type=int, default=0, help="mixed form: panels per trailing update, 1..6 (0 = plan default)")
    ap.add_argument("--split", type=int, default=0, help="mixed-form split: 3 bf16x3, 2 bf16x2, 16 fp16x2 (0 = plan default)")
    ap.add_argument("--solve-path", type=int, default=-1,
                    help="triangular solves: 0 per block, 1 one CTA per sample, 2/4/8 clusters (-1 = default)")
    ap.add_argument("--ref-steps", type=int, default=4, help="cap on timed steps of the reference arm")
    ap.add_argument("--first-batch", type=int, default=0,
                    help="batch of samples the warm-up and timed steps start from (0 = the whole job in order)")
    ap.add_argument("--workload", default="solves", choices=["solves", "fields", "grids", "mhem", "rods"],
                    help="solves: the per-sample HEM path (default); fields: post-processing along a line; "
                         "grids: 64 uneven grids in one call; mhem: the examples' mHEM model on the same grid; "
                         "rods: the 120 x 120 m grid with 50 rods, N = 17875, 512 samples")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "fields":
        return run_fields(args)
    if args.workload == "grids":
        return run_grids(args)
    if args.workload == "mhem":
        return run_mhem(args)
    if args.workload == "rods":
        return run_rods(args)

    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    pkg.build()
    elec, img, nodes, s, kappa, inj, centre = workload(pkg)
    m, n = elec.shape[0], nodes.shape[0]
    N = n + 2 * m
    mixed = args.precision == "mixed"
    B = args.batch or (128 if mixed else 8)          # samples per pass
    P = args.pipelines or (2 if mixed else 1)         # passes in flight per step
    SB = B * (args.step_passes or P)                  # samples per step
    plan = pkg.Plan(elec, img, nodes, pkg.MIXED if mixed else pkg.PLAIN_FP64, max_batch=B)
    if mixed and args.split:
        plan.set_split(args.split)
    if mixed and args.panels:
        plan.set_panels(args.panels)
    if mixed and args.tc_pairs >= 0:
        plan.set_tc_pairs(args.tc_pairs)
    if args.solve_path != -1 and pkg.lib().tags_debug_solve_path(args.solve_path) != 0:
        raise SystemExit(pkg.last_error())
    if P > 1:
        plan.set_pipelines(P)
    ns_total = len(s)
    # default steps: the 2048-sample job split over the ranks (total work
    # fixed: strong scaling); --steps K: K steps per rank (weak scaling)
    scaling = "strong" if args.steps <= 0 and world > 1 else "weak"
    if args.steps <= 0:
        args.steps = max(1, -(-ns_total // (SB * world)))
    dev = torch.device("cuda", local)
    # inputs resident in HBM; each rank takes its own strided share of samples
    s_d = torch.from_numpy(s).to(dev)
    k_d = torch.from_numpy(kappa).to(dev)
    ie_full = np.zeros((ns_total, n), np.complex128)
    ie_full[:, centre] = inj
    ie_d = torch.from_numpy(ie_full).to(dev)
    sol_d = torch.empty((SB, N), dtype=torch.complex128, device=dev)
    info_d = torch.empty((SB,), dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)   # > L2

    def batch_index(step):
        start = (((args.first_batch + step) * world + rank) * SB) % ns_total
        return start, min(SB, ns_total - start)

    def run_step(step):
        k0, nb = batch_index(step)
        return plan.run_device(s_d[k0:].data_ptr(), k_d[k0:].data_ptr(), nb, 1.0, ie_d[k0:].data_ptr(), centre,
                               sol_d.data_ptr(), info_d.data_ptr())

    for w in range(args.warmup):
        run_step(w)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    # the timed steps walk the sample set from its first (lowest-frequency,
    # hardest-to-refine) batch: 16 steps of 128 samples are the whole job
    step_ms = []

    def timed(profile):
        """K steps; each step's device time from the plan's events on its
        stream. profile=True: kernel by kernel with per-family events."""
        launches0 = pkg.launch_count()
        it_max, fb, dt, split = 0, 0, 0.0, 0
        step_ms.clear()
        if profile:
            pkg.lib().tags_gpu_profile(1)      # per-family CUDA events on the launching stream
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            for st_i in range(args.steps):
                flush.zero_()
                st = run_step(st_i)
                dt += st.seconds
                step_ms.append(round(st.seconds * 1e3, 3))
                it_max = max(it_max, st.max_iterations)
                fb += st.fallbacks
                split = st.split
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        prof = read_profile(pkg) if profile else None
        if profile:
            pkg.lib().tags_gpu_profile(0)
        return dt, it_max, fb, pkg.launch_count() - launches0, clk, wall, prof, split

    # the measured pass: every batch one CUDA-graph launch (the default path)
    plan.set_graphs(not args.no_graphs)
    dev_time, stats_iter, stats_fb, launches, clk, wall, _, split = timed(False)
    measured_step_ms = list(step_ms)
    # the same steps kernel by kernel with per-family events, one pass in flight
    # (kernels timed alone): kernel shares and roofline
    plan.set_graphs(False)
    plan.set_pipelines(1)
    prof_time, _, _, _, _, _, prof, _ = timed(True)
    plan.set_graphs(not args.no_graphs)
    plan.set_pipelines(P)
    if world > 1:
        t = torch.tensor([dev_time], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_time = float(t.item())
        dist.barrier()
    samples = sum(batch_index(st_i)[1] for st_i in range(args.steps)) * world
    value = samples / dev_time

    # end to end through the public API with host (pinned) buffers
    s_h = torch.from_numpy(s).pin_memory()
    k_h = torch.from_numpy(kappa).pin_memory()
    ie_h = torch.from_numpy(ie_full).pin_memory()
    sol_h = torch.empty((SB, N), dtype=torch.complex128).pin_memory()
    info_h = torch.empty((SB,), dtype=torch.int32).pin_memory()
    e2e_steps = max(1, args.steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for st_i in range(e2e_steps):
        k0, nb = batch_index(st_i)
        code = pkg.lib().tags_plan_run(plan.handle, s_h[k0:].data_ptr(), k_h[k0:].data_ptr(), 1.0, nb,
                                       ie_h[k0:].data_ptr(), centre, sol_h.data_ptr(), info_h.data_ptr(), 0, None)
        if code != 0:
            raise RuntimeError(pkg.last_error())
    e2e_t = time.perf_counter() - t0
    e2e_samples = sum(batch_index(st_i)[1] for st_i in range(e2e_steps))
    e2e = {"value": e2e_samples / e2e_t, "unit": "solves/s", "h2d_bytes_per_step": SB * 16 * (2 + n),
           "d2h_bytes_per_step": SB * (16 * N + 4)}

    # accuracy of the measured form: every sample, GPR included, against the
    # plain FP64 form (outside the timed region)
    accuracy, plain = None, None
    if mixed and rank == 0 and not args.no_accuracy:
        accuracy = gpr_accuracy(pkg, plan, s_d, k_d, ie_d, centre, n, SB, sol_d, info_d, s, TMAX, NT)
    if mixed and rank == 0 and not args.no_plain:
        plain = plain_fp64_record(pkg, elec, img, nodes, s_d, k_d, ie_d, centre, local, flush)

    if rank != 0:
        return 0
    peaks = measured_peaks()
    roof, fams = roofline(prof, peaks, split, samples_per_pass=B)
    if roof is not None and mixed:
        # the whole job in the dense complex LU count: (8/3) N^3 real flops per sample
        lu = 8.0 / 3.0 * float(N) ** 3 * value / 1e12
        roof["lu_equivalent"] = {"tflops": lu, "frac": lu / peaks["bf16_tflops"],
                                 "note": "(8/3) N^3 real flops per sample, the dense complex LU count with its "
                                         "structural zeros and symmetry, times the job's solves/s; same peak"}
    line = {"metric": "Laplace-sample solves/s (1560-segment grid, 2048 samples)", "value": value,
            "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_time / args.steps, "step_ms": measured_step_ms,
            "higher_is_better": True, "scaling": scaling,
            "vs_baseline": None, "dtype": "c128" if not mixed else "c64+c128",
            "data": "synthetic (reference grid generator, Alipio soil, 1.2/50 us current)",
            "config": {"workload": "grid 60x60 m, 12x12 meshes, 1560 segments, 1417 nodes, N=4537, 2048 Laplace "
                                   "samples (nt=4094, 10 MHz), Alipio soil sigma0=1 mS/m, centre injection",
                       "precision": args.precision, "samples_per_step": SB, "samples_per_pass": B,
                       "passes_in_flight": P, "l2": "flushed between steps (256 MB write)",
                       "timed_samples": "batches in frequency order from the first sample (the default steps cover all 2048 once)",
                       "cuda_graphs": not args.no_graphs},
            "roofline": roof, "kernel_families": fams,
            "profiled_pass": {"ms_per_step": 1e3 * prof_time / args.steps,
                              "note": "same steps launched kernel by kernel with per-family CUDA events; "
                                      "roofline and kernel_families come from this pass"},
            "gpu_launches": launches, "clocks": clk.summary(), "e2e": e2e,
            "refinement": {"max_iterations": stats_iter, "fallbacks": stats_fb, "split": split},
            "fill_pipes": FILL_PIPES if mixed else None,
            "accuracy": accuracy, "wall_s": wall}
    if plain is not None:
        line["plain_fp64"] = plain
        line["mixed_over_plain"] = value / plain["value"]
    if not args.no_cpu_baseline:
        nsamp = args.cpu_samples or (os.cpu_count() or 1)
        line["cpu_baseline"] = cpu_baseline(args, elec, img, nodes, s, kappa, inj, centre, nsamp)[0]
    print(json.dumps(line))
    plan.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
