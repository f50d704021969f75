"""GB300-native HEM hot path of TAGS (transient analysis of grounding systems).

Python host-side mirror of the reference C interface for the per-Laplace-sample
path, backed by the CUDA library ``libtags_gpu.so`` (built from ``csrc/`` by
``build.py``). The compute functions call the C-ABI declared in
``include/tags_gpu.h``; they raise if the library is missing instead of
falling back to any CPU code.

Reference interface mirrored here (pedrohnv/transient-analysis-grounding-systems):

* geometry, host side: ``populate_electrode`` (src/electrode.c:12-32),
  ``segment_electrode`` (:103-127), ``number_segments`` / ``number_nodes`` /
  ``electrode_grid`` (src/grid.c:9-92), ``images`` (examples/three_grids.c:206-214);
* soil: ``alipio_soil`` (src/auxiliary.c:60-70) and the medium terms of
  examples/three_grids.c:326-333;
* GPU drop-ins with the reference's names and semantics:
  ``calculate_impedances``, ``impedances_images``, ``fill_incidence_imm``,
  ``fill_impedance_imm``, ``solve_immittance``, ``laplace_trans``,
  ``inv_laplace_trans``;
* batched extension: :class:`Plan` (``tags_plan_*``) and :func:`hem_sweep`.

Electrode arrays are float64 ``(m, 11)`` arrays with the reference's field order
(start[3], end[3], middle[3], length, radius); nodes are ``(n, 3)``.
Impedance buffers are flat complex128 arrays of ``m*m`` in the reference's
column-major layout (``z[i*m + k]`` = row k, column i).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import math
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtags_gpu.so")

INTG_NONE, INTG_DOUBLE, INTG_SINGLE, INTG_MHEM = 1, 2, 3, 4
FILTER_NONE, FILTER_BLACKMAN, FILTER_HANNING, FILTER_LANCZOS, FILTER_RIESZ = range(5)
PLAIN_FP64, MIXED = 0, 1
RUN_DEVICE_PTRS = 1
TUNE_REFRESH = 256
E_ARG, E_CUDA, E_NOMEM, E_GEOMETRY, E_NONFINITE = -101, -102, -103, -104, -105
SPLIT_BF16_2, SPLIT_BF16_3, SPLIT_F16 = 2, 3, 16

# physical constants of the reference (src/auxiliary.c:17-21)
PI = 3.1415926535897932384626433832795029
TWO_PI = 6.283185307179586476925286766559
FOUR_PI = 12.5663706143591729538505735331
MU0 = 1.256637061435917e-6
EPS0 = 8.854187817620e-12

# C-ABI symbols declared in include/tags_gpu.h
EXPORTS = (
    "calculate_impedances", "impedances_images", "fill_incidence_imm", "fill_impedance_imm",
    "solve_immittance", "fill_incidence_adm", "fill_impedance_adm", "calculate_yla_ytb", "fill_impedance_adm2",
    "solve_admittance", "electrodes_file", "nodes_file", "alipio_soil", "smith_longmire_soil", "heidler", "laplace_trans",
    "inv_laplace_trans", "tags_plan_create", "tags_plan_run",
    "tags_plan_destroy", "tags_plan_set_graphs", "tags_plan_set_pipelines", "tags_plan_set_split", "tags_plan_set_panels", "tags_plan_tune", "tags_plan_set_fill", "tags_inv_laplace_batch", "tags_gpu_launch_count", "tags_gpu_last_error",
    "tags_plan_set_max_steps", "tags_debug_tc_wait_limit", "tags_plan_set_refine_tol", "tags_plan_set_tc_pairs",
    "tags_debug_tc_pairs", "tags_debug_solve_path", "tags_debug_mixed_fill", "tags_probe_fp64",
    "tags_gpu_set_memory_budget", "tags_gpu_set_tune_cache",
    "electric_potential", "magnetic_potential", "electric_field", "voltage", "tags_fields_batch",
    "tags_gpd_mhem_batch", "tags_voltage_batch", "tags_fields_evaluations", "tags_gpu_solve_batch",
    "tags_gpu_inlt", "tags_batch_create", "tags_batch_run", "tags_batch_destroy",
    "tags_gpu_set_quiet",
)


class c_complex(ctypes.Structure):
    """C99 ``double _Complex`` by value (two doubles in FP registers)."""

    _fields_ = [("re", ctypes.c_double), ("im", ctypes.c_double)]

    @classmethod
    def of(cls, z) -> "c_complex":
        z = complex(z)
        return cls(z.real, z.imag)


class TuneResult(ctypes.Structure):
    _fields_ = [("samples_per_pass", ctypes.c_int), ("panels_per_update", ctypes.c_int), ("split", ctypes.c_int),
                ("solves_per_second", ctypes.c_double), ("candidates", ctypes.c_int)]


class GridJob(ctypes.Structure):
    """tags_grid_job: one grid of a tags_gpu_solve_batch call (pointers as integers)."""

    _fields_ = [("electrodes", ctypes.c_void_p), ("images", ctypes.c_void_p), ("num_electrodes", ctypes.c_size_t),
                ("nodes", ctypes.c_void_p), ("num_nodes", ctypes.c_size_t), ("s", ctypes.c_void_p),
                ("kappa", ctypes.c_void_p), ("ns", ctypes.c_size_t), ("ie", ctypes.c_void_p),
                ("inj_node", ctypes.c_size_t), ("sol", ctypes.c_void_p), ("info", ctypes.c_void_p)]


class RunStats(ctypes.Structure):
    _fields_ = [("max_iterations", ctypes.c_int), ("fallbacks", ctypes.c_int),
                ("max_backward_error", ctypes.c_double), ("seconds", ctypes.c_double),
                ("split", ctypes.c_int)]


_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    from importlib import util
    spec = util.spec_from_file_location("_tags_gpu_build", os.path.join(HERE, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library; raises if it was not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (build.py)")
            L = ctypes.CDLL(LIB_PATH)
            C = c_complex
            L.calculate_impedances.argtypes = [_vp, _vp, _vp, _sz, C, C, ctypes.c_double, C, _sz,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_int]
            L.impedances_images.argtypes = [_vp, _vp, _vp, _vp, _sz, C, C, ctypes.c_double, C, C, C, _sz,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_int]
            L.fill_incidence_imm.argtypes = [_vp, _vp, _sz, _vp, _sz]
            L.fill_impedance_imm.argtypes = [_vp, _vp, _vp, _sz, _sz]
            L.solve_immittance.argtypes = [_vp, _vp, _sz, _sz]
            L.fill_incidence_adm.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz]
            L.fill_impedance_adm.argtypes = [_vp, _vp, _vp, _vp, _vp, _sz, _sz]
            L.calculate_yla_ytb.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _sz, _sz]
            L.fill_impedance_adm2.argtypes = [_vp, _vp, _vp, _vp, _vp, _sz, _sz]
            L.solve_admittance.argtypes = [_vp, _vp, _sz]
            L.electrodes_file.argtypes = [ctypes.c_char_p, _vp, _sz]
            L.nodes_file.argtypes = [ctypes.c_char_p, _vp, _sz]
            L.alipio_soil.argtypes = [_vp, _vp, ctypes.c_double, C, ctypes.c_double, ctypes.c_double, ctypes.c_double]
            L.smith_longmire_soil.argtypes = [_vp, _vp, ctypes.c_double, C, ctypes.c_double]
            L.heidler.argtypes = [ctypes.c_double] * 5
            L.heidler.restype = ctypes.c_double
            L.laplace_trans.argtypes = [_vp, _vp, _vp, ctypes.c_double, _sz]
            L.inv_laplace_trans.argtypes = [_vp, _vp, _vp, ctypes.c_double, _sz, ctypes.c_int]
            L.tags_plan_create.argtypes = [ctypes.POINTER(_vp), _vp, _vp, _sz, _vp, _sz, ctypes.c_int, _sz]
            L.tags_plan_run.argtypes = [_vp, _vp, _vp, ctypes.c_double, _sz, _vp, _sz, _vp, _vp,
                                        ctypes.c_int, ctypes.POINTER(RunStats)]
            L.tags_plan_destroy.argtypes = [_vp]
            L.tags_plan_set_graphs.argtypes = [_vp, ctypes.c_int]
            L.tags_plan_set_pipelines.argtypes = [_vp, ctypes.c_int]
            L.tags_plan_set_split.argtypes = [_vp, ctypes.c_int]
            L.tags_plan_set_panels.argtypes = [_vp, ctypes.c_int]
            L.tags_plan_set_fill.argtypes = [_vp, ctypes.c_int]
            L.tags_plan_set_max_steps.argtypes = [_vp, ctypes.c_int]
            L.tags_plan_set_refine_tol.argtypes = [_vp, ctypes.c_double]
            L.tags_plan_set_tc_pairs.argtypes = [_vp, ctypes.c_int]
            L.tags_debug_tc_pairs.argtypes = [ctypes.c_int]
            L.tags_debug_solve_path.argtypes = [ctypes.c_int]
            L.tags_gpu_set_memory_budget.argtypes = [ctypes.c_ulonglong]
            L.tags_gpu_set_memory_budget.restype = ctypes.c_int
            L.tags_gpu_set_tune_cache.argtypes = [ctypes.c_char_p]
            L.tags_gpu_set_tune_cache.restype = ctypes.c_int
            L.tags_probe_fp64.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
            L.tags_debug_tc_wait_limit.argtypes = [ctypes.c_longlong]
            L.tags_debug_mixed_fill.argtypes = [_vp, _vp, _vp, ctypes.c_double, _sz, _vp, _vp]
            L.tags_inv_laplace_batch.argtypes = [_vp, _vp, _vp, ctypes.c_double, _sz, _sz, ctypes.c_int, ctypes.c_int]
            L.tags_plan_tune.argtypes = [_vp, _vp, _vp, ctypes.c_double, _sz, _sz, ctypes.c_int,
                                         ctypes.POINTER(TuneResult)]
            d = ctypes.c_double
            L.electric_potential.argtypes = [_vp, _vp, _sz, _vp, C, C, _sz, d, d]
            L.electric_potential.restype = C
            L.magnetic_potential.argtypes = [_vp, _vp, _sz, _vp, C, d, _sz, d, d, _vp]
            L.electric_field.argtypes = [_vp, _vp, _sz, _vp, _vp, C, C, d, C, _sz, d, d, _vp]
            L.voltage.argtypes = [_vp, _vp, _vp, _sz, _vp, _vp, C, C, d, C, _sz, d, d]
            L.voltage.restype = C
            L.tags_fields_batch.argtypes = [_vp, _sz, _vp, _sz, _vp, _vp, _sz, _sz, _vp, _vp, d, _vp, _vp, _vp]
            L.tags_gpd_mhem_batch.argtypes = [_vp, _sz, _vp, _sz, _vp, _sz, _sz, _vp, _vp, _vp]
            L.tags_voltage_batch.argtypes = [_vp, _sz, _vp, _sz, _vp, _vp, _sz, _sz, _vp, _vp, _vp, d, _vp]
            L.tags_fields_evaluations.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
            L.tags_gpu_solve_batch.argtypes = [ctypes.POINTER(GridJob), _sz, ctypes.c_int, d, _sz, ctypes.c_int]
            L.tags_batch_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(GridJob), _sz, ctypes.c_int, d, _sz]
            L.tags_batch_run.argtypes = [_vp, ctypes.POINTER(GridJob), _sz, ctypes.POINTER(RunStats)]
            L.tags_batch_destroy.argtypes = [_vp]
            L.tags_gpu_inlt.argtypes = [_vp, _vp, _vp, d, _sz, _sz, ctypes.c_int, ctypes.c_int]
            L.tags_gpu_launch_count.restype = ctypes.c_longlong
            L.tags_gpu_last_error.restype = ctypes.c_char_p
            L.tags_gpu_set_quiet.argtypes = [ctypes.c_int]
            for name in ("calculate_impedances", "impedances_images", "fill_incidence_imm",
                         "fill_impedance_imm", "solve_immittance", "fill_incidence_adm", "fill_impedance_adm",
                         "calculate_yla_ytb", "fill_impedance_adm2", "solve_admittance", "electrodes_file",
                         "nodes_file", "alipio_soil", "smith_longmire_soil", "laplace_trans",
                         "inv_laplace_trans",
                         "tags_plan_create", "tags_plan_run", "tags_plan_destroy", "tags_plan_set_graphs",
                         "tags_plan_set_pipelines",
                         "tags_plan_set_split", "tags_plan_set_panels", "tags_plan_tune", "tags_plan_set_fill",
                         "tags_inv_laplace_batch",
                         "tags_plan_set_max_steps", "tags_debug_tc_wait_limit", "tags_plan_set_refine_tol",
                         "tags_plan_set_tc_pairs", "tags_debug_tc_pairs", "tags_debug_solve_path",
                         "tags_debug_mixed_fill", "tags_probe_fp64",
                         "magnetic_potential", "electric_field", "tags_fields_batch", "tags_gpd_mhem_batch",
                         "tags_voltage_batch", "tags_fields_evaluations", "tags_gpu_solve_batch", "tags_gpu_inlt",
                         "tags_batch_create", "tags_batch_run", "tags_batch_destroy"):
                getattr(L, name).restype = ctypes.c_int
            _lib = L
        return _lib


def set_memory_budget(nbytes: int = 0) -> None:
    """Cap the free device memory that plans and grid batches size themselves
    against (0 removes the cap)."""
    _ret(lib().tags_gpu_set_memory_budget(int(nbytes)))


def set_tune_cache(path=None) -> None:
    """Autotuner cache file (None switches it off): Plan.tune applies a stored
    configuration for the plan's shape and GPU instead of timing candidates,
    and appends each timed result."""
    _ret(lib().tags_gpu_set_tune_cache(None if path is None else os.fsencode(path)))


def last_error() -> str:
    return lib().tags_gpu_last_error().decode()


def launch_count() -> int:
    return int(lib().tags_gpu_launch_count())


def _addr(a: np.ndarray) -> int:
    return a.ctypes.data


def _check_c128(a, name, size=None):
    if not isinstance(a, np.ndarray) or a.dtype != np.complex128 or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous complex128 numpy array")
    if size is not None and a.size < size:
        raise ValueError(f"{name} must hold at least {size} values")


def _elec(e) -> np.ndarray:
    e = np.ascontiguousarray(e, dtype=np.float64)
    if e.ndim != 2 or e.shape[1] != 11:
        raise ValueError("electrodes must be an (m, 11) float64 array")
    return e


# ---- geometry (host side, restating the reference) -----------------------------

def vector_length(a, b) -> float:
    """src/auxiliary.c:110-125 (sum of squared differences, then sqrt)."""
    return math.sqrt(sum((a[i] - b[i]) ** 2 for i in range(3)))


def populate_electrode(start, end, radius) -> np.ndarray:
    """One electrode row (src/electrode.c:12-32)."""
    start = [float(v) for v in start]
    end = [float(v) for v in end]
    if all(abs(start[i] - end[i]) <= 2.220446049250313e-16 for i in range(3)):
        raise ValueError("start_point and end_point are equal")
    if radius <= 0:
        raise ValueError("radius must be > 0")
    mid = [(start[i] + end[i]) / 2.0 for i in range(3)]
    return np.array(start + end + mid + [vector_length(start, end), float(radius)])


def linspace(a: float, b: float, n: int) -> np.ndarray:
    """src/auxiliary.c:24-36: a + i*step with the last point pinned to b."""
    if n < 2:
        raise ValueError("n must be >= 2")
    c = (b - a) / (n - 1)
    u = np.array([a + i * c for i in range(n - 1)] + [b], dtype=np.float64)
    return u


def logspace(a: float, b: float, n: int) -> np.ndarray:
    """src/auxiliary.c:38-50."""
    c = (b - a) / (n - 1)
    return np.array([10.0 ** (a + i * c) for i in range(n - 1)] + [10.0 ** b])


def segment_electrode(start, end, num_segments: int, radius: float):
    """Split a conductor into equal segments (src/electrode.c:103-127)."""
    if num_segments < 1:
        raise ValueError("number of segments should be greater than 0")
    nn = num_segments + 1
    xyz = [linspace(start[d], end[d], nn) for d in range(3)]
    nodes = np.stack(xyz, axis=1)
    elec = np.stack([populate_electrode(nodes[i], nodes[i + 1], radius) for i in range(num_segments)])
    return elec, nodes


def number_segments(vx, vy, nx, ny) -> int:
    """src/grid.c:9-17."""
    return nx * vy * (vx - 1) + ny * vx * (vy - 1)


def number_nodes(vx, vy, nx, ny) -> int:
    """src/grid.c:19-27."""
    return vx * vy + vx * (vy - 1) * (ny - 1) + vy * (vx - 1) * (nx - 1)


def electrode_grid(vertices_x, vertices_y, length_x, length_y, edge_segments_x, edge_segments_y,
                   radius, depth):
    """Rectangular grid (src/grid.c:29-92): x-directed conductors row by row,
    then y-directed column by column, with the reference's node order."""
    vx, vy, nx, ny = int(vertices_x), int(vertices_y), int(edge_segments_x), int(edge_segments_y)
    lx = length_x / (nx * (vx - 1))
    ly = length_y / (ny * (vy - 1))
    elec, nodes = [], []
    for h in range(vy):
        for span in range(vx - 1):
            for k in range(nx):
                a = [lx * (span * nx + k), ly * ny * h, depth]
                b = [a[0] + lx, a[1], depth]
                elec.append(populate_electrode(a, b, radius))
                if span == 0 and k == 0:
                    nodes.append(a)
                nodes.append(b)
    for g in range(vx):
        for span in range(vy - 1):
            for k in range(ny):
                a = [lx * nx * g, ly * (span * ny + k), depth]
                b = [a[0], a[1] + ly, depth]
                elec.append(populate_electrode(a, b, radius))
                if k < ny - 1:
                    nodes.append(b)
    return np.array(elec), np.array(nodes, dtype=np.float64)


def grid_with_rods(vertices=25, length=120.0, edge_segments=5, radius=7e-3, depth=-0.5, rods=50,
                   rod_length=3.0, rod_segments=3, seed=0):
    """Square grid (electrode_grid) plus vertical rods at `rods` vertices drawn
    by numpy's default_rng(seed) without replacement, each from the grid's
    depth down by rod_length in rod_segments segments; a rod's top node is the
    grid vertex's node. Defaults: the 120 x 120 m grid with 24 x 24 meshes and
    50 rods of 3 m (6150 segments, 5575 nodes)."""
    elec, nodes = electrode_grid(vertices, vertices, length, length, edge_segments, edge_segments, radius, depth)
    pick = np.sort(np.random.default_rng(seed).choice(vertices * vertices, size=rods, replace=False))
    step = length / (vertices - 1)
    all_e, all_n = [elec], [nodes]
    for v in pick:
        gx, gy = int(v) % vertices, int(v) // vertices
        top = [step * gx, step * gy, depth]
        e, nd = segment_electrode(top, [top[0], top[1], depth - rod_length], rod_segments, radius)
        all_e.append(e)
        all_n.append(nd[1:])
    return np.concatenate(all_e), np.concatenate(all_n)


def images(elec) -> np.ndarray:
    """Mirror segments across the soil surface z = 0 (examples/three_grids.c:206-214)."""
    img = np.array(elec, dtype=np.float64, copy=True)
    img[:, [2, 5, 8]] *= -1.0
    return img


# ---- soil and medium --------------------------------------------------------------

def alipio_soil(sigma0: float, s: complex, h: float, g: float, eps_ratio: float):
    """Frequency-dependent soil (src/auxiliary.c:60-70): (sigma, epsr)."""
    f = complex(s) / (TWO_PI * 1j)
    sigma = sigma0 + sigma0 * h * (f / 1e6) ** g
    t = math.tan(PI * g / 2) / (TWO_PI * EPS0 * 1e6 ** g)
    epsr = eps_ratio + t * sigma0 * h * f ** (g - 1.0)
    return complex(sigma), complex(epsr)


def kappa_of(s, sigma, epsr):
    """Complex conductivity kappa = sigma + s epsr eps0 (examples/three_grids.c:331)."""
    return np.asarray(sigma) + np.asarray(s) * np.asarray(epsr) * EPS0


def medium(s, kappa, mur=1.0):
    """gamma = sqrt(s mur mu0 kappa), ref_t = (kappa - s eps0)/(kappa + s eps0)
    (examples/three_grids.c:326-333)."""
    s = complex(s)
    kappa = complex(kappa)
    gamma = complex(np.sqrt(s * mur * MU0 * kappa))
    ref_t = (kappa - s * EPS0) / (kappa + s * EPS0)
    return gamma, ref_t


def laplace_samples(nt: int, tmax: float) -> np.ndarray:
    """s_k = c + j k 2 pi / tmax, c = ln(nt^2)/tmax (src/auxiliary.c:247-252)."""
    ns = nt // 2 + 1
    c = math.log(float(nt) ** 2) / tmax
    dw = TWO_PI / tmax
    return np.array([c + 1j * dw * k for k in range(ns)])


# ---- GPU drop-ins (reference names and semantics) ------------------------------------

def _ret(code: int) -> int:
    if code in (E_ARG, E_CUDA, E_NOMEM, E_GEOMETRY, E_NONFINITE):
        raise RuntimeError(f"tags_gpu error {code}: {last_error()}")
    return code


def calculate_impedances(zl, zt, electrodes, gamma, s, mur, kappa, max_eval=0, req_abs_error=1e-6,
                         req_rel_error=1e-6, integration_type=INTG_DOUBLE) -> int:
    e = _elec(electrodes)
    m = e.shape[0]
    _check_c128(zl, "zl", m * m)
    _check_c128(zt, "zt", m * m)
    C = c_complex
    return _ret(lib().calculate_impedances(_addr(zl), _addr(zt), _addr(e), m, C.of(gamma), C.of(s), float(mur),
                                           C.of(kappa), int(max_eval), float(req_abs_error),
                                           float(req_rel_error), int(integration_type)))


def impedances_images(zl, zt, electrodes, imgs, gamma, s, mur, kappa, ref_l, ref_t, max_eval=0,
                      req_abs_error=1e-6, req_rel_error=1e-6, integration_type=INTG_DOUBLE) -> int:
    e = _elec(electrodes)
    im = _elec(imgs)
    m = e.shape[0]
    _check_c128(zl, "zl", m * m)
    _check_c128(zt, "zt", m * m)
    C = c_complex
    return _ret(lib().impedances_images(_addr(zl), _addr(zt), _addr(e), _addr(im), m, C.of(gamma), C.of(s),
                                        float(mur), C.of(kappa), C.of(ref_l), C.of(ref_t), int(max_eval),
                                        float(req_abs_error), float(req_rel_error), int(integration_type)))


def fill_incidence_imm(wg, electrodes, nodes) -> int:
    e = _elec(electrodes)
    nd = np.ascontiguousarray(nodes, dtype=np.float64)
    N = nd.shape[0] + 2 * e.shape[0]
    _check_c128(wg, "wg", N * N)
    return _ret(lib().fill_incidence_imm(_addr(wg), _addr(e), e.shape[0], _addr(nd), nd.shape[0]))


def fill_impedance_imm(wg, zl, zt, num_electrodes: int, num_nodes: int) -> int:
    m, n = int(num_electrodes), int(num_nodes)
    _check_c128(wg, "wg", (n + 2 * m) ** 2)
    _check_c128(zl, "zl", m * m)
    _check_c128(zt, "zt", m * m)
    return _ret(lib().fill_impedance_imm(_addr(wg), _addr(zl), _addr(zt), m, n))


def solve_immittance(wg, ie, num_electrodes: int, num_nodes: int) -> int:
    m, n = int(num_electrodes), int(num_nodes)
    N = n + 2 * m
    _check_c128(wg, "wg", N * N)
    _check_c128(ie, "ie", N)
    return _ret(lib().solve_immittance(_addr(wg), _addr(ie), m, n))


def electrodes_file(path: str, num_electrodes: int):
    """(code, electrodes m x 11) read by the reference's CSV rule (electrodes_file)."""
    e = np.zeros((int(num_electrodes), 11))
    code = lib().electrodes_file(os.fsencode(path), _addr(e), int(num_electrodes))
    return code, e


def nodes_file(path: str, num_nodes: int):
    """(code, nodes n x 3) read by the reference's CSV rule (nodes_file)."""
    nd = np.zeros((int(num_nodes), 3))
    code = lib().nodes_file(os.fsencode(path), _addr(nd), int(num_nodes))
    return code, nd


def smith_longmire_soil(sigma0: float, s: complex, erinf: float):
    """(sigma, eps_r) of the Smith-Longmire soil model at s."""
    out = np.zeros(2, dtype=np.complex128)
    lib().smith_longmire_soil(_addr(out[:1]), _addr(out[1:]), float(sigma0), c_complex.of(s), float(erinf))
    return complex(out[0]), complex(out[1])


def heidler(t: float, imax: float, tau1: float, tau2: float, n: float) -> float:
    """Heidler lightning current at time t (src/auxiliary.c:331-336)."""
    return lib().heidler(float(t), float(imax), float(tau1), float(tau2), float(n))


def inv_laplace_batch(g, s, tmax: float, nt: int, filt: int = FILTER_NONE) -> np.ndarray:
    """Inverse transform of every column of g (ns x nseries, sample-major, e.g.
    node potentials of all samples) at once: nt x nseries, scaled as the
    reference examples' output loop (tags_inv_laplace_batch)."""
    g = np.ascontiguousarray(g, dtype=np.complex128)
    if g.ndim == 1:
        g = g[:, None]
    ns, nser = g.shape
    if ns != nt // 2 + 1:
        raise ValueError("g needs nt // 2 + 1 rows")
    s = np.ascontiguousarray(s, dtype=np.complex128)
    f = np.zeros((nt, nser))
    _ret(lib().tags_inv_laplace_batch(_addr(f), _addr(g), _addr(s), float(tmax), int(nt), int(nser), int(filt), 0))
    return f


# post-processing: potentials, fields and path voltages (src/electrode.c:434-668)

def _currents(c, ns: int, m: int, name: str) -> np.ndarray:
    """Currents as [sample][injection][electrode] (complex128, contiguous) from
    an array shaped (m,), (ns, m) or (ns, nrhs, m)."""
    a = np.asarray(c, dtype=np.complex128)
    if a.ndim == 1:
        a = a[None, None, :]
    elif a.ndim == 2:
        a = a[:, None, :]
    if a.ndim != 3 or a.shape[0] != ns or a.shape[2] != m:
        raise ValueError(f"{name} must be (m,), (ns, m) or (ns, nrhs, m) with ns = {ns}, m = {m}")
    return np.ascontiguousarray(a)


def _per_sample(v, ns: int) -> np.ndarray:
    return np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.complex128), (ns,)))


def fields_batch(points, electrodes, il, it, gamma, kappa, mur: float = 1.0, want=("pot", "vecpot", "efield")):
    """Potential, vector potential and conservative field at many points for
    many samples and injections (tags_fields_batch). gamma/kappa: per sample
    (ns,); il/it: (ns, nrhs, m) (or (ns, m), or (m,) for one sample). Returns a
    dict with pot (ns, P, nrhs), vecpot and efield (ns, P, nrhs, 3) and the
    return code under "status" (0 or E_GEOMETRY); the full field is efield -
    s vecpot."""
    pts = np.ascontiguousarray(np.atleast_2d(points), dtype=np.float64)
    e = _elec(electrodes)
    g = np.atleast_1d(np.asarray(gamma, dtype=np.complex128))
    ns, m, P = g.shape[0], e.shape[0], pts.shape[0]
    g = _per_sample(g, ns)
    k = _per_sample(kappa, ns)
    itc = _currents(it, ns, m, "it")
    ilc = _currents(il, ns, m, "il")
    R = itc.shape[1]
    if ilc.shape[1] != R:
        raise ValueError("il and it need the same number of injections")
    out = {}
    pot = np.zeros((ns, P, R), np.complex128) if "pot" in want else None
    vec = np.zeros((ns, P, R, 3), np.complex128) if "vecpot" in want else None
    ef = np.zeros((ns, P, R, 3), np.complex128) if "efield" in want else None
    rc = lib().tags_fields_batch(_addr(pts), P, _addr(e), m, _addr(ilc), _addr(itc), R, ns, _addr(g), _addr(k),
                                 float(mur), _addr(pot) if pot is not None else None,
                                 _addr(vec) if vec is not None else None, _addr(ef) if ef is not None else None)
    if rc not in (0, E_GEOMETRY):
        _ret(rc)
    for name, arr in (("pot", pot), ("vecpot", vec), ("efield", ef)):
        if arr is not None:
            out[name] = arr
    out["status"] = rc
    return out


def fields_evaluations(reset: bool = False) -> int:
    """Rule-node x sample evaluations of the field kernels since the last reset."""
    n = ctypes.c_ulonglong(0)
    _ret(lib().tags_fields_evaluations(ctypes.byref(n), 1 if reset else 0))
    return int(n.value)


def gpd_mhem_batch(points, electrodes, it, gamma, kappa) -> np.ndarray:
    """Closed-form mHEM ground potential (ns, P, nrhs) (tags_gpd_mhem_batch);
    it (ns, nrhs, m) already multiplied by (1 + ref_t) where wanted."""
    pts = np.ascontiguousarray(np.atleast_2d(points), dtype=np.float64)
    e = _elec(electrodes)
    g = np.atleast_1d(np.asarray(gamma, dtype=np.complex128))
    ns, m, P = g.shape[0], e.shape[0], pts.shape[0]
    g = _per_sample(g, ns)
    k = _per_sample(kappa, ns)
    itc = _currents(it, ns, m, "it")
    R = itc.shape[1]
    out = np.zeros((ns, P, R), np.complex128)
    _ret(lib().tags_gpd_mhem_batch(_addr(pts), P, _addr(e), m, _addr(itc), R, ns, _addr(g), _addr(k), _addr(out)))
    return out


def voltage_batch(paths, electrodes, il, it, gamma, s, kappa, mur: float = 1.0) -> np.ndarray:
    """The reference's path voltage for paths (L, 6) = (p1, p2), every sample
    and injection: (ns, L, nrhs) (tags_voltage_batch)."""
    pa = np.ascontiguousarray(np.atleast_2d(paths), dtype=np.float64)
    if pa.shape[1] != 6:
        raise ValueError("paths must be (L, 6)")
    e = _elec(electrodes)
    g = np.atleast_1d(np.asarray(gamma, dtype=np.complex128))
    ns, m, NL = g.shape[0], e.shape[0], pa.shape[0]
    g = _per_sample(g, ns)
    sv = _per_sample(s, ns)
    k = _per_sample(kappa, ns)
    itc = _currents(it, ns, m, "it")
    ilc = _currents(il, ns, m, "il")
    R = itc.shape[1]
    out = np.zeros((ns, NL, R), np.complex128)
    rc = lib().tags_voltage_batch(_addr(pa), NL, _addr(e), m, _addr(ilc), _addr(itc), R, ns, _addr(g), _addr(sv),
                                  _addr(k), float(mur), _addr(out))
    if rc not in (0, E_GEOMETRY):
        _ret(rc)
    return out


def electric_potential(point, electrodes, it, gamma, kappa) -> complex:
    """Drop-in electric_potential (src/electrode.c:434-457) for one point."""
    p = np.ascontiguousarray(point, dtype=np.float64)
    e = _elec(electrodes)
    itc = np.ascontiguousarray(it, dtype=np.complex128)
    r = lib().electric_potential(_addr(p), _addr(e), e.shape[0], _addr(itc), c_complex.of(gamma),
                                 c_complex.of(kappa), 0, 0.0, 0.0)
    return complex(r.re, r.im)


def magnetic_potential(point, electrodes, il, gamma, mur: float = 1.0) -> np.ndarray:
    p = np.ascontiguousarray(point, dtype=np.float64)
    e = _elec(electrodes)
    ilc = np.ascontiguousarray(il, dtype=np.complex128)
    va = np.zeros(3, np.complex128)
    _ret(lib().magnetic_potential(_addr(p), _addr(e), e.shape[0], _addr(ilc), c_complex.of(gamma), float(mur), 0,
                                  0.0, 0.0, _addr(va)))
    return va


def electric_field(point, electrodes, il, it, gamma, s, kappa, mur: float = 1.0, ve=None) -> np.ndarray:
    """Drop-in electric_field: returns ve after the call (overwritten when |s|
    > DBL_EPSILON, added to otherwise, as the reference)."""
    p = np.ascontiguousarray(point, dtype=np.float64)
    e = _elec(electrodes)
    ilc = np.ascontiguousarray(il, dtype=np.complex128)
    itc = np.ascontiguousarray(it, dtype=np.complex128)
    out = np.zeros(3, np.complex128) if ve is None else np.array(ve, dtype=np.complex128)
    _ret(lib().electric_field(_addr(p), _addr(e), e.shape[0], _addr(ilc), _addr(itc), c_complex.of(gamma),
                              c_complex.of(s), float(mur), c_complex.of(kappa), 0, 0.0, 0.0, _addr(out)))
    return out


def voltage(p1, p2, electrodes, il, it, gamma, s, kappa, mur: float = 1.0) -> complex:
    a = np.ascontiguousarray(p1, dtype=np.float64)
    b = np.ascontiguousarray(p2, dtype=np.float64)
    e = _elec(electrodes)
    ilc = np.ascontiguousarray(il, dtype=np.complex128)
    itc = np.ascontiguousarray(it, dtype=np.complex128)
    r = lib().voltage(_addr(a), _addr(b), _addr(e), e.shape[0], _addr(ilc), _addr(itc), c_complex.of(gamma),
                      c_complex.of(s), float(mur), c_complex.of(kappa), 0, 0.0, 0.0)
    return complex(r.re, r.im)


# nodal admittance formulation (src/linalg.c:142-350), used by the reference's mHEM examples

def fill_incidence_adm(a, b, electrodes, nodes) -> int:
    """A and B (m x n column-major, flat complex128); a may be b (then A)."""
    e = _elec(electrodes)
    nd = np.ascontiguousarray(nodes, dtype=np.float64)
    _check_c128(a, "a", e.shape[0] * nd.shape[0])
    _check_c128(b, "b", e.shape[0] * nd.shape[0])
    return _ret(lib().fill_incidence_adm(_addr(a), _addr(b), _addr(e), e.shape[0], _addr(nd), nd.shape[0]))


def calculate_yla_ytb(yla, ytb, zl, zt, a, b, num_electrodes: int, num_nodes: int) -> int:
    m, n = int(num_electrodes), int(num_nodes)
    for arr, name, size in ((yla, "yla", m * n), (ytb, "ytb", m * n), (zl, "zl", m * m), (zt, "zt", m * m),
                            (a, "a", m * n), (b, "b", m * n)):
        _check_c128(arr, name, size)
    return _ret(lib().calculate_yla_ytb(_addr(yla), _addr(ytb), _addr(zl), _addr(zt), _addr(a), _addr(b), m, n))


def fill_impedance_adm2(yn, yla, ytb, a, b, num_electrodes: int, num_nodes: int) -> int:
    m, n = int(num_electrodes), int(num_nodes)
    for arr, name, size in ((yn, "yn", n * n), (yla, "yla", m * n), (ytb, "ytb", m * n), (a, "a", m * n),
                            (b, "b", m * n)):
        _check_c128(arr, name, size)
    return _ret(lib().fill_impedance_adm2(_addr(yn), _addr(yla), _addr(ytb), _addr(a), _addr(b), m, n))


def fill_impedance_adm(yn, zl, zt, a, b, num_electrodes: int, num_nodes: int) -> int:
    m, n = int(num_electrodes), int(num_nodes)
    for arr, name, size in ((yn, "yn", n * n), (zl, "zl", m * m), (zt, "zt", m * m), (a, "a", m * n),
                            (b, "b", m * n)):
        _check_c128(arr, name, size)
    return _ret(lib().fill_impedance_adm(_addr(yn), _addr(zl), _addr(zt), _addr(a), _addr(b), m, n))


def solve_admittance(yn, ic, num_nodes: int) -> int:
    n = int(num_nodes)
    _check_c128(yn, "yn", n * n)
    _check_c128(ic, "ic", n)
    return _ret(lib().solve_admittance(_addr(yn), _addr(ic), n))


def laplace_trans(f, tmax: float):
    """Returns (g, s) like the reference's laplace_trans."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    nt = f.shape[0]
    g = np.zeros(nt // 2 + 1, dtype=np.complex128)
    s = np.zeros(nt // 2 + 1, dtype=np.complex128)
    _ret(lib().laplace_trans(_addr(f), _addr(g), _addr(s), float(tmax), nt))
    return g, s


def inv_laplace_trans(g, s, tmax: float, nt: int, filt: int = FILTER_NONE) -> np.ndarray:
    g = np.ascontiguousarray(g, dtype=np.complex128)
    s = np.ascontiguousarray(s, dtype=np.complex128)
    f = np.zeros(nt, dtype=np.float64)
    _ret(lib().inv_laplace_trans(_addr(f), _addr(g), _addr(s), float(tmax), int(nt), int(filt)))
    return f


# ---- batched extension ------------------------------------------------------------------

class Plan:
    """Device-resident geometry + workspaces for many Laplace samples
    (tags_plan_create / tags_plan_run / tags_plan_destroy)."""

    def __init__(self, electrodes, imgs, nodes, precision=PLAIN_FP64, max_batch=0, graphs=True):
        self.elec = _elec(electrodes)
        self.img = None if imgs is None else _elec(imgs)
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.m, self.n = self.elec.shape[0], self.nodes.shape[0]
        self.N = self.n + 2 * self.m
        self.precision = precision
        h = ctypes.c_void_p()
        code = lib().tags_plan_create(ctypes.byref(h), _addr(self.elec),
                                      None if self.img is None else _addr(self.img), self.m,
                                      _addr(self.nodes), self.n, int(precision), int(max_batch))
        if code != 0:
            raise RuntimeError(f"tags_plan_create failed ({code}): {last_error()}")
        self.handle = h
        self.set_graphs(graphs)

    def set_pipelines(self, n):
        """1, 2 or 3 passes in flight (k > 1: k - 1 twin plans take passes as they free up)."""
        _ret(lib().tags_plan_set_pipelines(self.handle, int(n)))

    def set_panels(self, panels):
        """Panels of 128 columns per trailing update of the mixed form (1 .. 6; 0 = default 6)."""
        code = lib().tags_plan_set_panels(self.handle, int(panels))
        if code != 0:
            raise RuntimeError(f"tags_plan_set_panels failed ({code}): {last_error()}")

    def set_split(self, pieces):
        """Split form of the mixed form's tensor-core products: SPLIT_BF16_3,
        SPLIT_BF16_2 or SPLIT_F16 (see include/tags_gpu.h)."""
        code = lib().tags_plan_set_split(self.handle, int(pieces))
        if code != 0:
            raise RuntimeError(f"tags_plan_set_split failed ({code}): {last_error()}")

    def tune(self, s, kappa, mur=1.0, inj_node=0, refresh=False):
        """Autotune samples per pass, panels per trailing update and the split
        form on these samples (tags_plan_tune); returns the kept TuneResult.
        With a tune cache set (set_tune_cache) a stored entry is applied
        without timing unless refresh is true."""
        s = np.ascontiguousarray(s, dtype=np.complex128)
        kappa = np.ascontiguousarray(np.broadcast_to(kappa, s.shape), dtype=np.complex128)
        res = TuneResult()
        code = lib().tags_plan_tune(self.handle, _addr(s), _addr(kappa), float(mur), s.shape[0], int(inj_node),
                                    TUNE_REFRESH if refresh else 0, ctypes.byref(res))
        if code != 0:
            raise RuntimeError(f"tags_plan_tune failed ({code}): {last_error()}")
        return res

    def set_fill(self, integration_type):
        """Impedance model: INTG_DOUBLE (double line integrals) or INTG_MHEM
        (static potentials rescaled per sample, as the reference's mHEM examples)."""
        code = lib().tags_plan_set_fill(self.handle, int(integration_type))
        if code != 0:
            raise RuntimeError(f"tags_plan_set_fill failed ({code}): {last_error()}")

    def set_tc_pairs(self, mode):
        """Trailing updates: 0 one SM per tile, 1 two-SM clusters (tcgen05
        cta_group::2, complex products), 2 two-SM clusters with the complex
        update as one real product of N = 256 (True means 1)."""
        _ret(lib().tags_plan_set_tc_pairs(self.handle, int(mode)))

    def set_refine_tol(self, tol):
        """Refinement stopping tolerance of the mixed form (0 = default 1e-9)."""
        code = lib().tags_plan_set_refine_tol(self.handle, float(tol))
        if code != 0:
            raise RuntimeError(f"tags_plan_set_refine_tol failed ({code}): {last_error()}")

    def set_max_steps(self, steps):
        """Cap the mixed form's refinement steps per pass (1..40, 0 = 40);
        samples not converged by then are re-solved in plain FP64."""
        code = lib().tags_plan_set_max_steps(self.handle, int(steps))
        if code != 0:
            raise RuntimeError(f"tags_plan_set_max_steps failed ({code}): {last_error()}")

    def mixed_fill(self, s, kappa, mur=1.0):
        """The mixed form's ZL, ZT (ns x m x m, full) as its residual sees
        them: FP32 regular pairs, FP64 touching pairs and diagonal."""
        s = np.ascontiguousarray(s, dtype=np.complex128)
        ns = s.shape[0]
        kappa = np.ascontiguousarray(np.broadcast_to(kappa, (ns,)), dtype=np.complex128)
        zl = np.zeros((ns, self.m, self.m), np.complex128)
        zt = np.zeros((ns, self.m, self.m), np.complex128)
        code = lib().tags_debug_mixed_fill(self.handle, _addr(s), _addr(kappa), float(mur), ns, _addr(zl), _addr(zt))
        if code != 0:
            raise RuntimeError(f"tags_debug_mixed_fill failed ({code}): {last_error()}")
        # column-major buffers: element (k, i) at k + m i
        return zl.transpose(0, 2, 1), zt.transpose(0, 2, 1)

    def set_graphs(self, enable):
        """Run each pass as one CUDA-graph launch (True) or kernel by kernel."""
        code = lib().tags_plan_set_graphs(self.handle, 1 if enable else 0)
        if code != 0:
            raise RuntimeError(f"tags_plan_set_graphs failed ({code}): {last_error()}")

    def run(self, s, kappa, mur=1.0, ie=None, inj_node=0, want_solution=True):
        """Solve for every sample; returns (solution ns x N, info, RunStats)."""
        s = np.ascontiguousarray(s, dtype=np.complex128)
        ns = s.shape[0]
        kappa = np.ascontiguousarray(np.broadcast_to(kappa, (ns,)), dtype=np.complex128)
        iep = None
        if ie is not None:
            ie = np.ascontiguousarray(ie, dtype=np.complex128).reshape(ns, self.n)
            iep = _addr(ie)
        sol = np.zeros((ns, self.N), dtype=np.complex128) if want_solution else None
        info = np.zeros(ns, dtype=np.int32)
        st = RunStats()
        code = lib().tags_plan_run(self.handle, _addr(s), _addr(kappa), float(mur), ns, iep, int(inj_node),
                                   None if sol is None else _addr(sol), _addr(info), 0, ctypes.byref(st))
        if code != 0:
            raise RuntimeError(f"tags_plan_run failed ({code}): {last_error()}")
        return sol, info, st

    def run_resumable(self, s, kappa, directory, mur=1.0, ie=None, inj_node=0, chunk=256, columns=None):
        """run() over chunks of `chunk` samples with each finished chunk saved
        under `directory`, so a sweep that was interrupted resumes from its
        last saved chunk when called again with the same arguments. columns
        (optional indices into the N unknowns) keeps only those columns of the
        solution. Returns (solution, info, stats) with stats summed over the
        chunks: max_iterations, fallbacks, max_backward_error, seconds, and
        chunks_run (the chunks this call solved)."""
        s = np.ascontiguousarray(s, dtype=np.complex128)
        ns = s.shape[0]
        kappa = np.ascontiguousarray(np.broadcast_to(kappa, (ns,)), dtype=np.complex128)
        if ie is not None:
            ie = np.ascontiguousarray(ie, dtype=np.complex128).reshape(ns, self.n)
        cols = None if columns is None else np.ascontiguousarray(columns, dtype=np.int64)
        fp = sweep_fingerprint([self.elec, self.img, self.nodes, self.precision, float(mur), int(inj_node), s,
                                kappa, ie, cols])

        def run_chunk(k0, k1):
            sol, info, st = self.run(s[k0:k1], kappa[k0:k1], mur, None if ie is None else ie[k0:k1], inj_node)
            return ({"sol": sol if cols is None else sol[:, cols], "info": info},
                    {"max_iterations": st.max_iterations, "fallbacks": st.fallbacks,
                     "max_backward_error": st.max_backward_error, "seconds": st.seconds})

        out, stats, ran = resumable_sweep(run_chunk, ns, directory, chunk, fp)
        summary = {"max_iterations": int(max((t["max_iterations"] for t in stats), default=0)),
                   "fallbacks": int(sum(t["fallbacks"] for t in stats)),
                   "max_backward_error": max((t["max_backward_error"] for t in stats), default=0.0),
                   "seconds": sum(t["seconds"] for t in stats), "chunks_run": ran}
        return out["sol"], out["info"], summary

    def run_device(self, s_ptr, kappa_ptr, ns, mur, ie_ptr, inj_node, sol_ptr, info_ptr):
        """Same as run() on device pointers (integers); inputs stay in HBM."""
        st = RunStats()
        code = lib().tags_plan_run(self.handle, s_ptr, kappa_ptr, float(mur), int(ns), ie_ptr, int(inj_node),
                                   sol_ptr, info_ptr, RUN_DEVICE_PTRS, ctypes.byref(st))
        if code != 0:
            raise RuntimeError(f"tags_plan_run failed ({code}): {last_error()}")
        return st

    def close(self):
        if getattr(self, "handle", None):
            lib().tags_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def probe_fp64():
    """(DFMA, DMMA) FP64 throughput of the current device in TFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _ret(lib().tags_probe_fp64(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def debug_tc_wait_limit(ns: int = 0) -> None:
    """Test hook: per-wait limit (ns) of the tensor-core kernels' main loops on
    the current device; 0 restores the default (50 ms)."""
    _ret(lib().tags_debug_tc_wait_limit(int(ns)))


def hem_sweep(electrodes, imgs, nodes, s, kappa, mur=1.0, ie=None, inj_node=0, precision=PLAIN_FP64,
              max_batch=0, graphs=True, split=None, fill=None):
    """Solutions [U; I_L; I_T] for every Laplace sample (one plan, one run);
    fill = INTG_MHEM selects the mHEM impedance model."""
    if not max_batch:
        max_batch = min(len(np.atleast_1d(s)), 64)
    plan = Plan(electrodes, imgs, nodes, precision, max_batch, graphs)
    if split is not None:
        plan.set_split(split)
    if fill is not None:
        plan.set_fill(fill)
    try:
        return plan.run(s, kappa, mur, ie, inj_node)
    finally:
        plan.close()


def sweep_fingerprint(parts) -> str:
    """SHA-256 over a sweep's inputs (arrays by dtype, shape and bytes; other
    values by repr), which a saved sweep must match to be resumed."""
    h = hashlib.sha256()
    for x in parts:
        if x is None:
            h.update(b"none")
        elif isinstance(x, np.ndarray):
            h.update(f"{x.dtype}{x.shape}".encode())
            h.update(np.ascontiguousarray(x).tobytes())
        else:
            h.update(repr(x).encode())
        h.update(b"|")
    return h.hexdigest()


def _replace_atomic(path, write):
    tmp = path + ".tmp"
    write(tmp)
    os.replace(tmp, path)


def resumable_sweep(run_chunk, ns, directory, chunk, fingerprint):
    """Samples [0, ns) in chunks: run_chunk(k0, k1) returns (arrays, stats),
    the arrays' first axis k1 - k0, stats a dict of numbers. After each chunk
    its arrays go to directory/chunk_<k0>.npz and the manifest
    (directory/manifest.json: fingerprint, ns, chunk, finished chunks and their
    stats) records it; both are written under a temporary name and renamed, so
    an interruption leaves the last finished chunk recorded. A call on a
    directory with a manifest resumes when fingerprint, ns and chunk agree and
    raises ValueError otherwise. Returns (arrays concatenated over the samples,
    stats of every chunk in order, chunks run by this call)."""
    if ns <= 0 or chunk <= 0:
        raise ValueError("resumable_sweep: ns and chunk must be positive")
    os.makedirs(directory, exist_ok=True)
    man_path = os.path.join(directory, "manifest.json")
    man = {"version": 1, "fingerprint": fingerprint, "ns": int(ns), "chunk": int(chunk), "done": {}}
    if os.path.exists(man_path):
        with open(man_path) as f:
            old = json.load(f)
        if (old.get("version"), old.get("fingerprint"), old.get("ns"), old.get("chunk")) != \
                (1, fingerprint, int(ns), int(chunk)):
            raise ValueError(f"{man_path} belongs to another sweep (inputs, sample count or chunk differ)")
        man = old
    parts = {}
    ran = 0
    for k0 in range(0, ns, chunk):
        k1 = min(ns, k0 + chunk)
        name = os.path.join(directory, f"chunk_{k0:09d}.npz")
        if str(k0) in man["done"] and os.path.exists(name):
            with np.load(name) as z:
                arrays = {k: z[k] for k in z.files}
        else:
            arrays, stats = run_chunk(k0, k1)
            arrays = {k: np.asarray(v) for k, v in arrays.items()}
            for k, v in arrays.items():
                if v.shape[0] != k1 - k0:
                    raise ValueError(f"resumable_sweep: output {k} has {v.shape[0]} rows for {k1 - k0} samples")

            def write_npz(tmp, arrays=arrays):
                with open(tmp, "wb") as f:
                    np.savez(f, **arrays)
            _replace_atomic(name, write_npz)
            man["done"][str(k0)] = {k: float(v) for k, v in stats.items()}

            def write_man(tmp):
                with open(tmp, "w") as f:
                    json.dump(man, f)
            _replace_atomic(man_path, write_man)
            ran += 1
        for k, v in arrays.items():
            parts.setdefault(k, []).append(v)
    out = {k: np.concatenate(v, axis=0) for k, v in parts.items()}
    stats = [man["done"][str(k0)] for k0 in range(0, ns, chunk)]
    return out, stats, ran


def uneven_grids(count: int = 64, seed: int = 0):
    """A batch of square grids of uneven size (the 64-grid workload): side
    uniform in 5-40 m, 2-10 meshes per side, 1 m segmentation (ceil(mesh
    edge / 1 m) segments per edge, as the reference's examples divide edges),
    depth uniform 0.3-1.0 m, radius uniform 5-10 mm, soil resistivity
    log-uniform 50-5000 ohm m, relative permittivity uniform 5-40.
    Returns dicts with electrodes, nodes and the soil of each grid."""
    rng = np.random.default_rng(seed)
    grids = []
    for _ in range(count):
        side = float(rng.uniform(5.0, 40.0))
        meshes = int(rng.integers(2, 11))
        depth = float(rng.uniform(0.3, 1.0))
        radius = float(rng.uniform(5e-3, 10e-3))
        rho = float(np.exp(rng.uniform(np.log(50.0), np.log(5000.0))))
        epsr = float(rng.uniform(5.0, 40.0))
        div = int(math.ceil(side / meshes / 1.0))
        elec, nodes = electrode_grid(meshes + 1, meshes + 1, side, side, div, div, radius, -depth)
        grids.append({"electrodes": elec, "nodes": nodes, "rho": rho, "epsr": epsr, "side": side,
                      "meshes": meshes, "depth": depth, "radius": radius})
    return grids


def hem_sweep_grids(jobs, precision=MIXED, max_batch=0, workers=8, graphs=True, split=None):
    """Many grids at once: one plan per job, run from `workers` host threads,
    so the plans' passes (each a graph launch on the plan's own stream) share
    the GPU. A job is a dict with electrodes, images (or None), nodes, s,
    kappa and either ie (ns x n) or inj_node. Returns [(solution, info,
    RunStats)] in job order."""
    from concurrent.futures import ThreadPoolExecutor

    def one(job):
        ns = len(np.atleast_1d(job["s"]))
        plan = Plan(job["electrodes"], job.get("images"), job["nodes"], precision,
                    max_batch or min(ns, 256), graphs)
        try:
            if split is not None and precision == MIXED:
                plan.set_split(split)
            return plan.run(job["s"], job["kappa"], job.get("mur", 1.0), job.get("ie"), job.get("inj_node", 0))
        finally:
            plan.close()

    with ThreadPoolExecutor(max_workers=max(1, int(workers))) as ex:
        return list(ex.map(one, jobs))


def _grid_jobs(jobs):
    """ctypes job array for tags_gpu_solve_batch / tags_batch_*: the arrays it
    points into (kept alive by the caller) and the (solution, info) outputs."""
    keep, out = [], []
    arr = (GridJob * len(jobs))()
    for q, job in enumerate(jobs):
        e = _elec(job["electrodes"])
        im = None if job.get("images") is None else _elec(job["images"])
        nd = np.ascontiguousarray(job["nodes"], dtype=np.float64)
        sv = np.ascontiguousarray(np.atleast_1d(job["s"]), dtype=np.complex128)
        ns = sv.shape[0]
        kv = np.ascontiguousarray(np.broadcast_to(job["kappa"], (ns,)), dtype=np.complex128)
        ie = job.get("ie")
        if ie is not None:
            ie = np.ascontiguousarray(ie, dtype=np.complex128).reshape(ns, nd.shape[0])
        sol = np.zeros((ns, nd.shape[0] + 2 * e.shape[0]), np.complex128)
        info = np.zeros(ns, np.int32)
        keep += [e, im, nd, sv, kv, ie, sol, info]
        out.append((sol, info))
        arr[q] = GridJob(_addr(e), None if im is None else _addr(im), e.shape[0], _addr(nd), nd.shape[0], _addr(sv),
                         _addr(kv), ns, None if ie is None else _addr(ie), int(job.get("inj_node", 0)), _addr(sol),
                         _addr(info))
    return arr, keep, out


class GridBatch:
    """Many grids of uneven size in one CUDA graph (tags_batch_create /
    tags_batch_run / tags_batch_destroy): built once for the jobs' shapes,
    each run solves every sample of every grid with one graph launch."""

    def __init__(self, jobs, precision=MIXED, mur: float = 1.0, max_batch: int = 0):
        arr, keep, _ = _grid_jobs(jobs)
        h = ctypes.c_void_p()
        code = lib().tags_batch_create(ctypes.byref(h), arr, len(jobs), int(precision), float(mur), int(max_batch))
        if code != 0:
            raise RuntimeError(f"tags_batch_create failed ({code}): {last_error()}")
        self.handle = h
        self.count = len(jobs)

    def run(self, jobs):
        """[(solution ns x (n + 2m), info)] in job order, and the RunStats."""
        arr, keep, out = _grid_jobs(jobs)
        st = RunStats()
        code = lib().tags_batch_run(self.handle, arr, len(jobs), ctypes.byref(st))
        if code != 0:
            raise RuntimeError(f"tags_batch_run failed ({code}): {last_error()}")
        return out, st

    def close(self):
        if getattr(self, "handle", None):
            lib().tags_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_batch(jobs, precision=MIXED, mur: float = 1.0, max_batch: int = 0, workers: int = 4):
    """Many grids x many samples in one C call (tags_gpu_solve_batch). Jobs as
    for hem_sweep_grids (dicts with electrodes, images, nodes, s, kappa and ie
    or inj_node); returns [(solution ns x (n + 2m), info)] in job order."""
    keep, out = [], []
    arr = (GridJob * len(jobs))()
    for q, job in enumerate(jobs):
        e = _elec(job["electrodes"])
        im = None if job.get("images") is None else _elec(job["images"])
        nd = np.ascontiguousarray(job["nodes"], dtype=np.float64)
        sv = np.ascontiguousarray(np.atleast_1d(job["s"]), dtype=np.complex128)
        ns = sv.shape[0]
        kv = np.ascontiguousarray(np.broadcast_to(job["kappa"], (ns,)), dtype=np.complex128)
        ie = job.get("ie")
        if ie is not None:
            ie = np.ascontiguousarray(ie, dtype=np.complex128).reshape(ns, nd.shape[0])
        sol = np.zeros((ns, nd.shape[0] + 2 * e.shape[0]), np.complex128)
        info = np.zeros(ns, np.int32)
        keep += [e, im, nd, sv, kv, ie]
        out.append((sol, info))
        arr[q] = GridJob(_addr(e), None if im is None else _addr(im), e.shape[0], _addr(nd), nd.shape[0], _addr(sv),
                         _addr(kv), ns, None if ie is None else _addr(ie), int(job.get("inj_node", 0)), _addr(sol),
                         _addr(info))
    _ret(lib().tags_gpu_solve_batch(arr, len(jobs), int(precision), float(mur), int(max_batch), int(workers)))
    return out


# ---- multi-GPU helpers (host side) ------------------------------------------------------

def shard_samples(ns: int, rank: int, world: int) -> np.ndarray:
    """Laplace samples handled by `rank` of `world` processes (one GPU each):
    strided, so every rank sees low and high frequencies alike. The samples are
    independent, so ranks exchange nothing while they solve."""
    if not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    return np.arange(rank, ns, world)


def gather_samples(values: np.ndarray, ns: int, group=None):
    """Collect every rank's per-sample results (rows in shard_samples order)
    on rank 0 before the inverse Laplace transform; other ranks get None.
    The only exchange of the multi-GPU path, done on the host."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    parts = [None] * world if rank == 0 else None
    dist.gather_object(np.asarray(values), parts, dst=0, group=group)
    if rank != 0:
        return None
    first = np.asarray(parts[0])
    out = np.zeros((ns,) + first.shape[1:], dtype=first.dtype)
    for r, part in enumerate(parts):
        out[shard_samples(ns, r, world)] = part
    return out
