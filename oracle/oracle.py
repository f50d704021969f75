"""Test infrastructure only: Python bindings of the CPU oracle for the HEM hot path.

Two libraries share one calling convention:

* ``port`` -- ``oracle/libtags_oracle.so``, the project's plain-C restatement of
  the reference's per-sample path (``oracle/tags_oracle.c``). It builds from this
  repository alone, so it is the oracle everywhere the reference sources are
  absent.
* ``ref`` -- ``oracle/_ref/libtags_ref.so``, the reference's own
  ``src/{electrode,auxiliary,grid,linalg}.c`` compiled with the project-written
  shims for its missing third-party code (``make -C oracle ref``). It exists only
  where the reference sources were present at build time, and is used to pin the
  restatement and to generate the golden fixtures under ``tests/golden/``.

LAPACK comes from the OpenBLAS that ships inside scipy (``zsysv`` and friends are
bound at load time). Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` import this module; the GPU product never does.

Matrices are returned as numpy arrays in mathematical orientation: a
column-major ``m x m`` buffer ``z`` of the reference (``z[i*m + k]`` = row k,
column i) becomes ``Z[k, i]``.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "libtags_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libtags_ref.so")

INTG_NONE, INTG_DOUBLE, INTG_SINGLE, INTG_MHEM = 1, 2, 3, 4
FILTER_NONE, FILTER_BLACKMAN, FILTER_HANNING, FILTER_LANCZOS, FILTER_RIESZ = range(5)

# src/auxiliary.c:17-21
PI = 3.1415926535897932384626433832795029
TWO_PI = 6.283185307179586476925286766559
FOUR_PI = 12.5663706143591729538505735331
MU0 = 1.256637061435917e-6
EPS0 = 8.854187817620e-12


class c_complex(ctypes.Structure):
    """A C99 ``double _Complex`` passed by value (two doubles; same register
    class as the complex type on x86-64 SysV and AArch64 AAPCS64)."""

    _fields_ = [("re", ctypes.c_double), ("im", ctypes.c_double)]

    @classmethod
    def of(cls, z) -> "c_complex":
        z = complex(z)
        return cls(z.real, z.imag)

    def value(self) -> complex:
        return complex(self.re, self.im)


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_sz = ctypes.c_size_t


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _openblas_path() -> str | None:
    try:
        import scipy
    except ImportError:
        return None
    base = os.path.dirname(scipy.__file__)
    for pat in ("../scipy.libs/libscipy_openblas*.so", "../scipy_openblas*/lib/libscipy_openblas*.so"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return hits[0]
    return None


_lock = threading.Lock()
_libs: dict[str, "Oracle"] = {}


def reference_dir() -> str:
    """Where the reference's sources are read from to build ``ref``: the
    TAGS_REFERENCE_DIR environment variable, else a checkout named
    ``reference`` beside this repository."""
    return os.environ.get("TAGS_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build(ref: bool = False) -> None:
    """Compile the restatement (and, with ``ref``, the reference) via oracle/Makefile."""
    target = ["ref", "REF=" + reference_dir()] if ref else []
    subprocess.run(["make", "-s", "-C", HERE] + target, check=True)


class Oracle:
    """One loaded oracle library (``kind`` = "port" or "ref")."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        path = PORT_LIB if kind == "port" else REF_LIB
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} is not built")
        self.lib = ctypes.CDLL(path)
        self.p = "oracle_" if kind == "port" else ""
        self._bind_lapack()
        self._declare()

    # -- set-up ------------------------------------------------------------
    def _bind_lapack(self) -> None:
        path = _openblas_path()
        if path is None:
            raise RuntimeError("scipy's bundled OpenBLAS was not found; the oracle needs zsysv")
        ob = ctypes.CDLL(path)
        self.openblas = ob
        for name in ("zsysv", "zsytrf", "zsytri", "zsymm", "zgemm", "zgesv"):
            fn = getattr(ob, f"scipy_{name}_")
            self.lib.tags_lapack_bind(name.encode(), ctypes.cast(fn, ctypes.c_void_p))
        try:
            self._set_threads = ob.scipy_openblas_set_num_threads
            self._set_threads.argtypes = [ctypes.c_int]
        except AttributeError:
            self._set_threads = None
        self.blas_threads(1)

    def blas_threads(self, n: int) -> None:
        """Pin OpenBLAS threads, as the reference examples do (examples/grcev12pwrd01.c:88)."""
        if self._set_threads is not None:
            self._set_threads(int(n))

    def _fn(self, name: str):
        return getattr(self.lib, self.p + name)

    def _declare(self) -> None:
        C = c_complex
        f = self._fn("self_integral")
        f.argtypes = [_dp]
        f.restype = C if self.kind == "ref" else ctypes.c_double
        f = self._fn("calculate_impedances")
        f.argtypes = [_dp, _dp, _dp, _sz, C, C, ctypes.c_double, C, _sz, ctypes.c_double,
                      ctypes.c_double, ctypes.c_int]
        f.restype = ctypes.c_int
        f = self._fn("impedances_images")
        f.argtypes = [_dp, _dp, _dp, _dp, _sz, C, C, ctypes.c_double, C, C, C, _sz,
                      ctypes.c_double, ctypes.c_double, ctypes.c_int]
        f.restype = ctypes.c_int
        f = self._fn("integral")
        f.argtypes = [_dp, _dp, C, _sz, ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp]
        f.restype = ctypes.c_int
        for name in ("fill_incidence_imm",):
            f = self._fn(name)
            f.argtypes = [_dp, _dp, _sz, _dp, _sz]
            f.restype = ctypes.c_int
        f = self._fn("fill_impedance_imm")
        f.argtypes = [_dp, _dp, _dp, _sz, _sz]
        f.restype = ctypes.c_int
        f = self._fn("solve_immittance")
        f.argtypes = [_dp, _dp, _sz, _sz]
        f.restype = ctypes.c_int
        # nodal admittance formulation (src/linalg.c:142-321)
        f = self._fn("fill_incidence_adm")
        f.argtypes = [_dp, _dp, _dp, _sz, _dp, _sz]
        f.restype = ctypes.c_int
        f = self._fn("calculate_yla_ytb")
        f.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _sz, _sz]
        f.restype = ctypes.c_int
        for name in ("fill_impedance_adm2", "fill_impedance_adm"):
            f = self._fn(name)
            f.argtypes = [_dp, _dp, _dp, _dp, _dp, _sz, _sz]
            f.restype = ctypes.c_int
        f = self._fn("solve_admittance")
        f.argtypes = [_dp, _dp, _sz]
        f.restype = ctypes.c_int
        f = self._fn("laplace_trans")
        f.argtypes = [_dp, _dp, _dp, ctypes.c_double, _sz]
        f.restype = ctypes.c_int
        f = self._fn("inv_laplace_trans")
        f.argtypes = [_dp, _dp, _dp, ctypes.c_double, _sz, ctypes.c_int]
        f.restype = ctypes.c_int
        f = self._fn("alipio_soil")
        f.argtypes = [_dp, _dp, ctypes.c_double, C, ctypes.c_double, ctypes.c_double,
                      ctypes.c_double]
        f.restype = ctypes.c_int
        f = self._fn("heidler")
        f.argtypes = [ctypes.c_double] * 5
        f.restype = ctypes.c_double
        f = self._fn("segment_electrode")
        f.argtypes = [_dp, _dp, _sz, _dp, _dp, ctypes.c_double]
        f.restype = ctypes.c_int
        # post-processing (src/electrode.c:434-668); the restatement adds a
        # failure out-argument to the two functions that return the value
        tail = [_ip] if self.kind == "port" else []
        f = self._fn("electric_potential")
        f.argtypes = [_dp, _dp, _sz, _dp, C, C, _sz, ctypes.c_double, ctypes.c_double] + tail
        f.restype = C
        f = self._fn("magnetic_potential")
        f.argtypes = [_dp, _dp, _sz, _dp, C, ctypes.c_double, _sz, ctypes.c_double, ctypes.c_double, _dp]
        f.restype = ctypes.c_int
        f = self._fn("electric_field")
        f.argtypes = [_dp, _dp, _sz, _dp, _dp, C, C, ctypes.c_double, C, _sz, ctypes.c_double,
                      ctypes.c_double, _dp]
        f.restype = ctypes.c_int
        f = self._fn("voltage")
        f.argtypes = [_dp, _dp, _dp, _sz, _dp, _dp, C, C, ctypes.c_double, C, _sz, ctypes.c_double,
                      ctypes.c_double] + tail
        f.restype = C
        if self.kind == "port":
            f = self.lib.oracle_hem_sweep
            f.argtypes = [_dp, _dp, _sz, _dp, _sz, _dp, _dp, _sz, ctypes.c_double, _sz, _dp,
                          _sz, ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _ip]
            f.restype = ctypes.c_int
            f = self.lib.oracle_hem_impedances
            f.argtypes = [_dp, _dp, _sz, C, C, ctypes.c_double, _sz, ctypes.c_double,
                          ctypes.c_double, ctypes.c_int, _dp, _dp]
            f.restype = ctypes.c_int
            f = self.lib.oracle_mhem_impedances
            f.argtypes = [_dp, _dp, _sz, _dp, _dp, _dp, _dp, C, C, ctypes.c_double, _dp, _dp]
            f.restype = ctypes.c_int
            f = self.lib.oracle_gpd_mhem
            f.argtypes = [_dp, _sz, _dp, _sz, _dp, _sz, C, C, _dp]
            f.restype = ctypes.c_int
            f = self.lib.oracle_mhem_sweep
            f.argtypes = [_dp, _dp, _sz, _dp, _sz, _dp, _dp, _sz, ctypes.c_double, _sz, _dp,
                          _sz, ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _ip]
            f.restype = ctypes.c_int

    # -- geometry ------------------------------------------------------------
    def segment_electrode(self, a, b, nseg: int, radius: float):
        elec = np.zeros((nseg, 11))
        nodes = np.zeros((nseg + 1, 3))
        err = self._fn("segment_electrode")(_ptr(elec), _ptr(nodes), nseg,
                                            _ptr(np.ascontiguousarray(a, dtype=float)),
                                            _ptr(np.ascontiguousarray(b, dtype=float)), radius)
        if err:
            raise ValueError(f"segment_electrode failed: {err}")
        return elec, nodes

    def self_integral(self, elec_row) -> float:
        e = np.ascontiguousarray(elec_row, dtype=float)
        r = self._fn("self_integral")(_ptr(e))
        return r.value().real if self.kind == "ref" else float(r)

    # -- impedance fill ------------------------------------------------------
    def integral(self, sender, receiver, gamma, max_eval=0, req_abs=1e-6, req_rel=1e-6,
                 itype=INTG_DOUBLE):
        res = np.zeros(2)
        err = np.zeros(2)
        code = self._fn("integral")(_ptr(np.ascontiguousarray(sender, dtype=float)),
                                    _ptr(np.ascontiguousarray(receiver, dtype=float)),
                                    c_complex.of(gamma), max_eval, req_abs, req_rel, itype,
                                    _ptr(res), _ptr(err))
        return complex(res[0], res[1]), complex(err[0], err[1]), code

    def calculate_impedances(self, zl, zt, elec, gamma, s, mur, kappa, max_eval=0,
                             req_abs=1e-6, req_rel=1e-6, itype=INTG_DOUBLE) -> int:
        """Raw call: zl/zt are flat complex128 buffers of m*m (column-major)."""
        e = np.ascontiguousarray(elec, dtype=float)
        return self._fn("calculate_impedances")(
            _ptr(zl), _ptr(zt), _ptr(e), e.shape[0], c_complex.of(gamma), c_complex.of(s),
            mur, c_complex.of(kappa), max_eval, req_abs, req_rel, itype)

    def impedances_images(self, zl, zt, elec, img, gamma, s, mur, kappa, ref_l, ref_t,
                          max_eval=0, req_abs=1e-6, req_rel=1e-6, itype=INTG_DOUBLE) -> int:
        e = np.ascontiguousarray(elec, dtype=float)
        im = np.ascontiguousarray(img, dtype=float)
        return self._fn("impedances_images")(
            _ptr(zl), _ptr(zt), _ptr(e), _ptr(im), e.shape[0], c_complex.of(gamma),
            c_complex.of(s), mur, c_complex.of(kappa), c_complex.of(ref_l), c_complex.of(ref_t),
            max_eval, req_abs, req_rel, itype)

    def hem_impedances(self, elec, img, s, kappa, mur=1.0, max_eval=0, req_abs=1e-6,
                       req_rel=1e-6, itype=INTG_DOUBLE):
        """ZL, ZT (lower triangles, direct + images) of one sample as m x m arrays."""
        m = elec.shape[0]
        zl = np.zeros(m * m, dtype=np.complex128)
        zt = np.zeros(m * m, dtype=np.complex128)
        gamma, ref_t = medium(s, kappa, mur)
        err = self.calculate_impedances(zl, zt, elec, gamma, s, mur, kappa, max_eval,
                                        req_abs, req_rel, itype)
        if err:
            raise RuntimeError(f"calculate_impedances failed: {err}")
        if img is not None:
            err = self.impedances_images(zl, zt, elec, img, gamma, s, mur, kappa, 1.0, ref_t,
                                         max_eval, req_abs, req_rel, itype)
            if err:
                raise RuntimeError(f"impedances_images failed: {err}")
        return zl.reshape(m, m).T.copy(), zt.reshape(m, m).T.copy()

    # -- immittance system ---------------------------------------------------
    def fill_incidence_imm(self, wg_flat, elec, nodes) -> int:
        e = np.ascontiguousarray(elec, dtype=float)
        nd = np.ascontiguousarray(nodes, dtype=float)
        return self._fn("fill_incidence_imm")(_ptr(wg_flat), _ptr(e), e.shape[0], _ptr(nd),
                                              nd.shape[0])

    def fill_impedance_imm(self, wg_flat, zl_flat, zt_flat, m: int, n: int) -> int:
        return self._fn("fill_impedance_imm")(_ptr(wg_flat), _ptr(zl_flat), _ptr(zt_flat), m, n)

    def solve_immittance(self, wg_flat, ie, m: int, n: int) -> int:
        return self._fn("solve_immittance")(_ptr(wg_flat), _ptr(ie), m, n)

    # -- nodal admittance formulation -------------------------------------------
    def fill_incidence_adm(self, a_flat, b_flat, elec, nodes) -> int:
        e = np.ascontiguousarray(elec, dtype=float)
        nd = np.ascontiguousarray(nodes, dtype=float)
        return self._fn("fill_incidence_adm")(_ptr(a_flat), _ptr(b_flat), _ptr(e), e.shape[0], _ptr(nd),
                                              nd.shape[0])

    def calculate_yla_ytb(self, yla, ytb, zl, zt, a, b, m: int, n: int) -> int:
        return self._fn("calculate_yla_ytb")(_ptr(yla), _ptr(ytb), _ptr(zl), _ptr(zt), _ptr(a), _ptr(b), m, n)

    def fill_impedance_adm2(self, yn, yla, ytb, a, b, m: int, n: int) -> int:
        return self._fn("fill_impedance_adm2")(_ptr(yn), _ptr(yla), _ptr(ytb), _ptr(a), _ptr(b), m, n)

    def fill_impedance_adm(self, yn, zl, zt, a, b, m: int, n: int) -> int:
        return self._fn("fill_impedance_adm")(_ptr(yn), _ptr(zl), _ptr(zt), _ptr(a), _ptr(b), m, n)

    def solve_admittance(self, yn, ic, n: int) -> int:
        return self._fn("solve_admittance")(_ptr(yn), _ptr(ic), n)

    def mhem_sweep(self, elec, img, nodes, s, kappa, inj_node, inj, mur=1.0, max_eval=0, req_abs=1e-6,
                   req_rel=1e-6, threads=0):
        """Node potentials (ns x n) of the mHEM + nodal-admittance sample loop and the zsysv infos."""
        if self.kind != "port":
            raise NotImplementedError("the sweep driver is part of the restatement")
        e = np.ascontiguousarray(elec, dtype=float)
        im = np.ascontiguousarray(img, dtype=float)
        nd = np.ascontiguousarray(nodes, dtype=float)
        s = np.ascontiguousarray(s, dtype=np.complex128)
        kappa = np.ascontiguousarray(np.broadcast_to(kappa, s.shape), dtype=np.complex128)
        inj = np.ascontiguousarray(np.broadcast_to(inj, s.shape), dtype=np.complex128)
        m, n, ns = e.shape[0], nd.shape[0], s.shape[0]
        sol = np.zeros((ns, n), dtype=np.complex128)
        info = np.zeros(ns, dtype=np.int32)
        err = self.lib.oracle_mhem_sweep(_ptr(e), _ptr(im), m, _ptr(nd), n, _ptr(s), _ptr(kappa), ns, mur,
                                         inj_node, _ptr(inj), max_eval, req_abs, req_rel, threads, _ptr(sol),
                                         info.ctypes.data_as(_ip))
        if err:
            raise RuntimeError(f"mhem_sweep set-up failed: {err}")
        return sol, info

    # -- Laplace pair --------------------------------------------------------
    def laplace_trans(self, f, tmax: float):
        f = np.ascontiguousarray(f, dtype=float)
        nt = f.shape[0]
        ns = nt // 2 + 1
        g = np.zeros(ns, dtype=np.complex128)
        s = np.zeros(ns, dtype=np.complex128)
        err = self._fn("laplace_trans")(_ptr(f), _ptr(g), _ptr(s), tmax, nt)
        if err:
            raise RuntimeError("laplace_trans failed")
        return g, s

    def inv_laplace_trans(self, g, s, tmax: float, nt: int, filt: int = FILTER_NONE):
        g = np.ascontiguousarray(g, dtype=np.complex128)
        s = np.ascontiguousarray(s, dtype=np.complex128)
        f = np.zeros(nt)
        err = self._fn("inv_laplace_trans")(_ptr(f), _ptr(g), _ptr(s), tmax, nt, filt)
        if err:
            raise RuntimeError("inv_laplace_trans failed")
        return f

    def alipio_soil(self, sigma0, s, h, g, eps_ratio):
        sig = np.zeros(1, dtype=np.complex128)
        eps = np.zeros(1, dtype=np.complex128)
        self._fn("alipio_soil")(_ptr(sig), _ptr(eps), sigma0, c_complex.of(s), h, g, eps_ratio)
        return complex(sig[0]), complex(eps[0])

    # -- post-processing: potentials, fields, path voltage ------------------------
    def electric_potential(self, point, elec, it, gamma, kappa, max_eval=0, req_abs=1e-6, req_rel=1e-6):
        p = np.ascontiguousarray(point, dtype=float)
        e = np.ascontiguousarray(elec, dtype=float)
        it = np.ascontiguousarray(it, dtype=np.complex128)
        args = [_ptr(p), _ptr(e), e.shape[0], _ptr(it), c_complex.of(gamma), c_complex.of(kappa), max_eval,
                req_abs, req_rel]
        if self.kind == "port":
            fail = ctypes.c_int(0)
            v = self._fn("electric_potential")(*args, ctypes.byref(fail))
            if fail.value:
                raise RuntimeError(f"electric_potential failed: {fail.value}")
        else:
            v = self._fn("electric_potential")(*args)
        return v.value()

    def magnetic_potential(self, point, elec, il, gamma, mur=1.0, max_eval=0, req_abs=1e-6, req_rel=1e-6):
        p = np.ascontiguousarray(point, dtype=float)
        e = np.ascontiguousarray(elec, dtype=float)
        il = np.ascontiguousarray(il, dtype=np.complex128)
        va = np.zeros(3, dtype=np.complex128)
        code = self._fn("magnetic_potential")(_ptr(p), _ptr(e), e.shape[0], _ptr(il), c_complex.of(gamma), mur,
                                              max_eval, req_abs, req_rel, _ptr(va))
        if code:
            raise RuntimeError(f"magnetic_potential failed: {code}")
        return va

    def electric_field(self, point, elec, il, it, gamma, s, kappa, mur=1.0, max_eval=0, req_abs=1e-6,
                       req_rel=1e-6, ve=None):
        """E at a point; ``ve`` (3 complex) is the array the reference adds to when |s| is 0."""
        p = np.ascontiguousarray(point, dtype=float)
        e = np.ascontiguousarray(elec, dtype=float)
        il = np.ascontiguousarray(il, dtype=np.complex128)
        it = np.ascontiguousarray(it, dtype=np.complex128)
        ve = np.zeros(3, dtype=np.complex128) if ve is None else np.array(ve, dtype=np.complex128)
        code = self._fn("electric_field")(_ptr(p), _ptr(e), e.shape[0], _ptr(il), _ptr(it), c_complex.of(gamma),
                                          c_complex.of(s), mur, c_complex.of(kappa), max_eval, req_abs, req_rel,
                                          _ptr(ve))
        return ve, code

    def voltage(self, p1, p2, elec, il, it, gamma, s, kappa, mur=1.0, max_eval=0, req_abs=1e-6, req_rel=1e-6):
        a = np.ascontiguousarray(p1, dtype=float)
        b = np.ascontiguousarray(p2, dtype=float)
        e = np.ascontiguousarray(elec, dtype=float)
        il = np.ascontiguousarray(il, dtype=np.complex128)
        it = np.ascontiguousarray(it, dtype=np.complex128)
        args = [_ptr(a), _ptr(b), _ptr(e), e.shape[0], _ptr(il), _ptr(it), c_complex.of(gamma), c_complex.of(s),
                mur, c_complex.of(kappa), max_eval, req_abs, req_rel]
        if self.kind == "port":
            fail = ctypes.c_int(0)
            v = self._fn("voltage")(*args, ctypes.byref(fail))
        else:
            v = self._fn("voltage")(*args)
        return v.value()

    def gpd_mhem(self, points, elec, it, gamma, kappa):
        """Closed-form mHEM ground potential (np x nrhs); it is (m x nrhs)."""
        if self.kind != "port":
            raise NotImplementedError("the ground-potential loop belongs to an example, not the library")
        pts = np.ascontiguousarray(points, dtype=float)
        e = np.ascontiguousarray(elec, dtype=float)
        it = np.asarray(it, dtype=np.complex128)
        if it.ndim == 1:
            it = it[:, None]
        nrhs = it.shape[1]
        itc = np.ascontiguousarray(it.T)          # column-major (m x nrhs)
        out = np.zeros((pts.shape[0], nrhs), dtype=np.complex128)
        self.lib.oracle_gpd_mhem(_ptr(pts), pts.shape[0], _ptr(e), e.shape[0], _ptr(itc), nrhs,
                                 c_complex.of(gamma), c_complex.of(kappa), _ptr(out))
        return out

    def heidler(self, t, imax, tau1, tau2, n):
        return self._fn("heidler")(t, imax, tau1, tau2, n)

    # -- per-sample sweep (restatement only) -----------------------------------
    def hem_sweep(self, elec, img, nodes, s, kappa, inj_node, inj, mur=1.0, max_eval=0,
                  req_abs=1e-6, req_rel=1e-6, threads=0):
        """Solutions [U; I_L; I_T] for every sample (ns x N) and LAPACK infos."""
        if self.kind != "port":
            raise NotImplementedError("the sweep driver is part of the restatement")
        e = np.ascontiguousarray(elec, dtype=float)
        im = np.ascontiguousarray(img, dtype=float)
        nd = np.ascontiguousarray(nodes, dtype=float)
        s = np.ascontiguousarray(s, dtype=np.complex128)
        kappa = np.ascontiguousarray(np.broadcast_to(kappa, s.shape), dtype=np.complex128)
        inj = np.ascontiguousarray(np.broadcast_to(inj, s.shape), dtype=np.complex128)
        m, n, ns = e.shape[0], nd.shape[0], s.shape[0]
        sol = np.zeros((ns, n + 2 * m), dtype=np.complex128)
        info = np.zeros(ns, dtype=np.int32)
        err = self.lib.oracle_hem_sweep(_ptr(e), _ptr(im), m, _ptr(nd), n, _ptr(s), _ptr(kappa),
                                        ns, mur, inj_node, _ptr(inj), max_eval, req_abs, req_rel,
                                        threads, _ptr(sol), info.ctypes.data_as(_ip))
        if err:
            raise RuntimeError(f"hem_sweep set-up failed: {err}")
        return sol, info


def get(kind: str = "port") -> Oracle:
    """Load (building the restatement if needed) and cache an oracle library."""
    with _lock:
        if kind not in _libs:
            if kind == "port" and not os.path.exists(PORT_LIB):
                build(ref=False)
            _libs[kind] = Oracle(kind)
        return _libs[kind]


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind == "port" else REF_LIB)


# -- host-side helpers shared by tests (pure numpy restatements) -------------

def medium(s, kappa, mur=1.0):
    """gamma and the transversal reflection coefficient (examples/three_grids.c:326-333)."""
    s = complex(s)
    kappa = complex(kappa)
    gamma = np.sqrt(s * mur * MU0 * kappa)
    ref_t = (kappa - s * EPS0) / (kappa + s * EPS0)
    return complex(gamma), complex(ref_t)


def images(elec: np.ndarray) -> np.ndarray:
    """Mirror segments across z = 0 (examples/three_grids.c:206-214)."""
    img = np.array(elec, dtype=float, copy=True)
    img[:, 2] *= -1.0
    img[:, 5] *= -1.0
    img[:, 8] *= -1.0
    return img
