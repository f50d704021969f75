"""GPU checks of the mixed form's tensor-core LDL^T (tcgen05 GEMMs on split
products: bf16 pieces or scaled fp16 pairs, FP32 storage; trailing updates on
one SM per tile or on two-SM clusters) through its diagnostic entry points."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym_matrix(rng, N, dominance):
    a = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) / np.sqrt(N)
    a = a + a.T
    a += np.diag(dominance * (1.0 + 0.3j) * (1 + rng.random(N)))
    return a


def _ldl(pkg, mats, pieces=3, pairs=False):
    pkg.lib().tags_debug_tc_pairs(int(pairs))
    fn = pkg.lib().tags_debug_ldl
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    fn.restype = ctypes.c_int
    nb, N = mats.shape[0], mats.shape[1]
    buf = np.ascontiguousarray(np.transpose(mats, (0, 2, 1))).astype(np.complex128)   # column-major
    code = fn(buf.ctypes.data, N, nb, pieces)
    pkg.lib().tags_debug_tc_pairs(0)
    return code, np.transpose(buf, (0, 2, 1))


@pytest.mark.parametrize("pairs", [0, 1, 2])
@pytest.mark.parametrize("pieces,tol", [(2, 2e-5), (3, 2e-6), (16, 4e-6)])
@pytest.mark.parametrize("N", [128, 300, 517])
def test_tensor_core_ldl_reconstructs(gpu_pkg, N, pieces, tol, pairs):
    """L D L^T reproduces A to the accuracy of the split products: ~1e-5 with
    two bf16 pieces per value (three products), FP32 level with three (six),
    near FP32 level with two fp16 pieces of 2^8 x (three products); the
    trailing updates on one SM per tile, on two-SM clusters (pairs 1), or on
    two-SM clusters with real-form products of N = 256 (pairs 2; three bf16
    pieces fall back to 1)."""
    rng = np.random.default_rng(N)
    mats = np.stack([_sym_matrix(rng, N, 4.0), _sym_matrix(rng, N, 2.0), _sym_matrix(rng, N, 3.0)])
    code, fac = _ldl(gpu_pkg, mats, pieces, pairs)
    assert code == 0, gpu_pkg.last_error()
    for q in range(3):
        L = np.tril(fac[q], -1) + np.eye(N)
        D = np.diag(np.diag(fac[q]))
        err = np.linalg.norm(L @ D @ L.T - mats[q]) / np.linalg.norm(mats[q])
        assert err < tol, (N, q, err)


def test_tensor_core_ldl_matches_fp64_factors(gpu_pkg):
    rng = np.random.default_rng(7)
    N = 260
    A = _sym_matrix(rng, N, 3.0)
    code, fac = _ldl(gpu_pkg, A[None])
    assert code == 0
    # FP64 reference LDL^T without pivoting
    W = A.copy()
    Lr = np.eye(N, dtype=complex)
    d = np.zeros(N, dtype=complex)
    for k in range(N):
        d[k] = W[k, k]
        Lr[k + 1:, k] = W[k + 1:, k] / d[k]
        W[k + 1:, k + 1:] -= np.outer(Lr[k + 1:, k], W[k, k + 1:])
    assert np.max(np.abs(np.diag(fac[0]) - d)) < 1e-4 * np.max(np.abs(d))
    assert np.max(np.abs(np.tril(fac[0], -1) - np.tril(Lr, -1))) < 1e-4


def test_fp16_split_reports_out_of_range(gpu_pkg):
    """A block column with entries beyond the fp16 pair's range (|x| > 255
    after the 2^8 scale) is reported, not used: TAGS_E_NONFINITE."""
    rng = np.random.default_rng(3)
    N = 300
    A = _sym_matrix(rng, N, 3.0)
    A[200, 5] = A[5, 200] = 4.0e3
    gpu_pkg.lib().tags_gpu_set_quiet(1)
    code, _ = _ldl(gpu_pkg, A[None], 16)
    gpu_pkg.lib().tags_gpu_set_quiet(0)
    assert code == gpu_pkg.E_NONFINITE
    code, fac = _ldl(gpu_pkg, A[None], 3)
    assert code == 0


def _banded_sym(rng, N, zl_m, dominance):
    a = _sym_matrix(rng, N, dominance)
    if zl_m:
        a[zl_m:2 * zl_m, :zl_m] = 0.0
        a[:zl_m, zl_m:2 * zl_m] = 0.0
    return a


@pytest.mark.parametrize("pairs", [0, 1, 2])
@pytest.mark.parametrize("pieces,group", [(3, 6), (16, 6), (16, 5), (16, 4), (16, 3), (16, 2), (16, 1)])
@pytest.mark.parametrize("N,zl_m", [(300, 0), (517, 0), (700, 150), (1000, 300), (1500, 400)])
def test_tensor_core_solve_matches_numpy(gpu_pkg, N, zl_m, pieces, group, pairs):
    """One solve with the tensor-core factors (block-inverse sweeps, the
    diagonal, the zero ZL/ZT band skipped when zl_m > 0; 1 to 6 panels per
    trailing update) against numpy's solve of the same matrices: FP32-level
    agreement on these well-conditioned matrices, partial last blocks included."""
    fn = gpu_pkg.lib().tags_debug_ldl_solve
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_int]
    fn.restype = ctypes.c_int
    rng = np.random.default_rng(N + zl_m)
    mats = np.stack([_banded_sym(rng, N, zl_m, d) for d in (4.0, 3.0)])
    rhs = rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N))
    buf = np.ascontiguousarray(np.transpose(mats, (0, 2, 1))).astype(np.complex128)
    x = rhs.copy()
    gpu_pkg.lib().tags_debug_tc_pairs(int(pairs))
    try:
        code = fn(buf.ctypes.data, x.ctypes.data, N, 2, pieces, zl_m, group)
    finally:
        gpu_pkg.lib().tags_debug_tc_pairs(0)
    assert code == 0, gpu_pkg.last_error()
    for q in range(2):
        ref = np.linalg.solve(mats[q], rhs[q])
        assert np.linalg.norm(x[q] - ref) / np.linalg.norm(ref) < 2e-5, (N, zl_m, q)


@pytest.mark.parametrize("N,zl_m", [(517, 0), (1000, 300), (1500, 400)])
def test_solve_paths_are_identical(gpu_pkg, N, zl_m):
    """The solve block by block (two kernels per 128-row block and sweep), as
    one CTA per sample, and on clusters of 2, 4 and 8 CTAs per sample (rows
    spread over their shared memory) form every sum in the same order:
    identical results, partial last block and the zero ZL/ZT band included."""
    fn = gpu_pkg.lib().tags_debug_ldl_solve
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_int]
    fn.restype = ctypes.c_int
    rng = np.random.default_rng(N + 7 * zl_m)
    mats = np.stack([_banded_sym(rng, N, zl_m, d) for d in (4.0, 3.0)])
    rhs = rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N))
    out = {}
    for path in (0, 1, 2, 4, 8):
        buf = np.ascontiguousarray(np.transpose(mats, (0, 2, 1))).astype(np.complex128)
        x = rhs.copy()
        assert gpu_pkg.lib().tags_debug_solve_path(path) == 0
        try:
            code = fn(buf.ctypes.data, x.ctypes.data, N, 2, 16, zl_m, 4)
        finally:
            gpu_pkg.lib().tags_debug_solve_path(-1)
        assert code == 0, gpu_pkg.last_error()
        out[path] = x
    for path in (1, 2, 4, 8):
        assert np.array_equal(out[path], out[0]), path
