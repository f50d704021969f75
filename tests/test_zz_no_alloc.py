"""The solve entry point for callers that cannot allocate device memory.

Runs last (file name) so that a stop-at-first-failure run has already run every
other test. It calls tags_solve_immittance_noalloc through the C-ABI on device
buffers owned by the caller (here torch tensors) and checks two calls in a row
against the allocating solve_immittance, with the solve tolerance of the other
parity tests."""
import ctypes

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def _system(pkg, k):
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    img = pkg.images(e)
    m, n = e.shape[0], nodes.shape[0]
    N = n + 2 * m
    s, kappa = gd["s"][k], gd["kappa"][k]
    gamma, ref_t = pkg.medium(s, kappa)
    zl = np.zeros(m * m, np.complex128)
    zt = np.zeros(m * m, np.complex128)
    pkg.calculate_impedances(zl, zt, e, gamma, s, 1.0, kappa)
    pkg.impedances_images(zl, zt, e, img, gamma, s, 1.0, kappa, 1.0, ref_t)
    wg = np.zeros(N * N, np.complex128)
    assert pkg.fill_incidence_imm(wg, e, nodes) == 0
    pkg.fill_impedance_imm(wg, zl, zt, m, n)
    ie = np.zeros(N, np.complex128)
    ie[0] = gd["inj_s"][k]
    return wg, ie, m, n


def test_noalloc_solve_matches_allocating_solve(gpu_pkg):
    torch = pytest.importorskip("torch")
    pkg = gpu_pkg
    L = pkg.lib()
    fn = L.tags_solve_immittance_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    for k in (5, 900):                       # two calls in a row share the scratch
        wg, ie, m, n = _system(pkg, k)
        d_wg = torch.from_numpy(wg.copy()).to(dev)
        d_ie = torch.from_numpy(ie.copy()).to(dev)
        torch.cuda.synchronize()
        assert fn(d_wg.data_ptr(), d_ie.data_ptr(), m, n, None) == 0
        got = d_ie.cpu().numpy()
        want = ie.copy()
        assert pkg.solve_immittance(wg.copy(), want, m, n) == 0
        assert rel_err(got, want) < 1e-10


def test_noalloc_rejects_oversize_and_singular(gpu_pkg):
    torch = pytest.importorskip("torch")
    pkg = gpu_pkg
    fn = pkg.lib().tags_solve_immittance_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    pkg.lib().tags_gpu_set_quiet(1)
    dummy = torch.zeros(4, dtype=torch.complex128, device="cuda")
    assert fn(dummy.data_ptr(), dummy.data_ptr(), 20000, 1, None) == pkg.E_ARG
    assert "exceed" in pkg.last_error()
    w = torch.zeros(9, dtype=torch.complex128, device="cuda")
    w[0] = 1.0
    x = torch.ones(3, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    assert fn(w.data_ptr(), x.data_ptr(), 1, 1, None) > 0
    assert torch.all(x == 1).item()
    pkg.lib().tags_gpu_set_quiet(0)
