"""The mixed form's failure paths, driven without faulting or hanging the GPU.

* Refinement that does not converge: a cap of one refinement step
  (tags_plan_set_max_steps) leaves every sample unconverged, so each is
  re-solved by the plain FP64 path (partial pivoting).
* A tensor-core wait that runs out: the waits of the factorisation kernels'
  main loops are limited to 1 ns (tags_debug_tc_wait_limit), so the first
  wait not satisfied at once gives up. The kernel raises its error word, lets
  the copies and products it issued finish (those waits keep their 50 ms
  limit), frees its tensor memory and returns; the pass is re-solved in FP64.
Both must return the plain FP64 solution, and the plan must work normally
afterwards."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def _case(pkg, count=16):
    gd = golden("grid2.npz")
    e, nodes = gd["elec"], gd["nodes"]
    idx = np.linspace(0, len(gd["s"]) - 1, count).astype(int)
    s, kappa = gd["s"][idx], gd["kappa"][idx]
    ie = np.zeros((count, nodes.shape[0]), np.complex128)
    ie[:, 0] = gd["inj_s"][idx]
    plain, info, _ = pkg.hem_sweep(e, pkg.images(e), nodes, s, kappa, ie=ie, precision=pkg.PLAIN_FP64)
    assert np.all(info == 0)
    return e, nodes, s, kappa, ie, plain


@pytest.mark.parametrize("graphs", [True, False])
def test_refinement_cap_sends_samples_to_fp64(gpu_pkg, graphs):
    pkg = gpu_pkg
    e, nodes, s, kappa, ie, plain = _case(pkg)
    n = nodes.shape[0]
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=16, graphs=graphs)
    try:
        plan.set_max_steps(1)
        sol, info, st = plan.run(s, kappa, 1.0, ie)
        assert np.all(info == 0)
        assert st.fallbacks == len(s)
        assert rel_err(sol, plain) < 1e-10
        plan.set_max_steps(0)
        sol, info, st = plan.run(s, kappa, 1.0, ie)
        assert np.all(info == 0) and st.fallbacks == 0
        assert rel_err(sol[:, :n], plain[:, :n]) < 1e-6
    finally:
        plan.close()


def test_tensor_core_wait_expiry_falls_back_to_fp64(gpu_pkg):
    pkg = gpu_pkg
    e, nodes, s, kappa, ie, plain = _case(pkg)
    n = nodes.shape[0]
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=16)
    try:
        pkg.lib().tags_gpu_set_quiet(1)
        pkg.debug_tc_wait_limit(1)
        try:
            sol, info, st = plan.run(s, kappa, 1.0, ie)
        finally:
            pkg.debug_tc_wait_limit(0)
            pkg.lib().tags_gpu_set_quiet(0)
        assert "timeout" in pkg.last_error()
        assert np.all(info == 0)
        assert st.fallbacks == len(s)
        assert rel_err(sol, plain) < 1e-10
        # the limit restored, the same plan factorises on the tensor cores again
        sol, info, st = plan.run(s, kappa, 1.0, ie)
        assert np.all(info == 0) and st.fallbacks == 0
        assert rel_err(sol[:, :n], plain[:, :n]) < 1e-6
    finally:
        plan.close()


def test_invalid_samples_are_reported_and_the_plan_recovers(gpu_pkg):
    """A NaN Laplace sample from host memory is refused before any launch
    (TAGS_E_NONFINITE). From device memory it reaches the coefficient kernel,
    which reports it and hands the fill finite coefficients instead, so no
    quadrature order is derived from a NaN; a finite |gamma| beyond 1e5 / m is
    reported the same way (TAGS_E_ARG). The plan keeps its fp16 split and
    solves the next run normally."""
    torch = pytest.importorskip("torch")
    pkg = gpu_pkg
    e, nodes, s, kappa, ie, plain = _case(pkg)
    n, N = nodes.shape[0], plain.shape[1]
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED, max_batch=16)
    pkg.lib().tags_gpu_set_quiet(1)
    try:
        bad = s.copy()
        bad[3] = complex(np.nan, 0.0)
        with pytest.raises(RuntimeError, match=f"failed \\({pkg.E_NONFINITE}\\)"):
            plan.run(bad, kappa, 1.0, ie)
        dev = torch.device("cuda", 0)
        k_d = torch.from_numpy(kappa).to(dev)
        ie_d = torch.from_numpy(ie).to(dev)
        sol_d = torch.empty((len(s), N), dtype=torch.complex128, device=dev)
        info_d = torch.empty((len(s),), dtype=torch.int32, device=dev)
        for value, code in ((complex(np.nan, 0.0), pkg.E_NONFINITE), (complex(0.0, 1e20), pkg.E_ARG)):
            bad = s.copy()
            bad[5] = value
            s_d = torch.from_numpy(bad).to(dev)
            with pytest.raises(RuntimeError, match=f"failed \\({code}\\)"):
                plan.run_device(s_d.data_ptr(), k_d.data_ptr(), len(s), 1.0, ie_d.data_ptr(), 0, sol_d.data_ptr(),
                                info_d.data_ptr())
            torch.cuda.synchronize()
    finally:
        pkg.lib().tags_gpu_set_quiet(0)
    try:
        sol, info, st = plan.run(s, kappa, 1.0, ie)
        assert np.all(info == 0) and st.fallbacks == 0
        assert st.split == 16                       # the NaN did not switch the plan to bf16 pieces
        assert rel_err(sol[:, :n], plain[:, :n]) < 1e-6
    finally:
        plan.close()


def test_memory_budget_below_one_sample_reports_nomem(gpu_pkg):
    """With the process-wide memory budget below what one sample needs, a new
    plan fails with TAGS_E_NOMEM (nothing is left allocated); with the budget
    lifted the same plan builds and solves."""
    pkg = gpu_pkg
    e, nodes, s, kappa, ie, plain = _case(pkg, 4)
    n = nodes.shape[0]
    pkg.lib().tags_gpu_set_quiet(1)
    pkg.set_memory_budget(1 << 20)
    try:
        with pytest.raises(RuntimeError, match=f"failed \\({pkg.E_NOMEM}\\)"):
            pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED)
    finally:
        pkg.set_memory_budget(0)
        pkg.lib().tags_gpu_set_quiet(0)
    plan = pkg.Plan(e, pkg.images(e), nodes, pkg.MIXED)
    try:
        sol, info, st = plan.run(s, kappa, 1.0, ie)
        assert np.all(info == 0)
        assert rel_err(sol[:, :n], plain[:, :n]) < 1e-6
    finally:
        plan.close()
