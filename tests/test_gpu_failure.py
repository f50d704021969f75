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
