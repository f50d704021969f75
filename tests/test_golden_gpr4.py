"""The benchmark-grid GPR fixture (tests/golden/gpr4.npz) against the
reference: its plain FP64 values at 16 strided samples equal the reference's
own C code run at cubature tolerance 1e-11 (tests/golden/make_gpr4.py pin), and
its GPR is the reference's inverse transform (restated in the oracle) of its
node potential at the injection node. CPU only."""
import numpy as np

from conftest import golden, rel_err


def test_gpr4_fixture_is_pinned_to_the_reference_build():
    fx = golden("gpr4.npz")
    assert "ref_u_nodes" in fx.files, "fixture not pinned: run tests/golden/make_gpr4.py pin"
    assert float(fx["ref_tolerance"]) <= 1e-11
    err = rel_err(fx["u_nodes"], fx["ref_u_nodes"])
    assert err <= 1e-8, err
    c = int(fx["centre"])
    inj = np.abs(fx["u_nodes"][:, c] - fx["ref_u_nodes"][:, c]) / np.abs(fx["ref_u_nodes"][:, c])
    assert inj.max() <= 1e-8
    assert np.array_equal(fx["u_nodes"][:, c], fx["u_centre"][fx["pin_idx"]])


def test_gpr4_fixture_gpr_is_the_reference_transform(port):
    fx = golden("gpr4.npz")
    gpr = port.inv_laplace_trans(fx["u_centre"], fx["s"], float(fx["tmax"]), int(fx["nt"]))
    assert np.array_equal(gpr, fx["gpr"])
