"""GPU parity of the post-processing path (src/electrode.c:434-668 and the
closed-form mHEM ground potential of examples/visacro57emc01.c:406-430):
the four drop-ins and the three batched entry points against the reference's
own outputs (tests/golden/fields.npz, written by tests/golden/make_golden.py)
and against the oracle at tight cubature tolerance.

Tolerance: 1e-9 of the largest magnitude of each compared vector (the GPU
rules integrate to ~1e-12; the fixtures were made at 1e-11, the nested path
voltage at 1e-10, and path voltages are compared at 1e-8)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _close(got, want, axis=None):
    got = np.asarray(got)
    want = np.asarray(want)
    scale = np.max(np.abs(want), axis=axis, keepdims=axis is not None)
    err = np.abs(got - want) / np.maximum(scale, 1e-300)
    return float(np.max(err))


def _field_case():
    gd = golden("fields.npz")
    return {k: gd[k] for k in gd.files}


def test_fields_batch_matches_reference_fixture(gpu_pkg):
    pkg = gpu_pkg
    d = _field_case()
    before = pkg.launch_count()
    out = pkg.fields_batch(d["points"], d["elec"], d["il"], d["it"], d["gamma"], d["kappa"])
    assert pkg.launch_count() > before
    assert out["status"] == 0
    s = d["s"][:, None, None, None]
    full = out["efield"] - s * out["vecpot"]
    assert _close(out["pot"], d["pot"], axis=(1, 2)) <= TOL
    assert _close(out["vecpot"], d["vecpot"], axis=(1, 2, 3)) <= TOL
    assert _close(full, d["efield"], axis=(1, 2, 3)) <= TOL
    # s = 0 and a nonzero ve: the reference adds the conservative part to ve
    assert _close(out["efield"] + d["ve0"], d["efield_s0"], axis=(1, 2, 3)) <= TOL


def test_dropins_match_reference_fixture(gpu_pkg):
    pkg = gpu_pkg
    d = _field_case()
    e, pts = d["elec"], d["points"]
    for k in (0, 2):
        for r in range(d["il"].shape[1]):
            for p in (0, 4, 5, 6):
                u = pkg.electric_potential(pts[p], e, d["it"][k, r], d["gamma"][k], d["kappa"][k])
                assert abs(u - d["pot"][k, p, r]) <= TOL * abs(d["pot"][k, p, r])
                va = pkg.magnetic_potential(pts[p], e, d["il"][k, r], d["gamma"][k])
                assert _close(va, d["vecpot"][k, p, r]) <= TOL
                ve = pkg.electric_field(pts[p], e, d["il"][k, r], d["it"][k, r], d["gamma"][k], d["s"][k],
                                        d["kappa"][k], ve=[9.0, 9.0, 9.0])          # overwritten when |s| > 0
                assert _close(ve, d["efield"][k, p, r]) <= TOL
                ve0 = pkg.electric_field(pts[p], e, d["il"][k, r], d["it"][k, r], d["gamma"][k], 0.0, d["kappa"][k],
                                         ve=d["ve0"])                                 # added to when s = 0
                assert _close(ve0, d["efield_s0"][k, p, r]) <= TOL
            for l in range(d["paths"].shape[0]):
                v = pkg.voltage(d["paths"][l, :3], d["paths"][l, 3:], e, d["il"][k, r], d["it"][k, r], d["gamma"][k],
                                d["s"][k], d["kappa"][k])
                assert abs(v - d["voltage"][k, l, r]) <= 1e-8 * abs(d["voltage"][k, l, r])


def test_voltage_batch_matches_reference_fixture(gpu_pkg):
    pkg = gpu_pkg
    d = _field_case()
    v = pkg.voltage_batch(d["paths"], d["elec"], d["il"], d["it"], d["gamma"], d["s"], d["kappa"])
    assert v.shape == d["voltage"].shape
    assert _close(v, d["voltage"], axis=(1, 2)) <= 1e-8


def test_gpd_mhem_matches_oracle(gpu_pkg, port):
    pkg = gpu_pkg
    d = _field_case()
    rng = np.random.default_rng(3)
    pts = np.column_stack([rng.uniform(-6, 10, 40), rng.uniform(-6, 10, 40), np.zeros(40)])
    got = pkg.gpd_mhem_batch(pts, d["elec"], d["it"], d["gamma"], d["kappa"])
    for k in range(3):
        want = port.gpd_mhem(pts, d["elec"], d["it"][k].T, d["gamma"][k], d["kappa"][k])
        assert _close(got[k], want) <= 1e-12


def test_fields_many_samples_near_points_vs_oracle(gpu_pkg, port):
    """A sweep of 40 samples (60 Hz to 10 MHz, more than one warp of samples)
    at points from 1e-3 of an electrode length to far away, on a rod's axis
    beyond its tip and near a junction, against the oracle at 1e-12."""
    pkg = gpu_pkg
    from oracle import oracle as O
    grid, _ = pkg.electrode_grid(3, 3, 6.0, 6.0, 2, 2, 7e-3, -0.6)
    rod, _ = pkg.segment_electrode([6.0, 6.0, -0.6], [6.0, 6.0, -3.6], 2, 9e-3)
    e = np.vstack([grid, rod])
    m = e.shape[0]
    f = np.logspace(np.log10(60.0), 7, 40)
    s = 2j * np.pi * f + 1e3
    kappa = 1.0 / 150.0 + s * 9.0 * O.EPS0
    gamma = np.array([O.medium(a, b)[0] for a, b in zip(s, kappa)])
    rng = np.random.default_rng(21)
    il = rng.normal(size=(40, 1, m)) + 1j * rng.normal(size=(40, 1, m))
    it = rng.normal(size=(40, 1, m)) + 1j * rng.normal(size=(40, 1, m))
    pts = np.array([[1.5, 0.0015, -0.6], [1.5, 0.0, -0.603], [0.0, 0.0, -0.6 + 0.02], [6.0, 6.0, -3.7],
                    [6.0, 6.0, -5.0], [3.0, 2.9, -0.59], [2.0, 2.0, 0.0], [40.0, -30.0, 0.0]])
    out = pkg.fields_batch(pts, e, il, it, gamma, kappa)
    assert out["status"] == 0
    for k in (0, 13, 27, 39):
        for p in range(pts.shape[0]):
            u = port.electric_potential(pts[p], e, it[k, 0], gamma[k], kappa[k], 0, 1e-14, 1e-12)
            va = port.magnetic_potential(pts[p], e, il[k, 0], gamma[k], 1.0, 0, 1e-14, 1e-12)
            ve, _ = port.electric_field(pts[p], e, il[k, 0], it[k, 0], gamma[k], 0.0, kappa[k], 1.0, 0, 1e-14, 1e-12)
            assert abs(out["pot"][k, p, 0] - u) <= TOL * abs(u), (k, p)
            assert _close(out["vecpot"][k, p, 0], va) <= TOL, (k, p)
            assert _close(out["efield"][k, p, 0], ve) <= 1e-8, (k, p)


def test_point_on_electrode_is_flagged(gpu_pkg):
    pkg = gpu_pkg
    d = _field_case()
    e = d["elec"]
    on = e[0, 6:9].copy()                      # the midpoint of the first segment
    pkg.lib().tags_gpu_set_quiet(1)
    try:
        out = pkg.fields_batch(np.array([on, [9.0, 9.0, 0.0]]), e, d["il"], d["it"], d["gamma"], d["kappa"])
    finally:
        pkg.lib().tags_gpu_set_quiet(0)
    assert out["status"] == pkg.E_GEOMETRY
    assert np.all(np.isnan(out["pot"][:, 0]))
    assert np.all(np.isfinite(out["pot"][:, 1]))


def test_empty_and_zero_currents(gpu_pkg):
    pkg = gpu_pkg
    d = _field_case()
    z = np.zeros_like(d["il"])
    out = pkg.fields_batch(d["points"], d["elec"], z, z, d["gamma"], d["kappa"])
    assert not np.any(out["pot"]) and not np.any(out["vecpot"]) and not np.any(out["efield"])
    out = pkg.fields_batch(d["points"], d["elec"][:0], z[:, :, :0], z[:, :, :0], d["gamma"], d["kappa"])
    assert out["pot"].shape == (3, d["points"].shape[0], 2) and not np.any(out["pot"])


def test_more_injections_than_one_pass(gpu_pkg, port):
    """Six injections (the kernel takes four per pass over the electrodes) and
    a single sample: every injection against the oracle."""
    pkg = gpu_pkg
    d = _field_case()
    rng = np.random.default_rng(8)
    m = d["elec"].shape[0]
    il = rng.normal(size=(1, 6, m)) + 1j * rng.normal(size=(1, 6, m))
    it = rng.normal(size=(1, 6, m)) + 1j * rng.normal(size=(1, 6, m))
    pts = d["points"][:4]
    out = pkg.fields_batch(pts, d["elec"], il, it, d["gamma"][1:2], d["kappa"][1:2])
    for r in range(6):
        for p in range(pts.shape[0]):
            u = port.electric_potential(pts[p], d["elec"], it[0, r], d["gamma"][1], d["kappa"][1], 0, 1e-14, 1e-12)
            va = port.magnetic_potential(pts[p], d["elec"], il[0, r], d["gamma"][1], 1.0, 0, 1e-14, 1e-12)
            assert abs(out["pot"][0, p, r] - u) <= TOL * abs(u)
            assert _close(out["vecpot"][0, p, r], va) <= TOL
