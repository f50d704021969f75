"""GPU parity of the impedance fill (calculate_impedances / impedances_images
through the C-ABI) against the reference's golden fixtures and the oracle."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def unpack_lower(packed, m):
    z = np.zeros((m, m), dtype=np.complex128)
    r, c = np.tril_indices(m)
    z[r, c] = packed
    return z


def gpu_fill(pkg, elec, img, s, kappa, mur=1.0, itype=None):
    itype = itype or pkg.INTG_DOUBLE
    m = elec.shape[0]
    zl = np.zeros(m * m, dtype=np.complex128)
    zt = np.zeros(m * m, dtype=np.complex128)
    scaled = itype in (pkg.INTG_DOUBLE, pkg.INTG_SINGLE)
    gamma, ref_t = pkg.medium(s, kappa, mur) if scaled else (0.0, 0.0)
    assert pkg.calculate_impedances(zl, zt, elec, gamma, s, mur, kappa, 0, 1e-6, 1e-6, itype) == 0
    if img is not None:
        assert pkg.impedances_images(zl, zt, elec, img, gamma, s, mur, kappa, 1.0, ref_t, 0, 1e-6, 1e-6, itype) == 0
    return np.tril(zl.reshape(m, m).T), np.tril(zt.reshape(m, m).T)


def elementwise(a, b):
    mask = np.abs(b) > 0
    return float(np.max(np.abs(a[mask] - b[mask]) / np.abs(b[mask])))


# Tolerances: plain-form bar of 1e-8 relative on every entry against the
# reference run at 1e-11 cubature tolerance.
TOL = 1e-8


def test_rod_fill_matches_golden(gpu_pkg):
    pkg = gpu_pkg
    gd = golden("rod_zf.npz")
    e = gd["elec"]
    m = e.shape[0]
    img = pkg.images(e)
    for j, k in enumerate(gd["z_idx"]):
        zl, zt = gpu_fill(pkg, e, img, gd["s"][k], gd["kappa"][k])
        assert elementwise(zl, unpack_lower(gd["zl"][j], m)) < TOL
        assert elementwise(zt, unpack_lower(gd["zt"][j], m)) < TOL


def test_grid_fill_matches_golden(gpu_pkg):
    pkg = gpu_pkg
    gd = golden("grid2.npz")
    e = gd["elec"]
    m = e.shape[0]
    img = pkg.images(e)
    for j, k in enumerate(gd["z_idx"]):
        zl, zt = gpu_fill(pkg, e, img, gd["s"][k], gd["kappa"][k])
        assert elementwise(zl, unpack_lower(gd["zl"][j], m)) < TOL
        assert elementwise(zt, unpack_lower(gd["zt"][j], m)) < TOL


@pytest.mark.parametrize("name", ["mhem", "single", "none"])
def test_other_integration_types_match_golden(gpu_pkg, name):
    pkg = gpu_pkg
    gd = golden("rod_zf.npz")
    e = gd["elec"]
    m = e.shape[0]
    itype = {"mhem": pkg.INTG_MHEM, "single": pkg.INTG_SINGLE, "none": pkg.INTG_NONE}[name]
    zl, zt = gpu_fill(pkg, e, pkg.images(e), complex(gd["type_s"]), complex(gd["type_kappa"]), itype=itype)
    assert elementwise(zl, unpack_lower(gd[name + "_zl"], m)) < TOL
    assert elementwise(zt, unpack_lower(gd[name + "_zt"], m)) < TOL


def test_memory_contract_and_aliasing(gpu_pkg, port):
    """Lower triangle written, upper untouched; images accumulate; zl == zt
    follows the reference's write order."""
    pkg = gpu_pkg
    e, _ = pkg.electrode_grid(3, 3, 4.0, 4.0, 2, 2, 5e-3, -0.6)
    m = e.shape[0]
    img = pkg.images(e)
    s = 1e5 + 2j * np.pi * 2e6
    kappa = 0.005 + s * 12 * pkg.EPS0
    gamma, ref_t = pkg.medium(s, kappa)
    rng = np.random.default_rng(5)
    base = rng.standard_normal(m * m) + 1j * rng.standard_normal(m * m)
    zl, zt = base.copy(), base.copy()
    pkg.calculate_impedances(zl, zt, e, gamma, s, 1.0, kappa)
    upper = np.triu(np.ones((m, m), bool), 1).T.reshape(-1)   # positions i*m+k with k < i
    assert np.array_equal(zl[upper], base[upper]) and np.array_equal(zt[upper], base[upper])
    before = zl.copy()
    pkg.impedances_images(zl, zt, e, img, gamma, s, 1.0, kappa, 1.0, ref_t)
    assert np.array_equal(zl[upper], base[upper])
    ol, ot = base.copy(), base.copy()
    port.calculate_impedances(ol, ot, e, gamma, s, 1.0, kappa, 0, 0.0, 1e-11)
    port.impedances_images(ol, ot, e, img, gamma, s, 1.0, kappa, 1.0, ref_t, 0, 0.0, 1e-11)
    lower = ~upper
    assert elementwise(zl[lower], ol[lower]) < TOL and elementwise(zt[lower], ot[lower]) < TOL
    # aliasing zl == zt
    za = base.copy()
    pkg.calculate_impedances(za, za, e, gamma, s, 1.0, kappa)
    pkg.impedances_images(za, za, e, img, gamma, s, 1.0, kappa, 1.0, ref_t)
    oa = base.copy()
    port.calculate_impedances(oa, oa, e, gamma, s, 1.0, kappa, 0, 0.0, 1e-11)
    port.impedances_images(oa, oa, e, img, gamma, s, 1.0, kappa, 1.0, ref_t, 0, 0.0, 1e-11)
    assert elementwise(za[lower], oa[lower]) < TOL
    assert not np.array_equal(before, zl)


def test_unknown_type_and_degenerate_geometry(gpu_pkg, port):
    pkg = gpu_pkg
    e, _ = pkg.segment_electrode([0, 0, -1], [0, 0, -2], 3, 5e-3)
    m = e.shape[0]
    s, kappa = 2j * np.pi * 1e4, 0.01
    gamma, _ = pkg.medium(s, kappa)
    a = np.zeros(m * m, np.complex128)
    b = np.zeros(m * m, np.complex128)
    o1 = np.zeros(m * m, np.complex128)
    o2 = np.zeros(m * m, np.complex128)
    pkg.lib().tags_gpu_set_quiet(1)
    assert pkg.calculate_impedances(a, b, e, gamma, s, 1.0, kappa, integration_type=9) == -10
    assert port.calculate_impedances(o1, o2, e, gamma, s, 1.0, kappa, 0, 1e-6, 1e-6, 9) == -10
    assert abs(a[0] - o1[0]) < 1e-14 * abs(o1[0]) and np.all(a[1:] == 0)
    # a horizontal conductor lying on the surface coincides with its image:
    # the image integral diverges, reported as an error instead of a number
    h, _ = pkg.segment_electrode([0, 0, 0], [2, 0, 0], 2, 5e-3)
    z1 = np.zeros(4, np.complex128)
    z2 = np.zeros(4, np.complex128)
    with pytest.raises(RuntimeError, match="-104"):
        pkg.impedances_images(z1, z2, h, pkg.images(h), gamma, s, 1.0, kappa, 1.0, 0.5)
    pkg.lib().tags_gpu_set_quiet(0)


def test_full_size_pair_integrals(gpu_pkg, port):
    """60 x 60 m grid (1560 segments): the GPU fill against the oracle's
    tight-tolerance pair integrals on a sample of pairs, adjacent ones included."""
    pkg = gpu_pkg
    e, _ = pkg.electrode_grid(13, 13, 60.0, 60.0, 5, 5, 7e-3, -0.5)
    m = e.shape[0]
    img = pkg.images(e)
    s = 8.1e4 + 2j * np.pi * 4e6
    sig, epsr = pkg.alipio_soil(1e-3, s, 1.26, 0.54, 12)
    kappa = sig + s * epsr * pkg.EPS0
    zl, zt = gpu_fill(pkg, e, img, s, kappa)
    gamma, ref_t = pkg.medium(s, kappa)
    cT = 1.0 / (pkg.FOUR_PI * kappa)
    rng = np.random.default_rng(11)
    pairs = [(i, i + 1) for i in range(0, m - 1, 97)] + [tuple(sorted(rng.choice(m, 2, replace=False))) for _ in range(60)]
    for i, k in pairs:
        d, _, c1 = port.integral(e[i], e[k], gamma, 0, 0.0, 1e-11, pkg.INTG_DOUBLE)
        im, _, c2 = port.integral(e[i], img[k], gamma, 0, 0.0, 1e-11, pkg.INTG_DOUBLE)
        assert c1 == 0 and c2 == 0
        want = cT / (e[i, 9] * e[k, 9]) * d + ref_t * cT / (e[i, 9] * img[k, 9]) * im
        assert abs(zt[k, i] - want) <= TOL * abs(want), (i, k)


def _touching_pairs(e):
    """Lower-triangle pairs (k > i) of segments that share an endpoint."""
    ends = {}
    for j in range(e.shape[0]):
        for pt in (e[j, 0:3], e[j, 3:6]):
            ends.setdefault(tuple(np.round(pt, 9)), []).append(j)
    pairs = set()
    for segs in ends.values():
        for a in segs:
            for b in segs:
                if a != b:
                    pairs.add((max(a, b), min(a, b)))
    return pairs


@pytest.mark.parametrize("with_images", [False, True])
def test_mixed_fill_matches_fp64_fill(gpu_pkg, with_images):
    """60 x 60 m grid (1560 segments), a low and a high Laplace sample of the
    benchmark: the mixed form's fill as its residual sees it (float pairs hi +
    lo), against the FP64 fill. Pairs sharing an endpoint and the diagonal are
    computed in FP64 per sample (Duffy rule, closed-form self term); the
    regular pairs come from the moment expansion (FP64 geometry moments, series
    in float pairs). Both agree with the FP64 fill to ~1e-14."""
    pkg = gpu_pkg
    e, nodes = pkg.electrode_grid(13, 13, 60.0, 60.0, 5, 5, 7e-3, -0.5)
    m = e.shape[0]
    img = pkg.images(e) if with_images else None
    c = np.log(4094.0 ** 2) / 204.7e-6
    s = np.array([c + 2j * np.pi * 2e4, c + 2j * np.pi * 7e6])
    kappa = np.zeros_like(s)
    for j, sk in enumerate(s):
        sig, epsr = pkg.alipio_soil(1e-3, sk, 1.26, 0.54, 12)
        kappa[j] = sig + sk * epsr * pkg.EPS0
    plan = pkg.Plan(e, img, nodes, pkg.MIXED, max_batch=2)
    try:
        zl_m, zt_m = plan.mixed_fill(s, kappa)
    finally:
        plan.close()
    touch = _touching_pairs(e)
    spec = np.zeros((m, m), bool)
    spec[tuple(np.array(sorted(touch)).T)] = True
    spec[np.diag_indices(m)] = True
    low = np.tril(np.ones((m, m), bool))
    regular = low & ~spec
    worst = {}
    for b in range(len(s)):
        zl_p, zt_p = gpu_fill(pkg, e, img, s[b], kappa[b])
        for name, zm, zp in (("zl", zl_m[b], zl_p), ("zt", zt_m[b], zt_p)):
            # both triangles hold the same float pair
            assert np.array_equal(zm, zm.T)
            for part, mask in (("special", spec), ("regular", regular)):
                nz = mask & (np.abs(zp) > 0)
                assert np.all(zm[mask & (zp == 0)] == 0)
                err = float(np.max(np.abs(zm[nz] - zp[nz]) / np.abs(zp[nz])))
                worst[(name, part)] = max(worst.get((name, part), 0.0), err)
    print(f"\nmixed fill vs FP64 fill ({'with' if with_images else 'without'} images), "
          f"{len(touch)} touching pairs + {m} diagonal: " +
          ", ".join(f"{k[0]} {k[1]} {v:.2e}" for k, v in sorted(worst.items())))
    assert worst[("zl", "special")] <= 1e-13 and worst[("zt", "special")] <= 1e-13
    assert worst[("zl", "regular")] <= 1e-12 and worst[("zt", "regular")] <= 1e-12
