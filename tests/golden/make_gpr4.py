"""Fixture of the transient ground-potential rise on the 1560-segment grid.

The workload is the benchmark's: a 60 x 60 m grid with 12 x 12 meshes and 5
segments per edge (m = 1560 segments, n = 1417 nodes, N = n + 2m = 4537
unknowns), Alipio soil with sigma0 = 1 mS/m, a 1 kA 1.2/50 us current injected
at the centre node, 2048 Laplace samples (nt = 4094, omega_max = 2 pi 10 MHz).

Two steps, on two machines:

    python tests/golden/make_gpr4.py gpu [out.npz]
        On a GPU: the plain FP64 form of this library (FP64 fill, LU with
        partial pivoting) over all 2048 samples, about ten minutes. Writes
        the node potential at the injection node for every sample, all node
        potentials at 16 strided samples, and the GPR from the reference's
        inverse transform (src/auxiliary.c:265-329, restated in oracle/).

    python tests/golden/make_gpr4.py pin [fixture.npz]
        Where the reference sources are present: the same 16 strided samples
        through the reference's own C code (oracle/_ref, cubature tolerance
        1e-11, zsysv), added to the fixture as ref_u_nodes; prints the
        largest relative difference to the plain FP64 values (<= 1e-8 is
        the plain form's parity bar).

The fixture pins the denominator of the mixed form's accuracy claim: the GPU
test tests/test_gpu_gpr.py runs the mixed form over all 2048 samples and
compares its GPR with this one.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

FIXTURE = os.path.join(HERE, "gpr4.npz")
PIN_SAMPLES = 16


def pin_index(ns: int) -> np.ndarray:
    return np.linspace(0, ns - 1, PIN_SAMPLES).astype(int)


def make_gpu(out: str) -> None:
    import __graft_entry__ as entry
    import bench
    from oracle import oracle as O
    pkg = entry.load_package()
    pkg.build()
    elec, img, nodes, s, kappa, inj, centre = bench.workload(pkg)
    m, n = elec.shape[0], nodes.shape[0]
    ns = len(s)
    pidx = pin_index(ns)
    u_centre = np.zeros(ns, np.complex128)
    u_nodes = np.zeros((PIN_SAMPLES, n), np.complex128)
    plan = pkg.Plan(elec, img, nodes, pkg.PLAIN_FP64, max_batch=16)
    chunk = 128
    t0 = time.time()
    try:
        for k0 in range(0, ns, chunk):
            k1 = min(ns, k0 + chunk)
            ie = np.zeros((k1 - k0, n), np.complex128)
            ie[:, centre] = inj[k0:k1]
            sol, info, _ = plan.run(s[k0:k1], kappa[k0:k1], 1.0, ie)
            if np.any(info != 0):
                raise RuntimeError(f"plain FP64 solve failed at samples {k0}..{k1}: {info}")
            u_centre[k0:k1] = sol[:, centre]
            for j, k in enumerate(pidx):
                if k0 <= k < k1:
                    u_nodes[j] = sol[k - k0, :n]
            print(f"samples {k1}/{ns}: {time.time() - t0:.1f} s", flush=True)
    finally:
        plan.close()
    wall = time.time() - t0
    O.build(ref=False)
    port = O.get("port")
    gpr = port.inv_laplace_trans(u_centre, s, bench.TMAX, bench.NT, O.FILTER_NONE)
    np.savez_compressed(out, s=s, kappa=kappa, inj=inj, centre=centre, nt=bench.NT, tmax=bench.TMAX,
                        m=m, n=n, u_centre=u_centre, pin_idx=pidx, u_nodes=u_nodes, gpr=gpr,
                        plain_seconds=wall)
    print(f"plain FP64: {ns} samples in {wall:.1f} s ({ns / wall:.3f} solves/s); wrote {out}")


def make_pin(path: str) -> None:
    import make_golden as MG
    import __graft_entry__ as entry
    import bench
    from oracle import oracle as O
    O.build(ref=True)
    pkg = entry.load_package()
    elec, img, nodes, s, kappa, inj, centre = bench.workload(pkg)
    fx = dict(np.load(path))
    pidx = fx["pin_idx"]
    assert np.array_equal(fx["s"], s) and int(fx["centre"]) == centre
    t0 = time.time()
    sol = MG.sweep_parallel(elec, O.images(elec), nodes, s[pidx], kappa[pidx], centre, inj[pidx], 1e-11)
    n = nodes.shape[0]
    ref_u = sol[:, :n]
    fx["ref_u_nodes"] = ref_u
    fx["ref_tolerance"] = 1e-11
    np.savez_compressed(path, **fx)
    rel = np.max(np.abs(fx["u_nodes"] - ref_u), axis=1) / np.max(np.abs(ref_u), axis=1)
    rel_c = np.abs(fx["u_nodes"][:, centre] - ref_u[:, centre]) / np.abs(ref_u[:, centre])
    print(f"reference build, {len(pidx)} samples in {time.time() - t0:.1f} s")
    print(f"plain FP64 vs reference: node potentials max rel {rel.max():.3e}, injection node {rel_c.max():.3e}")


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else ""
    dest = sys.argv[2] if len(sys.argv) > 2 else FIXTURE
    if what == "gpu":
        make_gpu(dest)
    elif what == "pin":
        make_pin(dest)
    else:
        sys.exit(__doc__)
