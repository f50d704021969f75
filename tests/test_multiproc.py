"""Multi-process path on CPU (gloo, world size 2): sample sharding, per-rank
solves and the host-side gather before the inverse Laplace transform. No GPU
is involved: the oracle solves each rank's share."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rod_transient(pkg, orc):
    """The 3 m rod (10 segments) under a 1.2/50 us current: nt = 126 time
    steps over 20 us, 64 Laplace samples, soil 100 ohm m, eps_r 10."""
    elec, nodes = pkg.segment_electrode([0.0, 0.0, 0.0], [0.0, 0.0, -3.0], 10, 7e-3)
    nt, tmax = 126, 20e-6
    t = np.linspace(0.0, tmax, nt)
    i_t = 1000.0 * 1.037 * (np.exp(-t / 68.2e-6) - np.exp(-t / 0.405e-6))
    inj, s = orc.laplace_trans(i_t, tmax)
    kappa = 1.0 / 100.0 + s * 10.0 * pkg.EPS0
    return elec, pkg.images(elec), nodes, s, kappa, inj, nt, tmax


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    orc = entry.load_oracle().get("port")
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    elec, img, nodes, s, kappa, inj, nt, tmax = _rod_transient(pkg, orc)
    ns = len(s)
    idx = pkg.shard_samples(ns, rank, world)
    # this rank's share of the per-sample solves (the oracle stands in for one
    # GPU's plan), then the only exchange: U at the injection node to rank 0
    sol, info = orc.hem_sweep(elec, img, nodes, s[idx], kappa[idx], 0, inj[idx], req_abs=1e-10, req_rel=1e-8,
                              threads=1)
    assert np.all(info == 0)
    vals = np.stack([sol[:, 0], idx.astype(np.complex128)], axis=1)
    full = pkg.gather_samples(vals, ns)
    if rank == 0:
        gpr = orc.inv_laplace_trans(full[:, 0], s, tmax, nt)
        np.savez(out_path, u0=full[:, 0], order=full[:, 1].real, gpr=gpr)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_solves_gather_in_order(tmp_path):
    """World size 2: each rank solves its strided share of the rod's Laplace
    samples, rank 0 gathers U(s) and inverts the transform; the result equals
    one process solving every sample."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    orc = entry.load_oracle().get("port")
    world = 2
    out = str(tmp_path / "gathered.npz")
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    got = np.load(out)
    elec, img, nodes, s, kappa, inj, nt, tmax = _rod_transient(pkg, orc)
    sol, info = orc.hem_sweep(elec, img, nodes, s, kappa, 0, inj, req_abs=1e-10, req_rel=1e-8, threads=1)
    assert np.array_equal(got["order"], np.arange(len(s)))
    assert np.array_equal(got["u0"], sol[:, 0])
    assert np.array_equal(got["gpr"], orc.inv_laplace_trans(sol[:, 0], s, tmax, nt))


def test_shards_partition_the_samples():
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    for ns, world in ((2048, 8), (1024, 3), (5, 4)):
        parts = [pkg.shard_samples(ns, r, world) for r in range(world)]
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(ns))
    with pytest.raises(ValueError):
        pkg.shard_samples(10, 2, 2)
