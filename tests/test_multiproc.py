"""Multi-process path on CPU (gloo, world size 2): sample sharding and the
host-side gather before the inverse Laplace transform. No GPU is involved."""
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


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as entry
    pkg = entry.load_package()
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ns = 1023
    idx = pkg.shard_samples(ns, rank, world)
    # stand-in per-sample result: a function of the sample index only
    vals = np.stack([idx * 1.0 + 0.5j, -idx * 2.0 + 0j], axis=1)
    full = pkg.gather_samples(vals, ns)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_samples_gather_in_order(tmp_path):
    world = 2
    out = str(tmp_path / "gathered.npy")
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    full = np.load(out)
    k = np.arange(1023)
    assert full.shape == (1023, 2)
    assert np.array_equal(full[:, 0], k * 1.0 + 0.5j) and np.array_equal(full[:, 1], -k * 2.0 + 0j)


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
