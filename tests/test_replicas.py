"""Several GPUs run as replicas: each rank its own batch, no collective in the data
path; the whole-job number is the total segments over the slowest rank's time.
Checked with two gloo ranks on the CPU (every GPU run here has one GPU)."""
import json
import os
import socket
import tempfile

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from neuwon_gb300.replicas import aggregate, replica_seed
from neuwon_gb300.workloads import batched_trees


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    trees = batched_trees(8, seed=replica_seed(rank), processes=1, lo=50, hi=300)
    segments = sum(len(t) for t in trees)
    ms = 100.0 + 50.0 * rank                     # rank 1 is the slower one
    dist.barrier()
    res = aggregate(ms, segments, 40, dist)
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"segments": segments, "agg": res, "sizes": [len(t) for t in trees]}, f)
    dist.destroy_process_group()


def test_two_replicas_aggregate_over_gloo():
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank, args=(2, _free_port(), d), nprocs=2, start_method="spawn", join=True)
        r = [json.load(open(os.path.join(d, f"r{k}.json"))) for k in range(2)]
    total = r[0]["segments"] + r[1]["segments"]
    for k in range(2):
        assert r[k]["agg"]["ms"] == 150.0                      # the slowest rank's time
        assert r[k]["agg"]["segments"] == total
        assert abs(r[k]["agg"]["value"] - total * 40 / 0.150) < 1e-6 * total
    assert r[0]["sizes"] != r[1]["sizes"]                      # each rank its own batch


def test_single_process_aggregate_is_local():
    res = aggregate(10.0, 1000, 5)
    assert res == {"ms": 10.0, "segments": 1000, "value": 1000 * 5 / 0.01}
    a = batched_trees(4, seed=replica_seed(3), processes=1, lo=50, hi=100)
    b = batched_trees(4, seed=replica_seed(3), processes=1, lo=50, hi=100)
    assert all(np.array_equal(x.parent, y.parent) for x, y in zip(a, b))


def _exchange_rank(rank, world, port, out_dir):
    from neuwon_gb300.replicas import exchange_rings
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(rank)
    ring = rng.integers(0, 2 ** 32, (10, 4), dtype=np.uint64).astype(np.uint32)   # stale words everywhere
    offset, count = (0, 6) if rank == 0 else (6, 4)
    total = exchange_rings(ring, offset, count, dist)
    np.save(os.path.join(out_dir, f"ring{rank}.npy"), ring)
    np.save(os.path.join(out_dir, f"total{rank}.npy"), total)
    dist.destroy_process_group()


def test_spike_ring_exchange_over_gloo():
    """Two ranks own neurons 0-5 and 6-9; after the exchange both hold every
    neuron's words from its owner."""
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_exchange_rank, args=(2, _free_port(), d), nprocs=2, start_method="spawn", join=True)
        r0, r1 = (np.load(os.path.join(d, f"ring{k}.npy")) for k in range(2))
        t0, t1 = (np.load(os.path.join(d, f"total{k}.npy")) for k in range(2))
    expect = np.concatenate([r0[:6], r1[6:]])
    assert np.array_equal(t0, expect) and np.array_equal(t1, expect)
    assert t0.dtype == np.uint32
