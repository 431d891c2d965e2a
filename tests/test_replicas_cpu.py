"""The multi-GPU path is independent replicas: disjoint run keys per rank and one timing
reduction (slowest rank's time, units of all ranks).  world_size 2 over gloo on the CPU."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from jaxns_gb300.replicas import reduce_timing, replica_keys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        keys = replica_keys(rank, 8)
        ms, units = reduce_timing(10.0 * (rank + 1), 5 + rank)
        np.save(os.path.join(out_dir, f"r{rank}.npy"), np.concatenate([[ms, units], keys.ravel().astype(np.float64)]))
    finally:
        dist.destroy_process_group()


def test_replicas_two_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    # both ranks see the slowest rank's time and the total units
    assert r0[0] == r1[0] == 20.0
    assert r0[1] == r1[1] == 11
    # disjoint keys: rank 1 starts where rank 0 ends
    k0 = r0[2:].reshape(-1, 2)
    k1 = r1[2:].reshape(-1, 2)
    assert not set(map(tuple, k0)) & set(map(tuple, k1))
    from jaxns_gb300.replicas import replica_keys
    np.testing.assert_array_equal(k1, replica_keys(0, 16)[8:].astype(np.float64))


def test_reduce_timing_without_process_group():
    from jaxns_gb300.replicas import reduce_timing
    assert reduce_timing(3.5, 7) == (3.5, 7)
