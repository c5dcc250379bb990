"""The N-GPU path as independent replicas, on CPU with gloo (world size 2).

Each rank measures its round-robin shard of a list of small boxes (the oracle's
P(k) stands in for the GPU estimator, which is replicated unchanged per rank);
rank 0 gathers every box exactly once and the results equal a serial run of
all boxes.  The max-over-ranks timing and the whole-job throughput are checked
with planted per-rank times.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from pbi4_gb300 import replicas

N_BOXES = 5


def _measure(i):
    from oracle import pbi4_oracle as O
    from pbi4_gb300 import synthetic
    pos = synthetic.uniform_box(300 + 50 * i, seed=40 + i)
    p = dict(grid=16, box=1000.0, interpolation=3, interlacing=bool(i % 2), kbin=1.0, kcenter=1.0)
    npart, dcl = O.assign_grid(pos, p)
    d = O.compute_density(npart, dcl, p)
    out = O.measure_pk(16, 1000.0, 1.0, 1.0, 8, d, d)
    return np.asarray(out[1], dtype=np.float64)


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    w, r, _ = replicas.init("gloo")
    assert (w, r) == (world, rank)
    res = replicas.run_boxes(N_BOXES, _measure)
    tmax = replicas.max_over_ranks(1.0 + rank)        # planted: rank r took 1 + r seconds
    nsum = replicas.sum_over_ranks(len(replicas.shard(N_BOXES, w, r)))
    replicas.barrier()
    if rank == 0:
        np.savez(os.path.join(out_dir, "r0.npz"), keys=np.array(sorted(res)),
                 vals=np.stack([res[k] for k in sorted(res)]), tmax=tmax, nsum=nsum)
    else:
        assert res is None
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_round_robin():
    assert replicas.shard(5, 2, 0) == [0, 2, 4]
    assert replicas.shard(5, 2, 1) == [1, 3]
    assert replicas.shard(1, 4, 3) == []
    with pytest.raises(ValueError):
        replicas.shard(5, 2, 2)
    assert replicas.throughput(8, 2.0) == 4.0
    with pytest.raises(ValueError):
        replicas.throughput(8, 0.0)


def test_single_process_is_identity():
    res = replicas.run_boxes(2, lambda i: i * 10)
    assert res == {0: 0, 1: 10}
    assert replicas.max_over_ranks(3.5) == 3.5


def test_two_rank_gloo_replicas(tmp_path):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    z = np.load(tmp_path / "r0.npz")
    assert list(z["keys"]) == list(range(N_BOXES))
    serial = np.stack([_measure(i) for i in range(N_BOXES)])
    np.testing.assert_array_equal(z["vals"], serial)
    assert float(z["tmax"]) == 2.0
    assert float(z["nsum"]) == N_BOXES
