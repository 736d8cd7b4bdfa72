"""The multi-rank path of bench.py on CPU, world_size 2 over gloo.

Paths are independent, so N GPUs run N replicas of the workload (weak
scaling) with no data-path collective: each rank's replica has its own seed,
the job time is the maximum over ranks (an all-reduce of one number) and
the value is world * units / that time.  Here each rank prices its replica
with the oracle on the CPU and the helpers bench.py uses on the GPU run over
gloo.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle as O

    seed = bench.replica_seed(rank)
    paths = O.gbm(100.0, 0.05, 0.2, 1.0, 12, 500, seed=seed, threads=1)
    # rank 1 pretends to be the slow one: the job time must be its time
    t = 0.25 if rank == 1 else 0.1
    t_max = bench.rank_max(t, world, "cpu")
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([[t_max], paths[:, -1]]))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_and_max_over_ranks_gloo(oracle, tmp_path):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r0 = np.load(tmp_path / "rank0.npy")
    r1 = np.load(tmp_path / "rank1.npy")
    # every rank sees the slowest rank's time
    assert r0[0] == r1[0] == 0.25
    # each replica is exactly the single-process run with its own seed
    sys.path.insert(0, ROOT)
    import bench

    for rank, r in enumerate((r0, r1)):
        want = oracle.gbm(100.0, 0.05, 0.2, 1.0, 12, 500, seed=bench.replica_seed(rank), threads=1)[:, -1]
        assert np.array_equal(r[1:], want)
    # replicas are independent draws, not copies
    assert not np.array_equal(r0[1:], r1[1:])


def test_reference_arm_prints_on_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup = 1, 0

    bench.run_reference(A(), 1, 2)  # a non-zero rank does no work and prints nothing
    assert capsys.readouterr().out == ""
