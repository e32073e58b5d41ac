"""The N>1 path of bench.py on CPU with the gloo backend (world size 2): each
rank runs its own ensemble, the job time is the max over ranks and the value is
the units of all ranks over that time.  The GPU run uses the same functions
over NCCL."""

import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = [120.0, 80.0][rank]
    job_ms = bench.max_over_ranks(local_ms, dist, "cpu")
    out[rank] = (job_ms, bench.whole_job_rate(1_000_000, world, job_ms))
    # each rank's ensemble is seeded by its rank: independent replicas
    L0, _ = bench.ensemble_config(seed=bench.SEED + rank)
    out[10 + rank] = int(L0.sum())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation():
    port = free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 120.0
    assert res[0][1] == pytest.approx(2_000_000 / 0.12)
    assert res[10] != res[11]
