"""The bench's N>1 path: one replica per rank, job time = slowest rank (gloo, 2 ranks, CPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as td  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_env()
        assert (w, r) == (world, rank)
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, td, "cpu")
        out[rank] = (ms, bench.replica_throughput(1000, w, ms))
        td.barrier()
    finally:
        td.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] == pytest.approx(2 * 1000 / 0.015)


def test_single_process_is_its_own_max():
    assert bench.max_over_ranks(3.5) == 3.5


def _shard_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import ktruss_gb300 as kt

        n, u, v, off = kt.gen_batch(8, 64, 400, bench.shard_seed(5, rank))
        sizes = torch.tensor([n, len(u)], dtype=torch.int64)
        gathered = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
        td.all_gather(gathered, sizes)
        ms = bench.max_over_ranks(3.0 * (rank + 1), td, "cpu")
        out[rank] = ([g.tolist() for g in gathered], ms)
    finally:
        td.destroy_process_group()


def test_batch_shards_are_distinct_graphs_per_rank():
    """Under torchrun each rank decomposes its own shard of the batch (no exchange on the data
    path): rank 0 keeps the workload's seed, the others get their own graphs."""
    import ktruss_gb300 as kt

    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_shard_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    sizes0, ms0 = res[0]
    assert sizes0 == res[1][0] and ms0 == res[1][1] == 6.0
    assert sizes0[0] != sizes0[1]  # the two shards are different graphs
    n, u, _, _ = kt.gen_batch(8, 64, 400, 5)
    assert sizes0[0] == [n, len(u)]
