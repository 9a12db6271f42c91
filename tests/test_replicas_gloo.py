"""The multi-rank path of bench.py on CPU: two gloo ranks, each standing for
one replica, reduce their timings (max over ranks) and work (sum over
ranks) the way the GPU run does under torchrun."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mx, sm = bench.replica_reduce([1.0 + rank, 10.0 - rank, 0.5 * rank], [100.0 * (rank + 1), 7.0])
        with open(os.path.join(out, f"r{rank}.txt"), "w") as f:
            f.write(repr((mx, sm)))
    finally:
        dist.destroy_process_group()


def test_replica_reduce_two_ranks(tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        mx, sm = eval((tmp_path / f"r{r}.txt").read_text())
        assert mx == [2.0, 10.0, 0.5]
        assert sm == [300.0, 14.0]


def test_replica_reduce_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_reduce([3.0], [4.0, 5.0]) == ([3.0], [4.0, 5.0])
