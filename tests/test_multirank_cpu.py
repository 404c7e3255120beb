"""The N>1 path of bench.py on CPU: two gloo ranks take the max of their step
times over ranks and meet at the barriers; a non-zero rank's reference arm
does no work."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import argparse

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    v = bench.max_over_ranks(1.5 + rank, world)
    args = argparse.Namespace(steps=1, warmup=0, gpus=world)
    bench.run_reference(args, rank, world) if rank else None  # rank != 0: no work
    bench.barrier(world)
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr(v))
    dist.destroy_process_group()


def test_two_rank_max_and_barrier(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    vals = [float(open(tmp_path / f"r{r}.txt").read()) for r in range(2)]
    assert vals == [2.5, 2.5]
    del torch
