"""Replica (one process per GPU) host logic on CPU: two gloo ranks reduce
per-rank step statistics as the reference's cell loop does across MPI ranks
(MAX of rstep_error, sums of iterations), and take the slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, failed_on_rank):
    import torch.distributed as dist

    from pfgpu.replicas import max_over_ranks, reduce_step_stats
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        st = dict(cells=1000 + rank, failed_cells=(3 if rank == failed_on_rank else 0),
                  newton_iterations=10 * (rank + 1), max_newton_iterations=20 + rank, max_substeps=1 + 2 * rank)
        out = reduce_step_stats(st)
        exp_failed = 3 if 0 <= failed_on_rank < world else 0
        assert out["cells"] == sum(1000 + r for r in range(world))
        assert out["failed_cells"] == exp_failed
        assert out["rstep_error"] == (1 if exp_failed else 0)
        assert out["newton_iterations"] == sum(10 * (r + 1) for r in range(world))
        assert out["max_newton_iterations"] == 20 + world - 1
        assert out["max_substeps"] == 1 + 2 * (world - 1)
        assert max_over_ranks(1.5 * (rank + 1)) == 1.5 * world
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("failed_on_rank", [-1, 1])
def test_two_rank_reductions(failed_on_rank):
    import torch.multiprocessing as mp
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    mp.spawn(_worker, args=(2, _free_port(), failed_on_rank), nprocs=2, join=True)
