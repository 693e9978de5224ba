"""Replica runs: one process per GPU, each stepping its own cells.

The operator-split reaction step is cell-local; the reference's cell loop has
exactly two cross-cell operations, the MAX reduction of rstep_error over the
ranks and the sums of Newton iterations
(src/pflotran/pmc_subsurface_osrt.F90:367-381).  With the cells of a domain
split over GPUs, each rank runs pf_rstep on its own cells and these helpers
perform those reductions over a torch.distributed process group (NCCL between
GPUs, gloo on the host).  There is no data-path collective.
"""
from __future__ import annotations

STAT_SUMS = ("cells", "failed_cells", "newton_iterations")
STAT_MAXS = ("max_newton_iterations", "max_substeps")


def reduce_step_stats(stats: dict, group=None, device="cpu") -> dict:
    """Sum cells / failures / iterations and take the maxima over the ranks;
    adds rstep_error = 1 when any rank had a failed cell (the MPI_Allreduce
    MAX of the reference loop)."""
    import torch
    import torch.distributed as dist
    sums = torch.tensor([int(stats[k]) for k in STAT_SUMS], dtype=torch.int64, device=device)
    maxs = torch.tensor([int(stats[k]) for k in STAT_MAXS], dtype=torch.int64, device=device)
    dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(maxs, op=dist.ReduceOp.MAX, group=group)
    out = {k: int(v) for k, v in zip(STAT_SUMS, sums.tolist())}
    out.update({k: int(v) for k, v in zip(STAT_MAXS, maxs.tolist())})
    out["rstep_error"] = 1 if out["failed_cells"] > 0 else 0
    return out


def max_over_ranks(value: float, group=None, device="cpu") -> float:
    """The slowest rank's value (timed regions of replica runs)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
