"""Launch-configuration autotuner for the batched step kernel.

For one network and a sample of its cells, times every configuration the
library accepts -- threads per block (32..256), resident blocks per SM
(1..4), Jacobian in shared or local memory -- with CUDA events on the
launching stream, restoring the sample before each launch, and installs the
fastest with pf_network_set_launch.  Results are cached per (GPU, network
shape) in autotune_cache.json next to this file.
"""
from __future__ import annotations

import hashlib
import json
import os

from . import abi
from .network import CellState

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "autotune_cache.json")
MUTABLE = ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_volfrac",
           "mnrl_rate", "status", "newton_its", "num_substeps", "total_sorb", "ionx_ref_sorbed", "ln_act_h2o")


def network_key(eng, device_name: str | None = None) -> str:
    net = eng.net
    if device_name is None:
        import torch
        device_name = torch.cuda.get_device_name()
    h = hashlib.sha1()
    for a in (net.sec_nspec, net.sec_spec, net.mnrl_nspec, net.mnrl_spec):
        h.update(a.tobytes())
    return "%s|n%d|s%d|m%d|%s" % (device_name, net.ncomp, net.nsec, net.nmnrl, h.hexdigest()[:12])


def event_timer(fn) -> float:
    """Milliseconds of fn() between two CUDA events on the current stream."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def candidates(quick: bool = False):
    """One lane per cell: threads per block x blocks per SM x Jacobian in
    shared or local memory; a group of 4 or 8 lanes per cell: threads per
    block x blocks per SM (the library refuses what it cannot run)."""
    tpbs = (64, 128, 192, 256) if quick else range(32, 257, 32)
    bpss = (1, 2, 4) if quick else (1, 2, 3, 4)
    for js in (1, 0):
        for tpb in tpbs:
            for bps in bpss:
                yield dict(threads_per_block=tpb, blocks_per_sm=bps, jac_in_shared=js, lanes_per_cell=1)
    for g in (2, 4, 8):
        for tpb in (64, 128, 192, 256):
            for bps in (1, 2, 4):
                yield dict(threads_per_block=tpb, blocks_per_sm=bps, jac_in_shared=0, lanes_per_cell=g)


def tune(eng, state: CellState, dt: float, max_cells: int = 65536, reps: int = 2, use_cache: bool = True,
         verbose: bool = False, quick: bool = False, cost_order: bool = False, timer=event_timer,
         device_name: str | None = None, cache_path: str | None = None):
    """cost_order: time every configuration with the work queue ordered by a
    first step's Newton counts (longest cells first), as a time loop that
    orders by the previous step runs; without it the sample's tail of slow
    cells favours configurations that are only better on unordered queues.
    timer(fn) returns the milliseconds of one launch (CUDA events by
    default); device_name and cache_path default to the current GPU's name
    and the cache file next to this module."""
    import torch
    key = network_key(eng, device_name)
    cache_path = cache_path or CACHE
    cache = {}
    if use_cache and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
        except Exception:
            cache = {}
    if use_cache and key in cache:
        cfg = cache[key]["best"]
        if eng.set_launch_config(**cfg) == abi.PF_OK:
            return cfg, cache[key]["table"]
    n = min(state.ncells, max_cells)
    sample = state.subset(torch.arange(n, device=state.a["porosity"].device))
    pristine = {k: sample.a[k].clone() for k in MUTABLE if k in sample.a}
    order = None
    if cost_order:
        eng.rstep(sample, dt, stats=False)
        order = torch.argsort(sample.a["newton_its"].to(torch.int64), descending=True)
    table = []
    for cfg in candidates(quick):
        if eng.set_launch_config(**cfg) != abi.PF_OK:
            continue
        best = None
        for _ in range(reps + 1):
            for k, v in pristine.items():
                sample.a[k].copy_(v)
            ms = timer(lambda: eng.rstep(sample, dt, stats=False, order=order))
            best = ms if best is None else min(best, ms)
        table.append(dict(cfg, ms=best))
        if verbose:
            print(cfg, "%.3f ms" % best)
    if not table:
        raise RuntimeError("pf_network_set_launch accepted no candidate configuration for this network")
    table.sort(key=lambda r: r["ms"])
    keys = ("threads_per_block", "blocks_per_sm", "jac_in_shared", "lanes_per_cell")
    top = {k: table[0][k] for k in keys}
    # the library keeps the last one-lane configuration for the adjoint:
    # install the best one first, then the overall best
    lane1 = [r for r in table if r["lanes_per_cell"] <= 1]
    if lane1:
        eng.set_launch_config(**{k: lane1[0][k] for k in keys})
    eng.set_launch_config(**top)
    for k, v in pristine.items():
        sample.a[k].copy_(v)
    cache[key] = {"best": top, "table": table[:12], "cells": n, "cost_order": bool(cost_order)}
    try:
        json.dump(cache, open(cache_path, "w"), indent=1)
    except OSError:
        pass
    return top, table
