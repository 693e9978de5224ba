"""Parity on the benchmark's own inputs.

The throughput figures of bench.py come from two workloads: the 12/40/6
network over 1,000,000 cells (network seed 12, cells seed 2026, dt = 1 day),
whose timed step is the second operator-split step (its work queue in cell
order; the first step's Newton order is measured beside it and gives the
same results), and the eight heterogeneous
networks (ncomp 4 ... 24, network seeds 3000 + ncomp, per-cell dt
log-uniform in [1 h, 30 d]).  These tests build those states exactly as
bench.py does (bench.build_state, bench.build_c3: the same generator calls,
device equilibration and auxvar sequence), run the step on the GPU over every
cell, download the inputs and results, and run the oracle on a sample of the
cells from the same inputs: every cell the step failed, the cells with the
most Newton iterations, and a seeded random sample.  The comparison is
tests/parity.py's (default tolerances: path-identical cells at 1e-10, flips
and outliers within the oracle's own one-ulp counts; converged tolerances:
every cell with the oracle's substep count and status at 1e-10).
"""
import numpy as np
import pytest

import cases
import parity
from pfgpu import abi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

C2_CELLS = 1_000_000
C3_CELLS = 500_000


def _sample(got, nrand, seed, ntop=200):
    """Indices: failed cells, the ntop cells with the most Newton iterations,
    nrand random cells (sorted, unique)."""
    N = got.ncells
    fail = np.nonzero(got.a["status"] != 0)[0]
    top = np.argsort(got.a["newton_its"], kind="stable")[-ntop:]
    rnd = np.random.default_rng(seed).choice(N, size=min(nrand, N), replace=False)
    return np.unique(np.concatenate([fail, top, rnd])), fail


def _oracle_parity(oracle, net, inputs, got, idx, dt, label, converged=False):
    """The oracle on the sampled cells of `inputs` (and on one-ulp
    perturbations of them), compared with the GPU's results on the same
    cells."""
    sub0 = inputs.subset(idx)
    ref = sub0.copy()
    oracle.rstep(net, ref, dt, nthreads=16)
    perts = []
    for k, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = sub0.copy()
        p.a[k][:] = np.nextafter(p.a[k], to)
        oracle.rstep(net, p, dt, nthreads=16)
        perts.append(p)
    entry, ok = parity.compare(net, ref, got.subset(idx), dt, label, perts, its=not converged)
    return entry, ok, ref


@pytest.fixture(scope="module")
def c2():
    import bench
    net, eng, dev = bench.build_state("c2", C2_CELLS, "cuda")
    s0 = dev.numpy()
    return net, eng, dev, s0


@pytest.mark.parametrize("lanes", [1, 4], ids=["one-lane", "group4"])
def test_c2_bench_steps(oracle, c2, lanes):
    """Both timed configurations of the bench (one lane per cell, and the
    group of 4 lanes the autotuner picks), first and second step."""
    from pfgpu.engine import ReactionEngine
    net, _, dev0, s0 = c2
    eng = ReactionEngine(net)
    if lanes > 1:
        assert eng.set_launch_config(128, 2, 0, lanes) == abi.PF_OK
    else:
        assert eng.launch_config()["lanes_per_cell"] <= 1  # the default launch: one lane per cell
    dev = s0.to("cuda")
    stats1 = eng.rstep(dev, 86400.0)
    got1 = dev.numpy()
    idx, fail = _sample(got1, 20000, seed=1)
    entry, ok, ref = _oracle_parity(oracle, net, s0, got1, idx, 86400.0, "bench-c2/step1/lanes%d" % lanes)
    parity.check(entry, "c2 step 1", min_compared=int(0.95 * idx.size))
    # the failed cells: the oracle fails them too (within its own flip count)
    if fail.size:
        fe, _, _ = _oracle_parity(oracle, net, s0, got1, fail, 86400.0, "bench-c2/step1-failed/lanes%d" % lanes)
        assert fe["failed_ref"] >= fe["failed_gpu"] - 2 * fe["oracle_self_flips"] - 2, fe
    assert stats1["failed_cells"] == fail.size
    # second step: from the GPU's own state after the first, the queue in
    # cell order (what the bench times); the first step's Newton order gives
    # the same bits
    order = torch.argsort(dev.a["newton_its"].to(torch.int64), descending=True)
    s1 = got1
    dev2 = s1.to("cuda")
    eng.rstep(dev2, 86400.0)
    got2 = dev2.numpy()
    dev3 = s1.to("cuda")
    eng.rstep(dev3, 86400.0, order=order)
    got3 = dev3.numpy()
    for k in ("total", "pri_molal", "sec_molal", "mnrl_rate", "mnrl_volfrac", "newton_its", "status"):
        np.testing.assert_array_equal(got3.a[k], got2.a[k], err_msg=k)
    idx2, _ = _sample(got2, 20000, seed=2)
    entry2, _, _ = _oracle_parity(oracle, net, s1, got2, idx2, 86400.0, "bench-c2/step2/lanes%d" % lanes)
    parity.check(entry2, "c2 step 2", min_compared=int(0.95 * idx2.size))


def test_c2_bench_converged(oracle, c2):
    """The same inputs at converged tolerances: every sampled cell with the
    oracle's substep count and status agrees at 1e-10."""
    from pfgpu.engine import ReactionEngine
    net, _, _, s0 = c2
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(s0.ncells, 20000, replace=False))
    sub = s0.subset(idx)
    netc = net.with_options(**cases.CONVERGED)
    eng = ReactionEngine(netc)
    dev = sub.to("cuda")
    eng.rstep(dev, 86400.0)
    got = dev.numpy()
    entry, _, _ = _oracle_parity(oracle, netc, sub, got, np.arange(sub.ncells), 86400.0,
                                 "bench-c2/converged", converged=True)
    parity.check(entry, "c2 converged", min_compared=int(0.99 * sub.ncells))
    assert entry["outliers"] == 0, entry


@pytest.fixture(scope="module")
def c3():
    import bench
    members = bench.build_c3(C3_CELLS, "cuda")
    return [(eng, eng.net, dev.numpy()) for eng, dev in members]


def test_c3_bench_networks(oracle, c3):
    """Each of the eight heterogeneous networks of the bench, its default
    launch, per-cell dt: the sampled cells against the oracle, at the
    default and at converged tolerances."""
    from pfgpu.engine import ReactionEngine
    for eng0, net, s0 in c3:
        # the default launch and a group of lanes per cell (the autotuner's
        # pick from ncomp 8 up)
        for lanes in (0, 4, 8):
            eng = ReactionEngine(net)
            if lanes and eng.set_launch_config(128, 2, 0, lanes) != abi.PF_OK:
                continue
            dev = s0.to("cuda")
            eng.rstep(dev, 86400.0)
            got = dev.numpy()
            idx, _ = _sample(got, 3000, seed=net.ncomp, ntop=100)
            label = "bench-c3/n%d/%s" % (net.ncomp, "group%d" % lanes if lanes else "default")
            entry, _, _ = _oracle_parity(oracle, net, s0, got, idx, 86400.0, label)
            parity.check(entry, label)
        netc = net.with_options(**cases.CONVERGED)
        engc = ReactionEngine(netc)
        sub = s0.subset(idx)
        devc = sub.to("cuda")
        engc.rstep(devc, 86400.0)
        gotc = devc.numpy()
        label = "bench-c3/n%d/converged" % net.ncomp
        ec, _, _ = _oracle_parity(oracle, netc, sub, gotc, np.arange(sub.ncells), 86400.0, label, converged=True)
        parity.check(ec, label, min_compared=int(0.9 * sub.ncells))
        assert ec["outliers"] == 0, (label, ec)
