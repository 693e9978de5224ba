"""GPU parity: every kernel form against the CPU oracle on identical inputs.

The comparison, its scales and the classes of cells are in tests/parity.py.
Two regimes per case and kernel form:

  default tolerances (the reference's: relative change 1e-6, |r| < 1e-12,
      ||r||/||r0|| < 1e-8, 20 iterations, 10 cuts): every cell whose Newton
      path the GPU reproduces (same iteration count, substeps and status --
      single-RReact cells, cells with dt cuts and failed cells alike) is
      compared at 1e-10; path flips and outliers (path-identical cells whose
      values moved by 1e-10 or more) must stay within twice the oracle's own
      counts on inputs one ulp away, plus max(2, 1 %) of the cells.  The
      reference's stopping tests are absolute, so on the stiff networks the
      oracle itself moves converged cells by up to tens of percent under a
      one-ulp change of its inputs; the report states the GPU's and the
      oracle's own errors on flipped cells side by side.
  converged tolerances (converged_options: relative change 1e-12, residual
      tests off, 100 iterations): every cell is solved to rounding level, so
      every cell with the same substep count and status -- including the
      cells that flipped, cut or failed at the default tolerances -- must
      agree at 1e-10 in every quantity; substep-count differences are bounded
      by the oracle's own as above.
The per-case report is printed at the end of the pytest session.
"""
import numpy as np
import pytest

import cases
import parity
from pfgpu import abi
from pfgpu.network import CellState

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = parity.REL
GROUP = {"group2": 2, "group4": 4, "group8": 8}
KERNELS = [abi.PF_KERNEL_PLAIN, abi.PF_KERNEL_BATCHED, "group2", "group4", "group8"]
KERNEL_IDS = ["plain", "batched", "group2", "group4", "group8"]
_SELF = {}


def _engine(net):
    from pfgpu.engine import ReactionEngine
    return ReactionEngine(net)


def self_runs(oracle, net, st0, dt, key=None):
    """The oracle on three one-ulp perturbations of the inputs (totals up,
    totals down, initial molalities up), cached per key."""
    if key is not None and key in _SELF:
        return _SELF[key]
    perts = []
    for k, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        pert = st0.copy()
        pert.a[k][:] = np.nextafter(pert.a[k], to)
        oracle.rstep(net, pert, dt, nthreads=8)
        perts.append(pert)
    if key is not None:
        _SELF[key] = perts
    return perts


def gpu_step(net, st0, dt, kernel, launch_tpb=128, blocks_per_sm=2):
    """One pf_rstep of st0 on the device with the given kernel form; returns
    (host copy of the result, stats) or None when the library refuses that
    group size for the network."""
    eng = _engine(net)
    if kernel in GROUP:
        if eng.set_launch_config(launch_tpb, blocks_per_sm, 0, GROUP[kernel]) != abi.PF_OK:
            return None
        kernel = abi.PF_KERNEL_BATCHED
    dev = st0.to("cuda")
    stats = eng.rstep(dev, dt, kernel=kernel)
    torch.cuda.synchronize()
    return dev.numpy(), stats


def _kname(kernel):
    return kernel if kernel in GROUP else ("plain" if kernel == abi.PF_KERNEL_PLAIN else "batched")


def run_case(oracle, name, kernel, converged=False):
    net, st0 = cases.case(oracle, name)
    if converged:
        net = net.with_options(**cases.CONVERGED)
    dt = cases.CASE_DT[name]
    ref = st0.copy()
    oracle.rstep(net, ref, dt, nthreads=8)
    perts = self_runs(oracle, net, st0, dt, key=(name, converged))
    out = gpu_step(net, st0, dt, kernel)
    if out is None:
        pytest.skip("%s: ncomp %d not covered" % (kernel, net.ncomp))
    got, stats = out
    label = "%s/%s%s" % (name, _kname(kernel), "/converged" if converged else "")
    entry, ok = parity.compare(net, ref, got, dt, label, perts, its=not converged)
    return net, ref, got, stats, entry, ok, label


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
@pytest.mark.parametrize("name", ["calcite", "random12"] + ["hetero%d" % n for n in cases.HETERO])
def test_rstep_parity(oracle, name, kernel):
    net, ref, got, stats, entry, ok, label = run_case(oracle, name, kernel)
    parity.check(entry, label)
    assert stats["failed_cells"] == int((got.a["status"] != 0).sum())
    assert stats["newton_iterations"] == int(got.a["newton_its"].sum())
    assert stats["max_newton_iterations"] == int(got.a["newton_its"].max())


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
@pytest.mark.parametrize("name", ["calcite", "random12"] + ["hetero%d" % n for n in cases.HETERO])
def test_rstep_parity_converged(oracle, name, kernel):
    """Converged tolerances: 1e-10 on every quantity for every cell with the
    oracle's substep count and status, whatever its Newton count."""
    net, ref, got, stats, entry, ok, label = run_case(oracle, name, kernel, converged=True)
    parity.check(entry, label, min_compared=int(0.9 * ref.ncells))
    assert entry["outliers"] == 0, (label, entry)
    assert entry["compared"] == entry["compared_by_class"]["single"] + entry["compared_by_class"]["cut"] + \
        entry["compared_by_class"]["failed"]


def test_rstep_host_path_matches_device(oracle):
    net, st0 = cases.case(oracle, "calcite")
    eng = _engine(net)
    dev = st0.to("cuda")
    eng.rstep(dev, 3600.0)
    host = st0.copy()
    eng.rstep_host(host, 3600.0)
    d = dev.numpy()
    for k in ("total", "pri_molal", "sec_molal", "mnrl_rate", "mnrl_volfrac", "newton_its"):
        np.testing.assert_array_equal(host.a[k], d.a[k])


@pytest.mark.parametrize("with_order", [False, True], ids=["natural", "permuted"])
def test_rstep_host_pipeline_over_chunks_matches_device(oracle, with_order):
    """pf_rstep_host cuts a large state into chunks (copy-in, compute and
    copy-out overlapped on three streams): a tenth of the cells, the rest,
    a tenth (the last chunk takes the ragged end), the order restricted to
    each chunk.  600,000 cells give the device path's results
    bit for bit, with the same statistics; an order that is not a
    permutation is refused."""
    net, st0 = cases.case(oracle, "random12")
    reps = -(-600000 // st0.ncells)
    big = CellState(net, {k: (np.tile(v, reps)[..., :600000] if v.ndim == 1 else np.tile(v, (1, reps))[:, :600000])
                          for k, v in st0.a.items()})
    big.a["total"][:] *= np.random.default_rng(5).uniform(0.9, 1.1, big.a["total"].shape)
    eng = _engine(net)
    order_dev = order_host = None
    if with_order:
        perm = np.random.default_rng(6).permutation(600000).astype(np.int64)
        order_host, order_dev = perm, torch.from_numpy(perm).cuda()
    dev = big.to("cuda")
    s_dev = eng.rstep(dev, 86400.0, order=order_dev)
    host = big.copy()
    s_host = eng.rstep_host(host, 86400.0, order=order_host)
    d = dev.numpy()
    for k in ("total", "pri_molal", "pri_act_coef", "sec_molal", "mnrl_rate", "mnrl_volfrac", "newton_its",
              "num_substeps", "status"):
        np.testing.assert_array_equal(host.a[k], d.a[k], err_msg=k)
    assert s_host == s_dev
    if with_order:
        # a cell twice and another missing: across chunks, inside chunk 0,
        # inside the last chunk; an entry out of range.  Each is refused and
        # leaves the caller's state as it was.
        edge = ((600000 + 9) // 10 + 63) // 64 * 64
        tail = (600000 - edge) // 64 * 64
        first = np.flatnonzero(order_host < edge)[:2]
        last = np.flatnonzero(order_host >= tail)[:2]
        cross = np.array([np.flatnonzero(order_host < edge)[0], np.flatnonzero(order_host >= edge)[0]])
        for i, j, v in ((cross[0], cross[1], None), (first[0], first[1], None), (last[0], last[1], None),
                        (5, None, 600000)):
            bad = order_host.copy()
            bad[i] = bad[j] if v is None else v
            before = big.copy()
            arg = big.copy()
            with pytest.raises(abi.PfError) as e:
                eng.rstep_host(arg, 86400.0, order=bad)
            assert e.value.code == abi.PF_ERR_INVALID
            for k in ("total", "pri_molal", "status"):
                np.testing.assert_array_equal(arg.a[k], before.a[k], err_msg=k)


def test_cell_order_does_not_change_results(oracle):
    """The work-queue order only schedules cells; every cell's result is the
    same bit pattern in any order."""
    net, st0 = cases.case(oracle, "random12")
    eng = _engine(net)
    a = st0.to("cuda")
    eng.rstep(a, 86400.0)
    b = st0.to("cuda")
    order = torch.argsort(a.a["newton_its"].to(torch.int64), descending=True)
    eng.rstep(b, 86400.0, order=order)
    for k in ("total", "pri_molal", "sec_molal", "mnrl_rate", "mnrl_volfrac", "newton_its", "status"):
        assert torch.equal(a.a[k], b.a[k]), k


def test_zero_cells_and_bad_args(oracle):
    net, st0 = cases.case(oracle, "calcite")
    eng = _engine(net)
    empty = st0.subset(np.arange(0)).to("cuda")
    st = eng.rstep(empty, 3600.0)
    assert st["cells"] == 0
    dev = st0.to("cuda")
    with pytest.raises(abi.PfError):
        eng.rstep(dev, -1.0)
    with pytest.raises(abi.PfError):
        eng.rstep(dev, 3600.0, kernel=7)


def test_dry_and_floored_cells(oracle):
    """Saturation below rt_min_saturation (reactive_transport_aux.F90:19) and
    totals <= 1e-40 (RStep floor, reaction.F90:3618-3631) follow the oracle."""
    net, st0 = cases.case(oracle, "calcite")
    st0 = st0.subset(np.arange(64))
    st0.a["saturation"][:8] = 0.0
    st0.a["total"][1, 8:16] = -1.0e-3  # negative HCO3- total: floored, then restored
    ref = st0.copy()
    oracle.rstep(net, ref, 3600.0)
    for kernel in (abi.PF_KERNEL_PLAIN, abi.PF_KERNEL_BATCHED):
        eng = _engine(net)
        dev = st0.to("cuda")
        eng.rstep(dev, 3600.0, kernel=kernel)
        got = dev.numpy()
        np.testing.assert_array_equal(got.a["status"], ref.a["status"])
        same = got.a["newton_its"] == ref.a["newton_its"]
        np.testing.assert_allclose(got.a["total"][:, same], ref.a["total"][:, same], rtol=1e-10, atol=1e-25)
        np.testing.assert_allclose(got.a["pri_molal"][:, same], ref.a["pri_molal"][:, same], rtol=1e-10)


def test_failing_cells_report_status(oracle):
    """Cells that cannot converge: RStep cuts dt maximum_reaction_cuts times
    and reports ierror = 1 (reaction.F90:3657-3666); both forms agree with
    the oracle on which cells fail and how many Newton iterations they spent."""
    net, st0 = cases.case(oracle, "calcite")
    st0 = st0.subset(np.arange(32))
    net2 = net.with_options(maximum_reaction_iterations=2, maximum_reaction_cuts=3)
    ref = st0.copy()
    oracle.rstep(net2, ref, 3600.0)
    assert (ref.a["status"] != 0).any()
    for kernel in (abi.PF_KERNEL_PLAIN, abi.PF_KERNEL_BATCHED):
        eng = _engine(net2)
        dev = st0.to("cuda")
        stats = eng.rstep(dev, 3600.0, kernel=kernel)
        got = dev.numpy()
        np.testing.assert_array_equal(got.a["status"], ref.a["status"])
        np.testing.assert_array_equal(got.a["newton_its"], ref.a["newton_its"])
        assert stats["failed_cells"] == int((ref.a["status"] != 0).sum())


@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_group_kernel_order_invariant_and_close_to_one_lane(oracle, lanes):
    """The group-per-cell kernel: results do not depend on the work-queue
    order, and agree with the one-lane kernel to rounding on cells whose
    Newton path is the same."""
    net, st0 = cases.case(oracle, "random12")
    eng = _engine(net)
    assert eng.set_launch_config(128, 2, 0, lanes) == abi.PF_OK
    a = st0.to("cuda")
    eng.rstep(a, 86400.0)
    b = st0.to("cuda")
    order = torch.argsort(a.a["newton_its"].to(torch.int64), descending=True)
    eng.rstep(b, 86400.0, order=order)
    for k in ("total", "pri_molal", "sec_molal", "mnrl_rate", "mnrl_volfrac", "newton_its", "status"):
        assert torch.equal(a.a[k], b.a[k]), k
    one = _engine(net)
    c = st0.to("cuda")
    one.rstep(c, 86400.0)
    same = (a.a["newton_its"] == c.a["newton_its"]) & (a.a["status"] == 0) & (c.a["status"] == 0)
    assert same.float().mean() > 0.95
    d = (a.a["pri_molal"] - c.a["pri_molal"]).abs() / c.a["pri_molal"]
    assert float(d[:, same].max()) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("ncomp", [5, 7, 9, 11, 14])
def test_component_counts_without_one_lane_kernel(oracle, ncomp):
    """ncomp values with no one-lane instantiation run through the batched
    path on a group of lanes per cell (the default launch picks one) and meet
    the same parity bar as the other networks: path-identical cells to
    1e-10, flips and outliers within the oracle's own one-ulp sensitivity."""
    from pfgpu import abi, generate
    from pfgpu.engine import ReactionEngine
    from pfgpu.network import default_options
    net = generate.random_network(ncomp, 3 * ncomp, max(1, ncomp // 2), seed=900 + ncomp,
                                  options=default_options(isothermal=0))
    st, ct, cc = generate.random_cells(net, 400, seed=901 + ncomp, dt_range=(3600.0, 30 * 86400.0))
    st, _ = cases.prepare(oracle, net, st, ct, cc)
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, 86400.0, nthreads=8)
        perts.append(p)
    eng = ReactionEngine(net)
    assert eng.launch_config()["lanes_per_cell"] > 1
    assert eng.set_launch_config(128, 1, 0, 1) == abi.PF_ERR_UNSUPPORTED  # no one-lane kernel for this ncomp
    dev = st.to("cuda")
    eng.rstep(dev, 86400.0)
    got = dev.numpy()
    entry, ok = parity.compare(net, ref, got, 86400.0, "odd%d/default" % ncomp, perts)
    parity.check(entry, "odd%d" % ncomp, min_compared=50)


def _newton_iter_case(oracle, algo=None):
    from pfgpu import abi, generate
    from pfgpu.network import default_options
    opts = default_options(isothermal=0)
    opts["act_coef_update_frequency"] = abi.PF_ACT_COEF_NEWTON_ITER
    if algo is not None:
        opts["act_coef_update_algorithm"] = algo
    net = generate.random_network(12, 40, 6, seed=12, options=opts)
    st, ct, cc = generate.random_cells(net, 600, seed=4242)
    st, _ = cases.prepare(oracle, net, st, ct, cc)
    return net, st


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["batched", "group4", "group8", "plain"])
def test_activity_each_newton_iteration(oracle, kernel):
    """act_coef_update_frequency = NEWTON_ITERATION: the LAG activity
    coefficients follow every Newton iterate from the previous evaluation's
    complexes (reaction.F90:3857-3860); each kernel form against the oracle
    with the flip-aware comparison."""
    from pfgpu import abi
    from pfgpu.engine import ReactionEngine
    net, st = _newton_iter_case(oracle)
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, 86400.0, nthreads=8)
        perts.append(p)
    eng = ReactionEngine(net)
    k = abi.PF_KERNEL_PLAIN if kernel == "plain" else abi.PF_KERNEL_BATCHED
    if kernel.startswith("group"):
        assert eng.set_launch_config(128, 2, 0, int(kernel[5:])) == abi.PF_OK
    dev = st.to("cuda")
    eng.rstep(dev, 86400.0, kernel=k)
    got = dev.numpy()
    entry, ok = parity.compare(net, ref, got, 86400.0, "newton_iter/" + kernel, perts)
    parity.check(entry, "newton_iter/" + kernel, min_compared=100)
    np.testing.assert_allclose(got.a["pri_act_coef"][:, ok], ref.a["pri_act_coef"][:, ok], rtol=1e-10)


@pytest.mark.gpu
def test_newton_activity_each_newton_iteration(oracle):
    """act_coef_update_frequency = NEWTON_ITERATION with the NEWTON
    algorithm (reaction.F90:3857-3860, 4403-4551): the ionic-strength
    iteration at every Newton iterate runs in the plain kernel, against the
    oracle with the flip-aware comparison; the batched kernels refuse it."""
    from pfgpu import abi
    from pfgpu.engine import ReactionEngine
    net, st = _newton_iter_case(oracle, abi.PF_ACT_COEF_ALGO_NEWTON)
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, 86400.0, nthreads=8)
        perts.append(p)
    eng = ReactionEngine(net)
    dev = st.to("cuda")
    with pytest.raises(abi.PfError) as e:
        eng.rstep(dev, 86400.0, kernel=abi.PF_KERNEL_BATCHED)
    assert e.value.code == abi.PF_ERR_UNSUPPORTED
    assert eng.set_launch_config(128, 2, 0, 4) == abi.PF_ERR_UNSUPPORTED
    eng.rstep(dev, 86400.0, kernel=abi.PF_KERNEL_PLAIN)
    got = dev.numpy()
    entry, ok = parity.compare(net, ref, got, 86400.0, "newton_algo_iter/plain", perts)
    parity.check(entry, "newton_algo_iter/plain", min_compared=100)
    for key in ("pri_act_coef", "sec_act_coef"):
        np.testing.assert_allclose(got.a[key][:, ok], ref.a[key][:, ok], rtol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["batched", "group4", "plain"])
def test_non_finite_cell_fails_alone(oracle, kernel):
    """A cell with a non-finite total fails (status != 0, its factorisation
    falls back and gives up), and every other cell's result is bitwise the
    result of the same run without it."""
    from pfgpu import abi
    from pfgpu.engine import ReactionEngine
    net, st0 = cases.case(oracle, "random12")
    st = st0.subset(np.arange(300))
    bad = st.copy()
    bad.a["total"][3, 17] = np.nan
    eng = ReactionEngine(net)
    k = abi.PF_KERNEL_PLAIN if kernel == "plain" else abi.PF_KERNEL_BATCHED
    if kernel == "group4":
        assert eng.set_launch_config(128, 2, 0, 4) == abi.PF_OK
    outs = []
    for s in (st, bad):
        dev = s.to("cuda")
        eng.rstep(dev, 86400.0, kernel=k)
        outs.append(dev.numpy())
    good, gotbad = outs
    assert gotbad.a["status"][17] != 0
    keep = np.ones(300, bool)
    keep[17] = False
    for key in ("pri_molal", "total", "sec_molal", "mnrl_rate", "status", "newton_its"):
        np.testing.assert_array_equal(gotbad.a[key][..., keep], good.a[key][..., keep], err_msg=key)


def _mineral_options_case(oracle, log_formulation):
    """An 8-component network whose four kinetic minerals exercise every
    optional branch of RKineticMineral (reaction_mineral.F90:647-1078): rate
    limiter, Temkin constant with a minimum scale factor, affinity power,
    irreversibility with an affinity threshold, Arrhenius activation energy."""
    from pfgpu import generate
    from pfgpu.network import default_options
    opts = default_options(isothermal=0)
    opts["use_log_formulation"] = int(log_formulation)
    net = generate.random_network(8, 24, 4, seed=818, options=opts)
    nm = net.nmnrl
    net.mnrl_rate_limiter = np.array([0.5, 0.0, 0.0, 0.0])[:nm]
    net.mnrl_Temkin_const = np.array([1.0, 2.0, 1.0, 1.0])[:nm]
    net.mnrl_min_scale_factor = np.array([1.0, 1.5, 1.0, 1.0])[:nm]
    net.mnrl_affinity_power = np.array([1.0, 1.0, 2.0, 1.0])[:nm]
    net.mnrl_irreversible = np.array([0, 0, 0, 1], np.int32)[:nm]
    net.mnrl_affinity_threshold = np.array([0.0, 0.0, 0.0, 1.0e-3])[:nm]
    net.mnrl_activation_energy = np.array([3.0e4, 0.0, 5.0e4, 0.0])[:nm]
    st, ct, cc = generate.random_cells(net, 600, seed=8181)
    st, _ = cases.prepare(oracle, net, st, ct, cc)
    # put each mineral's logK at the median log Q of the cells, so that about
    # half of them precipitate (the threshold and irreversibility branches)
    la = np.log10(st.a["pri_molal"] * st.a["pri_act_coef"])
    for m in range(nm):
        lq = sum(net.mnrl_stoich[m, k] * la[net.mnrl_spec[m, k]] for k in range(net.mnrl_nspec[m]))
        delta = float(np.median(lq)) - net.mnrl_logK[m]
        net.mnrl_logK[m] += delta
        if net.mnrl_logKcoef is not None:
            net.mnrl_logKcoef[m, 1] += delta
    return net, st


@pytest.mark.gpu
@pytest.mark.parametrize("kernel,log_formulation", [("batched", True), ("group4", True), ("plain", True),
                                                     ("batched", False), ("plain", False)])
def test_mineral_rate_law_branches(oracle, kernel, log_formulation):
    from pfgpu import abi
    from pfgpu.engine import ReactionEngine
    net, st = _mineral_options_case(oracle, log_formulation)
    ref = st.copy()
    oracle.rstep(net, ref, 3600.0, nthreads=8)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, 3600.0, nthreads=8)
        perts.append(p)
    eng = ReactionEngine(net)
    k = abi.PF_KERNEL_PLAIN if kernel == "plain" else abi.PF_KERNEL_BATCHED
    if kernel.startswith("group"):
        assert eng.set_launch_config(128, 2, 0, int(kernel[5:])) == abi.PF_OK
    dev = st.to("cuda")
    eng.rstep(dev, 3600.0, kernel=k)
    got = dev.numpy()
    label = "mineral_options/%s/%s" % (kernel, "log" if log_formulation else "linear")
    entry, ok = parity.compare(net, ref, got, 3600.0, label, perts)
    parity.check(entry, label, min_compared=300)
    # every branch was taken somewhere: the reversible minerals both dissolve
    # and precipitate among the compared cells
    rates = ref.a["mnrl_rate"][:, ok]
    for m in range(3):
        assert (rates[m] > 0).any() and (rates[m] < 0).any(), m


def test_linear_formulation_after_group_launch(oracle):
    """pf_network_set_options after a group launch: the group kernel carries
    the log formulation only, so switching to the linear one puts the network
    back on one lane per cell (the step then follows the oracle's linear
    Newton), and the step never runs a kernel that ignores the option."""
    from pfgpu.engine import ReactionEngine
    net, st0 = cases.case(oracle, "random12")
    net = net.with_options()
    eng = ReactionEngine(net)
    assert eng.set_launch_config(128, 2, 0, 4) == abi.PF_OK
    eng.set_options(use_log_formulation=0)
    assert eng.launch_config()["lanes_per_cell"] <= 1
    ref = st0.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    dev = st0.to("cuda")
    eng.rstep(dev, 86400.0)
    got = dev.numpy()
    entry, ok = parity.compare(net, ref, got, 86400.0, "random12/linear-after-group4",
                               self_runs(oracle, net, st0, 86400.0))
    parity.check(entry, "random12/linear-after-group4", min_compared=int(0.9 * ref.ncells))
    # and back: the log formulation accepts the group launch again
    eng.set_options(use_log_formulation=1)
    assert eng.set_launch_config(128, 2, 0, 4) == abi.PF_OK
