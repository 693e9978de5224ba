"""GPU parity: both kernel forms against the CPU oracle on identical inputs.

Quantities and tolerances (FP64 throughout):
  pri_molal, sec_molal        1e-10 relative
  total                       1e-10 relative to the component's gross scale
                              den*(m_k + sum_i |nu_ik| s_i) (totals can cancel)
  mnrl_rate                   1e-10 relative to max(|rate|, 1e-30)
  mnrl_volfrac                1e-10 relative to max(volfrac, 1e-30)
  status, num_substeps        exact
The 1e-10 comparison covers every cell whose solve the oracle completes in a
single RReact (no dt cut) and whose Newton path the GPU reproduces (same
iteration count, substeps and status).  A cell whose path differs ("flip")
had a stopping test (relative change < 1e-6, |r| < 1e-12) or a dt cut
decided by rounding.  How often that happens is a property of the network,
not of the GPU: the oracle itself, re-run on inputs perturbed by one ulp,
flips the same kind of cells.  So each case also measures that rounding
sensitivity -- the union over three one-ulp perturbations (totals up, totals
down, initial molalities up) of the cells whose oracle path changes -- and
the GPU must stay within twice the oracle's own flip and outlier counts (plus
1 % of the cells): on the well-conditioned networks both
are zero and every compared value agrees to 1e-10; on the stiff
heterogeneous ones (kinetic minerals far from equilibrium, many cells
exhausting dt cuts in the reference) both rates are reported.  The
tight-tolerance test separates arithmetic error from stopping-rule noise.
"""
import json
import os

import numpy as np
import pytest

import cases
from pfgpu import abi
from pfgpu.network import CellState

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1.0e-10
OUT = os.environ.get("PFGPU_PARITY_OUT", os.path.join(os.path.dirname(os.path.dirname(__file__)),
                                                       "gpurun_out"))
_report = {}


def _engine(net):
    from pfgpu.engine import ReactionEngine
    return ReactionEngine(net)


def _gross_total(net, st):
    """den*(m_k + sum_i |nu_ik| s_i): the scale of total_k before cancellation."""
    g = st.a["pri_molal"].copy()
    for i in range(net.nsec):
        for s in range(net.sec_nspec[i]):
            g[net.sec_spec[i, s]] += abs(net.sec_stoich[i, s]) * st.a["sec_molal"][i]
    return g * st.a["den_kg"] * 1e-3


def _cell_err(net, ref, got):
    """Per-cell maximum relative difference over every compared quantity."""
    def r(a, b, scale):
        return (np.abs(a - b) / scale).reshape(-1, ref.ncells).max(axis=0)
    e = r(got.a["pri_molal"], ref.a["pri_molal"], np.abs(ref.a["pri_molal"]))
    if net.nsec:
        e = np.maximum(e, r(got.a["sec_molal"], ref.a["sec_molal"], np.maximum(np.abs(ref.a["sec_molal"]), 1e-300)))
    e = np.maximum(e, r(got.a["total"], ref.a["total"], _gross_total(net, ref)))
    if net.nmnrl:
        e = np.maximum(e, r(got.a["mnrl_rate"], ref.a["mnrl_rate"], np.maximum(np.abs(ref.a["mnrl_rate"]), 1e-30)))
        e = np.maximum(e, r(got.a["mnrl_volfrac"], ref.a["mnrl_volfrac"],
                            np.maximum(np.abs(ref.a["mnrl_volfrac"]), 1e-30)))
    return e


def _path_masks(net, ref, got):
    """(mask of flips among single-RReact cells, mask of path-identical single
    cells, mask of those with any compared quantity differing by REL or more)."""
    single = (ref.a["num_substeps"] == 1) & (ref.a["status"] == 0) & \
        (ref.a["newton_its"] <= net.options["maximum_reaction_iterations"])
    path = (ref.a["newton_its"] == got.a["newton_its"]) & (ref.a["num_substeps"] == got.a["num_substeps"]) & \
        (ref.a["status"] == got.a["status"])
    same = single & path
    bad = same & (_cell_err(net, ref, got) >= REL)
    return single & ~path, same, bad


def _path_stats(net, ref, got):
    """(flips among single-RReact cells, path-identical single cells, count of
    those with any compared quantity differing by REL or more).  got may be a
    list of perturbed oracle runs: a cell counts if any of them flips it."""
    if isinstance(got, (list, tuple)):
        fl = bad = None
        same = None
        for g in got:
            f, s_, b = _path_masks(net, ref, g)
            fl = f if fl is None else (fl | f)
            bad = b if bad is None else (bad | b)
            same = s_ if same is None else (same & s_)
        return int(fl.sum()), same, int((bad & ~fl).sum())
    f, same, b = _path_masks(net, ref, got)
    return int(f.sum()), same, int(b.sum())


def compare(net, ref, got, label, self_ref=None):
    """Returns (max errors dict over well-behaved cells, flips, mask of cells
    compared, outliers).  self_ref: the oracle on one-ulp-perturbed inputs
    (one run or a list of runs)."""
    its_r = ref.a["newton_its"]
    flips, same, outliers = _path_stats(net, ref, got)
    single = (ref.a["num_substeps"] == 1) & (ref.a["status"] == 0) & \
        (its_r <= net.options["maximum_reaction_iterations"])
    path = (its_r == got.a["newton_its"]) & (ref.a["num_substeps"] == got.a["num_substeps"]) & \
        (ref.a["status"] == got.a["status"])
    self_flips = self_out = None
    if self_ref is not None:
        self_flips, _, self_out = _path_stats(net, ref, self_ref)
    # value errors over the compared cells that are not outliers
    same_ok = same & (_cell_err(net, ref, got) < REL)
    errs = {}

    def rel(a, b, scale):
        return float(np.max(np.abs(a - b)[..., same_ok] / scale[..., same_ok])) if same_ok.any() else 0.0

    errs["pri_molal"] = rel(got.a["pri_molal"], ref.a["pri_molal"], np.abs(ref.a["pri_molal"]))
    if net.nsec:
        errs["sec_molal"] = rel(got.a["sec_molal"], ref.a["sec_molal"],
                                np.maximum(np.abs(ref.a["sec_molal"]), 1e-300))
    errs["total"] = rel(got.a["total"], ref.a["total"], _gross_total(net, ref))
    if net.nmnrl:
        errs["mnrl_rate"] = rel(got.a["mnrl_rate"], ref.a["mnrl_rate"],
                                np.maximum(np.abs(ref.a["mnrl_rate"]), 1e-30))
        errs["mnrl_volfrac"] = rel(got.a["mnrl_volfrac"], ref.a["mnrl_volfrac"],
                                   np.maximum(np.abs(ref.a["mnrl_volfrac"]), 1e-30))
    _report[label] = dict(cells=int(ref.ncells), single_rreact=int(single.sum()), compared=int(same.sum()),
                          flips=flips, outliers=outliers, oracle_self_flips=self_flips,
                          oracle_self_outliers=self_out, cut_cells=int((~single).sum()),
                          cut_cells_same_path=int((~single & path).sum()),
                          failed_ref=int((ref.a["status"] != 0).sum()),
                          failed_gpu=int((got.a["status"] != 0).sum()),
                          its_mean=float(its_r.mean()), its_max=int(its_r.max()),
                          substeps_max=int(ref.a["num_substeps"].max()), max_rel_err=errs)
    return errs, flips, same, outliers, self_flips, self_out


_SELF = {}


GROUP = {"group2": 2, "group4": 4, "group8": 8}


def run_pair(oracle, name, kernel, tight=False):
    net, st0 = cases.case(oracle, name, tight=tight)
    dt = cases.CASE_DT[name]
    ref = st0.copy()
    oracle.rstep(net, ref, dt, nthreads=8)
    if (name, tight) not in _SELF:
        perts = []
        for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
            pert = st0.copy()
            pert.a[key][:] = np.nextafter(pert.a[key], to)
            oracle.rstep(net, pert, dt, nthreads=8)
            perts.append(pert)
        _SELF[(name, tight)] = perts
    eng = _engine(net)
    if kernel in GROUP:
        # the group-per-cell kernel, where the library accepts the shape
        if eng.set_launch_config(128, 2, 0, GROUP[kernel]) != abi.PF_OK:
            pytest.skip("%s: ncomp %d not covered" % (kernel, net.ncomp))
        kernel = abi.PF_KERNEL_BATCHED
    dev = st0.to("cuda")
    stats = eng.rstep(dev, dt, kernel=kernel)
    torch.cuda.synchronize()
    got = dev.numpy()
    return net, ref, got, stats, _SELF[(name, tight)]


@pytest.mark.parametrize("kernel", [abi.PF_KERNEL_PLAIN, abi.PF_KERNEL_BATCHED, "group2", "group4", "group8"],
                         ids=["plain", "batched", "group2", "group4", "group8"])
@pytest.mark.parametrize("name", ["calcite", "random12"] + ["hetero%d" % n for n in cases.HETERO])
def test_rstep_parity(oracle, name, kernel):
    net, ref, got, stats, pert = run_pair(oracle, name, kernel)
    label = "%s/%s" % (name, kernel if kernel in GROUP else ("plain" if kernel == 0 else "batched"))
    errs, flips, same, outliers, self_flips, self_out = compare(net, ref, got, label, pert)
    n_single = int(same.sum()) + flips
    slack = max(2, 0.01 * n_single)
    assert flips <= 2 * self_flips + slack, (label, flips, self_flips, n_single)
    assert outliers <= 2 * self_out + slack, (label, outliers, self_out)
    for k, v in errs.items():
        assert v < REL, (label, k, v, errs)
    assert stats["failed_cells"] == int((got.a["status"] != 0).sum())
    assert stats["newton_iterations"] == int(got.a["newton_its"].sum())
    assert stats["max_newton_iterations"] == int(got.a["newton_its"].max())


@pytest.mark.parametrize("kernel", [abi.PF_KERNEL_BATCHED, "group8"], ids=["batched", "group8"])
@pytest.mark.parametrize("name", ["calcite", "random12", "hetero16"])
def test_rstep_parity_tight(oracle, name, kernel):
    """Tight tolerances: every solve converges to rounding level, separating
    arithmetic error from stopping-rule noise."""
    net, ref, got, stats, pert = run_pair(oracle, name, kernel, tight=True)
    compare(net, ref, got, "%s/%s/tight" % (name, kernel if kernel in GROUP else "batched"), pert)
    # tight solves converge far below the 1e-10 exit test, so even cells
    # whose iteration count flipped agree
    ok = (ref.a["status"] == 0) & (got.a["status"] == 0) & (ref.a["num_substeps"] == 1) & \
        (got.a["num_substeps"] == 1)
    assert ok.mean() > 0.9, ok.mean()
    e = np.max(np.abs(got.a["pri_molal"] - ref.a["pri_molal"])[:, ok] / ref.a["pri_molal"][:, ok])
    assert e < REL, (name, e)


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
    """pf_rstep_host cuts a large state into chunks of 2^18 cells (copy-in,
    compute and copy-out overlapped on three streams, the work-queue order
    restricted to each chunk): 600,000 cells (three chunks, the last one
    short) give the device path's results bit for bit, with the same
    statistics; an order that is not a permutation is refused."""
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
        bad = order_host.copy()
        bad[7] = bad[8]
        with pytest.raises(abi.PfError) as e:
            eng.rstep_host(big.copy(), 86400.0, order=bad)
        assert e.value.code == abi.PF_ERR_INVALID


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
    errs, flips, same, outliers, self_flips, self_out = compare(net, ref, got, "odd%d/default" % ncomp, perts)
    n_single = int(same.sum()) + flips
    slack = max(2, 0.01 * n_single)
    assert same.sum() > 50
    assert flips <= 2 * self_flips + slack, (flips, self_flips)
    assert outliers <= 2 * self_out + slack, (outliers, self_out)
    for k, v in errs.items():
        assert v < REL, (k, v, errs)


def _newton_iter_case(oracle):
    from pfgpu import abi, generate
    from pfgpu.network import default_options
    opts = default_options(isothermal=0)
    opts["act_coef_update_frequency"] = abi.PF_ACT_COEF_NEWTON_ITER
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
    errs, flips, same, outliers, self_flips, self_out = compare(net, ref, got, "newton_iter/" + kernel, perts)
    n_single = int(same.sum()) + flips
    slack = max(2, 0.01 * n_single)
    assert same.sum() > 100
    assert flips <= 2 * self_flips + slack, (flips, self_flips)
    assert outliers <= 2 * self_out + slack, (outliers, self_out)
    for kk, v in errs.items():
        assert v < REL, (kk, v, errs)
    np.testing.assert_allclose(got.a["pri_act_coef"][:, same], ref.a["pri_act_coef"][:, same], rtol=1e-10)


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
    errs, flips, same, outliers, self_flips, self_out = compare(net, ref, got, label, perts)
    n_single = int(same.sum()) + flips
    slack = max(2, 0.01 * n_single)
    assert same.sum() > 300, same.sum()
    assert flips <= 2 * self_flips + slack, (flips, self_flips)
    assert outliers <= 2 * self_out + slack, (outliers, self_out)
    for kk, v in errs.items():
        assert v < REL, (kk, v, errs)
    # every branch was taken somewhere: the reversible minerals both dissolve
    # and precipitate among the compared cells
    rates = ref.a["mnrl_rate"][:, same]
    for m in range(3):
        assert (rates[m] > 0).any() and (rates[m] < 0).any(), m


def test_write_parity_report():
    """Writes the per-case error/flip/iteration summary collected by the tests above (kept last in the module)."""
    if not _report:
        pytest.skip("no parity cases ran")
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(OUT, "parity_report.json"), "w") as f:
        json.dump(_report, f, indent=1, sort_keys=True)
