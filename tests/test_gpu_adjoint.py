"""Adjoint of the operator-split step (pf_adjoint) against central finite
differences, step 1e-6 in log space, of
  (a) the GPU forward pass (pf_rstep, batched kernel), and
  (b) the CPU oracle (the restatement of the reference's RStep),
for every parameter group: logK shifts of all complexes and kinetic minerals,
ln rate constants, per-cell ln areas and per-cell initial totals.

Loss: sum over cells of w*(total_final - target)^2, w ~ U[0,1], target = the
forward output perturbed by 5 % lognormal noise (the differentiation case of
the benchmark).  Two cases: the 12-component synthetic network at dt = 1 day
and the calcite system at dt = 1 h, where complexation controls the free Ca++
and HCO3- activities and hence the calcite rate (so the logK gradients of the
complexes are large enough for differences to resolve).  Tolerances: FD
truncation is O(h^2) ~ 1e-12 and the tight solver tolerance (relative update
< 1e-10) bounds FD noise; the comparison allows 1e-4 relative on summed and
per-cell gradients, plus the rounding floor of the difference quotient
(1e-14 * sum|loss| / h, ~100 ulp of the summed loss per step h): a gradient below that floor cannot be resolved by
differences and is only checked to be below it.
"""
import numpy as np
import pytest

import cases
from pfgpu import abi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-6
DTS = {"random12": 86400.0, "calcite": 3600.0}
DT = None    # set per case by the fixture
CASE = None


def _setup(oracle, name, lanes=1, ncells=240, tight=True):
    net, st0 = cases.case(oracle, name, tight=tight)
    st0 = st0.subset(np.arange(ncells))
    from pfgpu.engine import ReactionEngine
    eng = ReactionEngine(net)
    if lanes > 1:
        assert eng.set_launch_config(128, 2, 0, lanes) == abi.PF_OK
    dev = st0.to("cuda")
    eng.rstep(dev, DT)
    Tf = dev.a["total"].cpu().numpy()
    rng = np.random.default_rng(31)
    w = rng.uniform(0.0, 1.0, Tf.shape)
    tgt = Tf * np.exp(0.05 * rng.standard_normal(Tf.shape))
    return net, st0, eng, w, tgt


def _cell_loss(Tf, w, tgt):
    return (w * (Tf - tgt) ** 2).sum(axis=0)


def _gpu_loss(eng, st0, w, tgt, shift=None, area_scale=None, total_scale=None):
    st = st0.copy()
    if area_scale is not None:
        st.a["mnrl_area"] *= area_scale
    if total_scale is not None:
        st.a["total"] *= total_scale
    eng.shift_parameters(*(shift or (None, None, None)))
    dev = st.to("cuda")
    eng.rstep(dev, DT)
    eng.shift_parameters()
    got = dev.numpy()
    return _cell_loss(got.a["total"], w, tgt), got.a["newton_its"]


def _oracle_loss(oracle, net, st0, w, tgt, shift=None, area_scale=None, total_scale=None):
    n2 = net.with_options()
    n2.sec_logK, n2.mnrl_logK = net.sec_logK.copy(), net.mnrl_logK.copy()
    n2.sec_logKcoef = None if net.sec_logKcoef is None else net.sec_logKcoef.copy()
    n2.mnrl_logKcoef = None if net.mnrl_logKcoef is None else net.mnrl_logKcoef.copy()
    n2.mnrl_rate_constant = net.mnrl_rate_constant.copy()
    if shift:
        dks, dkm, dlnk = shift
        if dks is not None:
            n2.sec_logK += dks
            if n2.sec_logKcoef is not None:
                n2.sec_logKcoef[:, 1] += dks
        if dkm is not None:
            n2.mnrl_logK += dkm
            if n2.mnrl_logKcoef is not None:
                n2.mnrl_logKcoef[:, 1] += dkm
        if dlnk is not None:
            n2.mnrl_rate_constant = n2.mnrl_rate_constant * np.exp(dlnk)
    st = st0.copy()
    if area_scale is not None:
        st.a["mnrl_area"] *= area_scale
    if total_scale is not None:
        st.a["total"] *= total_scale
    oracle.rstep(n2, st, DT, nthreads=8)
    return _cell_loss(st.a["total"], w, tgt), st.a["newton_its"]


def _unit(k, n, h):
    v = np.zeros(n)
    v[k] = h
    return v


def _fd_global(lossfn, ns, nm):
    """Central differences, per cell, of the loss for every network parameter;
    also the mask of cells whose Newton path is the same in every run (a
    path that changes between +h and -h makes that cell's difference
    quotient meaningless)."""
    base_l, base_its = lossfn()
    stable = np.ones_like(base_its, dtype=bool)
    out = {"dL_dlogK_sec": [], "dL_dlogK_mnrl": [], "dL_dlnk": []}

    def fd(key, shift_p, shift_m):
        nonlocal stable
        lp, ip = lossfn(shift=shift_p)
        lm, im = lossfn(shift=shift_m)
        stable &= (ip == base_its) & (im == base_its)
        out[key].append((lp - lm) / (2 * H))
    for k in range(ns):
        fd("dL_dlogK_sec", (_unit(k, ns, H), None, None), (_unit(k, ns, -H), None, None))
    for k in range(nm):
        fd("dL_dlogK_mnrl", (None, _unit(k, nm, H), None), (None, _unit(k, nm, -H), None))
        fd("dL_dlnk", (None, None, _unit(k, nm, H)), (None, None, _unit(k, nm, -H)))
    return {k: np.array(v) for k, v in out.items()}, stable


def _rel(a, b):
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


@pytest.fixture(scope="module", params=[("random12", 1), ("random12", 8), ("calcite", 1), ("calcite", 8)],
                ids=["random12-lane", "random12-group8", "calcite-lane", "calcite-group8"])
def adjoint_case(oracle, request):
    """Both step kernels carry the adjoint: one lane per cell, and a group of
    8 lanes per cell (launch configuration lanes_per_cell = 8)."""
    global DT, CASE
    name, lanes = request.param
    DT, CASE = DTS[name], name
    net, st0, eng, w, tgt = _setup(oracle, name, lanes)
    dev = st0.to("cuda")
    g = eng.adjoint(dev, DT, weight=torch.from_numpy(w).cuda(), target=torch.from_numpy(tgt).cuda())
    g = {k: v.cpu().numpy() for k, v in g.items()}
    return net, st0, eng, w, tgt, g


def test_adjoint_status_and_loss(adjoint_case):
    net, st0, eng, w, tgt, g = adjoint_case
    assert (g["adj_status"] == 0).mean() > 0.95
    base, _ = _gpu_loss(eng, st0, w, tgt)
    assert g["loss"][0] == pytest.approx(base.sum(), rel=1e-12)


def _check_global(net, st0, eng, w, tgt, g, lossfn, rel=1e-4):
    fd, stable = _fd_global(lossfn, net.nsec, net.nmnrl)
    ok = stable & (g["adj_status"] == 0)
    assert ok.mean() > 0.9, ok.mean()
    idx = np.nonzero(ok)[0]
    sub = st0.subset(idx)
    gs = eng.adjoint(sub.to("cuda"), DT, weight=torch.from_numpy(np.ascontiguousarray(w[:, idx])).cuda(),
                     target=torch.from_numpy(np.ascontiguousarray(tgt[:, idx])).cuda())
    base, _ = lossfn()
    floor = 1e-14 * np.abs(base[ok]).sum() / H
    resolved = {}
    for k, v in fd.items():
        ref = v[:, ok].sum(axis=1)
        got = gs[k].cpu().numpy()
        err = np.abs(got - ref)
        assert np.all(err <= rel * np.abs(ref).max() + floor), (k, got, ref, floor)
        resolved[k] = int((np.abs(ref) > 30 * floor).sum())
    # the calcite case resolves every parameter group
    if CASE == "calcite":
        assert min(resolved.values()) > 0, resolved


def test_adjoint_global_vs_fd_gpu(adjoint_case):
    net, st0, eng, w, tgt, g = adjoint_case
    _check_global(net, st0, eng, w, tgt, g, lambda **kw: _gpu_loss(eng, st0, w, tgt, **kw))


def test_adjoint_global_vs_fd_oracle(adjoint_case, oracle):
    net, st0, eng, w, tgt, g = adjoint_case
    _check_global(net, st0, eng, w, tgt, g, lambda **kw: _oracle_loss(oracle, net, st0, w, tgt, **kw))


@pytest.mark.parametrize("which", ["gpu", "oracle"])
def test_adjoint_per_cell_vs_fd(adjoint_case, oracle, which):
    """Per-cell gradients: every cell's areas (resp. totals) are perturbed at
    once; cells are independent, so each cell's own loss difference is its
    derivative."""
    net, st0, eng, w, tgt, g = adjoint_case
    fn = (lambda **kw: _gpu_loss(eng, st0, w, tgt, **kw)) if which == "gpu" else \
        (lambda **kw: _oracle_loss(oracle, net, st0, w, tgt, **kw))
    ok = g["adj_status"] == 0
    base_l, base_its = fn()
    for m in range(net.nmnrl):
        scale_p = np.ones_like(st0.a["mnrl_area"])
        scale_p[m] = np.exp(H)
        scale_m = np.ones_like(st0.a["mnrl_area"])
        scale_m[m] = np.exp(-H)
        lp, ip = fn(area_scale=scale_p)
        lm, im = fn(area_scale=scale_m)
        fd = (lp - lm) / (2 * H)
        mask = ok & (ip == base_its) & (im == base_its)
        sc = max(np.abs(fd[mask]).max(), 1e-300)
        assert np.max(np.abs(g["dL_dlnarea"][m, mask] - fd[mask])) / sc < 1e-4, m
    for j in range(net.ncomp):
        t0 = st0.a["total"][j]
        scale_p = np.ones_like(st0.a["total"])
        scale_p[j] = 1.0 + H
        scale_m = np.ones_like(st0.a["total"])
        scale_m[j] = 1.0 - H
        lp, ip = fn(total_scale=scale_p)
        lm, im = fn(total_scale=scale_m)
        fd = (lp - lm) / (2 * H * t0)  # d/dT0 from a relative perturbation
        mask = ok & (ip == base_its) & (im == base_its) & (np.abs(t0) > 1e-40)
        sc = max(np.abs(fd[mask]).max(), 1e-300)
        assert np.max(np.abs(g["dL_dtotal0"][j, mask] - fd[mask])) / sc < 1e-4, j


def test_autograd_function_matches_adjoint(adjoint_case):
    """The autograd wrapper returns exactly what pf_adjoint returns for the
    same inputs and the same upstream gradient (up to the run-dependent
    order of the atomic cell sums), and leaves the network unshifted."""
    from pfgpu.autograd import rstep_totals
    net, st0, eng, w, tgt, g = adjoint_case
    dev = st0.to("cuda")
    ns, nm = net.nsec, net.nmnrl
    z = lambda n: torch.zeros(n, dtype=torch.float64, device="cuda", requires_grad=True)  # noqa: E731
    dks, dkm, dlnk = z(ns), z(nm), z(nm)
    lnarea = torch.log(dev.a["mnrl_area"]).clone().requires_grad_(True)
    total0 = dev.a["total"].clone().requires_grad_(True)
    Tf = rstep_totals(eng, dev, DT, dks, dkm, dlnk, lnarea, total0)
    W, TG = torch.from_numpy(w).cuda(), torch.from_numpy(tgt).cuda()
    loss = (W * (Tf - TG) ** 2).sum()
    loss.backward()
    # exp(log(area)) differs from area by an ulp: the loss agrees to the
    # solver tolerance, not bitwise
    assert float(loss.detach()) == pytest.approx(float(g["loss"][0]), rel=1e-8)
    same = dev.copy()
    same.a["mnrl_area"].copy_(torch.exp(lnarea.detach()))
    ref = eng.adjoint(same, DT, dL_dtotal=(2.0 * W * (Tf.detach() - TG)).contiguous())
    ref = {k: v.cpu().numpy() for k, v in ref.items()}
    assert _rel(dks.grad.cpu().numpy(), ref["dL_dlogK_sec"]) < 1e-9
    assert _rel(dkm.grad.cpu().numpy(), ref["dL_dlogK_mnrl"]) < 1e-9
    assert _rel(dlnk.grad.cpu().numpy(), ref["dL_dlnk"]) < 1e-9
    np.testing.assert_array_equal(lnarea.grad.cpu().numpy(), ref["dL_dlnarea"])
    np.testing.assert_array_equal(total0.grad.cpu().numpy(), ref["dL_dtotal0"])
    # the forward and backward calls restore the network's parameters
    after, _ = _gpu_loss(eng, st0, w, tgt)
    before = g["loss"][0]
    assert after.sum() == pytest.approx(before, rel=1e-12)


@pytest.mark.parametrize("lanes", [4, 8])
def test_group_adjoint_matches_one_lane(oracle, lanes):
    """The group kernel's adjoint and the one-lane kernel's agree per cell
    wherever the two forward solves took the same Newton path."""
    from pfgpu.engine import ReactionEngine
    net, st0 = cases.case(oracle, "random12")
    st0 = st0.subset(np.arange(1000))
    rng = np.random.default_rng(5)
    w = torch.from_numpy(rng.uniform(0, 1, st0.a["total"].shape)).cuda()
    tgt = torch.from_numpy(st0.a["total"] * np.exp(0.05 * rng.standard_normal(st0.a["total"].shape))).cuda()
    out = []
    for g in (1, lanes):
        eng = ReactionEngine(net)
        if g > 1:
            assert eng.set_launch_config(128, 2, 0, g) == abi.PF_OK
        dev = st0.to("cuda")
        gr = eng.adjoint(dev, 86400.0, weight=w, target=tgt)
        out.append(({k: v.cpu().numpy() for k, v in gr.items()}, dev.numpy()))
    (g1, s1), (g2, s2) = out
    same = (s1.a["newton_its"] == s2.a["newton_its"]) & (g1["adj_status"] == 0) & (g2["adj_status"] == 0)
    assert same.mean() > 0.95
    for k in ("dL_dtotal0", "dL_dlnarea"):
        a, b = g1[k][:, same], g2[k][:, same]
        assert np.max(np.abs(a - b)) <= 1e-8 * max(np.max(np.abs(a)), 1e-300), k
    assert g2["loss"][0] == pytest.approx(g1["loss"][0], rel=1e-9)


@pytest.mark.parametrize("lanes", [1, 4], ids=["lane", "group4"])
def test_adjoint_default_tolerances_vs_fd(oracle, lanes):
    """The adjoint at the solver's default tolerances, the ones the
    differentiation bench runs at (relative change 1e-6, residual 1e-12 and
    relative residual 1e-8, 20 iterations), on the 12-component network at
    dt = 1 day.  It differentiates the iterate where RReact stopped, which is
    within about the last Newton update (1e-6 relative in the molalities) of
    the root; the quantity it stands for is the gradient of the converged
    step.  So the reference here is central differences of the converged
    forward map (the same network and cells at the tight tolerances), and the
    bar is 1e-3 of the largest gradient of a group on the gradients summed
    over cells (logK of every complex and mineral, ln rate constants) and on
    the per-cell area gradients.  (Differences of the default-tolerance map
    itself measure where the stopping tests fire: a complex's logK moves the
    stopping point, and with it the totals by up to the stopped update, while
    the converged totals do not depend on it.)"""
    global DT, CASE
    DT, CASE = DTS["random12"], "random12"
    net, st0, eng, w, tgt = _setup(oracle, "random12", lanes, tight=False)
    net_t, st_t = cases.case(oracle, "random12", tight=True)
    st_t = st_t.subset(np.arange(st0.ncells))
    assert np.array_equal(st_t.a["total"], st0.a["total"])
    from pfgpu.engine import ReactionEngine
    eng_t = ReactionEngine(net_t)
    dev = st0.to("cuda")
    g = eng.adjoint(dev, DT, weight=torch.from_numpy(w).cuda(), target=torch.from_numpy(tgt).cuda())
    g = {k: v.cpu().numpy() for k, v in g.items()}
    lossfn = lambda **kw: _gpu_loss(eng_t, st0, w, tgt, **kw)  # noqa: E731
    _check_global(net, st0, eng, w, tgt, g, lossfn, rel=1e-3)
    ok = g["adj_status"] == 0
    base_l, base_its = lossfn()
    for m in range(net.nmnrl):
        sp = np.ones_like(st0.a["mnrl_area"])
        sp[m] = np.exp(H)
        sm = np.ones_like(st0.a["mnrl_area"])
        sm[m] = np.exp(-H)
        lp, ip = lossfn(area_scale=sp)
        lm, im = lossfn(area_scale=sm)
        fd = (lp - lm) / (2 * H)
        mask = ok & (ip == base_its) & (im == base_its)
        sc = max(np.abs(fd[mask]).max(), 1e-300)
        assert np.max(np.abs(g["dL_dlnarea"][m, mask] - fd[mask])) / sc < 1e-3, m
