"""Adjoint of the operator-split step (pf_adjoint) against central finite
differences, step 1e-6 in log space, of
  (a) the GPU forward pass (pf_rstep, batched kernel), and
  (b) the CPU oracle (the restatement of the reference's RStep),
for every parameter group: logK shifts of all complexes and kinetic minerals,
ln rate constants, per-cell ln areas and per-cell initial totals.

Loss: sum over cells of w*(total_final - target)^2, w ~ U[0,1], target = the
forward output perturbed by 5 % lognormal noise (the differentiation case of
the benchmark).  Tolerances: FD truncation is O(h^2) ~ 1e-12 and the tight
solver tolerance (relative update < 1e-10) bounds FD noise; the comparison
allows 1e-4 relative on summed gradients and 1e-4 on per-cell gradients
(reported maxima are far smaller).
"""
import numpy as np
import pytest

import cases
from pfgpu import abi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-6
DT = 86400.0


def _setup(oracle, ncells=240):
    net, st0 = cases.case(oracle, "random12", tight=True)
    st0 = st0.subset(np.arange(ncells))
    from pfgpu.engine import ReactionEngine
    eng = ReactionEngine(net)
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
    """Central differences of the summed loss for every network parameter."""
    out = {"dL_dlogK_sec": np.zeros(ns), "dL_dlogK_mnrl": np.zeros(nm), "dL_dlnk": np.zeros(nm)}
    for k in range(ns):
        lp, _ = lossfn(shift=(_unit(k, ns, H), None, None))
        lm, _ = lossfn(shift=(_unit(k, ns, -H), None, None))
        out["dL_dlogK_sec"][k] = (lp.sum() - lm.sum()) / (2 * H)
    for k in range(nm):
        lp, _ = lossfn(shift=(None, _unit(k, nm, H), None))
        lm, _ = lossfn(shift=(None, _unit(k, nm, -H), None))
        out["dL_dlogK_mnrl"][k] = (lp.sum() - lm.sum()) / (2 * H)
        lp, _ = lossfn(shift=(None, None, _unit(k, nm, H)))
        lm, _ = lossfn(shift=(None, None, _unit(k, nm, -H)))
        out["dL_dlnk"][k] = (lp.sum() - lm.sum()) / (2 * H)
    return out


def _rel(a, b):
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


@pytest.fixture(scope="module")
def adjoint_case(oracle):
    net, st0, eng, w, tgt = _setup(oracle)
    dev = st0.to("cuda")
    g = eng.adjoint(dev, DT, weight=torch.from_numpy(w).cuda(), target=torch.from_numpy(tgt).cuda())
    g = {k: v.cpu().numpy() for k, v in g.items()}
    return net, st0, eng, w, tgt, g


def test_adjoint_status_and_loss(adjoint_case):
    net, st0, eng, w, tgt, g = adjoint_case
    assert (g["adj_status"] == 0).mean() > 0.95
    base, _ = _gpu_loss(eng, st0, w, tgt)
    assert g["loss"][0] == pytest.approx(base.sum(), rel=1e-12)


def test_adjoint_global_vs_fd_gpu(adjoint_case):
    net, st0, eng, w, tgt, g = adjoint_case
    fd = _fd_global(lambda **kw: _gpu_loss(eng, st0, w, tgt, **kw), net.nsec, net.nmnrl)
    for k, v in fd.items():
        assert _rel(g[k], v) < 1e-4, (k, _rel(g[k], v))


def test_adjoint_global_vs_fd_oracle(adjoint_case, oracle):
    net, st0, eng, w, tgt, g = adjoint_case
    fd = _fd_global(lambda **kw: _oracle_loss(oracle, net, st0, w, tgt, **kw), net.nsec, net.nmnrl)
    for k, v in fd.items():
        assert _rel(g[k], v) < 1e-4, (k, _rel(g[k], v))


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
    assert float(loss) == pytest.approx(float(g["loss"][0]), rel=1e-12)
    assert _rel(dks.grad.cpu().numpy(), g["dL_dlogK_sec"]) < 1e-10
    assert _rel(dkm.grad.cpu().numpy(), g["dL_dlogK_mnrl"]) < 1e-10
    assert _rel(dlnk.grad.cpu().numpy(), g["dL_dlnk"]) < 1e-10
    assert _rel(lnarea.grad.cpu().numpy(), g["dL_dlnarea"]) < 1e-10
    assert _rel(total0.grad.cpu().numpy(), g["dL_dtotal0"]) < 1e-10
