"""Equilibrium sorption on the GPU (K_D isotherms and ion exchange in RTotal,
with the sorbed accumulation of RReact) against the oracle: the auxvar
update, constraint equilibration and the operator-split step (one-lane
batched kernel), and the entry points that refuse a network with sorption.
The global-implicit assembly with sorption is in test_gpu_girt.py."""
import numpy as np
import pytest

from pfgpu import abi
from pfgpu.network import CellState, ReactionNetwork, default_options

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# six primaries: a component count the batched kernel is compiled for
PRIMARY = ["Na+", "Ca++", "K+", "Cl-", "Tr", "Mg++"]
Z = [1.0, 2.0, 1.0, -1.0, 0.0, 2.0]
A0 = [4.0, 6.0, 3.0, 3.0, 3.0, 8.0]
SECS = [dict(name="NaCl(aq)", stoich={"Na+": 1.0, "Cl-": 1.0}, logK=0.5, Z=0.0, a0=3.0),
        dict(name="CaCl+", stoich={"Ca++": 1.0, "Cl-": 1.0}, logK=-0.4, Z=1.0, a0=4.0)]
MINS = [dict(name="Sylvite-like", stoich={"K+": 1.0, "Cl-": 1.0}, logK=-2.0, rate=1e-8, molar_vol=3.7e-5)]


def _net(sorption, minerals=True, options=None):
    net = ReactionNetwork.build(PRIMARY, Z, A0, SECS, MINS if minerals else [],
                                options=options or default_options())
    net.sorption = sorption
    return net


SORB = dict(kd=[dict(species="Tr", type="langmuir", coeff=80.0, b=3.0)],
            ionx=[dict(cations=[("Na+", 1.0), ("Ca++", 0.3), ("K+", 5.0), ("Mg++", 0.4)], cec=250.0)])
SORB_MIN = dict(kd=[dict(species="Tr", type="freundlich", coeff=20.0, n=1.5, mineral="Sylvite-like")],
                ionx=[dict(cations=[("Na+", 1.0), ("K+", 3.0)], cec=4000.0, mineral="Sylvite-like")])


def _cells(oracle, net, ncells, seed):
    rng = np.random.default_rng(seed)
    st = CellState.empty(net, ncells)
    st.a["pri_molal"][:] = 10.0 ** rng.uniform(-4.0, -2.0, (net.ncomp, ncells))
    st.a["porosity"][:] = rng.uniform(0.2, 0.4, ncells)
    st.a["den_kg"][:] = 997.0
    if net.nmnrl:
        st.a["mnrl_volfrac"][:] = rng.uniform(0.01, 0.1, (net.nmnrl, ncells))
        st.a["mnrl_area"][:] = rng.uniform(1.0, 50.0, (net.nmnrl, ncells))
    oracle.update_auxvars(net, st, False)
    oracle.update_activity_coefs(net, st)
    oracle.update_auxvars(net, st, False)
    # a disturbance of the aqueous totals, as transport would make
    st.a["total"][:] *= rng.uniform(0.7, 1.3, st.a["total"].shape)
    return st


@pytest.mark.parametrize("sorb", ["ionx+langmuir", "mineral-scaled"])
def test_auxvars_with_sorption_match_oracle(oracle, sorb):
    from pfgpu.engine import ReactionEngine
    net = _net(SORB if sorb == "ionx+langmuir" else SORB_MIN)
    st = _cells(oracle, net, 500, 1)
    ref = st.copy()
    oracle.update_auxvars(net, ref, True)
    dev = st.to("cuda")
    ReactionEngine(net).update_auxvars(dev, True)
    got = dev.numpy()
    for k in ("total", "total_sorb", "ionx_ref_sorbed", "sec_molal", "pri_act_coef"):
        np.testing.assert_allclose(got.a[k], ref.a[k], rtol=1e-12, atol=0, err_msg=k)


@pytest.mark.parametrize("kernel", ["batched", "group2", "group4", "plain"])
@pytest.mark.parametrize("sorb", ["ionx+langmuir", "mineral-scaled"])
def test_rstep_with_sorption_matches_oracle(oracle, sorb, kernel):
    from pfgpu.engine import ReactionEngine
    net = _net(SORB if sorb == "ionx+langmuir" else SORB_MIN)
    st = _cells(oracle, net, 800, 2)
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    eng = ReactionEngine(net)
    if kernel.startswith("group"):
        # a group of lanes per cell: one lane runs the sorption routine into
        # the rows of the pivoted LU
        assert eng.set_launch_config(128, 2, 0, int(kernel[5:])) == abi.PF_OK
    dev = st.to("cuda")
    eng.rstep(dev, 86400.0, kernel=abi.PF_KERNEL_PLAIN if kernel == "plain" else abi.PF_KERNEL_BATCHED)
    got = dev.numpy()
    ok = (got.a["newton_its"] == ref.a["newton_its"]) & (ref.a["status"] == 0) & (got.a["status"] == 0)
    assert ok.mean() > 0.9, (ok.mean(), (ref.a["status"] != 0).sum())
    for k in ("pri_molal", "total", "total_sorb", "mnrl_volfrac", "ionx_ref_sorbed"):
        a, b = got.a[k][:, ok], ref.a[k][:, ok]
        scale = np.maximum(np.abs(b), 1e-300)
        assert np.max(np.abs(a - b) / scale) < 1e-10, (k, np.max(np.abs(a - b) / scale))
    # aqueous + sorbed mass moved only by the mineral: conserved components
    # (Ca++ and the tracer, not in the mineral) keep psv*T + V*S
    psv = st.a["porosity"] * st.a["saturation"] * 1000.0 * st.a["volume"]
    for j in (1, 4):
        before = psv * st.a["total"][j] + st.a["volume"] * st.a["total_sorb"][j]
        after = psv * got.a["total"][j] + got.a["volume"] * got.a["total_sorb"][j]
        assert np.max(np.abs(after[ok] - before[ok]) / before[ok]) < 1e-5


def test_host_path_with_sorption_equals_device_path(oracle):
    from pfgpu.engine import ReactionEngine
    net = _net(SORB)
    st = _cells(oracle, net, 300, 3)
    eng = ReactionEngine(net)
    dev = st.to("cuda")
    eng.rstep(dev, 3600.0)
    host = st.copy()
    eng.rstep_host(host, 3600.0)
    got = dev.numpy()
    for k in ("pri_molal", "total", "total_sorb", "ionx_ref_sorbed"):
        np.testing.assert_array_equal(host.a[k], got.a[k], err_msg=k)


def test_constraint_with_sorption_matches_oracle(oracle):
    from pfgpu.engine import ReactionEngine
    net = _net(SORB, minerals=False)
    n = 400
    st = CellState.empty(net, n)
    rng = np.random.default_rng(4)
    st.a["den_kg"][:] = 997.0
    st.a["porosity"][:] = 0.3
    cconc = 10.0 ** rng.uniform(-4.0, -2.0, (net.ncomp, n))
    ctype = [abi.PF_CONSTRAINT_TOTAL] * net.ncomp
    ctype[3] = abi.PF_CONSTRAINT_CHARGE_BAL
    cconc[3] = 1e-3
    ref = st.copy()
    rc, its_ref = oracle.equilibrate(net, ref, ctype, cconc, nthreads=8)
    dev = st.to("cuda")
    its = ReactionEngine(net).equilibrate(dev, ctype, torch.from_numpy(cconc).cuda()).cpu().numpy()
    got = dev.numpy()
    ok = (its == its_ref) & (its_ref > 0)
    assert ok.mean() > 0.9
    for k in ("pri_molal", "total_sorb", "ionx_ref_sorbed"):
        a, b = got.a[k][:, ok], ref.a[k][:, ok]
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)) < 1e-10, k


def test_five_components_run_on_the_plain_kernel(oracle):
    """A component count without a batched instantiation: the plain kernel
    carries sorption as well."""
    from pfgpu.engine import ReactionEngine
    net = ReactionNetwork.build(PRIMARY[:5], Z[:5], A0[:5], SECS, MINS, options=default_options())
    net.sorption = dict(kd=[dict(species="Tr", coeff=50.0)],
                        ionx=[dict(cations=[("Na+", 1.0), ("Ca++", 0.3), ("K+", 5.0)], cec=250.0)])
    st = _cells(oracle, net, 400, 6)
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    dev = st.to("cuda")
    ReactionEngine(net).rstep(dev, 86400.0, kernel=abi.PF_KERNEL_PLAIN)
    got = dev.numpy()
    ok = (got.a["newton_its"] == ref.a["newton_its"]) & (ref.a["status"] == 0)
    assert ok.mean() > 0.9
    for k in ("pri_molal", "total_sorb"):
        a, b = got.a[k][:, ok], ref.a[k][:, ok]
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)) < 1e-10, k


def test_sorption_launches_and_refusals(oracle):
    from pfgpu.engine import ReactionEngine
    net = _net(SORB)
    st = _cells(oracle, net, 16, 5)
    eng = ReactionEngine(net)
    dev = st.to("cuda")
    assert eng.set_launch_config(128, 1, 0, 4) == abi.PF_OK  # the group kernel carries sorption
    assert eng.set_launch_config(128, 1, 1, 1) == abi.PF_OK
    # the adjoint has no sorption terms
    with pytest.raises(abi.PfError) as e:
        eng.adjoint(dev, 3600.0, dL_dtotal=torch.ones_like(dev.a["total"]))
    assert e.value.code == abi.PF_ERR_UNSUPPORTED
    # a state without the sorption arrays is an invalid argument
    bare = CellState(net, {k: v for k, v in dev.a.items() if k not in ("total_sorb", "ionx_ref_sorbed")})
    with pytest.raises(abi.PfError):
        eng.rstep(bare, 3600.0)
