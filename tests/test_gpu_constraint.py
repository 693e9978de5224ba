"""GPU constraint equilibration and auxvar kernels against the oracle and the
reference's own speciation gold values (regression_tests/ascem/batch)."""
import math

import numpy as np
import pytest

import kat
from pfgpu import abi, generate
from pfgpu.network import default_options

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _engine(net):
    from pfgpu.engine import ReactionEngine
    return ReactionEngine(net)


@pytest.mark.parametrize("name", ["calcite", "random12", "hetero20"])
def test_equilibrate_parity(oracle, name):
    if name == "calcite":
        net = generate.calcite_network()
        st, ct, cc = generate.calcite_cells(net, 1000, seed=5)
    elif name == "random12":
        net = generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
        st, ct, cc = generate.random_cells(net, 1000, seed=99)
    else:
        net = generate.random_network(20, 60, 10, seed=720, options=default_options(isothermal=0))
        st, ct, cc = generate.random_cells(net, 500, seed=98)
    ref = st.copy()
    rc, its_ref = oracle.equilibrate(net, ref, ct, cc, nthreads=8)
    eng = _engine(net)
    dev = st.to("cuda")
    its = eng.equilibrate(dev, ct, torch.from_numpy(cc).cuda()).cpu().numpy()
    got = dev.numpy()
    # identical Newton paths agree to 1e-10; a path that flipped on a
    # rounding-level test still lands within the constraint tolerance
    ok = (its_ref > 0) & (its == its_ref)
    assert ok.mean() > 0.85, (ok.mean(), (its != its_ref).sum())
    e = np.max(np.abs(got.a["pri_molal"][:, ok] - ref.a["pri_molal"][:, ok]) / ref.a["pri_molal"][:, ok])
    assert e < 1e-10, e
    both = (its_ref > 0) & (its > 0)
    assert both.mean() > 0.97
    tot_scale = np.abs(ref.a["total"][:, both]) + ref.a["pri_molal"][:, both]
    assert np.max(np.abs(got.a["total"][:, both] - ref.a["total"][:, both]) / tot_scale) < 1e-5
    np.testing.assert_allclose(got.a["pri_act_coef"][:, ok], ref.a["pri_act_coef"][:, ok], rtol=1e-10)


def test_update_auxvars_parity(oracle):
    net = generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
    st, ct, cc = generate.random_cells(net, 800, seed=3)
    oracle.equilibrate(net, st, ct, cc, nthreads=8)
    for act in (False, True):
        ref = st.copy()
        oracle.update_auxvars(net, ref, act)
        eng = _engine(net)
        dev = st.to("cuda")
        eng.update_auxvars(dev, act)
        got = dev.numpy()
        np.testing.assert_allclose(got.a["sec_molal"], ref.a["sec_molal"], rtol=1e-12)
        np.testing.assert_allclose(got.a["pri_act_coef"], ref.a["pri_act_coef"], rtol=1e-13)
        scale = np.abs(ref.a["pri_molal"]) + np.abs(ref.a["total"])
        assert np.max(np.abs(got.a["total"] - ref.a["total"]) / scale) < 1e-12


@pytest.mark.parametrize("algo", [abi.PF_ACT_COEF_ALGO_LAG, abi.PF_ACT_COEF_ALGO_NEWTON])
def test_activity_coefs_parity(oracle, algo):
    net = generate.calcite_network(default_options(act_coef_update_algorithm=algo))
    st, ct, cc = generate.calcite_cells(net, 500, seed=11)
    oracle.equilibrate(net, st, ct, cc, nthreads=8)
    ref = st.copy()
    oracle.update_activity_coefs(net, ref)
    eng = _engine(net)
    dev = st.to("cuda")
    eng.update_activity_coefs(dev)
    got = dev.numpy()
    np.testing.assert_allclose(got.a["pri_act_coef"], ref.a["pri_act_coef"], rtol=1e-12)
    np.testing.assert_allclose(got.a["sec_act_coef"], ref.a["sec_act_coef"], rtol=1e-12)


@pytest.mark.parametrize("name", kat.kat_names("speciation"))
def test_speciation_kat_on_gpu(name):
    """The reference's speciation gold values reproduced entirely on the GPU:
    constraint equilibration, then the initial auxvar sequence."""
    fx = kat.KAT[name]
    net = kat.network(fx, tight=False)
    den = generate.water_density(25.0)
    from pfgpu.network import CellState
    st = CellState.empty(net, 1)
    st.a["porosity"][:] = fx["porosity"]
    st.a["den_kg"][:] = den
    ctype = [kat.CON[fx["constraint"][s][0]] for s in net.primary]
    cconc = np.array([[fx["constraint"][s][1]] for s in net.primary])
    eng = _engine(net)
    dev = st.to("cuda")
    its = eng.equilibrate(dev, ctype, torch.from_numpy(cconc).cuda())
    assert int(its[0]) > 0
    dev.a["pri_molal"].copy_(dev.a["pri_molal"] * den / 1000.0 / den * 1000.0)
    dev.a["pri_act_coef"].fill_(1.0)
    dev.a["sec_act_coef"].fill_(1.0)
    dev.a["sec_molal"].fill_(0.0)
    eng.update_auxvars(dev, False)
    if net.options["act_coef_update_frequency"] != abi.PF_ACT_COEF_OFF:
        eng.update_auxvars(dev, True)
        eng.update_auxvars(dev, True)
    out = kat.outputs(fx, net, dev.numpy())
    for key, gold in fx["gold"].items():
        if key in ("Time Steps", "Newton Iterations"):
            continue
        assert out[key] == pytest.approx(gold, abs=1e-12), (key, out[key], gold)
