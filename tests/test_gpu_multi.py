"""pf_rstep_multi: the cells of several networks in one persistent launch.

Each cell's step in the multi-network launch is the group-per-cell kernel's
step with the same group size (the same device routine on the same tables,
scratch and work queue), so the results must be bit for bit those of one
single-network launch per network, with equal statistics, whatever the order
of the networks and of the cells; and they meet the parity bar of
tests/parity.py against the oracle.  The time loop runs it inside a CUDA
graph, replay equal to the eager steps.  A network the group kernel does not
carry makes the call refuse."""
import pytest

import cases
import parity
from pfgpu import abi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_rate", "mnrl_volfrac",
          "newton_its", "status", "num_substeps")


def same(x, y):
    """Equal element for element, a NaN equal to a NaN: a cell that failed
    keeps its last non-converged iterate, and the next step's auxvar update
    can turn that into NaN in both runs alike (torch.equal calls two NaN
    different)."""
    return x.shape == y.shape and bool(((x == y) | (torch.isnan(x) & torch.isnan(y))).all())


def _members(oracle, names=None):
    from pfgpu.engine import ReactionEngine
    names = names or ["hetero%d" % n for n in reversed(cases.HETERO)]  # costliest first
    out = []
    for name in names:
        net, st0 = cases.case(oracle, name)
        out.append((name, ReactionEngine(net), net, st0))
    return out


def _lanes(eng):
    from pfgpu.engine import ReactionEngine  # noqa: F401
    g = eng.launch_config()["lanes_per_cell"]
    if g in (4, 8):
        return g
    return 4 if eng.set_launch_config(128, 2, 0, 4) == abi.PF_OK else 8


def test_multi_equals_single_launches_and_oracle(oracle):
    from pfgpu.engine import ReactionEngine, rstep_multi
    mem = _members(oracle)
    devs = [st0.to("cuda") for _, _, _, st0 in mem]
    stats = rstep_multi([(eng, d) for (_, eng, _, _), d in zip(mem, devs)], 86400.0)
    torch.cuda.synchronize()
    for (name, eng, net, st0), d, sm in zip(mem, devs, stats):
        one = ReactionEngine(net)
        G = _lanes(eng)
        assert one.set_launch_config(128, 2, 0, G) == abi.PF_OK
        ref_dev = st0.to("cuda")
        s1 = one.rstep(ref_dev, 86400.0)
        for k in FIELDS:
            assert same(d.a[k], ref_dev.a[k]), (name, k)
        assert sm == s1, (name, sm, s1)
        got = d.numpy()
        ref = st0.copy()
        oracle.rstep(net, ref, 86400.0, nthreads=8)
        entry, _ = parity.compare(net, ref, got, 86400.0, "multi/" + name, [])
        assert entry["max_rel_err"]["pri_molal"] < parity.REL, (name, entry)


def test_multi_order_of_networks_and_cells_does_not_change_results(oracle):
    from pfgpu.engine import rstep_multi
    mem = _members(oracle, ["hetero12", "hetero6", "hetero20"])
    a = [st0.to("cuda") for _, _, _, st0 in mem]
    rstep_multi([(eng, d) for (_, eng, _, _), d in zip(mem, a)], 86400.0)
    b = [st0.to("cuda") for _, _, _, st0 in mem]
    orders = [torch.randperm(d.ncells, device="cuda", generator=torch.Generator("cuda").manual_seed(k))
              for k, d in enumerate(b)]
    rev = list(reversed(range(len(mem))))
    rstep_multi([(mem[k][1], b[k]) for k in rev], 86400.0, orders=[orders[k] for k in rev])
    for (name, _, _, _), x, y in zip(mem, a, b):
        for k in FIELDS:
            assert same(x.a[k], y.a[k]), (name, k)


def test_multi_time_loop_graph_equals_eager(oracle):
    from pfgpu.timeloop import OperatorSplitLoop
    mem = _members(oracle, ["hetero16", "hetero8", "hetero4"])
    eager = [st0.to("cuda") for _, _, _, st0 in mem]
    loop_e = OperatorSplitLoop([(eng, d) for (_, eng, _, _), d in zip(mem, eager)], dt=86400.0, multi=True)
    for _ in range(3):
        loop_e.step()
    graphed = [st0.to("cuda") for _, _, _, st0 in mem]
    loop_g = OperatorSplitLoop([(eng, d) for (_, eng, _, _), d in zip(mem, graphed)], dt=86400.0, multi=True)
    loop_g.step()  # eager warm step, as capture() asks
    snap = [{k: v.clone() for k, v in d.a.items()} for d in graphed]
    loop_g.capture(2)
    for d, sn in zip(graphed, snap):
        for k, v in sn.items():
            d.a[k].copy_(v)
    loop_g.replay()
    torch.cuda.synchronize()
    for (name, _, _, _), x, y in zip(mem, eager, graphed):
        for k in FIELDS:
            assert same(x.a[k], y.a[k]), (name, k)


def test_multi_refuses_networks_without_a_group_kernel(oracle):
    """The linear formulation has no group kernel (its Jacobian is not the
    symmetric log-form one the group kernel assembles)."""
    from pfgpu.engine import ReactionEngine, rstep_multi
    (_, e2, net, s2), = _members(oracle, ["hetero8"])
    eng = ReactionEngine(net.with_options(use_log_formulation=0))
    with pytest.raises(abi.PfError) as e:
        rstep_multi([(e2, s2.to("cuda")), (eng, s2.to("cuda"))], 3600.0)
    assert e.value.code == abi.PF_ERR_UNSUPPORTED


def test_multi_with_sorption_equals_single_launch(oracle):
    """A network with equilibrium sorption (ion exchange and a Langmuir K_D)
    among others in one launch: bit for bit its own group launch."""
    from pfgpu.engine import ReactionEngine, rstep_multi
    net, st, grid, total_k, sorb_k = cases.girt_sorption_case(oracle, "ionx+langmuir", 8, 6, 5)
    eng = ReactionEngine(net)
    (_, e2, _, s2), = _members(oracle, ["hetero12"])
    a, b = st.to("cuda"), s2.to("cuda")
    rstep_multi([(e2, b), (eng, a)], 86400.0)
    one = ReactionEngine(net)
    assert one.set_launch_config(128, 2, 0, _lanes(eng)) == abi.PF_OK
    ref = st.to("cuda")
    one.rstep(ref, 86400.0)
    for k in FIELDS + ("total_sorb", "ionx_ref_sorbed"):
        assert same(a.a[k], ref.a[k]), k
