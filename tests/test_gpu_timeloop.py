"""The operator-split time loop captured in one CUDA graph gives, bit for bit,
the results of the same steps run eagerly (RTUpdateAuxVars, the TIMESTEP
activity update and RStep per network per step, pm_osrt.F90:115-153), for
two networks of different size in one graph, sequential or on concurrent
per-network streams, with or without the transport solve before the
reaction step (pmc_subsurface_osrt.F90:259-330)."""
import numpy as np
import pytest

import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_volfrac", "mnrl_rate",
          "status", "newton_its", "num_substeps")


def _members(oracle):
    from pfgpu.engine import ReactionEngine
    out = []
    for name, n in (("hetero4", 400), ("random12", 600)):
        net, st = cases.case(oracle, name)
        st = st.subset(np.arange(min(n, st.ncells)))
        out.append((ReactionEngine(net), st))
    return out


def _run(members, eager_steps, graph_steps, concurrent, stages=None):
    from pfgpu.timeloop import OperatorSplitLoop
    devs = [(eng, st.to("cuda")) for eng, st in members]
    stages = stages or [None] * len(devs)
    loop = OperatorSplitLoop([(e, s, t) for (e, s), t in zip(devs, stages)], dt=86400.0, concurrent=concurrent)
    for _ in range(eager_steps):
        loop.step()
    if graph_steps:
        loop.capture(graph_steps)
        torch.cuda.synchronize()
        loop.replay()
    torch.cuda.synchronize()
    return [st.numpy() for _, st in devs], loop


@pytest.mark.parametrize("concurrent", [False, True], ids=["sequential", "concurrent"])
def test_graph_equals_eager(oracle, concurrent):
    members = _members(oracle)
    ref, _ = _run(members, 4, 0, False)
    got, loop = _run(members, 1, 3, concurrent)
    for a, b in zip(ref, got):
        for k in FIELDS:
            np.testing.assert_array_equal(a.a[k], b.a[k], err_msg=k)
    s = loop.summary()
    assert len(s) == 2 and all(m["cells"] > 0 for m in s)


def test_capture_leaves_state_untouched(oracle):
    from pfgpu.timeloop import OperatorSplitLoop
    members = _members(oracle)
    devs = [(eng, st.to("cuda")) for eng, st in members]
    loop = OperatorSplitLoop(devs, dt=86400.0)
    loop.step()
    torch.cuda.synchronize()
    before = [{k: st.a[k].clone() for k in FIELDS} for _, st in devs]
    loop.capture(2)
    torch.cuda.synchronize()
    for (_, st), b in zip(devs, before):
        for k in FIELDS:
            assert torch.equal(st.a[k], b[k]), k


def test_loop_requires_dt(oracle):
    from pfgpu.engine import ReactionEngine
    from pfgpu.timeloop import OperatorSplitLoop
    net, st = cases.case(oracle, "calcite")
    with pytest.raises(ValueError):
        OperatorSplitLoop([(ReactionEngine(net), st.subset(np.arange(8)).to("cuda"))], dt=0.0)


def _transport_stages(members):
    """A structured grid per member (ncells = nx*ny*nz) and a fixed schedule
    from an adaptive step."""
    from pfgpu.girt import StructuredGrid
    from pfgpu.timeloop import TransportStage
    from pfgpu.transport import OSTransport
    stages = []
    for k, (eng, st) in enumerate(members):
        N = st.ncells
        nz = max(z for z in range(1, 9) if N % z == 0)
        ny = max(y for y in range(1, 17) if (N // nz) % y == 0)
        nx = N // (nz * ny)
        rng = np.random.default_rng(70 + k)

        def q(shape):
            return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
        grid = StructuredGrid(nx, ny, nz, 1.0, 1.0, 1.0, q((nz, ny, nx - 1)), q((nz, ny - 1, nx)),
                              q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=1.0, dispersivity=0.0)
        solver = OSTransport(grid, eng.net.ncomp)
        dev = st.to("cuda")
        stats = solver.step(dev, 86400.0)
        inner, refs = OSTransport.schedule(stats)
        stages.append(TransportStage(solver, inner + 4, refs + 1))
    return stages


@pytest.mark.parametrize("concurrent", [False, True], ids=["sequential", "concurrent"])
def test_graph_with_transport_equals_eager(oracle, concurrent):
    members = _members(oracle)
    for _, st in members:
        st.a.pop("dt_cell", None)
    stages = _transport_stages(members)
    ref, _ = _run(members, 4, 0, False, stages)
    got, loop = _run(members, 1, 3, concurrent, stages)
    for a, b in zip(ref, got):
        for k in FIELDS:
            np.testing.assert_array_equal(a.a[k], b.a[k], err_msg=k)
    s = loop.summary()
    assert all(m["transport"]["converged"] == 1 for m in s), s
    # the transport moved the totals: the run differs from a reaction-only one
    plain, _ = _run(members, 4, 0, False)
    assert any(not np.array_equal(a.a["total"], b.a["total"]) for a, b in zip(ref, plain))
