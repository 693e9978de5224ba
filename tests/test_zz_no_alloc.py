"""pf_rstep_noalloc: the batched step for callers that may not allocate device
memory during the call (their GPU memory belongs to another framework's pool,
or their footprint is fixed up front).  Its scratch is a fixed array inside
the library, shared by every call, so each case here makes two calls in a
row -- the second reusing whatever the first left in that array -- and
checks them against the allocating entry point pf_rstep on the same launch
configuration.  The kernels, the launch and the per-cell arithmetic are the
same (only the scratch's address differs, and a cell's result does not
depend on where or when it is scheduled), so every field must agree bit for
bit, and the step statistics must be equal.  Cases: the default one-lane
launch of the 12-component network, a group of 4 lanes per cell on the same
network, and a 5-component network that has no one-lane kernel (its default
launch is a group).  Kept last in collection order so a failure here does
not hide other tests.
"""
import ctypes as C

import pytest

from pfgpu import abi, generate
from pfgpu.network import default_options

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_rate", "mnrl_volfrac",
          "newton_its", "status", "num_substeps")


def _state(net, ncells, seed):
    from pfgpu.engine import ReactionEngine
    st, ct, cc = generate.random_cells(net, ncells, seed=seed)
    eng = ReactionEngine(net)
    dev = st.to("cuda")
    its = eng.equilibrate(dev, ct, torch.from_numpy(cc).cuda())
    good = torch.nonzero(its > 0).flatten()
    dev = dev.subset(good)
    eng.update_auxvars(dev, True)
    torch.cuda.synchronize()
    return eng, dev


def _noalloc(eng, dev, dt):
    s = dev.struct()
    stats = abi.PfStepStats()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = eng.lib.pf_rstep_noalloc(eng.handle, C.byref(s), dt, stream, C.byref(stats))
    assert rc in (abi.PF_OK, abi.PF_CELL_FAILURES), rc
    torch.cuda.synchronize()
    return {k: getattr(stats, k) for k, _ in abi.PfStepStats._fields_}


def _net(ncomp):
    if ncomp == 12:
        return generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
    return generate.random_network(ncomp, 3 * ncomp, max(1, ncomp // 2), seed=900 + ncomp,
                                   options=default_options(isothermal=0))


@pytest.mark.parametrize("ncomp,lanes", [(12, None), (12, 4), (5, None)], ids=["n12-one-lane", "n12-group4", "n5-default"])
def test_noalloc_matches_allocating_step_twice(ncomp, lanes):
    net = _net(ncomp)
    eng, base = _state(net, 20000, seed=4242)
    if lanes is not None:
        assert eng.set_launch_config(128, 2, 0, lanes) == abi.PF_OK
    if ncomp == 5:
        assert eng.launch_config()["lanes_per_cell"] > 1  # no one-lane kernel for this ncomp
    ref = base.copy()
    ref_stats = eng.rstep(ref, 86400.0)
    torch.cuda.synchronize()
    for call in range(2):
        got = base.copy()
        got.a["status"].fill_(7)  # overwritten for every cell the step reaches
        stats = _noalloc(eng, got, 86400.0)
        assert stats == ref_stats, (call, stats, ref_stats)
        for k in FIELDS:
            assert torch.equal(got.a[k], ref.a[k]), (call, k)


def test_noalloc_rejects_oversized_state():
    net = generate.calcite_network()
    from pfgpu.engine import ReactionEngine
    eng = ReactionEngine(net)
    per_cell = net.ncomp + net.nsec + net.nmnrl
    n = (4 * 1024 * 1024) // per_cell + 1
    st = generate.calcite_cells(net, 1, seed=1)[0]
    big = {k: torch.zeros((v.shape[0], n) if v.ndim == 2 else (n,), dtype=torch.from_numpy(v).dtype,
                          device="cuda") for k, v in st.a.items()}
    from pfgpu.network import CellState
    bs = CellState(net, big)
    s = bs.struct()
    rc = eng.lib.pf_rstep_noalloc(eng.handle, C.byref(s), 3600.0,
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert rc == abi.PF_ERR_TOO_LARGE


def test_noalloc_in_a_cuda_graph():
    """A call outside any capture resolves the scratch array's address; a call
    captured into a CUDA graph then uses that address, and the replayed graph
    gives pf_rstep's results bit for bit."""
    net = _net(12)
    eng, base = _state(net, 20000, seed=4242)
    ref = base.copy()
    eng.rstep(ref, 86400.0)
    warm = base.copy()
    _noalloc(eng, warm, 86400.0)
    got = base.copy()
    s = got.struct()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = eng.lib.pf_rstep_noalloc(eng.handle, C.byref(s), 86400.0,
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert rc == abi.PF_OK
    g.replay()
    torch.cuda.synchronize()
    for k in FIELDS:
        assert torch.equal(got.a[k], ref.a[k]), k
