"""pf_rstep_noalloc: the batched step for callers that may not allocate device
memory during the call (their GPU memory belongs to another framework's pool,
or their footprint is fixed up front).  Its scratch is a fixed array inside the library, shared by every
call, so this test checks that two calls in a row -- the second reusing
whatever the first left in that array -- give the same results as the
allocating entry point pf_rstep, to the parity tolerance of the other tests
(1e-10 relative; the kernels are the same, so the results are identical).
Kept last in collection order so a failure here does not hide other tests.
"""
import ctypes as C

import numpy as np
import pytest

from pfgpu import abi, generate
from pfgpu.network import default_options

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-10


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
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = eng.lib.pf_rstep_noalloc(eng.handle, C.byref(s), dt, stream)
    assert rc == abi.PF_OK, rc
    torch.cuda.synchronize()


def test_noalloc_matches_allocating_step_twice():
    net = generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
    eng, base = _state(net, 20000, seed=4242)
    fields = ("total", "pri_molal", "sec_molal", "mnrl_rate", "mnrl_volfrac", "newton_its", "status",
              "num_substeps")
    ref = base.copy()
    eng.rstep(ref, 86400.0)
    torch.cuda.synchronize()
    for call in range(2):
        got = base.copy()
        _noalloc(eng, got, 86400.0)
        for k in fields:
            a, b = got.a[k], ref.a[k]
            if a.dtype.is_floating_point:
                scale = b.abs().clamp_min(1e-300)
                assert float(((a - b).abs() / scale).max()) < REL, (call, k)
            else:
                assert torch.equal(a, b), (call, k)


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
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == abi.PF_ERR_TOO_LARGE
