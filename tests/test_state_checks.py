"""Host-side checks of a cell state before a library call
(CellState.struct): every array has its field's dtype, rows x ncells values
and contiguous storage, and lives where the call reads it.  A buffer that
fails any of these would be read past its end by the kernels, so the check
raises before the call is made."""
import numpy as np
import pytest

from pfgpu import generate
from pfgpu.network import CellState


def _state(ncells=10):
    net = generate.calcite_network()
    st, _, _ = generate.calcite_cells(net, ncells, seed=3)
    return net, st


def test_valid_host_state_passes_and_fills_every_pointer():
    net, st = _state()
    s = st.struct("host")
    assert s.ncells == st.ncells
    assert bool(s.total) and bool(s.mnrl_area) and bool(s.status)
    st.struct()  # where=None accepts host arrays too


@pytest.mark.parametrize("field,bad", [
    ("total", lambda v: v.astype(np.float32)),
    ("status", lambda v: v.astype(np.int64)),
    ("porosity", lambda v: v[:-1].copy()),
    ("pri_molal", lambda v: np.concatenate([v, v], axis=1)),
    ("sec_molal", lambda v: np.asfortranarray(v)),
])
def test_bad_host_array_is_refused(field, bad):
    net, st = _state()
    st.a[field] = bad(st.a[field])
    with pytest.raises(ValueError, match=field):
        st.struct("host")


def test_rows_follow_the_calling_network():
    net, st = _state()
    bigger = generate.random_network(5, 12, 2, seed=1)
    with pytest.raises(ValueError, match="total"):
        st.struct(net=bigger)


def test_where_is_enforced():
    torch = pytest.importorskip("torch")
    net, st = _state()
    with pytest.raises(ValueError, match="host array"):
        st.struct("device")
    cpu = st.to("cpu")                      # torch tensors on the CPU
    cpu.struct()                            # fine for where=None
    with pytest.raises(ValueError, match="numpy"):
        cpu.struct("host")
    with pytest.raises(ValueError, match="CUDA"):
        cpu.struct("device")
    cpu.a["total"] = cpu.a["total"].to(torch.float32)
    with pytest.raises(ValueError, match="total"):
        cpu.struct()
    cpu2 = st.to("cpu")
    cpu2.a["sec_molal"] = cpu2.a["sec_molal"].t().contiguous().t()
    with pytest.raises(ValueError, match="not contiguous"):
        cpu2.struct()


def test_missing_optional_fields_stay_null():
    net, st = _state()
    st.a.pop("temperature")
    s = st.struct("host")
    assert not bool(s.temperature) and not bool(s.dt_cell)
    assert isinstance(st, CellState)
