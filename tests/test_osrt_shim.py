"""The operator-split step driven the way PFLOTRAN's Fortran caller would
drive it: per-cell records (tests/harness/osrt_shim.c, the C equivalent of
pfgpu_osrt_react in include/pfgpu_mod.F90) gathered into the C ABI's arrays,
one pf_rstep_host call, results scattered back into the records.

CPU: the harness compiles against pfgpu.h and links libpfgpu.so; its record
layout is the numpy dtype the test builds.  GPU: the records after the step
agree bit for bit with a direct pf_rstep_host call on the same state, and
with the oracle under the parity comparison of tests/parity.py."""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import cases
import parity
from pfgpu import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "harness", "osrt_shim.c")
FIELDS = [("total", "f8", abi.PF_MAX_NCOMP), ("pri_molal", "f8", abi.PF_MAX_NCOMP),
          ("pri_act_coef", "f8", abi.PF_MAX_NCOMP), ("sec_act_coef", "f8", abi.PF_MAX_NSEC),
          ("sec_molal", "f8", abi.PF_MAX_NSEC), ("mnrl_volfrac", "f8", abi.PF_MAX_NMNRL),
          ("mnrl_area", "f8", abi.PF_MAX_NMNRL), ("mnrl_rate", "f8", abi.PF_MAX_NMNRL),
          ("porosity", "f8", 1), ("saturation", "f8", 1), ("den_kg", "f8", 1), ("volume", "f8", 1),
          ("temperature", "f8", 1), ("status", "i4", 1), ("newton_its", "i4", 1), ("num_substeps", "i4", 1)]


@pytest.fixture(scope="module")
def shim():
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    lib = abi.LIB_PATH
    if not os.path.exists(lib):
        pytest.skip("libpfgpu.so not built")
    d = tempfile.mkdtemp()
    out = os.path.join(d, "libosrt_shim.so")
    libdir = os.path.dirname(lib)
    subprocess.run([gcc, "-O2", "-shared", "-fPIC", "-I", os.path.join(REPO, "include"), SRC, "-o", out,
                    "-L", libdir, "-lpfgpu", "-Wl,-rpath," + libdir], check=True)
    abi.load()  # the same libpfgpu.so the shim links against, loaded first
    h = C.CDLL(out)
    shutil.rmtree(d)
    h.shim_cell_size.restype = C.c_size_t
    h.shim_cell_offset.restype = C.c_size_t
    h.shim_cell_offset.argtypes = [C.c_int32]
    h.shim_osrt_react.restype = C.c_int32
    h.shim_osrt_react.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                  C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    names = [f[0] for f in FIELDS]
    fmts = [(f[1], (f[2],)) if f[2] > 1 else f[1] for f in FIELDS]
    offs = [h.shim_cell_offset(k) for k in range(len(FIELDS))]
    dtype = np.dtype({"names": names, "formats": fmts, "offsets": offs, "itemsize": h.shim_cell_size()})
    return h, dtype


def test_shim_record_layout(shim):
    h, dtype = shim
    assert dtype.itemsize == h.shim_cell_size()
    assert h.shim_cell_offset(len(FIELDS)) == C.c_size_t(-1).value


def to_records(dtype, st):
    net = st.net
    rec = np.zeros(st.ncells, dtype)
    for k, _, cnt in FIELDS:
        if k not in st.a:
            continue
        v = st.a[k]
        if cnt > 1:
            rec[k][:, :v.shape[0]] = v.T
        else:
            rec[k] = v
    return rec


def from_records(rec, st):
    out = st.copy()
    for k, _, cnt in FIELDS:
        if k not in out.a:
            continue
        if cnt > 1:
            out.a[k][:] = rec[k][:, :out.a[k].shape[0]].T
        else:
            out.a[k][:] = rec[k]
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["calcite", "random12"])
def test_shim_step_matches_library_and_oracle(oracle, shim, name):
    from pfgpu.engine import ReactionEngine
    h, dtype = shim
    net, st0 = cases.case(oracle, name)
    dt = cases.CASE_DT[name]
    eng = ReactionEngine(net)
    rec = to_records(dtype, st0)
    err, its = C.c_int32(-1), C.c_int64(0)
    rc = h.shim_osrt_react(eng.handle, rec.ctypes.data, st0.ncells, net.ncomp, net.nsec, net.nmnrl, dt,
                           C.byref(err), C.byref(its))
    assert rc in (abi.PF_OK, abi.PF_CELL_FAILURES), rc
    got = from_records(rec, st0)
    # the same call made directly
    direct = st0.copy()
    stats = eng.rstep_host(direct, dt)
    for k in ("total", "pri_molal", "pri_act_coef", "sec_molal", "mnrl_rate", "mnrl_volfrac", "status",
              "newton_its", "num_substeps"):
        np.testing.assert_array_equal(got.a[k], direct.a[k], err_msg=k)
    assert its.value == stats["newton_iterations"]
    assert err.value == (1 if stats["failed_cells"] else 0)
    # and against the oracle
    ref = st0.copy()
    oracle.rstep(net, ref, dt, nthreads=8)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st0.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, dt, nthreads=8)
        perts.append(p)
    entry, _ = parity.compare(net, ref, got, dt, "fortran-shim/" + name, perts)
    parity.check(entry, "fortran-shim/" + name, min_compared=int(0.95 * st0.ncells))
