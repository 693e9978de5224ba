"""Python front end of the C ABI: the host-side mirror of the reference's
per-cell reaction interface.

`ReactionEngine` owns one device network (pf_network_create) and exposes the
operations the reference's operator-split loop performs per time step
(pm_osrt.F90:115-153 and pmc_subsurface_osrt.F90:346-381):

    engine.update_auxvars(state)            # RTUpdateAuxVars(cells)
    engine.update_activity_coefs(state)     # RTUpdateActivityCoefficients
    stats = engine.rstep(state, dt)         # the RStep cell loop + rstep_error reduction

`state` is a CellState whose arrays are CUDA tensors (device path) or numpy
arrays (rstep_host: host buffers, copies inside the call).  Every call goes
through libpfgpu.so; there is no other implementation behind it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .network import CellState, ReactionNetwork


def _stream_ptr(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


class ReactionEngine:
    def __init__(self, net: ReactionNetwork, lib=None):
        self.lib = lib or abi.load()
        self.net = net
        self._desc = net.desc()
        h = C.c_void_p()
        abi.check("pf_network_create", self.lib.pf_network_create(C.byref(self._desc), C.byref(h)),
                  allow_cell_failures=False)
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pf_network_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ options
    def set_options(self, **kw):
        self.net.options.update(kw)
        o = self.net.options_struct()
        abi.check("pf_network_set_options", self.lib.pf_network_set_options(self.handle, C.byref(o)),
                  allow_cell_failures=False)

    def launch_config(self) -> dict:
        cfg = abi.PfLaunchConfig()
        abi.check("pf_network_get_launch", self.lib.pf_network_get_launch(self.handle, C.byref(cfg)))
        return {k: getattr(cfg, k) for k, _ in abi.PfLaunchConfig._fields_}

    def set_launch_config(self, threads_per_block, blocks_per_sm, jac_in_shared=0, lanes_per_cell=1):
        """Returns the PfStatus (PF_OK when the configuration is accepted)."""
        cfg = abi.PfLaunchConfig(int(threads_per_block), int(blocks_per_sm), int(jac_in_shared),
                                 int(lanes_per_cell))
        return self.lib.pf_network_set_launch(self.handle, C.byref(cfg))

    # ------------------------------------------------------------ steps
    def reserve(self, ncells: int):
        abi.check("pf_network_reserve", self.lib.pf_network_reserve(self.handle, int(ncells)),
                  allow_cell_failures=False)

    def rstep(self, state: CellState, dt: float, kernel: int = abi.PF_KERNEL_BATCHED, stream=None,
              stats: bool = True, order=None):
        """order: optional int64 CUDA tensor, a permutation of the cells giving
        the work-queue order of the batched kernel (results are unchanged)."""
        s = state.struct("device", self.net)
        if order is not None:
            assert order.dtype.is_floating_point is False and order.numel() == state.ncells
            s.cell_order = C.cast(order.data_ptr(), C.POINTER(C.c_int64))
        st = abi.PfStepStats() if stats else None
        rc = self.lib.pf_rstep(self.handle, C.byref(s), float(dt), int(kernel), _stream_ptr(stream),
                               C.byref(st) if stats else None)
        abi.check("pf_rstep", rc)
        if not stats:
            return None
        return {k: getattr(st, k) for k, _ in abi.PfStepStats._fields_}

    def rstep_host(self, state: CellState, dt: float, kernel: int = abi.PF_KERNEL_BATCHED, order=None):
        """order: optional int64 numpy array (host), the work-queue order."""
        s = state.struct("host", self.net)
        if order is not None:
            self._host_order = np.ascontiguousarray(order, np.int64)
            s.cell_order = C.cast(self._host_order.ctypes.data, C.POINTER(C.c_int64))
        st = abi.PfStepStats()
        rc = self.lib.pf_rstep_host(self.handle, C.byref(s), float(dt), int(kernel), C.byref(st))
        abi.check("pf_rstep_host", rc)
        return {k: getattr(st, k) for k, _ in abi.PfStepStats._fields_}

    def update_auxvars(self, state: CellState, update_activity_coefs: bool = False, stream=None):
        s = state.struct("device", self.net)
        abi.check("pf_update_auxvars",
                  self.lib.pf_update_auxvars(self.handle, C.byref(s), int(update_activity_coefs),
                                             _stream_ptr(stream)), allow_cell_failures=False)

    def equilibrate(self, state: CellState, ctype, cconc, use_prev: bool = False, stream=None, reactions=None):
        """Constraint equilibration on the device; cconc is a (ncomp, ncells)
        CUDA tensor.  reactions: {component: dict(spec, stoich, logK,
        logKcoef)} for MINERAL/GAS rows (pfgpu.database.constraint_reaction).
        Returns the per-cell iteration counts (-1 = failed)."""
        import torch
        ct = np.ascontiguousarray(ctype, np.int32)
        its = torch.empty(state.ncells, dtype=torch.int32, device=cconc.device)
        s = state.struct("device", self.net)
        cr = abi.constraint_reactions(len(ct), reactions)
        abi.check("pf_equilibrate_constraint_ex",
                  self.lib.pf_equilibrate_constraint_ex(
                      self.handle, C.byref(s), ct.ctypes.data_as(C.POINTER(C.c_int32)),
                      C.cast(cr, C.c_void_p) if cr is not None else None,
                      C.c_void_p(cconc.contiguous().data_ptr()), int(use_prev), C.c_void_p(its.data_ptr()),
                      _stream_ptr(stream)), allow_cell_failures=False)
        return its

    def shift_parameters(self, dlogK_sec=None, dlogK_mnrl=None, dlnk=None):
        """logK += shift for every secondary / kinetic mineral (at every
        temperature), rate constants *= exp(dlnk), from the values at
        creation.  Host sequences or None."""
        def arr(a, n):
            if a is None:
                return None, None
            a = np.ascontiguousarray(np.asarray(a, np.float64).reshape(n))
            return a, a.ctypes.data_as(C.POINTER(C.c_double))
        a1, p1 = arr(dlogK_sec, self.net.nsec)
        a2, p2 = arr(dlogK_mnrl, self.net.nmnrl)
        a3, p3 = arr(dlnk, self.net.nmnrl)
        abi.check("pf_network_shift_parameters",
                  self.lib.pf_network_shift_parameters(self.handle, p1, p2, p3), allow_cell_failures=False)

    def adjoint(self, state: CellState, dt: float, weight=None, target=None, dL_dtotal=None, order=None,
                stream=None):
        """Forward step (state is advanced as by rstep) plus the adjoint of the
        step.  Loss: sum weight*(total_final - target)^2 when weight/target
        are given, else dL/dtotal_final = dL_dtotal.  Returns a dict of CUDA
        tensors: dL_dtotal0 (ncomp, ncells), dL_dlnarea (nmnrl, ncells),
        dL_dlogK_sec (nsec), dL_dlogK_mnrl (nmnrl), dL_dlnk (nmnrl), loss (1),
        adj_status (ncells)."""
        import torch
        dev = state.a["porosity"].device
        n, ns, nm, N = self.net.ncomp, self.net.nsec, self.net.nmnrl, state.ncells
        f64 = dict(dtype=torch.float64, device=dev)
        out = dict(dL_dtotal0=torch.zeros((n, N), **f64), dL_dlnarea=torch.zeros((max(nm, 1), N), **f64),
                   dL_dlogK_sec=torch.zeros(max(ns, 1), **f64), dL_dlogK_mnrl=torch.zeros(max(nm, 1), **f64),
                   dL_dlnk=torch.zeros(max(nm, 1), **f64), loss=torch.zeros(1, **f64),
                   adj_status=torch.zeros(N, dtype=torch.int32, device=dev))
        a = abi.PfAdjointArgs()

        def ptr(t, ct=C.c_double):
            return C.cast(None if t is None else t.contiguous().data_ptr(), C.POINTER(ct))
        keep = [weight, target, dL_dtotal]
        a.weight, a.target, a.dL_dtotal = ptr(weight), ptr(target), ptr(dL_dtotal)
        a.dL_dtotal0, a.dL_dlnarea = ptr(out["dL_dtotal0"]), ptr(out["dL_dlnarea"])
        a.dL_dlogK_sec, a.dL_dlogK_mnrl = ptr(out["dL_dlogK_sec"]), ptr(out["dL_dlogK_mnrl"])
        a.dL_dlnk, a.loss = ptr(out["dL_dlnk"]), ptr(out["loss"])
        a.adj_status = ptr(out["adj_status"], C.c_int32)
        s = state.struct("device", self.net)
        if order is not None:
            s.cell_order = C.cast(order.data_ptr(), C.POINTER(C.c_int64))
        abi.check("pf_adjoint", self.lib.pf_adjoint(self.handle, C.byref(s), float(dt), C.byref(a),
                                                    _stream_ptr(stream)), allow_cell_failures=False)
        del keep
        if nm == 0:
            for k in ("dL_dlnarea", "dL_dlogK_mnrl", "dL_dlnk"):
                out[k] = out[k][:0]
        if ns == 0:
            out["dL_dlogK_sec"] = out["dL_dlogK_sec"][:0]
        return out

    def update_activity_coefs(self, state: CellState, stream=None):
        s = state.struct("device", self.net)
        abi.check("pf_update_activity_coefs",
                  self.lib.pf_update_activity_coefs(self.handle, C.byref(s), _stream_ptr(stream)),
                  allow_cell_failures=False)


def rstep_multi(members, dt: float, stream=None, stats: bool = True, orders=None):
    """One operator-split step for the cells of several networks in one
    persistent launch (pf_rstep_multi): members is a sequence of
    (ReactionEngine, CellState of CUDA tensors), processed in that order
    (costliest first); orders: optional per-member work-queue permutations.
    Returns a list of per-member statistics dicts (stats=True)."""
    lib = members[0][0].lib
    n = len(members)
    handles = (C.c_void_p * n)(*[eng.handle.value for eng, _ in members])
    structs = (abi.PfCellState * n)()
    for k, (eng, st) in enumerate(members):
        s = st.struct("device", eng.net)
        if orders is not None and orders[k] is not None:
            s.cell_order = C.cast(orders[k].data_ptr(), C.POINTER(C.c_int64))
        structs[k] = s
    out = (abi.PfStepStats * n)() if stats else None
    rc = lib.pf_rstep_multi(handles, structs, n, float(dt), _stream_ptr(stream), out)
    abi.check("pf_rstep_multi", rc)
    if not stats:
        return None
    return [{k: getattr(o, k) for k, _ in abi.PfStepStats._fields_} for o in out]
