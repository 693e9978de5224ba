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

    def set_launch_config(self, threads_per_block, blocks_per_sm, jac_in_shared):
        cfg = abi.PfLaunchConfig(int(threads_per_block), int(blocks_per_sm), int(jac_in_shared), 0)
        return self.lib.pf_network_set_launch(self.handle, C.byref(cfg))

    # ------------------------------------------------------------ steps
    def reserve(self, ncells: int):
        abi.check("pf_network_reserve", self.lib.pf_network_reserve(self.handle, int(ncells)),
                  allow_cell_failures=False)

    def rstep(self, state: CellState, dt: float, kernel: int = abi.PF_KERNEL_BATCHED, stream=None,
              stats: bool = True, order=None):
        """order: optional int64 CUDA tensor, a permutation of the cells giving
        the work-queue order of the batched kernel (results are unchanged)."""
        s = state.struct()
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
        s = state.struct()
        if order is not None:
            self._host_order = np.ascontiguousarray(order, np.int64)
            s.cell_order = C.cast(self._host_order.ctypes.data, C.POINTER(C.c_int64))
        st = abi.PfStepStats()
        rc = self.lib.pf_rstep_host(self.handle, C.byref(s), float(dt), int(kernel), C.byref(st))
        abi.check("pf_rstep_host", rc)
        return {k: getattr(st, k) for k, _ in abi.PfStepStats._fields_}

    def update_auxvars(self, state: CellState, update_activity_coefs: bool = False, stream=None):
        s = state.struct()
        abi.check("pf_update_auxvars",
                  self.lib.pf_update_auxvars(self.handle, C.byref(s), int(update_activity_coefs),
                                             _stream_ptr(stream)), allow_cell_failures=False)

    def equilibrate(self, state: CellState, ctype, cconc, use_prev: bool = False, stream=None):
        """Constraint equilibration on the device; cconc is a (ncomp, ncells)
        CUDA tensor.  Returns the per-cell iteration counts (-1 = failed)."""
        import torch
        ct = np.ascontiguousarray(ctype, np.int32)
        its = torch.empty(state.ncells, dtype=torch.int32, device=cconc.device)
        s = state.struct()
        abi.check("pf_equilibrate_constraint",
                  self.lib.pf_equilibrate_constraint(
                      self.handle, C.byref(s), ct.ctypes.data_as(C.POINTER(C.c_int32)),
                      C.c_void_p(cconc.contiguous().data_ptr()), int(use_prev), C.c_void_p(its.data_ptr()),
                      _stream_ptr(stream)), allow_cell_failures=False)
        return its

    def update_activity_coefs(self, state: CellState, stream=None):
        s = state.struct()
        abi.check("pf_update_activity_coefs",
                  self.lib.pf_update_activity_coefs(self.handle, C.byref(s), _stream_ptr(stream)),
                  allow_cell_failures=False)
