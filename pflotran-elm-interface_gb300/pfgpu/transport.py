"""The transport half of the operator-split step (pf_transport_step).

`OSTransport` owns the device work space of one structured grid and solves,
per step, (psv/dt + A) T_k+1 = psv T_k / dt for every component at once
(A: advection by the face Darcy fluxes, upwinded, plus dispersion-
diffusion, zero-flux outer boundaries), as the reference's operator-split
time step does before its reaction step (pmc_subsurface_osrt.F90:259-330).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .engine import _stream_ptr


class OSTransport:
    def __init__(self, grid, ncomp: int, lib=None, device="cuda"):
        """grid: a pfgpu.girt.StructuredGrid (geometry, face fluxes and
        transport coefficients)."""
        import torch
        self.lib = lib or abi.load()
        self.grid, self.ncomp = grid, int(ncomp)
        h = C.c_void_p()
        abi.check("pf_transport_create",
                  self.lib.pf_transport_create(grid.nx, grid.ny, grid.nz, self.ncomp, C.byref(h)),
                  allow_cell_failures=False)
        self.handle = h
        f64 = dict(dtype=torch.float64, device=device)
        self._q = [torch.as_tensor(np.ascontiguousarray(q), dtype=torch.float64).reshape(-1).to(device)
                   if np.size(q) else torch.zeros(1, **f64) for q in (grid.qx, grid.qy, grid.qz)]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pf_transport_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _args(self, state, dt: float, rtol: float, max_iterations: int):
        import torch
        g = self.grid
        N = g.nx * g.ny * g.nz
        for key, size in (("porosity", N), ("saturation", N), ("volume", N), ("total", self.ncomp * N)):
            t = state.a[key]
            if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous() or t.numel() != size:
                raise ValueError("state.%s must be a contiguous float64 CUDA tensor of %d values" % (key, size))
        a = abi.PfTransportArgs()
        dp = C.POINTER(C.c_double)
        a.nx, a.ny, a.nz, a.ncomp = g.nx, g.ny, g.nz, self.ncomp
        a.dx, a.dy, a.dz = g.dx, g.dy, g.dz
        a.qx, a.qy, a.qz = (C.cast(q.data_ptr(), dp) for q in self._q)
        a.diffusion_coefficient, a.tortuosity, a.dispersivity = g.diffusion, g.tortuosity, g.dispersivity
        a.porosity = C.cast(state.a["porosity"].data_ptr(), dp)
        a.saturation = C.cast(state.a["saturation"].data_ptr(), dp)
        a.volume = C.cast(state.a["volume"].data_ptr(), dp)
        a.dt = float(dt)
        a.total = C.cast(state.a["total"].data_ptr(), dp)
        a.rtol = float(rtol)
        a.max_iterations = int(max_iterations)
        return a

    @staticmethod
    def _stats(st):
        return {k: getattr(st, k) for k, _ in abi.PfTransportStats._fields_}

    def step(self, state, dt: float, rtol: float = 1e-10, max_iterations: int = 1000, stream=None) -> dict:
        """Transport the totals of `state` (a CellState of CUDA tensors on
        this grid) over dt, in place.  Returns the solver statistics; raises
        PfError if the solve did not converge within max_iterations."""
        a = self._args(state, dt, rtol, max_iterations)
        st = abi.PfTransportStats()
        rc = self.lib.pf_transport_step(self.handle, C.byref(a), _stream_ptr(stream), C.byref(st))
        abi.check("pf_transport_step", rc, allow_cell_failures=False)
        return self._stats(st)

    def enqueue(self, state, dt: float, inner_iterations: int, refinements: int, rtol: float = 1e-10,
                stream=None) -> None:
        """The same solve with a fixed schedule (refinements cycles of
        inner_iterations inner iterations), enqueued without host
        synchronisation, so that it can be captured in a CUDA graph.  The
        pointers of `state` are baked into a captured graph.  Check the
        outcome with read_stats()."""
        a = self._args(state, dt, rtol, 1)
        abi.check("pf_transport_enqueue",
                  self.lib.pf_transport_enqueue(self.handle, C.byref(a), int(inner_iterations), int(refinements),
                                                _stream_ptr(stream)), allow_cell_failures=False)

    def read_stats(self, rtol: float = 1e-10, stream=None) -> dict:
        """Statistics of the last solve (synchronises the stream); key
        'converged' tells whether a fixed schedule met rtol."""
        st = abi.PfTransportStats()
        rc = self.lib.pf_transport_read_stats(self.handle, float(rtol), _stream_ptr(stream), C.byref(st))
        abi.check("pf_transport_read_stats", rc, allow_cell_failures=True)
        return self._stats(st)

    @staticmethod
    def schedule(stats: dict) -> tuple:
        """A fixed schedule (inner_iterations, refinements) with margin from
        an adaptive step's statistics."""
        return int(stats["max_cycle_iterations"]) + 2, int(stats["refinements"]) + 1
