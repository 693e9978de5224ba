"""The transport half of the operator-split step (pf_transport_step).

`OSTransport` owns the device work space of one structured grid and solves,
per step, (psv/dt + A) T_k+1 = psv T_k / dt + b_bc for every component at
once (A: advection by the face Darcy fluxes, upwinded, plus dispersion-
diffusion; boundary conditions on the outer faces and sources/sinks add to
the diagonal and to b_bc), as the reference's operator-split time step does
before its reaction step (pmc_subsurface_osrt.F90:259-330,
RTCalculateTransportMatrix and RTCalculateRHS_t1).  Faces without a
boundary condition are closed (zero flux).
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
        self.device = device
        self._q = [torch.as_tensor(np.ascontiguousarray(q), dtype=torch.float64).reshape(-1).to(device)
                   if np.size(q) else torch.zeros(1, **f64) for q in (grid.qx, grid.qy, grid.qz)]
        self._bc = [None] * 6   # per face: (type, q tensor or None, total tensor, saturation)
        self._src = None        # (cell, type, q, total) tensors

    FACES = {"x-": 0, "x+": 1, "y-": 2, "y+": 3, "z-": 4, "z+": 5}

    def face_cells(self, face: int) -> int:
        g = self.grid
        return (g.ny * g.nz, g.ny * g.nz, g.nx * g.nz, g.nx * g.nz, g.nx * g.ny, g.nx * g.ny)[face]

    def set_boundary(self, face, bc_type, total, q=None, saturation=1.0):
        """A boundary condition on one outer face (0..5 or "x-", "x+", "y-",
        "y+", "z-", "z+"): bc_type PF_BC_*; total (ncomp, face cells) or
        (ncomp,) totals of the boundary water, mol/L; q (face cells,) or a
        scalar Darcy flux through the face, m/s, positive into the domain;
        saturation at the boundary.  Face cells are indexed j + ny*k (x
        faces), i + nx*k (y faces), i + nx*j (z faces).  bc_type
        PF_BC_ZERO_FLUX closes the face again."""
        import torch
        f = self.FACES[face] if isinstance(face, str) else int(face)
        if bc_type == abi.PF_BC_ZERO_FLUX:
            self._bc[f] = None
            return
        nf = self.face_cells(f)
        tot = np.asarray(total, np.float64)
        if tot.ndim == 1:
            tot = np.repeat(tot[:, None], nf, axis=1)
        if tot.shape != (self.ncomp, nf):
            raise ValueError("boundary totals must be (ncomp, %d) or (ncomp,)" % nf)
        qt = None
        if q is not None:
            qa = np.broadcast_to(np.asarray(q, np.float64), (nf,))
            qt = torch.from_numpy(np.ascontiguousarray(qa)).to(self.device)
        self._bc[f] = (int(bc_type), qt, torch.from_numpy(np.ascontiguousarray(tot)).to(self.device),
                       float(saturation))

    def set_sources(self, cell=None, src_type=None, q=None, total=None):
        """Sources and sinks, applied in the given order: cell indices, types
        PF_SRC_*, q in m^3/s (positive: injection), total (ncomp, nsrc) in
        mol/L (mol/s for PF_SRC_MASS_RATE).  No arguments: none."""
        import torch
        if cell is None or len(cell) == 0:
            self._src = None
            return
        n = len(cell)
        tot = np.asarray(total, np.float64).reshape(self.ncomp, n)
        dev = self.device
        self._src = (torch.from_numpy(np.ascontiguousarray(cell, np.int32)).to(dev),
                     torch.from_numpy(np.ascontiguousarray(np.broadcast_to(src_type, (n,)), np.int32)).to(dev),
                     torch.from_numpy(np.ascontiguousarray(np.broadcast_to(q, (n,)), np.float64)).to(dev),
                     torch.from_numpy(np.ascontiguousarray(tot)).to(dev))

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
        for f, b in enumerate(self._bc):
            if b is None:
                continue
            a.bc_type[f] = b[0]
            a.bc_q[f] = C.cast(b[1].data_ptr(), dp) if b[1] is not None else None
            a.bc_total[f] = C.cast(b[2].data_ptr(), dp)
            a.bc_saturation[f] = b[3]
        if self._src is not None:
            ip = C.POINTER(C.c_int32)
            a.nsrc = int(self._src[0].numel())
            a.src_cell = C.cast(self._src[0].data_ptr(), ip)
            a.src_type = C.cast(self._src[1].data_ptr(), ip)
            a.src_q = C.cast(self._src[2].data_ptr(), dp)
            a.src_total = C.cast(self._src[3].data_ptr(), dp)
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
