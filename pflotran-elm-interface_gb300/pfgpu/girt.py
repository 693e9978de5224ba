"""Global-implicit (GIRT) residual and block Jacobian on a structured grid.

`StructuredGrid` holds the grid geometry, the face Darcy fluxes and the
transport coefficients; `GirtAssembler` owns the SeqBAIJ pattern on the device
and calls pf_girt_assemble, which replaces RTResidual / RTJacobian
(reactive_transport.F90:1964, :2788) for that grid: per connection the
TFluxCoef / TFlux / TFluxDerivative terms (transport.F90:378-565), per cell
RTAccumulation[Derivative] and RReaction[Derivative], then the log-formulation
column scaling.  The residual is block-interleaved (cell-major, ncomp per
cell) and every ncomp x ncomp block is stored column-major, both as PETSc's
SeqBAIJ holds them, so the arrays can back a MatCreateSeqBAIJWithArrays /
VecPlaceArray pair directly.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .engine import ReactionEngine, _stream_ptr
from .network import CellState


def girt_pattern(nx: int, ny: int, nz: int, lib=None):
    """Host (rowptr[ncells+1], colidx[nnzb]) of the 7-point block pattern,
    block columns ascending (pf_girt_pattern)."""
    lib = lib or abi.load()
    nnzb = lib.pf_girt_pattern(nx, ny, nz, None, None)
    abi.check("pf_girt_pattern", min(int(nnzb), 0), allow_cell_failures=False)
    rowptr = np.zeros(nx * ny * nz + 1, np.int32)
    colidx = np.zeros(nnzb, np.int32)
    ip = C.POINTER(C.c_int32)
    rc = lib.pf_girt_pattern(nx, ny, nz, rowptr.ctypes.data_as(ip), colidx.ctypes.data_as(ip))
    abi.check("pf_girt_pattern", min(int(rc), 0), allow_cell_failures=False)
    return rowptr, colidx


@dataclass
class StructuredGrid:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    qx: object  # [nz][ny][nx-1] Darcy flux, m/s, + from i to i+1
    qy: object  # [nz][ny-1][nx]
    qz: object  # [nz-1][ny][nx]
    diffusion: float = 1.0e-9
    tortuosity: float = 1.0
    dispersivity: float = 0.0

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    def as_dict(self) -> dict:
        def host(a):
            return a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
        return dict(nx=self.nx, ny=self.ny, nz=self.nz, dx=self.dx, dy=self.dy, dz=self.dz,
                    qx=host(self.qx), qy=host(self.qy), qz=host(self.qz), diffusion=self.diffusion,
                    tortuosity=self.tortuosity, dispersivity=self.dispersivity)


class GirtAssembler:
    def __init__(self, engine: ReactionEngine, grid: StructuredGrid, device="cuda"):
        import torch
        self.engine, self.grid = engine, grid
        rp, ci = girt_pattern(grid.nx, grid.ny, grid.nz, engine.lib)
        self.rowptr_host, self.colidx_host = rp, ci
        self.rowptr = torch.from_numpy(rp).to(device)
        self.colidx = torch.from_numpy(ci).to(device)
        n = engine.net.ncomp
        f64 = dict(dtype=torch.float64, device=device)
        self.residual = torch.zeros(grid.ncells * n, **f64)
        self.values = torch.zeros(len(ci) * n * n, **f64)
        self._k_cache = None  # per-cell K of the reactions (k_cache="fill" / "read")
        self._q = [torch.as_tensor(np.ascontiguousarray(q), dtype=torch.float64).reshape(-1).to(device)
                   if np.size(q) else torch.zeros(1, **f64) for q in (grid.qx, grid.qy, grid.qz)]

    @property
    def nnzb(self) -> int:
        return len(self.colidx_host)

    def args(self, total_k, dt: float, total_sorb_k=None, numerical_derivatives=False, k_cache="off",
             ) -> abi.PfGirtArgs:
        g = self.grid
        a = abi.PfGirtArgs()
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        a.nx, a.ny, a.nz = g.nx, g.ny, g.nz
        a.dx, a.dy, a.dz = g.dx, g.dy, g.dz
        a.qx, a.qy, a.qz = (C.cast(q.data_ptr(), dp) for q in self._q)
        a.diffusion_coefficient, a.tortuosity, a.dispersivity = g.diffusion, g.tortuosity, g.dispersivity
        a.total_k = C.cast(total_k.data_ptr(), dp)
        a.dt = float(dt)
        a.rowptr, a.colidx = C.cast(self.rowptr.data_ptr(), ip), C.cast(self.colidx.data_ptr(), ip)
        a.residual, a.values = C.cast(self.residual.data_ptr(), dp), C.cast(self.values.data_ptr(), dp)
        if total_sorb_k is not None:
            a.total_sorb_k = C.cast(total_sorb_k.data_ptr(), dp)
        a.numerical_derivatives = int(bool(numerical_derivatives))
        if k_cache not in ("off", "fill", "read"):
            raise ValueError("k_cache: 'off', 'fill' or 'read'")
        if k_cache != "off":
            import torch
            net = self.engine.net
            shape = (net.nsec + net.nmnrl, self.grid.ncells)
            if k_cache == "fill" and (self._k_cache is None or tuple(self._k_cache.shape) != shape):
                self._k_cache = torch.empty(shape, dtype=torch.float64, device=self.values.device)
            if self._k_cache is None:
                raise ValueError("k_cache='read' before a k_cache='fill' assembly")
            a.k_cache = C.cast(self._k_cache.data_ptr(), dp)
            a.k_cache_valid = int(k_cache == "read")
        return a

    def assemble(self, state: CellState, total_k, dt: float, stream=None, total_sorb_k=None,
                 numerical_derivatives=False, k_cache="off"):
        """Residual and Jacobian values at the iterate in `state` (CUDA
        tensors); total_k: totals at the start of the step [ncomp][ncells];
        total_sorb_k: the sorbed totals at the start of the step (required
        when the network has sorption); numerical_derivatives: the reaction
        part of the Jacobian by forward differences (the reference's
        NUMERICAL_JACOBIAN transport option); k_cache: "off", or "fill" (the
        first assembly of a time step: each cell's K of every reaction is
        computed and kept in this assembler) then "read" (the step's later
        Newton iterations, temperatures and activity coefficients unchanged:
        the kept K are used).  Returns (residual, values), views of this
        assembler's buffers."""
        total_k = total_k.contiguous()
        if self.engine.net.has_sorption and total_sorb_k is None:
            raise ValueError("a network with sorption needs total_sorb_k")
        if total_sorb_k is not None:
            total_sorb_k = total_sorb_k.contiguous()
        a = self.args(total_k, dt, total_sorb_k, numerical_derivatives, k_cache)
        s = state.struct("device", self.engine.net)
        abi.check("pf_girt_assemble",
                  self.engine.lib.pf_girt_assemble(self.engine.handle, C.byref(s), C.byref(a), _stream_ptr(stream)),
                  allow_cell_failures=False)
        return self.residual, self.values

    def to_scipy(self, values=None):
        """The assembled matrix as scipy.sparse.bsr_matrix (tests, small grids)."""
        import scipy.sparse as sp
        n = self.engine.net.ncomp
        v = (self.values if values is None else values)
        v = v.cpu().numpy() if hasattr(v, "cpu") else np.asarray(v)
        blocks = v.reshape(-1, n, n).transpose(0, 2, 1)  # column-major blocks -> row-major
        N = self.grid.ncells
        return sp.bsr_matrix((blocks, self.colidx_host, self.rowptr_host), shape=(N * n, N * n))
