"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and reference legs use
this module; the product path never imports it.  The C++ restatement it
wraps is oracle/rxn_oracle.hpp (see the file header for the reference
routines it follows).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
LIB_COUNT = os.path.join(HERE, "_build", "liboracle_count.so")

_REPO = os.path.dirname(HERE)
_PKG = os.path.join(_REPO, "pflotran-elm-interface_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from pfgpu import abi  # noqa: E402  (struct layouts shared with the product)

CON_TOTAL, CON_FREE, CON_PH, CON_CHARGE_BAL, CON_LOG = 1, 2, 3, 4, 5


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "oracle_count.cpp", "rxn_oracle.hpp",
                                            "flop_real.hpp")]
    stale = force or not all(os.path.exists(x) for x in (LIB, LIB_COUNT)) or any(
        os.path.getmtime(s) > min(os.path.getmtime(LIB), os.path.getmtime(LIB_COUNT)) for s in srcs)
    if stale:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


class Oracle:
    def __init__(self):
        build()
        lib = C.CDLL(LIB)
        S, D = C.POINTER(abi.PfCellState), C.POINTER(abi.PfNetworkDesc)
        lib.oracle_rstep.argtypes = [D, S, C.c_double, C.c_int]
        lib.oracle_rreact.argtypes = [D, S, C.c_double, C.c_int]
        lib.oracle_update_kinetic_state.argtypes = [D, S, C.c_double]
        lib.oracle_implicit_step.argtypes = [D, S, C.c_double, C.c_double, C.c_int]
        lib.oracle_update_auxvars.argtypes = [D, S, C.c_int, C.c_int]
        lib.oracle_update_activity_coefs.argtypes = [D, S, C.c_int]
        lib.oracle_equilibrate.argtypes = [D, S, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_double),
                                           C.c_int, C.POINTER(C.c_int32), C.c_int]
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        lib.oracle_girt_assemble.argtypes = [D, S, ip, dp, dp, dp, dp, dp, dp, C.c_double, ip, ip, dp, dp, C.c_int]
        lib.oracle_ifc67_density.argtypes = [C.c_double, C.c_double]
        lib.oracle_ifc67_density.restype = C.c_double
        for f in ("oracle_rstep", "oracle_rreact", "oracle_implicit_step", "oracle_update_kinetic_state",
                  "oracle_update_auxvars", "oracle_update_activity_coefs", "oracle_equilibrate",
                  "oracle_girt_assemble"):
            getattr(lib, f).restype = C.c_int
        self.lib = lib

    @staticmethod
    def _args(net, state):
        d = net.desc()
        s = state.struct()
        return d, s

    def rstep(self, net, state, dt, nthreads=1):
        d, s = self._args(net, state)
        return self.lib.oracle_rstep(C.byref(d), C.byref(s), dt, nthreads)

    def rreact(self, net, state, dt, nthreads=1):
        d, s = self._args(net, state)
        return self.lib.oracle_rreact(C.byref(d), C.byref(s), dt, nthreads)

    def implicit_step(self, net, state, dt, rel_tol=1e-10, max_its=100):
        d, s = self._args(net, state)
        return self.lib.oracle_implicit_step(C.byref(d), C.byref(s), dt, rel_tol, max_its)

    def update_kinetic_state(self, net, state, dt):
        d, s = self._args(net, state)
        return self.lib.oracle_update_kinetic_state(C.byref(d), C.byref(s), dt)

    def update_auxvars(self, net, state, update_act=False, nthreads=1):
        d, s = self._args(net, state)
        return self.lib.oracle_update_auxvars(C.byref(d), C.byref(s), int(update_act), nthreads)

    def update_activity_coefs(self, net, state, nthreads=1):
        d, s = self._args(net, state)
        return self.lib.oracle_update_activity_coefs(C.byref(d), C.byref(s), nthreads)

    def equilibrate(self, net, state, ctype, cconc, use_prev=False, nthreads=1, reactions=None):
        """reactions: None, or per component a dict (species indices, stoich,
        logK, logKcoef) for MINERAL/GAS rows (pfgpu.abi.constraint_reactions
        builds the C array)."""
        from pfgpu import abi
        d, s = self._args(net, state)
        ct = np.ascontiguousarray(ctype, np.int32)
        cc = np.ascontiguousarray(cconc, np.float64)
        its = np.zeros(state.ncells, np.int32)
        cr = abi.constraint_reactions(len(ct), reactions) if reactions else None
        rc = self.lib.oracle_equilibrate(C.byref(d), C.byref(s),
                                         ct.ctypes.data_as(C.POINTER(C.c_int32)),
                                         C.cast(cr, C.c_void_p) if cr is not None else None,
                                         cc.ctypes.data_as(C.POINTER(C.c_double)),
                                         int(use_prev), its.ctypes.data_as(C.POINTER(C.c_int32)),
                                         nthreads)
        return rc, its

    def girt_assemble(self, net, state, grid, total_k, dt, rowptr, colidx, total_sorb_k=None,
                      numerical_derivatives=False):
        """Global-implicit residual [ncells*ncomp] and SeqBAIJ values
        [nnzb*ncomp*ncomp] (blocks column-major) of a structured grid.
        grid: dict nx, ny, nz, dx, dy, dz, qx, qy, qz, diffusion, tortuosity,
        dispersivity; total_sorb_k: sorbed totals at the start of the step
        (networks with sorption); numerical_derivatives: the reaction
        Jacobian by forward differences.  Updates state's total and sec_molal
        (and total_sorb, the ion-exchange warm start)."""
        d, s = self._args(net, state)
        f = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
        gi = np.array([grid["nx"], grid["ny"], grid["nz"]], np.int32)
        gd = f([grid["dx"], grid["dy"], grid["dz"], grid["diffusion"], grid["tortuosity"], grid["dispersivity"]])
        q = [f(grid[k]) if np.size(grid[k]) else np.zeros(1) for k in ("qx", "qy", "qz")]
        tk = f(total_k)
        sk = f(total_sorb_k) if total_sorb_k is not None else None
        rp, ci = np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32)
        n = net.ncomp
        r = np.zeros(state.ncells * n)
        vals = np.zeros(int(rp[-1]) * n * n)
        dp = C.POINTER(C.c_double)
        P = lambda a: a.ctypes.data_as(dp)  # noqa: E731
        rc = self.lib.oracle_girt_assemble(C.byref(d), C.byref(s), gi.ctypes.data_as(C.POINTER(C.c_int32)), P(gd),
                                           P(q[0]), P(q[1]), P(q[2]), P(tk),
                                           P(sk) if sk is not None else None, float(dt),
                                           rp.ctypes.data_as(C.POINTER(C.c_int32)),
                                           ci.ctypes.data_as(C.POINTER(C.c_int32)), P(r), P(vals),
                                           int(bool(numerical_derivatives)))
        if rc:
            raise RuntimeError("oracle_girt_assemble: %d" % rc)
        return r, vals

    def transport_matrix(self, grid, porosity, saturation, volume, dt, rowptr, colidx):
        """Values of the operator-split transport matrix (7-point pattern,
        block size 1) of a structured grid, as RTCalculateTransportMatrix
        assembles it."""
        f = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
        gi = np.array([grid["nx"], grid["ny"], grid["nz"]], np.int32)
        gd = f([grid["dx"], grid["dy"], grid["dz"], grid["diffusion"], grid["tortuosity"], grid["dispersivity"]])
        q = [f(grid[k]) if np.size(grid[k]) else np.zeros(1) for k in ("qx", "qy", "qz")]
        por, sat, vol = f(porosity), f(saturation), f(volume)
        rp, ci = np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32)
        vals = np.zeros(int(rp[-1]))
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        P = lambda a: a.ctypes.data_as(dp)  # noqa: E731
        fn = self.lib.oracle_transport_matrix
        fn.argtypes = [ip, dp, dp, dp, dp, dp, dp, dp, C.c_double, ip, ip, dp]
        fn.restype = C.c_int
        rc = fn(gi.ctypes.data_as(ip), P(gd), P(q[0]), P(q[1]), P(q[2]), P(por), P(sat), P(vol), float(dt),
                rp.ctypes.data_as(ip), ci.ctypes.data_as(ip), P(vals))
        if rc:
            raise RuntimeError("oracle_transport_matrix: %d" % rc)
        return vals

    def transport_bc_terms(self, grid, porosity, saturation, volume, ncomp, bc=None, sources=None):
        """Boundary and source terms of the operator-split transport system
        (the boundary and source/sink loops of RTCalculateTransportMatrix
        and RTCalculateRHS_t1): returns (diag_add [N], rhs_add [ncomp, N]).
        bc: dict(type=[6 ints], q=[6 arrays or None], total=[6 arrays
        (ncomp, face cells) or None], sat=[6 floats]), faces x-, x+, y-, y+,
        z-, z+; sources: dict(cell, type, q, total (ncomp, nsrc)) or None."""
        f = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
        gi = np.array([grid["nx"], grid["ny"], grid["nz"]], np.int32)
        gd = f([grid["dx"], grid["dy"], grid["dz"], grid["diffusion"], grid["tortuosity"], grid["dispersivity"]])
        N = int(gi.prod())
        por, sat, vol = f(porosity), f(saturation), f(volume)
        bc = bc or dict(type=[0] * 6, q=[None] * 6, total=[None] * 6, sat=[1.0] * 6)
        keep = []
        dp = C.POINTER(C.c_double)
        qptr = (dp * 6)()
        tptr = (dp * 6)()
        for k in range(6):
            for arr, dst in ((bc["q"][k], qptr), (bc["total"][k], tptr)):
                if arr is not None:
                    a = f(arr)
                    keep.append(a)
                    dst[k] = a.ctypes.data_as(dp)
        btype = np.ascontiguousarray(bc["type"], np.int32)
        bsat = f(bc["sat"])
        src = sources or dict(cell=np.zeros(0), type=np.zeros(0), q=np.zeros(0), total=np.zeros((ncomp, 0)))
        scell = np.ascontiguousarray(src["cell"], np.int32)
        stype = np.ascontiguousarray(src["type"], np.int32)
        sq = f(src["q"])
        stot = f(src["total"])
        diag = np.zeros(N)
        rhs = np.zeros((ncomp, N))
        ip = C.POINTER(C.c_int32)
        P = lambda a: a.ctypes.data_as(dp)  # noqa: E731
        fn = self.lib.oracle_transport_bc_terms
        fn.argtypes = [ip, dp, dp, dp, dp, C.c_int32, ip, C.POINTER(dp), C.POINTER(dp), dp, C.c_int32, ip, ip, dp,
                       dp, dp, dp]
        fn.restype = C.c_int
        rc = fn(gi.ctypes.data_as(ip), P(gd), P(por), P(sat), P(vol), int(ncomp), btype.ctypes.data_as(ip),
                qptr, tptr, P(bsat), int(scell.size), scell.ctypes.data_as(ip), stype.ctypes.data_as(ip), P(sq),
                P(stot), P(diag), P(rhs))
        if rc:
            raise RuntimeError("oracle_transport_bc_terms: %d" % rc)
        return diag, rhs

    def count_rstep(self, net, state, dt):
        """RStep of every cell with counted arithmetic (single thread; the
        state is advanced).  Returns per-cell (flops, transcendental calls,
        Newton iterations) of the reference algorithm: add/sub/mul/div/sqrt
        one flop, fma two; exp/log/pow counted apart."""
        if not hasattr(self, "_count"):
            lib = C.CDLL(LIB_COUNT)
            lib.oracle_count_rstep.argtypes = [C.POINTER(abi.PfNetworkDesc), C.POINTER(abi.PfCellState),
                                               C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
            lib.oracle_count_rstep.restype = C.c_int
            self._count = lib
        d, s = self._args(net, state)
        n = state.ncells
        fl = np.zeros(n, np.int64)
        tr = np.zeros(n, np.int64)
        its = np.zeros(n, np.int32)
        rc = self._count.oracle_count_rstep(C.byref(d), C.byref(s), float(dt), fl.ctypes.data, tr.ctypes.data,
                                            its.ctypes.data)
        if rc:
            raise RuntimeError("oracle_count_rstep: %d" % rc)
        return fl, tr, its

    def density(self, t, p):
        return self.lib.oracle_ifc67_density(t, p)


LOG_TO_LN = 2.30258509299  # pflotran_constants.F90:84


def surface_complexation_eq(pri_molal, pri_act_coef, complexes, site_density, free_site_guess=1.0e-9,
                            ln_act_h2o=0.0):
    """Equilibrium surface complexation of one site (one reaction), a
    pure-Python restatement of RTotalSorbEqSurfCplx1
    (reaction_surf_complex.F90:641-900) for a single cell.

    complexes: list of dicts with spec (primary indices), stoich, free_site_stoich,
    logK (log10 at the cell's temperature) and optionally h2o_stoich.
    site_density: mol sites / m^3 bulk (the NULL_SURFACE case, :720-722).
    Returns (free_site_conc, cplx_conc[ncplx], total_sorb[ncomp],
    dtotal_sorb[ncomp][ncomp]) in mol/m^3 bulk and kg water/m^3 bulk."""
    n = len(pri_molal)
    ln_act = [math.log(pri_molal[i]) + math.log(pri_act_coef[i]) for i in range(n)]  # :686-687
    ncplx = len(complexes)
    total_sorb = [0.0] * n
    dtotal = [[0.0] * n for _ in range(n)]
    if site_density < 1.0e-40:  # :728-737
        return 0.0, [0.0] * ncplx, total_sorb, dtotal
    stoich_flag = any(c["free_site_stoich"] > 1.0 for c in complexes)  # reaction_database.F90:2801-2803
    free = max(free_site_guess, 1.0e-40)  # :691
    conc = [0.0] * ncplx
    one_more, its, damping = False, 0, 1.0
    while True:  # :743-799
        its += 1
        total = free
        ln_free = math.log(free)
        for j, c in enumerate(complexes):
            lnQK = -c["logK"] * LOG_TO_LN
            if c.get("h2o_stoich", 0.0):
                lnQK += c["h2o_stoich"] * ln_act_h2o
            lnQK += c["free_site_stoich"] * ln_free
            for i, nu in zip(c["spec"], c["stoich"]):
                lnQK += nu * ln_act[i]
            conc[j] = math.exp(lnQK)
            total += c["free_site_stoich"] * conc[j]
        if one_more:
            break
        if stoich_flag:  # Newton on the site balance (:770-790)
            res = site_density - total
            dres = 1.0
            for j, c in enumerate(complexes):
                dres += c["free_site_stoich"] * conc[j] / free
            dfree = res / dres
            if its > 1000:
                damping = 0.5
            free = free + damping * dfree
            if abs(dfree / free) < 1.0e-12:
                one_more = True
        else:  # every complex holds one site: closed form (:792-797)
            total = total / free
            free = site_density / total
            one_more = True
    # derivatives (:803-824, 846-893)
    dSx = [0.0] * n
    tempreal = 0.0
    for j, c in enumerate(complexes):
        for i, nu in zip(c["spec"], c["stoich"]):
            dSx[i] += nu * c["free_site_stoich"] * conc[j]
        tempreal += c["free_site_stoich"] * c["free_site_stoich"] * conc[j]
    tempreal = tempreal / free + 1.0
    dSx = [-v / tempreal / pri_molal[i] for i, v in enumerate(dSx)]
    for j, c in enumerate(complexes):
        for i, nu in zip(c["spec"], c["stoich"]):
            total_sorb[i] += nu * conc[j]
        nui_Si_over_Sx = c["free_site_stoich"] * conc[j] / free
        for jc, nuj in zip(c["spec"], c["stoich"]):
            t = nuj * conc[j] / pri_molal[jc] + nui_Si_over_Sx * dSx[jc]
            for ic, nui in zip(c["spec"], c["stoich"]):
                dtotal[ic][jc] += nui * t
    return free, conc, total_sorb, dtotal
