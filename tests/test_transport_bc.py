"""Boundary conditions and sources of the operator-split transport step.

Oracle (CPU): its restatement of the boundary and source loops of
RTCalculateTransportMatrix / RTCalculateRHS_t1 (oracle transport_bc_terms)
added to its transport matrix and solved directly reproduces the exact
discrete solutions these terms must give: a column fed at its inflow face by
a Dirichlet condition stays at the inflow totals (advection in, zero-
gradient outflow); pure diffusion between two Dirichlet faces gives the
linear profile; each source type changes a closed box's mass by exactly its
rate over the step.

GPU: pf_transport_step with boundary conditions on several faces (every
type, both flux signs, a face with no flow) and sources of every type (two
in one cell) agrees with the oracle's system solved directly to 1e-9
relative, and on a 1-D column the component masses change by exactly the
boundary fluxes and source terms of the solution (1e-9)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from pfgpu import abi
from pfgpu.girt import girt_pattern

DT = 86400.0


def _grid(nx, ny, nz, q, disp=0.1, diffusion=1e-9, tortuosity=0.5, dx=2.0, dy=1.5, dz=0.5):
    return dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, qx=np.full((nz, ny, nx - 1), q[0]),
                qy=np.full((nz, ny - 1, nx), q[1]), qz=np.full((nz - 1, ny, nx), q[2]), diffusion=diffusion,
                tortuosity=tortuosity, dispersivity=disp)


def _system(oracle, grid, por, sat, vol, ncomp, bc, sources, dt=DT, storage=True):
    rp, ci = girt_pattern(grid["nx"], grid["ny"], grid["nz"])
    # storage=False: the steady system (dt so large that psv/dt vanishes
    # next to the flux terms, rather than subtracting it, which cancels)
    vals = oracle.transport_matrix(grid, por, sat, vol, dt if storage else 1e300, rp, ci)
    N = len(rp) - 1
    A = sp.csr_matrix((vals, ci, rp), shape=(N, N))
    diag, rhs = oracle.transport_bc_terms(grid, por, sat, vol, ncomp, bc, sources)
    A = A + sp.diags(diag)
    return A.tocsc(), rhs


def _bc(**faces):
    b = dict(type=[0] * 6, q=[None] * 6, total=[None] * 6, sat=[1.0] * 6)
    for name, (t, q, tot) in faces.items():
        f = {"xm": 0, "xp": 1, "ym": 2, "yp": 3, "zm": 4, "zp": 5}[name]
        b["type"][f], b["q"][f], b["total"][f] = t, q, tot
    return b


def test_oracle_column_keeps_the_inflow_totals(oracle):
    nx, n = 40, 3
    q = 1.0e-5
    grid = _grid(nx, 1, 1, (q, 0, 0))
    por, sat, vol = np.full(nx, 0.3), np.ones(nx), np.full(nx, 3.0)
    c_in = np.array([1e-3, 2e-5, 7e-4])
    bc = _bc(xm=(abi.PF_BC_DIRICHLET, np.array([q]), c_in[:, None].copy()),
             xp=(abi.PF_BC_ZERO_GRADIENT, np.array([-q]), np.zeros((n, 1))))
    A, rhs = _system(oracle, grid, por, sat, vol, n, bc, None)
    psv = por * sat * 1000.0 * vol
    for c in range(n):
        T = spla.spsolve(A, psv * c_in[c] / DT + rhs[c])
        np.testing.assert_allclose(T, c_in[c], rtol=1e-13)


def test_oracle_diffusion_between_two_dirichlet_faces_is_linear(oracle):
    nx = 25
    grid = _grid(nx, 1, 1, (0.0, 0, 0), disp=0.0)
    por, sat, vol = np.full(nx, 0.25), np.ones(nx), np.full(nx, 1.5)
    cl, cr = 1e-3, 4e-4
    bc = _bc(xm=(abi.PF_BC_DIRICHLET, None, np.array([[cl]])), xp=(abi.PF_BC_DIRICHLET, None, np.array([[cr]])))
    A, rhs = _system(oracle, grid, por, sat, vol, 1, bc, None, storage=False)
    T = spla.spsolve(A, rhs[0])
    x = (np.arange(nx) + 0.5) / nx
    np.testing.assert_allclose(T, cl + (cr - cl) * x, rtol=1e-12)


@pytest.mark.parametrize("stype,q", [(abi.PF_SRC_VOLUMETRIC, 2e-6), (abi.PF_SRC_VOLUMETRIC, -2e-6),
                                     (abi.PF_SRC_EQUILIBRIUM, 0.0), (abi.PF_SRC_MASS_RATE, 0.0)],
                         ids=["injection", "extraction", "equilibrium", "mass-rate"])
def test_oracle_sources_change_the_mass_by_their_rate(oracle, stype, q):
    nx, ny, nz, n = 5, 4, 3, 2
    rng = np.random.default_rng(4)
    grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=rng.uniform(-1e-6, 1e-6, (nz, ny, nx - 1)),
                qy=rng.uniform(-1e-6, 1e-6, (nz, ny - 1, nx)), qz=rng.uniform(-1e-6, 1e-6, (nz - 1, ny, nx)),
                diffusion=1e-9, tortuosity=0.5, dispersivity=0.1)
    N = nx * ny * nz
    por, sat, vol = rng.uniform(0.1, 0.4, N), np.ones(N), np.full(N, 1.5)
    Tk = 10.0 ** rng.uniform(-5, -3, (n, N))
    cell = 17
    csrc = np.array([[3e-3], [1e-6]])
    src = dict(cell=np.array([cell]), type=np.array([stype]), q=np.array([q]), total=csrc)
    A, rhs = _system(oracle, grid, por, sat, vol, n, None, src)
    psv = por * sat * 1000.0 * vol
    for c in range(n):
        T = spla.spsolve(A, psv * Tk[c] / DT + rhs[c])
        dm = np.sum(psv * (T - Tk[c])) / DT
        if stype == abi.PF_SRC_VOLUMETRIC:
            want = q * 1000.0 * csrc[c, 0] if q > 0 else q * 1000.0 * T[cell]
        elif stype == abi.PF_SRC_EQUILIBRIUM:
            want = 1e-3 * (csrc[c, 0] - T[cell])
        else:
            want = csrc[c, 0]
        assert abs(dm - want) <= 1e-11 * max(abs(want), np.max(psv * Tk[c]) / DT), (c, dm, want)


# ---------------------------------------------------------------------- GPU
def _gpu_solver(grid, ncomp):
    from pfgpu.girt import StructuredGrid
    from pfgpu.transport import OSTransport
    g = StructuredGrid(grid["nx"], grid["ny"], grid["nz"], grid["dx"], grid["dy"], grid["dz"], grid["qx"],
                       grid["qy"], grid["qz"], diffusion=grid["diffusion"], tortuosity=grid["tortuosity"],
                       dispersivity=grid["dispersivity"])
    return OSTransport(g, ncomp)


def _state(por, sat, vol, T):
    import torch
    from pfgpu.network import CellState
    st = CellState.__new__(CellState)
    st.net, st.ncells = None, len(por)
    st.a = {"porosity": torch.from_numpy(por).cuda(), "saturation": torch.from_numpy(sat).cuda(),
            "volume": torch.from_numpy(vol).cuda(), "total": torch.from_numpy(np.ascontiguousarray(T)).cuda()}
    return st


@pytest.mark.gpu
def test_gpu_boundaries_and_sources_match_the_oracle(oracle):
    pytest.importorskip("torch")
    nx, ny, nz, n = 12, 8, 6, 5
    rng = np.random.default_rng(11)
    grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5,
                qx=rng.uniform(1e-7, 1e-5, (nz, ny, nx - 1)) * rng.choice([-1.0, 1.0], (nz, ny, nx - 1)),
                qy=rng.uniform(1e-7, 1e-5, (nz, ny - 1, nx)) * rng.choice([-1.0, 1.0], (nz, ny - 1, nx)),
                qz=rng.uniform(1e-7, 1e-5, (nz - 1, ny, nx)) * rng.choice([-1.0, 1.0], (nz - 1, ny, nx)),
                diffusion=1e-9, tortuosity=0.5, dispersivity=0.1)
    N = nx * ny * nz
    por, sat, vol = rng.uniform(0.1, 0.5, N), np.ones(N), np.full(N, 1.5)
    sat[[3, 200]] = 0.0  # dry cells (one on the x- face)
    Tk = 10.0 ** rng.uniform(-6, -2, (n, N))
    nfx, nfy, nfz = ny * nz, nx * nz, nx * ny
    bc = _bc(xm=(abi.PF_BC_DIRICHLET, rng.uniform(1e-7, 1e-5, nfx), 10.0 ** rng.uniform(-5, -3, (n, nfx))),
             xp=(abi.PF_BC_ZERO_GRADIENT, -rng.uniform(1e-7, 1e-5, nfx), np.zeros((n, nfx))),
             ym=(abi.PF_BC_DIRICHLET_ZERO_GRADIENT, rng.uniform(-1e-5, 1e-5, nfy),
                 10.0 ** rng.uniform(-5, -3, (n, nfy))),
             zp=(abi.PF_BC_DIRICHLET, None, 10.0 ** rng.uniform(-5, -3, (n, nfz))))
    bc["sat"][2] = 0.8
    src = dict(cell=np.array([40, 40, 300, 77, 500]),
               type=np.array([abi.PF_SRC_VOLUMETRIC, abi.PF_SRC_EQUILIBRIUM, abi.PF_SRC_VOLUMETRIC,
                              abi.PF_SRC_MASS_RATE, abi.PF_SRC_VOLUMETRIC]),
               q=np.array([3e-6, 0.0, -2e-6, 0.0, 0.0]), total=10.0 ** rng.uniform(-5, -3, (n, 5)))
    A, rhs = _system(oracle, grid, por, sat, vol, n, bc, src)
    psv = por * sat * 1000.0 * vol
    tr = _gpu_solver(grid, n)
    for f in range(6):
        if bc["type"][f]:
            tr.set_boundary(f, bc["type"][f], bc["total"][f], q=bc["q"][f], saturation=bc["sat"][f])
    tr.set_sources(src["cell"], src["type"], src["q"], src["total"])
    st = _state(por, sat, vol, Tk)
    stats = tr.step(st, DT, rtol=1e-13, max_iterations=5000)
    got = st.a["total"].cpu().numpy()
    for c in range(n):
        b = np.where(psv > 0, psv * Tk[c] / DT, 0.0) + rhs[c]
        Ad = A.tolil()
        for d in np.nonzero(A.diagonal() == 0)[0]:  # dry cells: identity rows keep their totals
            Ad[d, d] = 1.0
            b[d] = Tk[c, d]
        want = spla.spsolve(Ad.tocsc(), b)
        np.testing.assert_allclose(got[c], want, rtol=1e-9, err_msg="component %d" % c)
    assert stats["converged"] == 1


@pytest.mark.gpu
def test_gpu_column_mass_balance_with_boundary_fluxes():
    """A 1-D column: inflow through x- (Dirichlet), outflow through x+ (zero
    gradient), one injection and one extraction well.  The change of each
    component's mass over the step equals the flux through the two faces
    and the wells, evaluated at the solution (the implicit step's balance)."""
    pytest.importorskip("torch")
    nx, n = 200, 4
    q = 2.0e-6
    grid = _grid(nx, 1, 1, (q, 0, 0), disp=0.05, dx=0.5, dy=1.0, dz=1.0)
    rng = np.random.default_rng(21)
    por, sat, vol = rng.uniform(0.2, 0.4, nx), np.ones(nx), np.full(nx, 0.5)
    Tk = 10.0 ** rng.uniform(-6, -4, (n, nx))
    c_in = 10.0 ** rng.uniform(-4, -3, n)
    c_well = 10.0 ** rng.uniform(-4, -3, n)
    tr = _gpu_solver(grid, n)
    tr.set_boundary("x-", abi.PF_BC_DIRICHLET, c_in, q=q)
    tr.set_boundary("x+", abi.PF_BC_ZERO_GRADIENT, np.zeros(n), q=-q)
    tr.set_sources([60, 150], abi.PF_SRC_VOLUMETRIC, [1e-7, -5e-8], np.stack([c_well, np.zeros(n)], axis=1))
    st = _state(por, sat, vol, Tk)
    tr.step(st, DT, rtol=1e-13, max_iterations=5000)
    T = st.a["total"].cpu().numpy()
    psv = por * sat * 1000.0 * vol
    area = 1.0
    dist0 = 0.25
    # TDispersionBC at the inflow face: boundary saturation 1, the cell's porosity
    hd = max(0.05 * q + 1.0 * 1.0 * por[0] * grid["tortuosity"] * grid["diffusion"], 1e-40) / dist0
    for c in range(n):
        dm = np.sum(psv * (T[c] - Tk[c])) / DT
        inflow = (hd + q) * area * 1000.0 * c_in[c] - hd * area * 1000.0 * T[c, 0]
        outflow = q * area * 1000.0 * T[c, -1]
        wells = 1e-7 * 1000.0 * c_well[c] - 5e-8 * 1000.0 * T[c, 150]
        want = inflow - outflow + wells
        assert abs(dm - want) <= 1e-9 * (abs(inflow) + abs(outflow) + abs(wells)), (c, dm, want)
