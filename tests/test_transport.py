"""The transport half of the operator-split step (pf_transport_step)
against the oracle's restatement of RTCalculateTransportMatrix solved
directly (scipy), and the conservation property of the zero-flux system.

CPU: the oracle matrix conserves mass (the flux part of every column sums to
zero: what a connection adds to one row it takes from the other) and has a
positive diagonal.  GPU: the Jacobi-BiCGStab solution of all components at
rtol 1e-13 agrees with the direct solution to 1e-9 relative (the solve's own
residual bound times the matrix's condition), on grids with both flux signs,
dry cells and 1-D shapes; at 64x64x32 cells the component masses
sum(psv*T) are conserved to 1e-10; a solve capped at too few iterations
reports non-convergence."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from pfgpu.girt import girt_pattern


def _grid(nx, ny, nz, seed, disp=0.1):
    rng = np.random.default_rng(seed)

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    return dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=q((nz, ny, nx - 1)), qy=q((nz, ny - 1, nx)),
                qz=q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=0.5, dispersivity=disp)


def _cells(N, seed, dry=()):
    rng = np.random.default_rng(seed)
    por = rng.uniform(0.1, 0.5, N)
    sat = np.ones(N)
    sat[list(dry)] = 0.0
    vol = 2.0 * 1.5 * 0.5 * np.ones(N)
    return por, sat, vol


def _matrix(oracle, grid, por, sat, vol, dt):
    rp, ci = girt_pattern(grid["nx"], grid["ny"], grid["nz"])
    vals = oracle.transport_matrix(grid, por, sat, vol, dt, rp, ci)
    N = len(rp) - 1
    return sp.csr_matrix((vals, ci, rp), shape=(N, N))


@pytest.mark.parametrize("dims", [(6, 5, 4), (20, 1, 1), (1, 1, 12)])
def test_oracle_matrix_conserves_mass(oracle, dims):
    grid = _grid(*dims, seed=1)
    N = int(np.prod(dims))
    por, sat, vol = _cells(N, 2)
    dt = 86400.0
    A = _matrix(oracle, grid, por, sat, vol, dt)
    psv_dt = por * sat * 1000.0 * vol / dt
    flux = A - sp.diags(psv_dt)
    assert np.max(np.abs(np.asarray(flux.sum(axis=0)).ravel())) <= 1e-12 * np.max(np.abs(flux.data))
    assert np.all(A.diagonal() > 0)


def test_oracle_matrix_dry_cells_have_no_flux(oracle):
    grid = _grid(4, 3, 2, seed=3)
    por, sat, vol = _cells(24, 4, dry=(5,))
    A = _matrix(oracle, grid, por, sat, vol, 3600.0).toarray()
    assert np.all(A[5, :] == 0.0) and np.all(A[:, 5] == 0.0)


def _gpu_case(oracle, dims, ncomp, seed, dry=(), rtol=1e-13, max_iterations=5000):
    torch = pytest.importorskip("torch")
    from pfgpu.girt import StructuredGrid
    from pfgpu.network import CellState
    from pfgpu.transport import OSTransport
    grid = _grid(*dims, seed=seed)
    N = int(np.prod(dims))
    por, sat, vol = _cells(N, seed + 1, dry)
    dt = 86400.0
    rng = np.random.default_rng(seed + 2)
    T0 = 10.0 ** rng.uniform(-6, -2, (ncomp, N))
    a = {"porosity": torch.from_numpy(por).cuda(), "saturation": torch.from_numpy(sat).cuda(),
         "volume": torch.from_numpy(vol).cuda(), "total": torch.from_numpy(T0.copy()).cuda()}
    st = CellState.__new__(CellState)
    st.a, st.ncells, st.net = a, N, None
    tr = OSTransport(StructuredGrid(**grid), ncomp)
    stats = tr.step(st, dt, rtol=rtol, max_iterations=max_iterations)
    got = a["total"].cpu().numpy()
    A = _matrix(oracle, grid, por, sat, vol, dt).tolil()
    psv = por * sat * 1000.0 * vol
    rhs = psv[None, :] * T0 / dt
    for c in dry:  # an empty (dry) row: the cell keeps its total
        A[c, c] = 1.0
        rhs[:, c] = T0[:, c]
    A = A.tocsc()
    ref = np.stack([spla.spsolve(A, rhs[c]) for c in range(ncomp)])
    return got, ref, T0, psv, stats


@pytest.mark.gpu
@pytest.mark.parametrize("dims,ncomp", [((6, 5, 4), 3), ((10, 7, 6), 12), ((40, 1, 1), 5), ((1, 1, 30), 2)])
def test_gpu_transport_matches_direct_solve(oracle, dims, ncomp):
    got, ref, T0, psv, stats = _gpu_case(oracle, dims, ncomp, seed=11)
    assert stats["converged"] == 1
    err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300))
    assert err < 1e-9, (err, stats)


@pytest.mark.gpu
def test_gpu_transport_conserves_mass():
    torch = pytest.importorskip("torch")
    from pfgpu.girt import StructuredGrid
    from pfgpu.network import CellState
    from pfgpu.transport import OSTransport
    dims, ncomp = (64, 64, 32), 12
    grid = _grid(*dims, seed=21)
    N = int(np.prod(dims))
    por, sat, vol = _cells(N, 22)
    rng = np.random.default_rng(23)
    T0 = 10.0 ** rng.uniform(-6, -2, (ncomp, N))
    a = {"porosity": torch.from_numpy(por).cuda(), "saturation": torch.from_numpy(sat).cuda(),
         "volume": torch.from_numpy(vol).cuda(), "total": torch.from_numpy(T0.copy()).cuda()}
    st = CellState.__new__(CellState)
    st.a, st.ncells, st.net = a, N, None
    tr = OSTransport(StructuredGrid(**grid), ncomp)
    stats = tr.step(st, 86400.0, rtol=1e-12, max_iterations=5000)
    got = a["total"].cpu().numpy()
    psv = por * sat * 1000.0 * vol
    m0, m1 = (psv * T0).sum(axis=1), (psv * got).sum(axis=1)
    assert np.max(np.abs(m1 - m0) / m0) < 1e-10, stats
    # the totals moved (the step is not the identity)
    assert np.max(np.abs(got - T0) / T0) > 1e-3


@pytest.mark.gpu
def test_gpu_transport_dry_cells_keep_their_totals(oracle):
    got, ref, T0, psv, stats = _gpu_case(oracle, (6, 5, 4), 4, seed=31, dry=(0, 17, 59))
    # an identity row goes through the iterations: its value to an ulp or two
    np.testing.assert_allclose(got[:, [0, 17, 59]], T0[:, [0, 17, 59]], rtol=1e-13, atol=0)
    err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300))
    assert err < 1e-9, err


@pytest.mark.gpu
def test_gpu_transport_reports_non_convergence(oracle):
    from pfgpu import abi
    with pytest.raises(abi.PfError):
        _gpu_case(oracle, (10, 7, 6), 3, seed=5, max_iterations=2)


def _state(dims, ncomp, seed):
    torch = pytest.importorskip("torch")
    from pfgpu.network import CellState
    N = int(np.prod(dims))
    por, sat, vol = _cells(N, seed + 1)
    rng = np.random.default_rng(seed + 2)
    T0 = 10.0 ** rng.uniform(-6, -2, (ncomp, N))
    st = CellState.__new__(CellState)
    st.a = {"porosity": torch.from_numpy(por).cuda(), "saturation": torch.from_numpy(sat).cuda(),
            "volume": torch.from_numpy(vol).cuda(), "total": torch.from_numpy(T0.copy()).cuda()}
    st.ncells, st.net = N, None
    return st, T0


@pytest.mark.gpu
def test_gpu_fixed_schedule_equals_adaptive():
    """pf_transport_enqueue with the schedule an adaptive step suggests gives
    bit for bit the adaptive step's totals (converged components make the
    extra launches no-ops); a schedule that is too short is reported by
    pf_transport_read_stats, and it leaves a partly converged answer."""
    torch = pytest.importorskip("torch")
    from pfgpu.girt import StructuredGrid
    from pfgpu.transport import OSTransport
    dims, ncomp = (12, 9, 7), 6
    tr = OSTransport(StructuredGrid(**_grid(*dims, seed=41)), ncomp)
    st, T0 = _state(dims, ncomp, 42)
    stats = tr.step(st, 86400.0, rtol=1e-12)
    ref = st.a["total"].clone()
    inner, refs = OSTransport.schedule(stats)
    assert stats["converged"] == 1 and stats["iterations"] >= stats["max_cycle_iterations"] >= 1
    st.a["total"].copy_(torch.from_numpy(T0))
    tr.enqueue(st, 86400.0, inner, refs, rtol=1e-12)
    fixed = tr.read_stats(1e-12)
    assert fixed["converged"] == 1
    assert fixed["iterations"] == stats["iterations"] and fixed["refinements"] == stats["refinements"]
    assert torch.equal(st.a["total"], ref)
    st.a["total"].copy_(torch.from_numpy(T0))
    tr.enqueue(st, 86400.0, 1, 1, rtol=1e-12)
    short = tr.read_stats(1e-12)
    assert short["converged"] == 0 and short["max_rel_residual"] > 1e-12


@pytest.mark.gpu
def test_gpu_fixed_schedule_in_cuda_graph():
    """The fixed schedule captured in a CUDA graph and replayed equals the
    same schedule enqueued eagerly."""
    torch = pytest.importorskip("torch")
    from pfgpu.girt import StructuredGrid
    from pfgpu.transport import OSTransport
    dims, ncomp = (16, 8, 8), 5
    tr = OSTransport(StructuredGrid(**_grid(*dims, seed=51)), ncomp)
    st, T0 = _state(dims, ncomp, 52)
    tr.enqueue(st, 3600.0, 12, 3)
    tr.enqueue(st, 3600.0, 12, 3)
    torch.cuda.synchronize()
    eager = st.a["total"].clone()
    st.a["total"].copy_(torch.from_numpy(T0))
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # warm-up outside the capture
        tr.enqueue(st, 3600.0, 12, 3)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    st.a["total"].copy_(torch.from_numpy(T0))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        tr.enqueue(st, 3600.0, 12, 3)
        tr.enqueue(st, 3600.0, 12, 3)
    st.a["total"].copy_(torch.from_numpy(T0))
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(st.a["total"], eager)
    assert tr.read_stats(1e-10)["converged"] == 1
