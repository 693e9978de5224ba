"""CPU checks of the global-implicit (GIRT) assembly: the block pattern that
pf_girt_pattern builds on the host, and the oracle's residual / Jacobian.

The oracle's Jacobian is checked against central differences (step 1e-6 in
ln m) of its own residual, with the water density at 1000 kg/m^3 so that the
reference's den*1e-3 factor on the mineral derivative is 1, and the residual's
flux terms against mass conservation (every internal connection adds to one
cell what it takes from the other, so the cell sum of the residual is the
cell sum of the accumulation and reaction terms).
"""
import numpy as np
import pytest

import cases
from pfgpu import abi
from pfgpu.girt import girt_pattern


@pytest.mark.parametrize("dims", [(1, 1, 1), (4, 1, 1), (3, 2, 1), (4, 3, 2), (5, 4, 3)])
def test_pattern(dims):
    nx, ny, nz = dims
    rp, ci = girt_pattern(nx, ny, nz)
    N = nx * ny * nz
    assert len(rp) == N + 1 and rp[0] == 0
    assert rp[-1] == 7 * N - 2 * (ny * nz + nx * nz + nx * ny)
    dense = np.zeros((N, N), bool)
    for X in range(N):
        cols = ci[rp[X]:rp[X + 1]]
        assert np.all(np.diff(cols) > 0)
        dense[X, cols] = True
        i, j, k = X % nx, (X // nx) % ny, X // (nx * ny)
        want = {X}
        for d, lim, s in ((i, nx, 1), (j, ny, nx), (k, nz, nx * ny)):
            if d > 0:
                want.add(X - s)
            if d < lim - 1:
                want.add(X + s)
        assert set(cols.tolist()) == want
    assert np.array_equal(dense, dense.T)


def test_pattern_bad_args():
    lib = abi.load()
    assert lib.pf_girt_pattern(0, 1, 1, None, None) == abi.PF_ERR_INVALID
    assert lib.pf_girt_pattern(2000, 2000, 2000, None, None) == abi.PF_ERR_TOO_LARGE


def _dense(net, rp, ci, vals):
    n = net.ncomp
    N = len(rp) - 1
    A = np.zeros((N * n, N * n))
    blk = vals.reshape(-1, n, n)
    for X in range(N):
        for b in range(rp[X], rp[X + 1]):
            A[X * n:(X + 1) * n, ci[b] * n:(ci[b] + 1) * n] = blk[b].T  # column-major blocks
    return A


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
@pytest.mark.parametrize("name", ["calcite", "random12"])
def test_oracle_jacobian_matches_fd(oracle, name, logf):
    nx, ny, nz = 3, 2, 2
    net, st, grid, tk = cases.girt_case(oracle, name, nx, ny, nz, log_formulation=logf)
    st.a["den_kg"][:] = 1000.0
    rp, ci = girt_pattern(nx, ny, nz)
    dt = 86400.0
    _, vals = oracle.girt_assemble(net, st.copy(), grid, tk, dt, rp, ci)
    A = _dense(net, rp, ci, vals)
    n, N = net.ncomp, st.ncells
    h = 1e-6
    fd = np.zeros_like(A)
    for c in range(N):
        for j in range(n):
            cols = []
            for sgn in (1.0, -1.0):
                s2 = st.copy()
                s2.a["pri_molal"][j, c] *= np.exp(sgn * h)
                r, _ = oracle.girt_assemble(net, s2, grid, tk, dt, rp, ci)
                cols.append(r)
            # log formulation: d r / d ln m; linear: d r / d m
            fd[:, c * n + j] = (cols[0] - cols[1]) / (2 * h) / (1.0 if logf else st.a["pri_molal"][j, c])
    scale = np.maximum(np.abs(fd).max(axis=0, keepdims=True), 1e-300)
    err = np.abs(A - fd) / scale
    assert err.max() < 1e-5, err.max()
    # the pattern holds every nonzero
    assert np.all((fd == 0) | (A != 0) | (np.abs(fd) < 1e-8 * scale))


def test_oracle_residual_conserves_mass(oracle):
    nx, ny, nz = 4, 3, 2
    net, st, grid, tk = cases.girt_case(oracle, "random12", nx, ny, nz)
    rp, ci = girt_pattern(nx, ny, nz)
    dt = 86400.0
    st2 = st.copy()
    r, _ = oracle.girt_assemble(net, st2, grid, tk, dt, rp, ci)
    # the same cells with no connection at all: accumulation + reaction only
    still = dict(grid, qx=np.zeros_like(grid["qx"]), qy=np.zeros_like(grid["qy"]), qz=np.zeros_like(grid["qz"]),
                 diffusion=0.0, dispersivity=0.0)
    r0, _ = oracle.girt_assemble(net, st.copy(), still, tk, dt, rp, ci)
    n = net.ncomp
    flux = (r - r0).reshape(-1, n)
    gross = np.abs(flux).sum(axis=0)
    assert np.all(np.abs(flux.sum(axis=0)) <= 1e-12 * np.maximum(gross, 1e-300))
    assert np.any(gross > 0)


def test_oracle_dry_cell_rows(oracle):
    """A dry cell (saturation below the minimum) has no connections, no
    accumulation and no reaction: its residual row is zero and its diagonal
    block is the identity (scaled by m in the log formulation)."""
    nx, ny, nz = 3, 2, 1
    net, st, grid, tk = cases.girt_case(oracle, "random12", nx, ny, nz, dry=(2,))
    rp, ci = girt_pattern(nx, ny, nz)
    r, vals = oracle.girt_assemble(net, st.copy(), grid, tk, 86400.0, rp, ci)
    n = net.ncomp
    assert np.all(r.reshape(-1, n)[2] == 0.0)
    A = _dense(net, rp, ci, vals)
    np.testing.assert_array_equal(A[2 * n:3 * n, 2 * n:3 * n], np.diag(st.a["pri_molal"][:, 2]))
    off = np.concatenate([A[2 * n:3 * n, :2 * n], A[2 * n:3 * n, 3 * n:]], axis=1)
    assert np.all(off == 0.0)


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
@pytest.mark.parametrize("sorb", ["ionx+langmuir", "mineral-scaled", "surface-same"])
def test_oracle_jacobian_with_sorption_matches_fd(oracle, sorb, logf):
    """With equilibrium sorption the diagonal blocks carry dtotal_sorb*V/dt
    (RAccumulationSorbDerivative) on top of the aqueous terms; a dry cell
    keeps its sorbed accumulation (the reference adds it unconditionally)."""
    nx, ny, nz = 3, 2, 1
    net, st, grid, tk, sk = cases.girt_sorption_case(oracle, sorb, nx, ny, nz, log_formulation=logf,
                                                     dry=(4,), den=1000.0)
    rp, ci = girt_pattern(nx, ny, nz)
    dt = 86400.0
    r0, vals = oracle.girt_assemble(net, st.copy(), grid, tk, dt, rp, ci, total_sorb_k=sk)
    A = _dense(net, rp, ci, vals)
    n, N = net.ncomp, st.ncells
    # the dry cell's identity (RTAccumulationDerivative) is no derivative of
    # the residual: take it out before comparing with the differences
    A[4 * n:5 * n, 4 * n:5 * n] -= np.diag(st.a["pri_molal"][:, 4] if logf else np.ones(n))
    # a wider step for the surface sites: their free-site Newton (the
    # reference's, whose update uses nu_f where the site balance's derivative
    # has nu_f^2) stops at a relative change of 1e-12, noise that a 1e-6 step
    # would magnify to 1e-5
    h = 1e-4 if sorb.startswith("surface") else 1e-6
    fd = np.zeros_like(A)
    for c in range(N):
        for j in range(n):
            cols = []
            for sgn in (1.0, -1.0):
                s2 = st.copy()
                s2.a["pri_molal"][j, c] *= np.exp(sgn * h)
                r, _ = oracle.girt_assemble(net, s2, grid, tk, dt, rp, ci, total_sorb_k=sk)
                cols.append(r)
            fd[:, c * n + j] = (cols[0] - cols[1]) / (2 * h) / (1.0 if logf else st.a["pri_molal"][j, c])
    scale = np.maximum(np.abs(fd).max(axis=0, keepdims=True), 1e-300)
    err = np.abs(A - fd) / scale
    assert err.max() < 1e-5, err.max()
    # the dry cell: no aqueous accumulation, connections or reaction; its row
    # is the sorbed accumulation alone and its block is I (x m) + dS V/dt
    st2 = st.copy()
    oracle.girt_assemble(net, st2, grid, tk, dt, rp, ci, total_sorb_k=sk)
    V = st.a["volume"][4]
    want = (st2.a["total_sorb"][:, 4] - sk[:, 4]) * V / dt
    np.testing.assert_allclose(r0.reshape(-1, n)[4], want, rtol=1e-13, atol=0)
    assert np.any(np.abs(want) > 0)


def test_oracle_girt_sorption_needs_fixed_sorbed_totals(oracle):
    net, st, grid, tk, sk = cases.girt_sorption_case(oracle, "ionx+langmuir", 2, 1, 1)
    rp, ci = girt_pattern(2, 1, 1)
    with pytest.raises(RuntimeError):
        oracle.girt_assemble(net, st.copy(), grid, tk, 3600.0, rp, ci)


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
@pytest.mark.parametrize("name", ["random12", "prefactors"])
def test_oracle_numerical_reaction_derivative(oracle, name, logf):
    """RReactionDerivative's forward differences (reaction.F90:4176-4230):
    the residual is the analytical mode's bit for bit, the Jacobian agrees
    with the analytical one to the forward-difference error (perturbation
    1e-5 of each molality), dry cells keep their identity block."""
    nx, ny, nz = 3, 2, 2
    if name == "prefactors":
        net, st = cases.prefactor_case(oracle, ncells=40, log_formulation=logf, with_secondary=False)
        st = st.subset(np.arange(nx * ny * nz))
        st.net = net
        grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=np.full((nz, ny, nx - 1), 2e-6),
                    qy=np.full((nz, ny - 1, nx), -1e-6), qz=np.full((nz - 1, ny, nx), 3e-6), diffusion=1e-9,
                    tortuosity=0.5, dispersivity=0.1)
        tk = st.a["total"] * 1.01
    else:
        net, st, grid, tk = cases.girt_case(oracle, name, nx, ny, nz, log_formulation=logf)
    st.a["saturation"][5] = 0.0
    st.a["den_kg"][:] = 1000.0  # the analytical mineral derivative's den*1e-3 factor is then 1
    rp, ci = girt_pattern(nx, ny, nz)
    r_a, v_a = oracle.girt_assemble(net, st.copy(), grid, tk, 86400.0, rp, ci)
    r_n, v_n = oracle.girt_assemble(net, st.copy(), grid, tk, 86400.0, rp, ci, numerical_derivatives=True)
    np.testing.assert_array_equal(r_n, r_a)
    A, B = _dense(net, rp, ci, v_a), _dense(net, rp, ci, v_n)
    n = net.ncomp
    assert np.array_equal(A[5 * n:6 * n, 5 * n:6 * n], B[5 * n:6 * n, 5 * n:6 * n])
    a = np.abs(A)
    scale = np.maximum(np.maximum(a.max(axis=0, keepdims=True), a.max(axis=1, keepdims=True)), 1e-300)
    err = np.abs(A - B) / scale
    assert err.max() < 1e-3, err.max()
    assert np.any(A != B)  # the reaction blocks did come from differences
