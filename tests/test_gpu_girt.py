"""GPU parity of pf_girt_assemble (global-implicit residual and SeqBAIJ
Jacobian on a structured grid) against the oracle's restatement of
RTResidual / RTJacobian.

Both sum every entry in the reference's order (connections x, y, z; then
accumulation; then reaction; then the log column scaling), so the entries
agree to rounding of the per-cell derivative terms.  Tolerance: 1e-10
relative to the largest entry of the same block row (matrix; with the
reaction part by forward differences, 1e-6 of it on the diagonal blocks
plus 4x the oracle's own movement under a 64-eps change of the molalities,
see fd_noise) and to the
gross magnitude of the same component's residual terms -- the accumulation
psv*|total|/dt, the sorbed V*|S|/dt, the minerals' sum |nu| |rate| V --
(residual, whose terms cancel at convergence).
"""
import numpy as np
import pytest

import cases
from pfgpu import abi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-10


def _run(oracle, name, dims, logf, dry=(), numjac=False):
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    nx, ny, nz = dims
    net, st, grid, tk = cases.girt_case(oracle, name, nx, ny, nz, log_formulation=logf, dry=dry)
    dt = 86400.0
    eng = ReactionEngine(net)
    g = StructuredGrid(**grid)
    asm = GirtAssembler(eng, g)
    dev = st.to("cuda")
    r, v = asm.assemble(dev, torch.from_numpy(tk).cuda(), dt, numerical_derivatives=numjac)
    torch.cuda.synchronize()
    ref_st = st.copy()
    r_ref, v_ref = oracle.girt_assemble(net, ref_st, grid, tk, dt, asm.rowptr_host, asm.colidx_host,
                                        numerical_derivatives=numjac)
    out = (net, st, ref_st, dev.numpy(), asm, r.cpu().numpy(), v.cpu().numpy(), r_ref, v_ref, tk, dt)
    if numjac:
        return out, fd_noise(oracle, net, st, grid, tk, dt, asm.rowptr_host, asm.colidx_host)
    return out


def _mineral_gross(net, ref_st):
    """[cell][comp] sum over minerals of |nu| |rate| V: the gross size of the
    kinetic-mineral terms of each residual row."""
    g = np.zeros((ref_st.ncells, net.ncomp))
    for m in range(net.nmnrl):
        for j in range(net.mnrl_nspec[m]):
            g[:, net.mnrl_spec[m, j]] += np.abs(net.mnrl_stoich[m, j] * ref_st.a["mnrl_rate"][m]) * ref_st.a["volume"]
    return g


def fd_noise(oracle, net, st, grid, tk, dt, rp, ci, total_sorb_k=None):
    """How far the oracle's forward-difference Jacobian moves when the
    molalities move by 64 eps of themselves either way (elementwise maximum):
    the step of 1e-5 m_j turns last-bit differences of the mineral residual
    into 1e5 times larger ones, more still next to equilibrium where 1 - Q/K
    cancels.  64 eps in ln m is the size of the rounding of ln Q/K itself (a
    sum of terms of magnitude 10-50, fused into multiply-adds on the GPU and
    not on the host), which a one-ulp change of m (1e-16 in ln m) does not
    reach."""
    _, v0 = oracle.girt_assemble(net, st.copy(), grid, tk, dt, rp, ci, total_sorb_k=total_sorb_k,
                                 numerical_derivatives=True)
    noise = np.zeros_like(v0)
    for sgn in (1.0, -1.0):
        p = st.copy()
        p.a["pri_molal"][:] *= 1.0 + sgn * 64 * np.finfo(float).eps
        _, vp = oracle.girt_assemble(net, p, grid, tk, dt, rp, ci, total_sorb_k=total_sorb_k,
                                     numerical_derivatives=True)
        noise = np.maximum(noise, np.abs(vp - v0))
    return noise


def _check(net, st, ref_st, got_st, asm, r, v, r_ref, v_ref, tk, dt, sk=None, noise=None):
    n, N = net.ncomp, st.ncells
    # matrix: per block row (cell, component i)
    blocks = v.reshape(-1, n, n)          # [b][col][row]
    blocks_ref = v_ref.reshape(-1, n, n)
    rows = np.repeat(np.arange(N), np.diff(asm.rowptr_host))
    row_scale = np.zeros((N, n))
    np.maximum.at(row_scale, rows, np.abs(blocks_ref).max(axis=1))
    tol = REL * np.maximum(row_scale[rows], 1e-300)[:, None, :] * np.ones((1, n, 1))
    if noise is not None:
        # reaction part by forward differences (diagonal blocks): 1e-6 of the
        # block row plus 4x the oracle's own spread (fd_noise); a wrong step or
        # a missing term would be O(1) there, rounding through the 1e-5 step
        # reaches ~1e-9.  Off-diagonal (flux) blocks keep the 1e-10.
        diag = asm.colidx_host == rows
        tol[diag] = 1e-6 * np.maximum(row_scale[rows[diag]], 1e-300)[:, None, :] + \
            4 * noise.reshape(blocks.shape)[diag]
    diff = np.abs(blocks - blocks_ref)
    assert np.all(diff <= tol), ("values", float((diff / tol).max()))
    err = diff.max(axis=1) / np.maximum(row_scale[rows], 1e-300)
    # exact zeros where the reference has exact zeros (dry cells, connections)
    assert np.array_equal(blocks == 0.0, blocks_ref == 0.0)
    # residual, relative to the gross magnitude of its terms per component
    psv = st.a["porosity"] * st.a["saturation"] * 1000.0 * st.a["volume"]
    acc = (psv * np.maximum(np.abs(tk), np.abs(ref_st.a["total"])) / dt).T  # [cell][comp]
    if sk is not None:
        acc = acc + (st.a["volume"] * np.maximum(np.abs(sk), np.abs(ref_st.a["total_sorb"])) / dt).T
    # the kinetic-mineral terms' gross magnitude sum_m |nu_mj| |rate_m| V
    acc = acc + _mineral_gross(net, ref_st)
    scale = np.maximum(acc.max(axis=0, keepdims=True), 1e-300)
    er = np.abs(r - r_ref).reshape(N, n) / scale
    assert er.max() < REL, ("residual", er.max())
    # the auxvars it updates: totals relative to their gross size den (m +
    # sum |nu| s) -- a total with negative coefficients cancels, and the
    # complexes are a product of powers on the device, exp of a sum on the
    # host, equal to a few ulp
    import parity
    gross = parity.gross_total(net, ref_st)
    et = np.abs(got_st.a["total"] - ref_st.a["total"]) / np.maximum(gross, 1e-300)
    assert et.max() < 1e-13, ("total", float(et.max()))
    if net.nsec:
        np.testing.assert_allclose(got_st.a["sec_molal"], ref_st.a["sec_molal"], rtol=1e-13, atol=1e-300)
    if sk is not None:
        for k in ("total_sorb", "ionx_ref_sorbed"):
            np.testing.assert_allclose(got_st.a[k], ref_st.a[k], rtol=1e-12, atol=0, err_msg=k)
    return err.max(), er.max()


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
@pytest.mark.parametrize("name,dims", [("calcite", (8, 6, 5)), ("random12", (10, 7, 6)),
                                       ("hetero24", (7, 6, 4))])
def test_girt_parity(oracle, name, dims, logf):
    _check(*_run(oracle, name, dims, logf))


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
@pytest.mark.parametrize("sorb", ["ionx+langmuir", "mineral-scaled", "surface", "surface+ionx+kd"])
def test_girt_parity_with_sorption(oracle, sorb, logf):
    """Sorbed accumulation (S - S_k) V/dt in the residual and dS/dm V/dt on
    the diagonal blocks, dry cells included, against the oracle."""
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    net, st, grid, tk, sk = cases.girt_sorption_case(oracle, sorb, 9, 7, 5, log_formulation=logf,
                                                     dry=(0, 11, 100, 314))
    dt = 86400.0
    eng = ReactionEngine(net)
    asm = GirtAssembler(eng, StructuredGrid(**grid))
    dev = st.to("cuda")
    with pytest.raises(ValueError):
        asm.assemble(dev, torch.from_numpy(tk).cuda(), dt)
    r, v = asm.assemble(dev, torch.from_numpy(tk).cuda(), dt, total_sorb_k=torch.from_numpy(sk).cuda())
    torch.cuda.synchronize()
    ref_st = st.copy()
    r_ref, v_ref = oracle.girt_assemble(net, ref_st, grid, tk, dt, asm.rowptr_host, asm.colidx_host,
                                        total_sorb_k=sk)
    _check(net, st, ref_st, dev.numpy(), asm, r.cpu().numpy(), v.cpu().numpy(), r_ref, v_ref, tk, dt, sk=sk)


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
def test_girt_parity_numerical_reaction_derivative(oracle, logf):
    """The reaction Jacobian by forward differences (the reference's
    NUMERICAL_JACOBIAN transport option) against the oracle's, with dry
    cells; a network whose minerals react (16 components)."""
    out, noise = _run(oracle, "hetero16", (7, 6, 4), logf, dry=(2, 50), numjac=True)
    _check(*out, noise=noise)
    # the allowance stays small: most entries agree to the analytical tolerance
    assert np.median(noise[noise > 0] / np.abs(out[8][noise > 0])) < 1e-8


def test_girt_parity_dry_cells_and_thin_grids(oracle):
    _check(*_run(oracle, "random12", (6, 5, 4), True, dry=(0, 7, 33, 119)))
    _check(*_run(oracle, "random12", (40, 1, 1), True))
    _check(*_run(oracle, "random12", (1, 1, 30), False))
    _check(*_run(oracle, "calcite", (1, 1, 1), True))


def test_girt_matches_scipy_product(oracle):
    """The BAIJ arrays describe the same operator as the oracle's (matrix-
    vector product through scipy's BSR)."""
    net, st, ref_st, got, asm, r, v, r_ref, v_ref, tk, dt = _run(oracle, "random12", (5, 4, 3), True)
    A, B = asm.to_scipy(v), asm.to_scipy(v_ref)
    x = np.random.default_rng(3).standard_normal(A.shape[1])
    ya, yb = A @ x, B @ x
    assert np.max(np.abs(ya - yb)) <= 1e-10 * np.max(np.abs(B) @ np.abs(x))


def test_girt_bad_args(oracle):
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    net, st, grid, tk = cases.girt_case(oracle, "calcite", 4, 3, 2)
    eng = ReactionEngine(net)
    asm = GirtAssembler(eng, StructuredGrid(**grid))
    bad = st.subset(np.arange(20)).to("cuda")  # 20 != 4*3*2 cells
    with pytest.raises(abi.PfError):
        asm.assemble(bad, torch.from_numpy(tk[:, :20].copy()).cuda(), 86400.0)
    with pytest.raises(abi.PfError):
        asm.assemble(st.to("cuda"), torch.from_numpy(tk).cuda(), 0.0)


@pytest.mark.parametrize("name,logf", [("random12", True), ("hetero16", False), ("calcite", True)])
def test_girt_k_cache(oracle, name, logf):
    """The per-cell K cache: an assembly that fills it and one that reads it
    give the values, residual and auxvars of an assembly without it, bit for
    bit (the same K, the same arithmetic after), over two Newton iterates of
    one step; reading before any fill is refused."""
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    net, st, grid, tk = cases.girt_case(oracle, name, 6, 5, 4, log_formulation=logf, dry=(3,))
    eng = ReactionEngine(net)
    plain = GirtAssembler(eng, StructuredGrid(**grid))
    cached = GirtAssembler(eng, StructuredGrid(**grid))
    with pytest.raises(ValueError):
        cached.assemble(st.to("cuda"), torch.from_numpy(tk).cuda(), 86400.0, k_cache="read")
    tkd = torch.from_numpy(tk).cuda()
    for it, mode in enumerate(("fill", "read", "read")):
        a, b = st.to("cuda"), st.to("cuda")
        for d in (a, b):  # a later Newton iterate: other molalities, same temperatures
            d.a["pri_molal"].mul_(1.0 + 0.01 * it)
        r0, v0 = plain.assemble(a, tkd, 86400.0)
        r1, v1 = cached.assemble(b, tkd, 86400.0, k_cache=mode)
        torch.cuda.synchronize()
        assert torch.equal(v0, v1) and torch.equal(r0, r1), mode
        for k in ("total", "sec_molal", "mnrl_rate"):
            assert torch.equal(a.a[k], b.a[k]), (mode, k)
