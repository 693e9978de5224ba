"""GPU parity of pf_girt_assemble (global-implicit residual and SeqBAIJ
Jacobian on a structured grid) against the oracle's restatement of
RTResidual / RTJacobian.

Both sum every entry in the reference's order (connections x, y, z; then
accumulation; then reaction; then the log column scaling), so the entries
agree to rounding of the per-cell derivative terms.  Tolerance: 1e-10
relative to the largest entry of the same block row (matrix) and to the
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


def _run(oracle, name, dims, logf, dry=()):
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    nx, ny, nz = dims
    net, st, grid, tk = cases.girt_case(oracle, name, nx, ny, nz, log_formulation=logf, dry=dry)
    dt = 86400.0
    eng = ReactionEngine(net)
    g = StructuredGrid(**grid)
    asm = GirtAssembler(eng, g)
    dev = st.to("cuda")
    r, v = asm.assemble(dev, torch.from_numpy(tk).cuda(), dt)
    torch.cuda.synchronize()
    ref_st = st.copy()
    r_ref, v_ref = oracle.girt_assemble(net, ref_st, grid, tk, dt, asm.rowptr_host, asm.colidx_host)
    return net, st, ref_st, dev.numpy(), asm, r.cpu().numpy(), v.cpu().numpy(), r_ref, v_ref, tk, dt


def _check(net, st, ref_st, got_st, asm, r, v, r_ref, v_ref, tk, dt, sk=None):
    n, N = net.ncomp, st.ncells
    # matrix: per block row (cell, component i)
    blocks = v.reshape(-1, n, n)          # [b][col][row]
    blocks_ref = v_ref.reshape(-1, n, n)
    rows = np.repeat(np.arange(N), np.diff(asm.rowptr_host))
    row_scale = np.zeros((N, n))
    np.maximum.at(row_scale, rows, np.abs(blocks_ref).max(axis=1))
    err = np.abs(blocks - blocks_ref).max(axis=1) / np.maximum(row_scale[rows], 1e-300)
    assert err.max() < REL, ("values", err.max())
    # exact zeros where the reference has exact zeros (dry cells, connections)
    assert np.array_equal(blocks == 0.0, blocks_ref == 0.0)
    # residual, relative to the gross magnitude of its terms per component
    psv = st.a["porosity"] * st.a["saturation"] * 1000.0 * st.a["volume"]
    acc = (psv * np.maximum(np.abs(tk), np.abs(ref_st.a["total"])) / dt).T  # [cell][comp]
    if sk is not None:
        acc = acc + (st.a["volume"] * np.maximum(np.abs(sk), np.abs(ref_st.a["total_sorb"])) / dt).T
    # the kinetic-mineral terms' gross magnitude sum_m |nu_mj| |rate_m| V
    for m in range(net.nmnrl):
        for j in range(net.mnrl_nspec[m]):
            acc[:, net.mnrl_spec[m, j]] += np.abs(net.mnrl_stoich[m, j] * ref_st.a["mnrl_rate"][m]) * st.a["volume"]
    scale = np.maximum(acc.max(axis=0, keepdims=True), 1e-300)
    er = np.abs(r - r_ref).reshape(N, n) / scale
    assert er.max() < REL, ("residual", er.max())
    # the auxvars it updates
    np.testing.assert_allclose(got_st.a["total"], ref_st.a["total"], rtol=1e-13, atol=0)
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
@pytest.mark.parametrize("sorb", ["ionx+langmuir", "mineral-scaled"])
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
