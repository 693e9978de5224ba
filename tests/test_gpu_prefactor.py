"""Kinetic-mineral rate prefactors on the GPU against the oracle: the plain
step kernel (RStep with the prefactor rate and derivative of
RKineticMineral, reaction_mineral.F90:820-858, 976-1070) in the log and
linear formulations, the group-per-cell kernel, the global-implicit
assembly, and the entry points that refuse such a network."""
import numpy as np
import pytest

import cases
from pfgpu import abi
import parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.mark.parametrize("kernel,logf", [("plain", True), ("plain", False), ("group4", True), ("group8", True),
                                         ("group2", True)])
def test_rstep_with_prefactors_matches_oracle(oracle, kernel, logf):
    """The plain kernel (log and linear formulations) and the group-per-cell
    kernel (log formulation: its pivoted LU takes the prefactor derivative,
    which is not symmetric, into full rows)."""
    from pfgpu.engine import ReactionEngine
    net, st = cases.prefactor_case(oracle, ncells=1000, log_formulation=logf)
    ref = st.copy()
    assert oracle.rstep(net, ref, 3600.0, nthreads=8) == 0
    # the oracle on one-ulp-perturbed inputs: how far rounding alone moves
    # it (minerals near equilibrium amplify it by 1/|1 - Q/K|)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, 3600.0, nthreads=8)
        perts.append(p)
    eng = ReactionEngine(net)
    if kernel.startswith("group"):
        assert eng.set_launch_config(128, 2, 0, int(kernel[5:])) == abi.PF_OK
    dev = st.to("cuda")
    eng.rstep(dev, 3600.0, kernel=abi.PF_KERNEL_PLAIN if kernel == "plain" else abi.PF_KERNEL_BATCHED)
    got = dev.numpy()
    label = "prefactors/%s/%s" % (kernel, "log" if logf else "linear")
    entry, ok = parity.compare(net, ref, got, 3600.0, label, perts)
    parity.check(entry, label, min_compared=int(0.9 * st.ncells))
    r = ref.a["mnrl_rate"][:, ok]
    assert all((r[m] > 0).any() and (r[m] < 0).any() for m in range(net.nmnrl))


def test_kernels_without_prefactors_refuse_them(oracle):
    """The one-lane kernel (LDL^T of a symmetric Jacobian) and the adjoint
    have no prefactor terms; the group kernel carries them, but not with
    activity coefficients moving each Newton iteration."""
    from pfgpu.engine import ReactionEngine
    net, st = cases.prefactor_case(oracle, ncells=64)
    eng = ReactionEngine(net)
    dev = st.to("cuda")
    assert eng.set_launch_config(128, 1, 0, 1) == abi.PF_ERR_UNSUPPORTED
    for lanes in (2, 4, 8):
        assert eng.set_launch_config(128, 1, 0, lanes) == abi.PF_OK
    with pytest.raises(abi.PfError) as e:
        eng.adjoint(dev, 3600.0, dL_dtotal=torch.ones_like(dev.a["total"]))
    assert e.value.code == abi.PF_ERR_UNSUPPORTED
    ni = ReactionEngine(net.with_options(act_coef_update_frequency=abi.PF_ACT_COEF_NEWTON_ITER))
    for lanes in (1, 2, 4, 8):
        assert ni.set_launch_config(128, 1, 0, lanes) == abi.PF_ERR_UNSUPPORTED


@pytest.mark.parametrize("numjac", [False, True], ids=["analytical", "numerical"])
@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
def test_girt_with_prefactors_matches_oracle(oracle, logf, numjac):
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    from test_gpu_girt import _check, fd_noise
    nx, ny, nz = 8, 6, 5
    net, st = cases.prefactor_case(oracle, ncells=600, log_formulation=logf)
    st = st.subset(np.arange(nx * ny * nz))
    st.net = net
    st.a["saturation"][[3, 77]] = 0.0  # dry cells
    rng = np.random.default_rng(17)

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=q((nz, ny, nx - 1)), qy=q((nz, ny - 1, nx)),
                qz=q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=0.5, dispersivity=0.1)
    tk = st.a["total"] * np.exp(0.05 * rng.standard_normal(st.a["total"].shape))
    dt = 86400.0
    asm = GirtAssembler(ReactionEngine(net), StructuredGrid(**grid))
    dev = st.to("cuda")
    r, v = asm.assemble(dev, torch.from_numpy(tk).cuda(), dt, numerical_derivatives=numjac)
    torch.cuda.synchronize()
    ref_st = st.copy()
    r_ref, v_ref = oracle.girt_assemble(net, ref_st, grid, tk, dt, asm.rowptr_host, asm.colidx_host,
                                        numerical_derivatives=numjac)
    noise = fd_noise(oracle, net, st, grid, tk, dt, asm.rowptr_host, asm.colidx_host) if numjac else None
    _check(net, st, ref_st, dev.numpy(), asm, r.cpu().numpy(), v.cpu().numpy(), r_ref, v_ref, tk, dt,
           noise=noise)
    # rates relative to their gross size |rate| (1 + Q/K / |1 - Q/K|): next to
    # equilibrium 1 - Q/K cancels, and the rounding of Q/K (a product of
    # powers on the device, exp of a sum on the host) is what remains
    import parity
    got_rate = dev.numpy().a["mnrl_rate"]
    err = np.abs(got_rate - ref_st.a["mnrl_rate"]) / np.maximum(parity.gross_rate(net, ref_st), 1e-300)
    assert np.all(np.where(got_rate == ref_st.a["mnrl_rate"], 0.0, err) < 1e-12), float(err.max())
