"""The water activity option (ACTIVITY_H2O) on the GPU against the oracle:
the auxvar and activity update (LAG and NEWTON algorithms), RStep in every
kernel form that carries it (one-lane and group kernels with the water term
folded into the set-up pre-pass; the plain kernel also with activity updated
at each Newton iteration), the global-implicit assembly and constraint
equilibration; the kernels that refuse it."""
import numpy as np
import pytest

import cases
from pfgpu import abi
import parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.mark.parametrize("algo", [abi.PF_ACT_COEF_ALGO_LAG, abi.PF_ACT_COEF_ALGO_NEWTON], ids=["lag", "newton"])
def test_auxvars_with_water_activity(oracle, algo):
    from pfgpu.engine import ReactionEngine
    net, st = cases.water_case(oracle, ncells=400, act_coef_update_algorithm=algo)
    ref = st.copy()
    oracle.update_auxvars(net, ref, True)
    dev = st.to("cuda")
    ReactionEngine(net).update_auxvars(dev, True)
    got = dev.numpy()
    ok = np.isfinite(ref.a["pri_act_coef"]).all(axis=0)
    assert ok.mean() > 0.95
    for k in ("ln_act_h2o", "pri_act_coef", "sec_act_coef", "sec_molal", "total"):
        np.testing.assert_allclose(got.a[k][..., ok], ref.a[k][..., ok], rtol=1e-12, atol=0, err_msg=k)


@pytest.mark.parametrize("kernel,freq,algo", [("batched", abi.PF_ACT_COEF_TIMESTEP, abi.PF_ACT_COEF_ALGO_LAG),
                                              ("group4", abi.PF_ACT_COEF_TIMESTEP, abi.PF_ACT_COEF_ALGO_LAG),
                                              ("plain", abi.PF_ACT_COEF_TIMESTEP, abi.PF_ACT_COEF_ALGO_LAG),
                                              ("plain", abi.PF_ACT_COEF_NEWTON_ITER, abi.PF_ACT_COEF_ALGO_LAG),
                                              ("plain", abi.PF_ACT_COEF_NEWTON_ITER, abi.PF_ACT_COEF_ALGO_NEWTON)],
                         ids=["batched", "group4", "plain", "plain-lag-each-iteration",
                              "plain-newton-each-iteration"])
def test_rstep_with_water_activity(oracle, kernel, freq, algo):
    from pfgpu.engine import ReactionEngine
    net, st = cases.water_case(oracle, ncells=800, act_coef_update_frequency=freq, act_coef_update_algorithm=algo)
    ref = st.copy()
    assert oracle.rstep(net, ref, 3600.0, nthreads=8) == 0
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
    label = "water/%s/%d%s" % (kernel, freq, "/newton" if algo == abi.PF_ACT_COEF_ALGO_NEWTON else "")
    entry, ok = parity.compare(net, ref, got, 3600.0, label, perts)
    parity.check(entry, label, min_compared=int(0.9 * st.ncells))
    if freq == abi.PF_ACT_COEF_NEWTON_ITER:
        np.testing.assert_allclose(got.a["ln_act_h2o"][ok], ref.a["ln_act_h2o"][ok], rtol=1e-10, atol=0)


def test_water_activity_each_iteration_refused_by_the_fast_kernels(oracle):
    from pfgpu.engine import ReactionEngine
    net, st = cases.water_case(oracle, ncells=64, act_coef_update_frequency=abi.PF_ACT_COEF_NEWTON_ITER)
    eng = ReactionEngine(net)
    with pytest.raises(abi.PfError) as e:
        eng.rstep(st.to("cuda"), 3600.0, kernel=abi.PF_KERNEL_BATCHED)
    assert e.value.code == abi.PF_ERR_UNSUPPORTED
    for lanes in (1, 4):
        assert eng.set_launch_config(128, 1, 0, lanes) == abi.PF_ERR_UNSUPPORTED
    bare = st.copy()
    del bare.a["ln_act_h2o"]
    with pytest.raises(abi.PfError):
        eng.rstep(bare.to("cuda"), 3600.0, kernel=abi.PF_KERNEL_PLAIN)


def test_girt_with_water_activity(oracle):
    from pfgpu.engine import ReactionEngine
    from pfgpu.girt import GirtAssembler, StructuredGrid
    from test_gpu_girt import _check
    nx, ny, nz = 8, 6, 5
    net, st = cases.water_case(oracle, ncells=600)
    st = st.subset(np.arange(nx * ny * nz))
    st.net = net
    rng = np.random.default_rng(19)

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=q((nz, ny, nx - 1)), qy=q((nz, ny - 1, nx)),
                qz=q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=0.5, dispersivity=0.1)
    tk = st.a["total"] * np.exp(0.05 * rng.standard_normal(st.a["total"].shape))
    asm = GirtAssembler(ReactionEngine(net), StructuredGrid(**grid))
    dev = st.to("cuda")
    r, v = asm.assemble(dev, torch.from_numpy(tk).cuda(), 86400.0)
    torch.cuda.synchronize()
    ref_st = st.copy()
    r_ref, v_ref = oracle.girt_assemble(net, ref_st, grid, tk, 86400.0, asm.rowptr_host, asm.colidx_host)
    _check(net, st, ref_st, dev.numpy(), asm, r.cpu().numpy(), v.cpu().numpy(), r_ref, v_ref, tk, 86400.0)
    # ln a_H2O follows the molalities: no K cache across Newton iterates
    with pytest.raises(abi.PfError) as e:
        asm.assemble(st.to("cuda"), torch.from_numpy(tk).cuda(), 86400.0, k_cache="fill")
    assert e.value.code == abi.PF_ERR_UNSUPPORTED


def test_constraint_with_water_activity(oracle):
    from pfgpu import generate
    from pfgpu.engine import ReactionEngine
    net, _ = cases.water_case(oracle, ncells=64)
    st, ct, cc = generate.random_cells(net, 400, seed=4242)
    eq = net.with_options(max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12,
                          max_rel_residual_tolerance=1e-8)
    ref = st.copy()
    rc, its_ref = oracle.equilibrate(eq, ref, ct, cc, nthreads=8)
    dev = st.to("cuda")
    its = ReactionEngine(eq).equilibrate(dev, ct, torch.from_numpy(np.ascontiguousarray(cc)).cuda()).cpu().numpy()
    got = dev.numpy()
    ok = (its == its_ref) & (its_ref > 0)
    assert ok.mean() > 0.9, ok.mean()
    for k in ("pri_molal", "ln_act_h2o"):
        a, b = got.a[k][..., ok], ref.a[k][..., ok]
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)) < 1e-10, k
    assert np.all(ref.a["ln_act_h2o"][ok] < 0)
