"""Equilibrium surface complexation (RTotalSorbEqSurfCplx1,
reaction_surf_complex.F90:641-900) in the C++ oracle and on the GPU.

Oracle (CPU): its total_sorb with surface complexation agrees with the
single-cell Python restatement (oracle.surface_complexation_eq, itself
pinned to the reference's surface-complexation-1 gold) on random cells, for
each site: a fixed site density with one-site complexes (closed-form free
site), sites on a kinetic mineral with a bidentate complex (the free-site
Newton) and sites per kg of solid.

GPU: the auxvar update (RTotal with sorption) against the oracle to 1e-12;
the operator-split step with the sorbed accumulation (plain and one-lane
batched kernels) under the parity comparison of tests/parity.py; the
surface-complexation-1 known answer through the library."""
import numpy as np
import pytest

import cases
import kat
from pfgpu.network import CellState, ReactionNetwork, default_options


def _net(sorb, options=None):
    net = ReactionNetwork.build(cases.SORB_PRIMARY, cases.SORB_Z, cases.SORB_A0, cases.SORB_SECS,
                                cases.SORB_MINS, options=options or default_options())
    net.sorption = cases.SORPTIONS[sorb]
    return net


def _cells(oracle, net, ncells, seed):
    rng = np.random.default_rng(seed)
    st = CellState.empty(net, ncells)
    st.a["pri_molal"][:] = 10.0 ** rng.uniform(-4.0, -2.0, (net.ncomp, ncells))
    st.a["porosity"][:] = rng.uniform(0.2, 0.4, ncells)
    st.a["den_kg"][:] = 997.0
    st.a["mnrl_volfrac"][:] = rng.uniform(0.01, 0.1, (net.nmnrl, ncells))
    st.a["mnrl_area"][:] = rng.uniform(1.0, 50.0, (net.nmnrl, ncells))
    oracle.update_auxvars(net, st, False)
    oracle.update_activity_coefs(net, st)
    oracle.update_auxvars(net, st, False)
    st.a["total"][:] *= rng.uniform(0.7, 1.3, st.a["total"].shape)
    return st


def test_oracle_surface_complexation_matches_the_single_cell_restatement(oracle):
    from oracle import oracle as om
    net = _net("surface")
    st = _cells(oracle, net, 40, 3)
    guess = st.a["srfcplx_free_site"].copy()  # the warm start of the evaluation below
    oracle.update_auxvars(net, st, False)
    sites = cases.SURFACE_SITES
    names = net.primary
    k0 = 0
    for r, site in enumerate(sites):
        cplx = [dict(spec=[names.index(s) for s in c["stoich"]], stoich=list(c["stoich"].values()),
                     free_site_stoich=c["free_site_stoich"], logK=c["logK"]) for c in site["complexes"]]
        for cell in range(st.ncells):
            if site.get("surface") == "mineral":
                dens = site["site_density"] * st.a["mnrl_volfrac"][0, cell]
            elif site.get("surface") == "rock":
                dens = site["site_density"] * 2650.0 * (1.0 - st.a["porosity"][cell])
            else:
                dens = site["site_density"]
            free, conc, ts, dts = om.surface_complexation_eq(
                list(st.a["pri_molal"][:, cell]), list(st.a["pri_act_coef"][:, cell]), cplx, dens,
                free_site_guess=guess[r, cell])
            assert st.a["srfcplx_free_site"][r, cell] == pytest.approx(free, rel=1e-12)
            for k, v in enumerate(conc):
                assert st.a["srfcplx_conc"][k0 + k, cell] == pytest.approx(v, rel=1e-12, abs=1e-300)
        k0 += len(site["complexes"])
    # the sorbed totals are the complexes' sums
    tot = np.zeros((net.ncomp, st.ncells))
    k = 0
    for site in sites:
        for c in site["complexes"]:
            for s_, nu in c["stoich"].items():
                tot[names.index(s_)] += nu * st.a["srfcplx_conc"][k]
            k += 1
    np.testing.assert_allclose(st.a["total_sorb"], tot, rtol=1e-12, atol=0)


def test_oracle_surface_complexation_step_conserves_mass(oracle):
    """RStep with surface complexation moves mass between the aqueous and the
    sorbed totals only (no mineral acts here: its rate constant is set to
    zero): psv*T + S*V is the same before and after."""
    net = _net("surface")
    net.mnrl_rate_constant = net.mnrl_rate_constant * 0.0
    st = _cells(oracle, net, 60, 4)
    # the fixed accumulation's sorbed part is that of the disturbed state
    oracle.update_auxvars(net, st, False)
    before = st.a["total"].copy()
    sorb0 = st.a["total_sorb"].copy()
    psv = st.a["porosity"] * st.a["saturation"] * 1000.0 * st.a["volume"]
    oracle.rstep(net, st, 86400.0)
    assert np.all(st.a["status"] == 0)
    m0 = psv * before + sorb0 * st.a["volume"]
    m1 = psv * st.a["total"] + st.a["total_sorb"] * st.a["volume"]
    np.testing.assert_allclose(m1, m0, rtol=1e-9)


# ---------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("sorb", ["surface", "surface+ionx+kd"])
def test_gpu_auxvars_with_surface_complexation(oracle, sorb):
    pytest.importorskip("torch")
    from pfgpu.engine import ReactionEngine
    net = _net(sorb)
    st = _cells(oracle, net, 500, 5)
    ref = st.copy()
    oracle.update_auxvars(net, ref, True)
    dev = st.to("cuda")
    ReactionEngine(net).update_auxvars(dev, True)
    got = dev.numpy()
    for k in ("total", "sec_molal", "pri_act_coef"):
        np.testing.assert_allclose(got.a[k], ref.a[k], rtol=1e-12, atol=0, err_msg=k)
    # the free-site Newton stops once its relative change is below 1e-12
    # (reaction_surf_complex.F90:677, :793): the two sides may stop one
    # iteration apart, so the free site and what is sorbed agree to a few
    # 1e-12 -- up to the complexes' site stoichiometry times that
    for k in ("srfcplx_free_site", "srfcplx_conc", "total_sorb"):
        np.testing.assert_allclose(got.a[k], ref.a[k], rtol=1e-10, atol=0, err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["batched", "group4", "plain"])
@pytest.mark.parametrize("sorb", ["surface", "surface+ionx+kd"])
def test_gpu_rstep_with_surface_complexation(oracle, sorb, kernel):
    pytest.importorskip("torch")
    import parity
    from pfgpu import abi
    from pfgpu.engine import ReactionEngine
    net = _net(sorb)
    st = _cells(oracle, net, 800, 6)
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    perts = []
    for key, to in (("total", np.inf), ("total", -np.inf), ("pri_molal", np.inf)):
        p = st.copy()
        p.a[key][:] = np.nextafter(p.a[key], to)
        oracle.rstep(net, p, 86400.0, nthreads=8)
        perts.append(p)
    eng = ReactionEngine(net)
    if kernel.startswith("group"):
        assert eng.set_launch_config(128, 2, 0, int(kernel[5:])) == abi.PF_OK
    dev = st.to("cuda")
    eng.rstep(dev, 86400.0, kernel=abi.PF_KERNEL_PLAIN if kernel == "plain" else abi.PF_KERNEL_BATCHED)
    got = dev.numpy()
    label = "surface/%s/%s" % (sorb, kernel)
    entry, ok = parity.compare(net, ref, got, 86400.0, label, perts)
    parity.check(entry, label, min_compared=int(0.9 * st.ncells))
    for k in ("total_sorb", "srfcplx_free_site", "srfcplx_conc"):
        np.testing.assert_allclose(got.a[k][..., ok], ref.a[k][..., ok], rtol=1e-10, atol=0, err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", kat.kat_names("surface"))
def test_gpu_surface_complexation_kat(oracle, name):
    """The surface-complexation-1 gold through the library: the constraint's
    speciation, then RTotal with the deck's surface complexation on the GPU."""
    pytest.importorskip("torch")
    from pfgpu.engine import ReactionEngine
    fx = kat.KAT[name]
    st = kat.initial_state(fx, kat.network(fx), oracle, oracle.density(25.0, 101325.0))
    net = kat.network(fx)
    sc = fx["surface_complexation"]
    net.sorption = dict(surface=[dict(site_density=sc["site_density"], complexes=[
        dict(name=c["name"], stoich=c["stoich"], free_site_stoich=c["free_site_stoich"], logK=c["logK"])
        for c in sc["complexes"]])])
    full = CellState.empty(net, st.ncells)
    for k in full.a:
        if k in st.a:
            full.a[k][...] = st.a[k]
    dev = full.to("cuda")
    ReactionEngine(net).update_auxvars(dev, False)
    got = dev.numpy()
    gold = fx["gold"]
    TOL = 1e-12
    assert got.a["srfcplx_free_site"][0, 0] == pytest.approx(gold["Free " + sc["site"]],
                                                            abs=max(TOL, 1e-12 * gold["Free " + sc["site"]]))
    for k, c in enumerate(sc["complexes"]):
        g = gold[c["name"]]
        assert got.a["srfcplx_conc"][k, 0] == pytest.approx(g, abs=max(TOL, 1e-12 * abs(g))), c["name"]
    for j, s_ in enumerate(net.primary):
        g = gold.get("Total Sorbed " + s_)
        if g is not None:
            assert got.a["total_sorb"][j, 0] == pytest.approx(g, abs=max(TOL, 1e-12 * abs(g))), s_
