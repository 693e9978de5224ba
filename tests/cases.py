"""Parity cases: seeded networks + cells equilibrated by the oracle's
constraint restatement (reaction.F90:1328-2115 subset), with the reference's
initial auxvar sequence (condition_control.F90:1638-1649) and one TIMESTEP
activity refresh (pm_osrt.F90:145-151), i.e. the state the operator-split
cell loop sees at the start of a step.
"""
import numpy as np

from pfgpu import abi, generate
from pfgpu.network import CellState, default_options, tight_options


def prepare(oracle, net, st, ctype, cconc):
    # constraints always equilibrate with the reference's default tolerances
    eq = net.with_options(max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12,
                          max_rel_residual_tolerance=1e-8)
    rc, its = oracle.equilibrate(eq, st, ctype, cconc, nthreads=8)
    ok = its > 0
    st = st.subset(np.nonzero(ok)[0])
    den = st.a["den_kg"]
    st.a["pri_molal"][:] = st.a["pri_molal"] * den / 1000.0 / den * 1000.0
    st.a["pri_act_coef"][:] = 1.0
    st.a["sec_act_coef"][:] = 1.0
    st.a["sec_molal"][:] = 0.0
    oracle.update_auxvars(net, st, False, nthreads=8)
    if net.options["act_coef_update_frequency"] != abi.PF_ACT_COEF_OFF:
        oracle.update_auxvars(net, st, True, nthreads=8)
        oracle.update_auxvars(net, st, True, nthreads=8)
        oracle.update_auxvars(net, st, False, nthreads=8)
        oracle.update_activity_coefs(net, st, nthreads=8)
    return st, int((~ok).sum())


_CACHE = {}


def case(oracle, name, tight=False):
    key = (name, tight)
    if key in _CACHE:
        net, st = _CACHE[key]
        return net, st.copy()
    mk = tight_options if tight else default_options
    if name == "calcite":
        net = generate.calcite_network(mk())
        st, ct, cc = generate.calcite_cells(net, 1000, seed=20261203)
        dt = 3600.0
    elif name == "random12":
        net = generate.random_network(12, 40, 6, seed=12, options=mk(isothermal=0))
        st, ct, cc = generate.random_cells(net, 1500, seed=1212)
        dt = 86400.0
    elif name.startswith("hetero"):
        n = int(name[6:])
        net = generate.random_network(n, 3 * n, max(1, n // 2), seed=700 + n, options=mk(isothermal=0))
        st, ct, cc = generate.random_cells(net, 400, seed=7000 + n, dt_range=(3600.0, 30 * 86400.0))
        dt = 86400.0
    else:
        raise KeyError(name)
    st, nfail = prepare(oracle, net, st, ct, cc)
    assert nfail < 0.05 * len(ct and cc[0]), (name, nfail)
    _CACHE[key] = (net, st)
    return net, st.copy()


# converged tolerances: every Newton solve runs to rounding level (relative
# change below 1e-12, residual tests off, up to 100 iterations), so the result
# does not depend on where a loose stopping test happened to fire
CONVERGED = dict(max_relative_change_tolerance=1e-12, max_residual_tolerance=1e-300,
                 max_rel_residual_tolerance=1e-300, maximum_reaction_iterations=100)

CASE_DT = {"calcite": 3600.0, "random12": 86400.0, "random12raw": 86400.0}
CASE_DT.update({"hetero%d" % n: 86400.0 for n in (4, 6, 8, 10, 12, 16, 20, 24)})
HETERO = (4, 6, 8, 10, 12, 16, 20, 24)


def girt_case(oracle, name, nx, ny, nz, seed=5, log_formulation=True, dry=()):
    """A structured-grid GIRT case: the first nx*ny*nz prepared cells of
    `name`, face Darcy fluxes |q| ~ U[1e-7, 1e-5] m/s with random sign,
    D_m = 1e-9 m^2/s, tortuosity 0.5, dispersivity 0.1 m, and the previous
    time level's totals = the current ones times 5 % lognormal noise."""
    net, st = case(oracle, name)
    net = net.with_options(use_log_formulation=int(log_formulation))
    st = st.subset(np.arange(nx * ny * nz))
    st.net = net
    for c in dry:
        st.a["saturation"][c] = 0.0
    rng = np.random.default_rng(seed)

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=q((nz, ny, nx - 1)), qy=q((nz, ny - 1, nx)),
                qz=q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=0.5, dispersivity=0.1)
    total_k = st.a["total"] * np.exp(0.05 * rng.standard_normal(st.a["total"].shape))
    return net, st, grid, total_k


# a six-primary network with equilibrium sorption (ion exchange of four
# cations, a Langmuir isotherm or a mineral-scaled Freundlich one) for the
# global-implicit assembly
SORB_PRIMARY = ["Na+", "Ca++", "K+", "Cl-", "Tr", "Mg++"]
SORB_Z = [1.0, 2.0, 1.0, -1.0, 0.0, 2.0]
SORB_A0 = [4.0, 6.0, 3.0, 3.0, 3.0, 8.0]
SORB_SECS = [dict(name="NaCl(aq)", stoich={"Na+": 1.0, "Cl-": 1.0}, logK=0.5, Z=0.0, a0=3.0),
             dict(name="CaCl+", stoich={"Ca++": 1.0, "Cl-": 1.0}, logK=-0.4, Z=1.0, a0=4.0)]
SORB_MINS = [dict(name="Sylvite-like", stoich={"K+": 1.0, "Cl-": 1.0}, logK=-2.0, rate=1e-8, molar_vol=3.7e-5)]
# equilibrium surface complexation on three sites: a fixed site density with
# one-site complexes (closed form), sites on the kinetic mineral with a
# bidentate complex (the free-site Newton), and sites per kg of solid
SURFACE_SITES = [
    dict(site_density=500.0, complexes=[
        dict(name=">A-Na", stoich={"Na+": 1.0}, free_site_stoich=1.0, logK=-1.0),
        dict(name=">A-Ca+", stoich={"Ca++": 1.0}, free_site_stoich=1.0, logK=-2.0),
        dict(name=">A-Tr", stoich={"Tr": 1.0}, free_site_stoich=1.0, logK=-1.5)]),
    dict(site_density=2.0e4, surface="mineral", mineral="Sylvite-like", complexes=[
        dict(name=">B2-Mg", stoich={"Mg++": 1.0}, free_site_stoich=2.0, logK=-3.0),
        dict(name=">B-K", stoich={"K+": 1.0}, free_site_stoich=1.0, logK=-1.2),
        dict(name=">B-CaCl", stoich={"Ca++": 1.0, "Cl-": 1.0}, free_site_stoich=1.0, logK=-2.5)]),
    dict(site_density=0.05, surface="rock", complexes=[
        dict(name=">C-NaCl", stoich={"Na+": 1.0, "Cl-": 1.0}, free_site_stoich=1.0, logK=-0.5)]),
]

# sites whose complexes all hold the same components: there the reference's
# sorbed-total derivative (which spreads the free site's response over each
# complex's own species only, reaction_surf_complex.F90:874-893) is the exact
# derivative, so the oracle's Jacobian can be checked against differences
SURFACE_SITES_SAME = [
    dict(site_density=500.0, complexes=[
        dict(name=">A-Na", stoich={"Na+": 1.0}, free_site_stoich=1.0, logK=-1.0),
        dict(name=">A-Na2", stoich={"Na+": 2.0}, free_site_stoich=1.0, logK=-2.5)]),
    dict(site_density=2.0e4, surface="mineral", mineral="Sylvite-like", complexes=[
        dict(name=">B2-Mg", stoich={"Mg++": 1.0}, free_site_stoich=2.0, logK=-3.0),
        dict(name=">B-Mg", stoich={"Mg++": 1.0}, free_site_stoich=1.0, logK=-1.2)]),
]

SORPTIONS = {
    "surface-same": dict(surface=SURFACE_SITES_SAME, soil_particle_density=2650.0),
    "surface": dict(surface=SURFACE_SITES, soil_particle_density=2650.0),
    "surface+ionx+kd": dict(surface=SURFACE_SITES[:2], soil_particle_density=2650.0,
                            kd=[dict(species="Tr", type="linear", coeff=5.0)],
                            ionx=[dict(cations=[("Na+", 1.0), ("K+", 3.0)], cec=100.0)]),
    "ionx+langmuir": dict(kd=[dict(species="Tr", type="langmuir", coeff=80.0, b=3.0)],
                          ionx=[dict(cations=[("Na+", 1.0), ("Ca++", 0.3), ("K+", 5.0), ("Mg++", 0.4)],
                                     cec=250.0)]),
    "mineral-scaled": dict(kd=[dict(species="Tr", type="freundlich", coeff=20.0, n=1.5, mineral="Sylvite-like")],
                           ionx=[dict(cations=[("Na+", 1.0), ("K+", 3.0)], cec=4000.0, mineral="Sylvite-like")]),
}


def girt_sorption_case(oracle, sorb, nx, ny, nz, seed=9, log_formulation=True, dry=(), den=997.0):
    """A GIRT case on the sorption network: random molalities, porosity and
    mineral state, auxvars and activity coefficients from the oracle, the
    grid of girt_case, and the previous time level's aqueous and sorbed
    totals = the current ones times 5 % lognormal noise."""
    from pfgpu.network import ReactionNetwork
    net = ReactionNetwork.build(SORB_PRIMARY, SORB_Z, SORB_A0, SORB_SECS, SORB_MINS,
                                options=default_options(use_log_formulation=int(log_formulation)))
    net.sorption = SORPTIONS[sorb]
    N = nx * ny * nz
    rng = np.random.default_rng(seed)
    st = CellState.empty(net, N)
    st.a["pri_molal"][:] = 10.0 ** rng.uniform(-4.0, -2.0, (net.ncomp, N))
    st.a["porosity"][:] = rng.uniform(0.2, 0.4, N)
    st.a["saturation"][:] = rng.uniform(0.5, 1.0, N)
    st.a["den_kg"][:] = den
    st.a["mnrl_volfrac"][:] = rng.uniform(0.01, 0.1, (net.nmnrl, N))
    st.a["mnrl_area"][:] = rng.uniform(1.0, 50.0, (net.nmnrl, N))
    oracle.update_auxvars(net, st, False)
    oracle.update_activity_coefs(net, st)
    oracle.update_auxvars(net, st, False)
    for c in dry:
        st.a["saturation"][c] = 0.0

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    grid = dict(nx=nx, ny=ny, nz=nz, dx=2.0, dy=1.5, dz=0.5, qx=q((nz, ny, nx - 1)), qy=q((nz, ny - 1, nx)),
                qz=q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=0.5, dispersivity=0.1)
    total_k = st.a["total"] * np.exp(0.05 * rng.standard_normal(st.a["total"].shape))
    sorb_k = st.a["total_sorb"] * np.exp(0.05 * rng.standard_normal(st.a["total_sorb"].shape))
    return net, st, grid, total_k, sorb_k


def prefactor_network(net, with_secondary=True):
    """Attach rate prefactors to the five minerals of the 10-component test
    network: M0 an H+ term with a denominator (alpha 0.37, K 1e9, beta 1) and
    a plain power of P4; M1 two parallel prefactors, one with an activation
    energy; M2 a secondary species followed by a primary one (the primary
    species' derivative then walks the complex's species count, 3 of M2's 4
    species); M3 none; M4 a secondary species alone.  with_secondary=False
    keeps only the primary-species terms."""
    k = net.mnrl_rate_constant
    three = next(net.secondary[i] for i in range(net.nsec) if net.sec_nspec[i] == 3)
    two = next(net.secondary[i] for i in range(net.nsec) if net.sec_nspec[i] == 2)
    pf = {
        "M0": [dict(rate=k[0], species=[dict(name="H+", alpha=0.37, atten_coef=1e9, beta=1.0),
                                        dict(name="P4", alpha=0.31)])],
        "M1": [dict(rate=k[1], activation_energy=2.0e4,
                    species=[dict(name="P2", alpha=0.5, atten_coef=10.0, beta=0.5)]),
               dict(rate=0.3 * k[1], species=[dict(name="P6", alpha=1.0)])],
        "M2": [dict(rate=k[2], species=([dict(name=three, alpha=0.25, atten_coef=3.0, beta=0.7)]
                                        if with_secondary else []) + [dict(name="P5", alpha=0.2)])],
    }
    if with_secondary:
        pf["M4"] = [dict(rate=2.0 * k[4], species=[dict(name=two, alpha=0.4, atten_coef=5.0, beta=0.8)])]
    net.prefactors = pf
    return net


def prefactor_case(oracle, ncells=600, log_formulation=True, with_secondary=True):
    """The 10-component network (30 complexes, 5 kinetic minerals) with rate
    prefactors, cells from the constraint equilibrator, and each mineral's
    logK at the cells' median log Q so that about half of them precipitate."""
    opts = default_options(isothermal=0)
    opts["use_log_formulation"] = int(log_formulation)
    net = generate.random_network(10, 30, 5, seed=710, options=opts)
    st, ct, cc = generate.random_cells(net, ncells, seed=7101)
    st, _ = prepare(oracle, net, st, ct, cc)
    la = np.log10(st.a["pri_molal"] * st.a["pri_act_coef"])
    for m in range(net.nmnrl):
        lq = sum(net.mnrl_stoich[m, j] * la[net.mnrl_spec[m, j]] for j in range(net.mnrl_nspec[m]))
        delta = float(np.median(lq)) - net.mnrl_logK[m]
        net.mnrl_logK[m] += delta
        if net.mnrl_logKcoef is not None:
            net.mnrl_logKcoef[m, 1] += delta
    prefactor_network(net, with_secondary)
    st.net = net
    return net, st


def water_case(oracle, ncells=600, **opts):
    """The 8-component random network (24 complexes, 4 minerals) with water
    in a third of the complexes' and in two minerals' reactions and the
    ACTIVITY_H2O option on; cells from the constraint equilibrator, each
    mineral's logK at the cells' median log Q (log Q with the water term)."""
    o = default_options(isothermal=0, use_activity_h2o=1)
    o.update(opts)
    net = generate.random_network(8, 24, 4, seed=818, options=o)
    rng = np.random.default_rng(8188)
    net.sec_h2o_stoich = np.where(rng.uniform(size=net.nsec) < 0.35, rng.choice([-2.0, -1.0, 1.0, 3.0], net.nsec), 0.0)
    net.mnrl_h2o_stoich = np.array([1.0, 0.0, -2.0, 0.0])[:net.nmnrl]
    st, ct, cc = generate.random_cells(net, ncells, seed=8181)
    assert "ln_act_h2o" in st.a
    st, _ = prepare(oracle, net, st, ct, cc)
    la = np.log10(st.a["pri_molal"] * st.a["pri_act_coef"])
    for m in range(net.nmnrl):
        lq = sum(net.mnrl_stoich[m, k] * la[net.mnrl_spec[m, k]] for k in range(net.mnrl_nspec[m]))
        lq = lq + net.mnrl_h2o_stoich[m] * st.a["ln_act_h2o"] / np.log(10.0)
        delta = float(np.median(lq)) - net.mnrl_logK[m]
        net.mnrl_logK[m] += delta
        if net.mnrl_logKcoef is not None:
            net.mnrl_logKcoef[m, 1] += delta
    return net, st
