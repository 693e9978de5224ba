"""Seeded synthetic networks and cell inputs for the benchmark configurations.

calcite_network / calcite_cells
    The calcite system of the 10x10x10 operator-split case: primaries H+,
    HCO3-, Ca++; six aqueous complexes; kinetic calcite.  Ion size
    parameters a0, charges and the calcite molar volume are those of the
    reference's calcite database (regression_tests/ascem/batch/calcite.dat);
    logK values are the rounded 25 C values of the case definition.
random_network / random_cells
    Synthetic networks: integer stoichiometry at density 0.3 -- in {-2..2}
    for H+ and in {1, 2} for the other primaries, so every total is
    increasing in every free-ion molality and each constraint has one
    solution (random negative coefficients on non-proton components make
    most draws infeasible) -- log10 K ~ U[-15, 15], species charges in
    {-2..2}, an OH- complex (H2O - H+) so that a charge balance on H+ is
    always attainable, kinetic rate constants log10 U[-10, -5], logK linear
    in temperature (fit coefficients (0, a, b, 0, 0) of
    ReactionInterpolateLogK).  Cells: totals log10 U[-6, -2], H+ by charge
    balance, T ~ U[5, 60] C.

Every generator takes an explicit seed (numpy default_rng) and is the only
source of inputs for the tests and the benchmark; no public dataset is used.
"""
from __future__ import annotations

import numpy as np

from . import abi
from .network import CellState, ReactionNetwork, default_options

# calcite.dat:4-20 (a0, Z) and :26 (molar volume, cm^3/mol)
_CALCITE_PRI = [("H+", 1.0, 9.0), ("HCO3-", -1.0, 4.0), ("Ca++", 2.0, 6.0)]
_CALCITE_SEC = [
    ("OH-", {"H+": -1.0}, 13.99, -1.0, 3.5),
    ("CO3--", {"H+": -1.0, "HCO3-": 1.0}, 10.33, -2.0, 4.5),
    ("CO2(aq)", {"H+": 1.0, "HCO3-": 1.0}, -6.34, 0.0, 3.0),
    ("CaOH+", {"H+": -1.0, "Ca++": 1.0}, 12.85, 1.0, 4.0),
    ("CaHCO3+", {"Ca++": 1.0, "HCO3-": 1.0}, -1.04, 1.0, 4.0),
    ("CaCO3(aq)", {"H+": -1.0, "Ca++": 1.0, "HCO3-": 1.0}, 7.01, 0.0, 3.0),
]


def calcite_network(options=None) -> ReactionNetwork:
    sec = [dict(name=n, stoich=st, logK=k, Z=z, a0=a) for n, st, k, z, a in _CALCITE_SEC]
    mins = [dict(name="Calcite", stoich={"H+": -1.0, "Ca++": 1.0, "HCO3-": 1.0}, logK=1.85,
                 rate=1.0e-6, molar_vol=36.934 * 1.0e-6)]
    return ReactionNetwork.build([p[0] for p in _CALCITE_PRI], [p[1] for p in _CALCITE_PRI],
                                 [p[2] for p in _CALCITE_PRI], sec, mins,
                                 options=options or default_options())


def calcite_cells(net: ReactionNetwork, ncells: int, seed: int = 20261203):
    """Per-cell draws of the calcite case.  Returns (state, ctype, cconc) where
    ctype/cconc describe the constraint (H+ by pH, HCO3- and Ca++ TOTAL)."""
    rng = np.random.default_rng(seed)
    st = CellState.empty(net, ncells)
    pH = rng.uniform(5.0, 9.0, ncells)
    ca = 10.0 ** rng.uniform(-5.0, -2.0, ncells)
    hco3 = 10.0 ** rng.uniform(-4.0, -2.0, ncells)
    st.a["mnrl_volfrac"][0] = rng.uniform(0.0, 0.1, ncells)
    st.a["mnrl_area"][0] = rng.uniform(1.0, 100.0, ncells)
    st.a["porosity"][:] = rng.uniform(0.1, 0.5, ncells)
    st.a["saturation"][:] = 1.0
    st.a["temperature"][:] = 25.0
    st.a["den_kg"][:] = water_density(25.0)
    st.a["volume"][:] = 1.0
    ctype = [abi.PF_CONSTRAINT_PH, abi.PF_CONSTRAINT_TOTAL, abi.PF_CONSTRAINT_TOTAL]
    cconc = np.stack([pH, hco3, ca])
    return st, ctype, cconc


def water_density(t_c: float, p_pa: float = 101325.0) -> float:
    """Liquid water density, IFC-67 industrial formulation (1967 IFC), kg/m^3.
    The same published formulation PFLOTRAN uses by default
    (src/pflotran/eos_water.F90:1583-1748); used only to fill den_kg."""
    aa = [6.824687741e03, -5.422063673e02, -2.096666205e04, 3.941286787e04, -6.733277739e04,
          9.902381028e04, -1.093911774e05, 8.590841667e04, -4.511168742e04, 1.418138926e04,
          -2.017271113e03, 7.982692717e00, -2.616571843e-2, 1.522411790e-3, 2.284279054e-2,
          2.421647003e02, 1.269716088e-10, 2.074838328e-7, 2.174020350e-8, 1.105710498e-9,
          1.293441934e01, 1.308119072e-5, 6.047626338e-14]
    a1, a2, a3, a4, a5, a6 = 8.438375405e-1, 5.362162162e-4, 1.72, 7.342278489e-2, 4.975858870e-2, 6.5371543e-1
    a7, a8, a9, a10, a11, a12 = 1.15e-6, 1.5108e-5, 1.4188e-1, 7.002753165, 2.995284926e-4, 2.04e-1
    theta = (t_c + 273.15) / 647.3
    beta = p_pa / 22.064e6
    th2 = theta * theta
    th18 = theta ** 18.0
    th20 = th18 * th2
    yy = 1.0 - a1 * th2 - a2 * theta ** (-6.0)
    xx = a3 * yy * yy - 2.0 * (a4 * theta - a5 * beta)
    xx = np.sqrt(xx) if xx > 0 else 1e-6
    zz = yy + xx
    u1 = aa[11] * a5 * zz ** (-5.0 / 17.0)
    u2 = 1.0 / (a8 + theta ** 11.0)
    u3 = aa[17] + (2.0 * aa[18] + 3.0 * aa[19] * beta) * beta
    u4 = 1.0 / (a7 + th18 * theta)
    u5 = (a10 + beta) ** (-4.0)
    u6 = a11 - 3.0 * u5
    u7 = aa[20] * th18 * (a9 + th2)
    u8 = aa[15] * (a6 - theta) ** 9.0
    vr = (u1 + aa[12] + theta * (aa[13] + aa[14] * theta) + u8 * (a6 - theta) + aa[16] * u4 - u2 * u3
          - u6 * u7 + (3.0 * aa[21] * (a12 - theta) + 4.0 * aa[22] * beta / th20) * beta * beta)
    return 1.0 / (vr * 0.00317)


def random_network(ncomp: int, nsec: int, nmnrl: int, seed: int, temperature_dependent: bool = True,
                   options=None, signed: bool = False) -> ReactionNetwork:
    """signed: the non-H coefficients drawn from {-2, -1, 1, 2} (each row
    keeps at least one positive one); some TOTAL constraints of such a
    network have no solution, and the cells whose equilibration fails are
    dropped by the callers (resampled from a larger draw)."""
    rng = np.random.default_rng(seed)
    primary = ["H+"] + ["P%d" % k for k in range(1, ncomp)]
    pri_Z = np.concatenate([[1.0], rng.integers(-2, 3, ncomp - 1).astype(float)])
    pri_a0 = np.concatenate([[9.0], rng.uniform(3.0, 9.0, ncomp - 1)])
    tref = 298.15

    def rxn_row():
        while True:
            mask = rng.random(ncomp) < 0.3
            nu = rng.choice([-2.0, -1.0, 1.0, 2.0] if signed else [1.0, 2.0], ncomp) * mask
            nu[0] = rng.choice([-2.0, -1.0, 1.0, 2.0]) * mask[0]
            if not (nu[1:] > 0).any():
                continue
            z = float(nu @ pri_Z)
            if abs(z) <= 2.0:
                return nu, z

    def linear_T(logK):
        b = rng.uniform(-0.02, 0.02)
        return [0.0, logK - b * tref, b, 0.0, 0.0]

    secs = []
    oh = dict(name="OH-", stoich={"H+": -1.0}, logK=13.99, Z=-1.0, a0=3.5)
    if temperature_dependent:
        oh["logKcoef"] = linear_T(13.99)
    secs.append(oh)
    for i in range(nsec - 1):
        nu, z = rxn_row()
        logK = rng.uniform(-15.0, 15.0)
        d = dict(name="S%d" % i, stoich={primary[k]: nu[k] for k in np.nonzero(nu)[0]}, logK=logK, Z=z,
                 a0=rng.uniform(3.0, 5.0))
        if temperature_dependent:
            d["logKcoef"] = linear_T(logK)
        secs.append(d)
    mins = []
    for m in range(nmnrl):
        nu, _ = rxn_row()
        logK = rng.uniform(-15.0, 15.0)
        d = dict(name="M%d" % m, stoich={primary[k]: nu[k] for k in np.nonzero(nu)[0]}, logK=logK,
                 rate=10.0 ** rng.uniform(-10.0, -5.0), molar_vol=rng.uniform(2.0e-5, 6.0e-5))
        if temperature_dependent:
            d["logKcoef"] = linear_T(logK)
        mins.append(d)
    opts = options or default_options(isothermal=0 if temperature_dependent else 1)
    return ReactionNetwork.build(primary, pri_Z, pri_a0, secs, mins, options=opts)


def random_cells(net: ReactionNetwork, ncells: int, seed: int, dt_range=None, free: bool = False):
    """Cells for a random network.  Returns (state, ctype, cconc); the
    constraint is TOTAL for every component but H+, which carries the charge
    balance (initial guess 1e-7).  dt_range=(lo, hi) adds a per-cell dt drawn
    log-uniformly.  free: FREE constraints instead (free molalities log10
    U[-8, -4], H+ 10^-U[5, 9]), for networks with signed stoichiometry whose
    TOTAL constraints mostly have no solution."""
    rng = np.random.default_rng(seed)
    st = CellState.empty(net, ncells, with_dt=dt_range is not None)
    n = net.ncomp
    totals = 10.0 ** rng.uniform(-6.0, -2.0, (n, ncells))
    cconc = totals.copy()
    h = net.h_ion_id
    cconc[h] = 1.0e-7
    ctype = [abi.PF_CONSTRAINT_TOTAL] * n
    ctype[h] = abi.PF_CONSTRAINT_CHARGE_BAL
    if free:
        # free-ion constraints: any molalities are an equilibrium state,
        # whatever the signs of the stoichiometry
        cconc = 10.0 ** rng.uniform(-8.0, -4.0, (n, ncells))
        cconc[h] = 10.0 ** -rng.uniform(5.0, 9.0, ncells)
        ctype = [abi.PF_CONSTRAINT_FREE] * n
    if net.nmnrl:
        st.a["mnrl_volfrac"][:] = rng.uniform(0.0, 0.1, (net.nmnrl, ncells))
        st.a["mnrl_area"][:] = rng.uniform(1.0, 100.0, (net.nmnrl, ncells))
    st.a["porosity"][:] = rng.uniform(0.1, 0.5, ncells)
    st.a["saturation"][:] = 1.0
    st.a["temperature"][:] = rng.uniform(5.0, 60.0, ncells)
    st.a["den_kg"][:] = water_density(25.0)
    st.a["volume"][:] = 1.0
    if dt_range is not None:
        lo, hi = dt_range
        st.a["dt_cell"][:] = np.exp(rng.uniform(np.log(lo), np.log(hi), ncells))
    return st, ctype, cconc


def heterogeneous_networks(seed: int = 7, ncomps=(4, 6, 8, 10, 12, 16, 20, 24)):
    """The eight networks of the heterogeneous mix: secondaries = 3 x ncomp,
    kinetic minerals = ncomp / 2."""
    return [random_network(n, 3 * n, max(1, n // 2), seed=seed * 100 + n) for n in ncomps]
