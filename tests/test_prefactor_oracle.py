"""Kinetic-mineral rate prefactors in the oracle (RKineticMineral,
reaction_mineral.F90:820-858 and the derivative :976-1070).  No reference
test holds a batch cell with prefactors (the reference's one deck with them,
default/column/mineral_prefactor, is a transport column), so the
restatement is checked by its definition: the rates against the prefactor
formula evaluated here in numpy, the Jacobian against central differences
of the oracle's own residual where the reference's derivative is exact
(primary prefactor species), and, with a secondary prefactor species,
against central differences plus the two departures the reference's
derivative makes there, computed here independently."""
import ctypes as C

import numpy as np
import pytest

import cases
from pfgpu import abi
from pfgpu.girt import girt_pattern

LOG_TO_LN = 2.30258509299
R_GAS = 8.31446


def _arrhenius(ea, temp):
    return np.exp(ea / R_GAS * (1.0 / 298.15 - 1.0 / (temp + 273.15))) if ea > 0 else np.ones_like(temp)


def _logK(coef, temp):
    tk = temp + 273.15
    return coef[0] * np.log(tk) + coef[1] + coef[2] * tk + coef[3] / tk + coef[4] / tk ** 2


def _lnact(net, st):
    la = np.log(st.a["pri_molal"]) + np.log(st.a["pri_act_coef"])
    lsa = np.log(st.a["sec_molal"]) + np.log(st.a["sec_act_coef"])
    return la, lsa


def _factor(net, la, lsa, sp):
    """exp(alpha ln a - ln(1 + K a^beta)) of one prefactor species."""
    name = sp["name"]
    lna = la[net.primary.index(name)] if name in net.primary else lsa[net.secondary.index(name)]
    K, a, b = sp.get("atten_coef", 0.0), sp.get("alpha", 0.0), sp.get("beta", 0.0)
    return np.exp(a * lna - np.log1p(K * np.exp(b * lna))), lna


def _sum_rate(net, st, m, la, lsa):
    """sum_prefactor_rate of mineral m and, per prefactor, its product P_p."""
    temp = st.a["temperature"]
    name = net.minerals[m]
    prefs = (net.prefactors or {}).get(name, [])
    if not prefs:
        return net.mnrl_rate_constant[m] * _arrhenius(net.mnrl_activation_energy[m], temp), []
    total, prods = 0.0, []
    for pr in prefs:
        P = np.ones(st.ncells)
        for sp in pr.get("species", ()):
            P = P * _factor(net, la, lsa, sp)[0]
        prods.append(P)
        total = total + pr["rate"] * _arrhenius(pr.get("activation_energy", 0.0), temp) * P
    return total, prods


def _prepared(oracle, with_secondary=True, ncells=200):
    net, st = cases.prefactor_case(oracle, ncells=ncells, with_secondary=with_secondary)
    for key in ("mnrl_rate_limiter", "mnrl_affinity_threshold"):
        assert np.all(getattr(net, key) == 0.0)
    assert not np.any(net.mnrl_irreversible)
    assert net.mnrl_min_scale_factor is None and net.mnrl_Temkin_const is None
    assert net.mnrl_affinity_power is None
    oracle.update_auxvars(net, st, False)
    return net, st


def test_rates_follow_the_prefactor_formula(oracle):
    net, st = _prepared(oracle)
    got = st.copy()
    oracle.update_kinetic_state(net, got, 0.0)
    la, lsa = _lnact(net, st)
    temp = st.a["temperature"]
    for m in range(net.nmnrl):
        lnQK = -_logK(net.mnrl_logKcoef[m], temp) * LOG_TO_LN
        for j in range(net.mnrl_nspec[m]):
            lnQK = lnQK + net.mnrl_stoich[m, j] * la[net.mnrl_spec[m, j]]
        aff = 1.0 - np.exp(lnQK)
        sign = np.where(aff >= 0.0, 1.0, -1.0)
        active = (st.a["mnrl_volfrac"][m] > 0) | (sign < 0)
        S, _ = _sum_rate(net, st, m, la, lsa)
        want = np.where(active, -st.a["mnrl_area"][m] * sign * np.abs(aff) * S, 0.0)
        np.testing.assert_allclose(got.a["mnrl_rate"][m], want, rtol=1e-11, atol=0, err_msg=net.minerals[m])
        assert np.any(want != 0.0)
    # the prefactors change the rates: the plain rate constants give others
    plain = st.copy()
    net2 = cases.prefactor_case(oracle, ncells=200)[0]
    net2.prefactors = None
    oracle.update_kinetic_state(net2, plain, 0.0)
    assert not np.allclose(plain.a["mnrl_rate"][:3], got.a["mnrl_rate"][:3])
    np.testing.assert_array_equal(plain.a["mnrl_rate"][3], got.a["mnrl_rate"][3])


def _dense_block(net, vals):
    n = net.ncomp
    return vals.reshape(-1, n, n)[0].T  # the one cell's block, row-major


def _grid1():
    z = np.zeros((1, 1, 0))
    return dict(nx=1, ny=1, nz=1, dx=1.0, dy=1.0, dz=1.0, qx=z, qy=z.reshape(1, 0, 1), qz=z.reshape(0, 1, 1),
                diffusion=1e-9, tortuosity=0.5, dispersivity=0.0)


def _jac_and_fd(oracle, net, cell_state, logf, h=1e-6):
    """Reaction + accumulation Jacobian of one cell (GIRT, 1x1x1 grid) and
    its central differences in ln m (log form) or m (linear form)."""
    grid = _grid1()
    rp, ci = girt_pattern(1, 1, 1)
    tk = cell_state.a["total"].copy()
    s0 = cell_state.copy()
    _, vals = oracle.girt_assemble(net, s0, grid, tk, 86400.0, rp, ci)
    A = _dense_block(net, vals)
    n = net.ncomp
    fd = np.zeros((n, n))
    for j in range(n):
        cols = []
        for sgn in (1.0, -1.0):
            s2 = cell_state.copy()
            s2.a["pri_molal"][j, 0] *= np.exp(sgn * h)
            r, _ = oracle.girt_assemble(net, s2, grid, tk, 86400.0, rp, ci)
            cols.append(r)
        fd[:, j] = (cols[0] - cols[1]) / (2 * h) / (1.0 if logf else cell_state.a["pri_molal"][j, 0])
    return A, fd, s0


def _scale(fd):
    """Per entry, the larger of its row's and its column's largest
    difference quotient: a column of tiny derivatives (a trace species)
    carries the residual's rounding noise divided by the step."""
    a = np.abs(fd)
    return np.maximum(np.maximum(a.max(axis=0, keepdims=True), a.max(axis=1, keepdims=True)), 1e-300)


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
def test_jacobian_with_primary_prefactor_species_matches_fd(oracle, logf):
    net, st = _prepared(oracle, with_secondary=False)
    net = net.with_options(use_log_formulation=int(logf))
    st.a["den_kg"][:] = 1000.0  # the reference's den*1e-3 factor on dQK/dm is then 1
    checked = 0
    for c in range(12):
        cell = st.subset(np.array([c]))
        if not np.any(cell.a["mnrl_volfrac"][:3, 0] > 0):
            continue
        A, fd, _ = _jac_and_fd(oracle, net, cell, logf)
        assert np.max(np.abs(A - fd) / _scale(fd)) < 1e-5, c
        checked += 1
    assert checked >= 6


@pytest.mark.parametrize("logf", [True, False], ids=["log", "linear"])
def test_jacobian_with_secondary_prefactor_species_is_the_references(oracle, logf):
    """With a secondary prefactor species the reference's derivative (a) puts
    dIm/ds ds/dm_j on the rows of the complex's species with the complex's
    stoichiometry instead of the mineral's, and (b) lets the primary species
    that follows (M2's P5) walk the complex's 3 species instead of M2's 4.
    The oracle's Jacobian must equal central differences plus exactly those
    two departures."""
    net, st = _prepared(oracle, with_secondary=True)
    net = net.with_options(use_log_formulation=int(logf))
    st.a["den_kg"][:] = 1000.0
    n = net.ncomp
    checked = 0
    for c in range(40):
        cell = st.subset(np.array([c]))
        A, fd, s0 = _jac_and_fd(oracle, net, cell, logf)
        la, lsa = _lnact(net, s0)
        m_ = s0.a["pri_molal"][:, 0]
        dev = np.zeros((n, n))
        V = s0.a["volume"][0]
        for mname, prefs in net.prefactors.items():
            m = net.minerals.index(mname)
            Im = s0.a["mnrl_rate"][m, 0] * V
            if Im == 0.0:
                continue
            S, prods = _sum_rate(net, s0, m, la, lsa)
            temp = s0.a["temperature"]
            mspec = list(net.mnrl_spec[m, :net.mnrl_nspec[m]])
            mnu = list(net.mnrl_stoich[m, :net.mnrl_nspec[m]])
            count = len(mspec)
            for p, pr in enumerate(prefs):
                kp = pr["rate"] * _arrhenius(pr.get("activation_energy", 0.0), temp)[0]
                for sp in pr.get("species", ()):
                    f, lna = _factor(net, la[:, :1], lsa[:, :1], sp)
                    K, a, b = sp.get("atten_coef", 0.0), sp.get("alpha", 0.0), sp.get("beta", 0.0)
                    Kab = K * np.exp(b * lna[0])
                    dlnf_dlna = a - b * Kab / (1.0 + Kab)
                    if sp["name"] in net.primary:
                        jc = net.primary.index(sp["name"])
                        dIm = Im / S[0] * kp * prods[p][0] * dlnf_dlna / m_[jc]
                        for r, nu in zip(mspec[count:], mnu[count:]):  # rows the reference skips
                            dev[r, jc] -= nu * dIm
                        continue
                    ic = net.secondary.index(sp["name"])
                    s = s0.a["sec_molal"][ic, 0]
                    dIm_ds = Im / S[0] * kp * prods[p][0] * dlnf_dlna / s
                    cspec = list(net.sec_spec[ic, :net.sec_nspec[ic]])
                    cnu = list(net.sec_stoich[ic, :net.sec_nspec[ic]])
                    for jc, nuj in zip(cspec, cnu):
                        ds_dm = nuj * s / m_[jc]
                        for r, nur in zip(cspec, cnu):
                            dev[r, jc] += nur * dIm_ds * ds_dm
                        for r, nur in zip(mspec, mnu):
                            dev[r, jc] -= nur * dIm_ds * ds_dm
                    count = len(cspec)
        if logf:
            dev = dev * m_[None, :]
        scale = _scale(fd)
        assert np.max(np.abs(A - fd - dev) / scale) < 1e-5, c
        # the departures are well above the tolerance in these cells
        if np.max(np.abs(dev) / scale) > 1e-3:
            checked += 1
    assert checked >= 5, checked


def _reordered(oracle):
    """M0 (2 species) with a 3-species complex before a primary species: the
    reference's derivative would walk 3 of M0's 2 species."""
    net, st = _prepared(oracle, ncells=20)
    three = next(net.secondary[i] for i in range(net.nsec) if net.sec_nspec[i] == 3)
    net.prefactors = {"M0": [dict(rate=1e-9, species=[dict(name=three, alpha=0.5), dict(name="P4", alpha=0.3)])]}
    return net, st


def test_unsafe_prefactor_order_is_refused(oracle):
    net, st = _reordered(oracle)
    assert oracle.rstep(net, st.copy(), 3600.0) == abi.PF_ERR_UNSUPPORTED
    lib = abi.load()
    d = net.desc()
    h = C.c_void_p()
    assert lib.pf_network_create(C.byref(d), C.byref(h)) == abi.PF_ERR_UNSUPPORTED


def test_prefactor_counts_are_validated(oracle):
    net, st = _prepared(oracle, ncells=20)
    net.prefactors = {"M0": [dict(rate=1e-9, species=[dict(name="H+", alpha=0.5)])] * 5}
    with pytest.raises(ValueError):
        net.desc()
    lib = abi.load()
    net.prefactors = {"M0": [dict(rate=1e-9, species=[dict(name="H+", alpha=0.5)])]}
    d = net.desc()
    d.prefactors.contents.spec[0] = net.ncomp  # out of range
    h = C.c_void_p()
    assert lib.pf_network_create(C.byref(d), C.byref(h)) == abi.PF_ERR_INVALID
