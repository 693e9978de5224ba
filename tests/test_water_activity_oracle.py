"""The water activity option (ACTIVITY_H2O, reaction%use_activity_h2o) in the
oracle: RActivityCoefficients sets ln a_H2O = ln(1 - 0.017 (sum of primary
and secondary molalities)) (reaction.F90:4539-4547 NEWTON, 4604-4611 LAG),
and every complex and mineral with water in its reaction adds its water
coefficient times ln a_H2O to ln Q/K (:4715-4717, reaction_mineral.F90:
769-772).  The reference's one deck with the option (default/constraint/
pe.in) needs PE constraints, which are not built, so the restatement is
checked by these definitions (parity unpinned against the reference)."""
import numpy as np

import cases
from pfgpu import abi

LOG_TO_LN = 2.30258509299


def _logK(coef, temp):
    tk = temp + 273.15
    return coef[0] * np.log(tk) + coef[1] + coef[2] * tk + coef[3] / tk + coef[4] / tk ** 2


def test_lag_water_activity_uses_the_previous_complexes(oracle):
    net, st = cases.water_case(oracle, ncells=200)
    got = st.copy()
    oracle.update_activity_coefs(net, got)
    want = np.log(1.0 - 0.017 * (st.a["pri_molal"].sum(axis=0) + st.a["sec_molal"].sum(axis=0)))
    np.testing.assert_allclose(got.a["ln_act_h2o"], want, rtol=1e-13, atol=0)
    assert np.all(want < 0)


def test_speciation_carries_the_water_term(oracle):
    net, st = cases.water_case(oracle, ncells=200)
    got = st.copy()
    oracle.update_auxvars(net, got, False)
    la = np.log(st.a["pri_molal"]) + np.log(st.a["pri_act_coef"])
    temp = st.a["temperature"]
    for i in range(net.nsec):
        lnQK = -_logK(net.sec_logKcoef[i], temp) * LOG_TO_LN + net.sec_h2o_stoich[i] * st.a["ln_act_h2o"]
        for k in range(net.sec_nspec[i]):
            lnQK = lnQK + net.sec_stoich[i, k] * la[net.sec_spec[i, k]]
        np.testing.assert_allclose(got.a["sec_molal"][i], np.exp(lnQK) / st.a["sec_act_coef"][i], rtol=1e-12)
    assert np.count_nonzero(net.sec_h2o_stoich) >= 5


def test_newton_algorithm_ends_on_its_last_complexes(oracle):
    net, st = cases.water_case(oracle, ncells=200, act_coef_update_algorithm=abi.PF_ACT_COEF_ALGO_NEWTON)
    got = st.copy()
    oracle.update_activity_coefs(net, got)
    ok = np.isfinite(got.a["pri_act_coef"]).all(axis=0)
    assert ok.mean() > 0.95
    want = np.log(1.0 - 0.017 * (got.a["pri_molal"].sum(axis=0) + got.a["sec_molal"].sum(axis=0)))
    np.testing.assert_allclose(got.a["ln_act_h2o"][ok], want[ok], rtol=1e-13, atol=0)


def test_option_off_is_the_network_without_water(oracle):
    """Off, ln a_H2O stays 0 (RTAuxVarInit) and the water coefficients change
    nothing: the step is bit for bit that of the same network without them."""
    net, st = cases.water_case(oracle, ncells=200)
    off = net.with_options(use_activity_h2o=0)
    plain = net.with_options(use_activity_h2o=0)
    plain.sec_h2o_stoich = plain.mnrl_h2o_stoich = None
    a, b = st.copy(), st.copy()
    oracle.rstep(off, a, 3600.0)
    oracle.rstep(plain, b, 3600.0)
    for k in ("pri_molal", "sec_molal", "total", "mnrl_rate"):
        np.testing.assert_array_equal(a.a[k], b.a[k])
    # and on, the water terms move the result
    c = st.copy()
    oracle.rstep(net, c, 3600.0)
    assert not np.allclose(c.a["sec_molal"], a.a["sec_molal"], rtol=1e-8, atol=0)
