"""MINERAL and GAS constraint rows of ReactionEquilibrateConstraint
(reaction.F90:1755-1811): the equilibrated state puts the mineral at
saturation, ln(Q/K) = 0, or the gas at its partial pressure, ln(Q/K) = ln p,
with the other rows met (TOTAL, PH, CHARGE_BAL), isothermal and at the cell
temperature.  CPU: the oracle against these properties; GPU: the kernel
against the oracle.  No reference test holds an equilibrated MINERAL/GAS
state (the decks that use them report transport runs), so the restatement is
checked by the defining equations."""
import math

import numpy as np
import pytest

from pfgpu import abi, generate
from pfgpu import database as dbm
from pfgpu.network import default_options

LOG_TO_LN = 2.30258509299  # pflotran_constants.F90:84


def _db_text():
    """The carbonate-like test database with a CO2(g) gas record (values
    chosen for this test)."""
    temps = [0.0, 25.0, 60.0, 100.0, 150.0, 200.0, 250.0, 300.0]

    def col(k25, slope):
        return " ".join("%.6f" % (k25 + slope * (t - 25.0)) for t in temps)
    lines = ["'temperature points' 8 " + " ".join("%.1f" % t for t in temps),
             "'H+' 9.0 1.0 1.0", "'Ca++' 6.0 2.0 40.0", "'HCO3-' 4.0 -1.0 61.0", "'null' 0. 0. 0."]
    for name, st, ks, a0, z in [("OH-", "2 1.0 'H2O' -1.0 'H+'", col(14.0, -0.03), 3.5, -1.0),
                                ("CO3--", "2 -1.0 'H+' 1.0 'HCO3-'", col(10.3, -0.01), 4.5, -2.0),
                                ("CO2(aq)", "3 -1.0 'H2O' 1.0 'H+' 1.0 'HCO3-'", col(-6.3, 0.005), 3.0, 0.0),
                                ("CaHCO3+", "2 1.0 'Ca++' 1.0 'HCO3-'", col(-1.0, -0.005), 4.0, 1.0)]:
        lines.append("'%s' %s %s %.1f %.1f 1.0" % (name, st, ks, a0, z))
    lines.append("'null' 1 0. 'null' " + " ".join(["0."] * 8) + " 0. 0. 0.")
    lines.append("'CO2(g)' 0.0 3 -1.0 'H2O' 1.0 'H+' 1.0 'HCO3-' %s 44.0" % col(-7.8, 0.01))
    lines.append("'null' 0. 1 0. 'null' " + " ".join(["0."] * 8) + " 0.")
    lines.append("'Calcite' 36.9 3 -1.0 'H+' 1.0 'Ca++' 1.0 'HCO3-' %s 100.0" % col(1.85, -0.012))
    lines.append("'null' 0. 1 0. 'null' " + " ".join(["0."] * 8) + " 0.")
    return "\n".join(lines) + "\n"


PRIMARY = ["H+", "Ca++", "HCO3-"]


def _setup(kind, isothermal, ncells=300, seed=3):
    db = dbm.read_database(_db_text())
    opts = default_options(isothermal=1 if isothermal else 0)
    net = dbm.build_network(db, PRIMARY, minerals={"Calcite": dict(rate=1e-8)}, options=opts)
    st, _, _ = generate.random_cells(net, ncells, seed=seed)
    rng = np.random.default_rng(seed + 1)
    cconc = np.zeros((3, ncells))
    if kind == "mineral":
        # H+ by pH, HCO3- by total, Ca++ at calcite saturation
        ctype = [abi.PF_CONSTRAINT_PH, abi.PF_CONSTRAINT_MINERAL, abi.PF_CONSTRAINT_TOTAL]
        cconc[0] = rng.uniform(6.5, 8.5, ncells)
        cconc[1] = 5e-4
        cconc[2] = 10.0 ** rng.uniform(-3.5, -2.0, ncells)
        rx = {1: dbm.constraint_reaction(db, PRIMARY, "Calcite", "mineral", isothermal=isothermal)}
    else:
        # charge balance on H+, HCO3- from the CO2(g) partial pressure, Ca++ by total
        ctype = [abi.PF_CONSTRAINT_CHARGE_BAL, abi.PF_CONSTRAINT_TOTAL, abi.PF_CONSTRAINT_GAS]
        cconc[0] = 1e-7
        cconc[1] = 10.0 ** rng.uniform(-4.0, -2.5, ncells)
        cconc[2] = rng.uniform(-3.5, -1.5, ncells)  # log10 bar
        rx = {2: dbm.constraint_reaction(db, PRIMARY, "CO2(g)", "gas", isothermal=isothermal)}
    return db, net, st, ctype, cconc, rx


def _lnQK(db, st, name, kind, isothermal):
    r = (db.minerals if kind == "mineral" else db.gases)[name]
    nu = {sp: v for sp, v in r.stoich if sp != "H2O"}
    coefs = dbm.fit_logK_coefs(db.temperatures, r.logK)
    out = np.zeros(st.ncells)
    for i in range(st.ncells):
        logK = r.logK[1] if isothermal else dbm.eval_logK(coefs, st.a["temperature"][i])
        ln = -logK * LOG_TO_LN
        for sp, v in nu.items():
            k = PRIMARY.index(sp)
            ln += v * math.log(st.a["pri_molal"][k, i] * st.a["pri_act_coef"][k, i])
        out[i] = ln
    return out


@pytest.mark.parametrize("isothermal", [True, False], ids=["isothermal", "cell-temperature"])
@pytest.mark.parametrize("kind", ["mineral", "gas"])
def test_oracle_meets_mineral_and_gas_rows(oracle, kind, isothermal):
    db, net, st, ctype, cconc, rx = _setup(kind, isothermal)
    rc, its = oracle.equilibrate(net, st, ctype, cconc, nthreads=4, reactions=rx)
    ok = its > 0
    assert ok.mean() > 0.98, (rc, (~ok).sum())
    name = "Calcite" if kind == "mineral" else "CO2(g)"
    ln = _lnQK(db, st, name, kind, isothermal)[ok]
    if kind == "mineral":
        assert np.max(np.abs(ln)) < 1e-9
        # the pH row and the total row hold as well
        h = st.a["pri_molal"][0] * st.a["pri_act_coef"][0]
        np.testing.assert_allclose(-np.log10(h[ok]), cconc[0][ok], rtol=0, atol=1e-10)
        np.testing.assert_allclose(st.a["total"][2][ok], cconc[2][ok], rtol=1e-9)
    else:
        np.testing.assert_allclose(ln, np.log(10.0 ** cconc[2][ok]), rtol=0, atol=1e-9)
        charge = sum(z * st.a["total"][k] for k, z in enumerate([1.0, 2.0, -1.0]))
        assert np.max(np.abs(charge[ok]) / st.a["total"][1][ok]) < 1e-8


def test_constraint_reaction_arguments():
    """Argument checks without a GPU: the C ABI refuses a null network, and
    the ctypes builder refuses species and stoichiometry lists of different
    length."""
    import ctypes as C
    lib = abi.load()
    ct = (C.c_int32 * 3)(abi.PF_CONSTRAINT_PH, abi.PF_CONSTRAINT_MINERAL, abi.PF_CONSTRAINT_TOTAL)
    assert lib.pf_equilibrate_constraint_ex(None, None, ct, None, None, 0, None, None) == abi.PF_ERR_INVALID
    with pytest.raises(ValueError):
        abi.constraint_reactions(3, {1: dict(spec=[0, 1], stoich=[1.0], logK=0.0)})
    arr = abi.constraint_reactions(3, {1: dict(spec=[0, 1, 2], stoich=[-1.0, 1.0, 1.0], logK=1.85,
                                               logKcoef=[0.0, 1.0, 0.0, 0.0, 0.0])})
    assert arr[1].nspec == 3 and arr[1].temperature_dependent == 1 and arr[0].nspec == 0


@pytest.mark.gpu
@pytest.mark.parametrize("isothermal", [True, False], ids=["isothermal", "cell-temperature"])
@pytest.mark.parametrize("kind", ["mineral", "gas"])
def test_gpu_mineral_and_gas_rows_match_oracle(oracle, kind, isothermal):
    torch = pytest.importorskip("torch")
    from pfgpu.engine import ReactionEngine
    db, net, st, ctype, cconc, rx = _setup(kind, isothermal, ncells=500, seed=11)
    ref = st.copy()
    rc, its_ref = oracle.equilibrate(net, ref, ctype, cconc, nthreads=4, reactions=rx)
    dev = st.to("cuda")
    its = ReactionEngine(net).equilibrate(dev, ctype, torch.from_numpy(cconc).cuda(), reactions=rx).cpu().numpy()
    got = dev.numpy()
    ok = (its_ref > 0) & (its == its_ref)
    assert ok.mean() > 0.95, (ok.mean(), (its != its_ref).sum())
    e = np.max(np.abs(got.a["pri_molal"][:, ok] - ref.a["pri_molal"][:, ok]) / ref.a["pri_molal"][:, ok])
    assert e < 1e-10, e
    name = "Calcite" if kind == "mineral" else "CO2(g)"
    ln = _lnQK(db, got, name, kind, isothermal)[ok]
    target = 0.0 if kind == "mineral" else np.log(10.0 ** cconc[2][ok])
    assert np.max(np.abs(ln - target)) < 1e-9


@pytest.mark.gpu
def test_gpu_rejects_mineral_row_without_reaction():
    torch = pytest.importorskip("torch")
    from pfgpu.engine import ReactionEngine
    db, net, st, ctype, cconc, rx = _setup("mineral", True, ncells=8)
    eng = ReactionEngine(net)
    dev = st.to("cuda")
    with pytest.raises(abi.PfError):
        eng.equilibrate(dev, ctype, torch.from_numpy(cconc).cuda())
    bad = {1: dict(spec=[0, 1, 2], stoich=[-1.0, 1.0, 1.0], logK=1.85)}
    bad[1]["spec"][2] = 5
    with pytest.raises(abi.PfError):
        eng.equilibrate(dev, ctype, torch.from_numpy(cconc).cuda(), reactions=bad)
