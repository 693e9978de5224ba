"""The .dat database reader and basis set-up (pfgpu.database).

Against the reference: the known-answer fixtures (tests/golden/kat_batch.json)
were generated from the reference's regression databases through this
reader; where the reference tree is present (PFGPU_REFERENCE_ROOT), the
networks built by build_network from those databases are compared with the
fixtures' networks.  Everywhere: a synthetic database round trip, the logK
temperature fit (ReactionFitLogKCoef), the Debye-Hueckel table, water and
basis handling."""
import math
import os

import numpy as np
import pytest

from pfgpu import database as dbm

# the reference tree's root, when the test should read it (no default)
REF = os.environ.get("PFGPU_REFERENCE_ROOT", "")
BATCH = os.path.join(REF, "regression_tests", "ascem", "batch") if REF else ""


def _coef_fn(c, t):
    tk = t + 273.15
    return c[0] * math.log(tk) + c[1] + c[2] * tk + c[3] / tk + c[4] / (tk * tk)


def _synthetic(seed=3):
    """A database text with 4 basis species, 5 complexes (one with water),
    a gas and 2 minerals, logK from known five-term functions; one logK at
    300 C marked missing (500)."""
    rng = np.random.default_rng(seed)
    temps = [0.0, 25.0, 60.0, 100.0, 150.0, 200.0, 250.0, 300.0]
    prim = [("H+", 9.0, 1.0), ("Ca++", 6.0, 2.0), ("HCO3-", 4.0, -1.0), ("Mg++", 8.0, 2.0)]
    coefs = {}
    lines = ["'temperature points' 8 " + " ".join("%.1f" % t for t in temps)]
    for name, a0, z in prim:
        lines.append("'%s' %.1f %.1f 1.0" % (name, a0, z))
    lines.append("'null' 0. 0. 0.")

    def logks(name, missing=False):
        c = [rng.uniform(-1, 1) * 1e-2, rng.uniform(-5, 5), rng.uniform(-1, 1) * 1e-3,
             rng.uniform(-1, 1) * 1e2, rng.uniform(-1, 1) * 1e3]
        coefs[name] = c
        vals = [_coef_fn(c, t) for t in temps]
        if missing:
            vals[-1] = 500.0
        return " ".join("%.12e" % v for v in vals)
    secs = [("OH-", [(1.0, "H2O"), (-1.0, "H+")], -1.0), ("CO3--", [(-1.0, "H+"), (1.0, "HCO3-")], -2.0),
            ("CaHCO3+", [(1.0, "Ca++"), (1.0, "HCO3-")], 1.0), ("MgCO3(aq)", [(-1.0, "H+"), (1.0, "Mg++"),
                                                                          (1.0, "HCO3-")], 0.0),
            ("NaCl(aq)", [(1.0, "Na+"), (1.0, "Cl-")], 0.0)]
    for name, st, z in secs:
        pairs = " ".join("%.1f '%s'" % (nu, sp) for nu, sp in st)
        lines.append("'%s' %d %s %s 4.0 %.1f 10.0" % (name, len(st), pairs, logks(name, name == "CO3--"), z))
    lines.append("'null' 1 0. 'null' " + " ".join(["0."] * 8) + " 0. 0. 0.")
    lines.append("'CO2(g)' 22.4 3 -1.0 'H2O' 1.0 'H+' 1.0 'HCO3-' %s 44.0" % logks("CO2(g)"))
    lines.append("'null' 0. 1 0. 'null' " + " ".join(["0."] * 8) + " 0.")
    lines.append("'Calcite' 36.934 3 -1.0 'H+' 1.0 'Ca++' 1.0 'HCO3-' %s 100.0" % logks("Calcite"))
    lines.append("'Dolomite' 64.34 5 -2.0 'H+' 1.0 'Ca++' 1.0 'Mg++' 2.0 'HCO3-' 0.0 'H2O' %s 184.4"
                 % logks("Dolomite"))
    lines.append("'null' 0. 1 0. 'null' " + " ".join(["0."] * 8) + " 0.")
    return "\n".join(lines) + "\n", temps, coefs


def test_synthetic_round_trip():
    text, temps, coefs = _synthetic()
    db = dbm.read_database(text)
    assert db.temperatures == temps
    assert list(db.primary) == ["H+", "Ca++", "HCO3-", "Mg++"]
    assert db.primary["Ca++"][:2] == (6.0, 2.0)
    assert list(db.secondary) == ["OH-", "CO3--", "CaHCO3+", "MgCO3(aq)", "NaCl(aq)"]
    assert db.secondary["OH-"].stoich == [("H2O", 1.0), ("H+", -1.0)]
    assert db.secondary["CO3--"].logK[-1] == 500.0
    assert list(db.gases) == ["CO2(g)"]
    assert list(db.minerals) == ["Calcite", "Dolomite"]
    assert db.minerals["Dolomite"].molar_vol_cm3 == 64.34


def test_logK_fit_recovers_the_function():
    text, temps, coefs = _synthetic()
    db = dbm.read_database(text)
    for name in ("CaHCO3+", "Calcite"):
        r = db.secondary.get(name) or db.minerals[name]
        c = dbm.fit_logK_coefs(temps, r.logK)
        for t in (5.0, 25.0, 42.0, 90.0, 280.0):
            assert abs(dbm.eval_logK(c, t) - _coef_fn(coefs[name], t)) < 1e-7, (name, t)
    # a missing value (500) is left out of the fit
    c = dbm.fit_logK_coefs(temps, db.secondary["CO3--"].logK)
    assert abs(dbm.eval_logK(c, 250.0) - _coef_fn(coefs["CO3--"], 250.0)) < 1e-6


def test_debye_huckel_table():
    assert dbm.debye_huckel(25.0) == (0.5114, 0.3288, 0.0410)
    a, b, bd = dbm.debye_huckel(42.5)
    assert a == pytest.approx(0.5 * (0.5114 + 0.5465))
    assert b == pytest.approx(0.5 * (0.3288 + 0.3346))
    assert bd == pytest.approx(0.5 * (0.0410 + 0.0440))
    assert dbm.debye_huckel(0.0) == (0.4939, 0.3253, 0.0374)
    assert dbm.debye_huckel(400.0) == (1.2180, 0.3925, 0.0)


def test_build_network_basis_water_and_selection():
    text, temps, coefs = _synthetic()
    db = dbm.read_database(text)
    net = dbm.build_network(db, ["H+", "Ca++", "HCO3-"], minerals={"Calcite": dict(rate=1e-6)})
    # automatic selection: complexes made of the primaries (and water)
    assert net.secondary == ["OH-", "CO3--", "CaHCO3+"]
    oh = net.secondary.index("OH-")
    assert net.sec_nspec[oh] == 1 and net.primary[net.sec_spec[oh, 0]] == "H+"
    assert net.sec_stoich[oh, 0] == -1.0
    # water leaves the species list and is kept as the reaction's water
    # coefficient (eqcplxh2ostoich): OH- = H2O - H+, the others have none
    np.testing.assert_array_equal(net.sec_h2o_stoich, [1.0, 0.0, 0.0])
    # isothermal at a database temperature: the database column
    assert net.sec_logK[2] == db.secondary["CaHCO3+"].logK[1]
    assert net.mnrl_molar_vol[0] == pytest.approx(36.934e-6)
    assert (net.debyeA, net.debyeB, net.debyeBdot) == (0.5114, 0.3288, 0.0410)
    # non-isothermal: the fit's coefficients travel with the network
    hot = dbm.build_network(db, ["H+", "Ca++", "HCO3-"], options=dict(isothermal=0), reference_temperature=30.0)
    assert hot.sec_logKcoef.shape == (3, 5)
    assert hot.sec_logK[2] == pytest.approx(_coef_fn(coefs["CaHCO3+"], 30.0), abs=1e-7)
    # a complex of a species that is not primary (and not swapped in) is refused
    with pytest.raises(KeyError):
        dbm.build_network(db, ["H+", "Ca++", "HCO3-"], secondary=["MgCO3(aq)"])
    with pytest.raises(KeyError):
        dbm.build_network(db, ["H+", "Na+"])


@pytest.mark.skipif(not BATCH or not os.path.isdir(BATCH),
                    reason="PFGPU_REFERENCE_ROOT does not name the reference tree")
def test_reference_databases_build_the_fixture_networks():
    import kat
    from golden import make_golden
    for name, fx in kat.KAT.items():
        if name.startswith("_"):
            continue
        deck = make_golden.read_deck(os.path.join(BATCH, name + ".in"))
        db = dbm.read_database(os.path.join(BATCH, deck["database"].lstrip("./")))
        mins = {m["name"]: dict(rate=m["rate"]) for m in fx["minerals"]}
        net = dbm.build_network(db, fx["primary"], secondary=[s["name"] for s in fx["secondaries"]],
                                minerals=mins)
        assert list(net.pri_Z) == fx["pri_Z"] and list(net.pri_a0) == fx["pri_a0"]
        for i, s in enumerate(fx["secondaries"]):
            assert net.sec_logK[i] == s["logK"] and net.sec_Z[i] == s["Z"] and net.sec_a0[i] == s["a0"]
            got = {net.primary[net.sec_spec[i, k]]: net.sec_stoich[i, k] for k in range(net.sec_nspec[i])}
            assert got == s["stoich"], (name, s["name"])
        for m, mx in enumerate(fx["minerals"]):
            assert net.mnrl_logK[m] == mx["logK"] and net.mnrl_molar_vol[m] == mx["molar_vol"]


def test_mineral_surface_area_units():
    """MineralProcessConstraint (reaction_mineral.F90:590-640): bulk-volume
    units scale directly; per-mass units go through molar weight / molar
    volume and the volume fraction; the reference's refusals are errors."""
    calcite = dbm.Reaction([], [], molar_vol_cm3=36.934, molar_weight=100.0872)
    assert dbm.mineral_surface_area(1.0, "cm^2/cm^3", calcite, 0.2) == pytest.approx(100.0, rel=1e-15)
    assert dbm.mineral_surface_area(3.0, "m^2/m^3", calcite, 0.2) == 3.0
    assert dbm.mineral_surface_area(2.0, "m^2/L", calcite, 0.2) == pytest.approx(2000.0, rel=1e-15)
    # 1.8450910805777365 cm^2/g of calcite at 20 % is 1 cm^2/cm^3 of bulk
    # (the comment of regression_tests/ascem/batch/calcite-area-per-mass.in)
    a = dbm.mineral_surface_area(1.8450910805777365, "cm^2/g", calcite, 0.2, "Calcite")
    assert a == pytest.approx(100.0, rel=1e-14)
    # m^2/kg and cm^2/g differ by 10; m^2/g and cm^2/g by 1e4
    assert dbm.mineral_surface_area(1.0, "m^2/kg", calcite, 0.2) == pytest.approx(
        10.0 * dbm.mineral_surface_area(1.0, "cm^2/g", calcite, 0.2), rel=1e-15)
    assert dbm.mineral_surface_area(1.0, "m^2/g", calcite, 0.2) == pytest.approx(
        1.0e4 * dbm.mineral_surface_area(1.0, "cm^2/g", calcite, 0.2), rel=1e-15)
    # per-cell datasets: arrays of areas and volume fractions
    vf = np.array([0.1, 0.2, 0.4])
    arr = dbm.mineral_surface_area(np.array([1.0, 1.0, 2.0]), "cm^2/g", calcite, vf)
    assert arr.shape == (3,) and arr[1] == pytest.approx(2.0 * arr[0]) and arr[2] == pytest.approx(8.0 * arr[0])
    with pytest.raises(ValueError, match="volume fraction"):
        dbm.mineral_surface_area(1.0, "cm^2/g", calcite, 0.0)
    with pytest.raises(ValueError, match="molar weight"):
        dbm.mineral_surface_area(1.0, "cm^2/g", dbm.Reaction([], [], molar_vol_cm3=36.9, molar_weight=500.0), 0.2)
    with pytest.raises(ValueError, match="molar volume"):
        dbm.mineral_surface_area(1.0, "cm^2/g", dbm.Reaction([], [], molar_vol_cm3=0.0, molar_weight=100.0), 0.2)
    for bad in ("cm/cm^3", "cm^2", "cm^2/ft^3", "cm^2/lb"):
        with pytest.raises(ValueError):
            dbm.mineral_surface_area(1.0, bad, calcite, 0.2)


def test_reader_keeps_mineral_molar_weight():
    db = dbm.read_database(_carbonate_like())
    assert db.minerals["Calcite"].molar_weight == 100.0
    assert db.minerals["Dolomite"].molar_weight == 184.0 and db.minerals["Dolomite"].molar_vol_cm3 == 64.3


def _carbonate_like():
    """A small carbonate-system database in the .dat format: logK near
    typical 25 C values, varying linearly with temperature (values chosen
    for this test, not taken from any database)."""
    temps = [0.0, 25.0, 60.0, 100.0, 150.0, 200.0, 250.0, 300.0]

    def col(k25, slope):
        return " ".join("%.6f" % (k25 + slope * (t - 25.0)) for t in temps)
    lines = ["'temperature points' 8 " + " ".join("%.1f" % t for t in temps),
             "'H+' 9.0 1.0 1.0", "'Ca++' 6.0 2.0 40.0", "'HCO3-' 4.0 -1.0 61.0", "'Mg++' 8.0 2.0 24.3",
             "'null' 0. 0. 0."]
    secs = [("OH-", "2 1.0 'H2O' -1.0 'H+'", col(14.0, -0.03), 3.5, -1.0),
            ("CO3--", "2 -1.0 'H+' 1.0 'HCO3-'", col(10.3, -0.01), 4.5, -2.0),
            ("CO2(aq)", "3 -1.0 'H2O' 1.0 'H+' 1.0 'HCO3-'", col(-6.3, 0.005), 3.0, 0.0),
            ("CaHCO3+", "2 1.0 'Ca++' 1.0 'HCO3-'", col(-1.0, -0.005), 4.0, 1.0),
            ("CaCO3(aq)", "3 -1.0 'H+' 1.0 'Ca++' 1.0 'HCO3-'", col(7.0, -0.02), 3.0, 0.0),
            ("MgHCO3+", "2 1.0 'Mg++' 1.0 'HCO3-'", col(-1.0, -0.004), 4.0, 1.0)]
    for name, st, ks, a0, z in secs:
        lines.append("'%s' %s %s %.1f %.1f 1.0" % (name, st, ks, a0, z))
    lines.append("'null' 1 0. 'null' " + " ".join(["0."] * 8) + " 0. 0. 0.")
    lines.append("'null' 0. 1 0. 'null' " + " ".join(["0."] * 8) + " 0.")
    lines.append("'Calcite' 36.9 3 -1.0 'H+' 1.0 'Ca++' 1.0 'HCO3-' %s 100.0" % col(1.85, -0.012))
    lines.append("'Dolomite' 64.3 5 -2.0 'H+' 1.0 'Ca++' 1.0 'Mg++' 2.0 'HCO3-' 0.0 'H2O' %s 184.0"
                 % col(2.5, -0.02))
    lines.append("'null' 0. 1 0. 'null' " + " ".join(["0."] * 8) + " 0.")
    return "\n".join(lines) + "\n"


@pytest.mark.gpu
def test_database_network_runs_on_the_gpu(oracle):
    """A network read from a database (non-isothermal, two kinetic minerals)
    goes through the C ABI: the GPU step agrees with the oracle."""
    torch = pytest.importorskip("torch")
    import cases
    from pfgpu import generate
    from pfgpu.engine import ReactionEngine
    from pfgpu.network import default_options
    db = dbm.read_database(_carbonate_like())
    net = dbm.build_network(db, ["H+", "Ca++", "HCO3-", "Mg++"],
                            minerals={"Calcite": dict(rate=1e-7), "Dolomite": dict(rate=1e-9)},
                            options=default_options(isothermal=0))
    assert net.sec_logKcoef is not None and net.nsec == 6
    st, ct, cc = generate.random_cells(net, 500, seed=77)
    st, nfail = cases.prepare(oracle, net, st, ct, cc)
    assert st.ncells > 450
    ref = st.copy()
    oracle.rstep(net, ref, 86400.0, nthreads=8)
    dev = st.to("cuda")
    ReactionEngine(net).rstep(dev, 86400.0)
    got = dev.numpy()
    same = (got.a["newton_its"] == ref.a["newton_its"]) & (ref.a["status"] == 0)
    assert same.mean() > 0.9
    err = np.max(np.abs(got.a["pri_molal"][:, same] - ref.a["pri_molal"][:, same]) / ref.a["pri_molal"][:, same])
    assert err < 1e-10, err


# ------------------------------------------------------------ basis swapping
def _speciate(oracle, net, free, gamma1=True):
    """Secondary molalities of `net` at the free-ion molalities `free`
    (ncomp, ncells), activity coefficients one (OFF), through the oracle's
    RTotal."""
    from pfgpu.network import CellState
    st = CellState.empty(net, free.shape[1])
    st.a["pri_molal"][:] = free
    st.a["den_kg"][:] = 1000.0
    oracle.update_auxvars(net, st, False)
    return st


def _swap_case(db, prim0, sec0, prim1, sec1, mins, t_c, oracle, isothermal):
    from pfgpu.network import default_options
    from pfgpu import abi
    opts = default_options(isothermal=int(isothermal), act_coef_update_frequency=abi.PF_ACT_COEF_OFF)
    net0 = dbm.build_network(db, prim0, sec0, minerals=mins, options=opts)
    net1 = dbm.build_network(db, prim1, sec1, minerals=mins, options=opts)
    rng = np.random.default_rng(7)
    N = 50
    free0 = 10.0 ** rng.uniform(-6.0, -2.0, (len(prim0), N))
    st0 = _speciate(oracle, net0, free0)
    if not isothermal:
        st0.a["temperature"][:] = t_c
        oracle.update_auxvars(net0, st0, False)
    # every species' molality in the unswapped network
    conc = {p: st0.a["pri_molal"][k] for k, p in enumerate(prim0)}
    conc.update({s: st0.a["sec_molal"][k] for k, s in enumerate(net0.secondary)})
    from pfgpu.network import CellState
    st1 = CellState.empty(net1, N)
    st1.a["pri_molal"][:] = np.stack([conc[p] for p in prim1])
    st1.a["den_kg"][:] = 1000.0
    st1.a["temperature"][:] = t_c
    oracle.update_auxvars(net1, st1, False)
    for k, s in enumerate(net1.secondary):
        np.testing.assert_allclose(st1.a["sec_molal"][k], conc[s], rtol=1e-11 if isothermal else 1e-9, err_msg=s)
    # minerals: the same ln Q/K written in either basis
    for m, name in enumerate(net0.minerals):
        def lnqk(net, st, mi):
            lq = np.zeros(N)
            for j in range(net.mnrl_nspec[mi]):
                lq += net.mnrl_stoich[mi, j] * np.log(st.a["pri_molal"][net.mnrl_spec[mi, j]])
            logK = net.mnrl_logK[mi] if isothermal else dbm.eval_logK(net.mnrl_logKcoef[mi], t_c)
            return lq - logK * 2.30258509299
        np.testing.assert_allclose(lnqk(net1, st1, net1.minerals.index(name)), lnqk(net0, st0, m),
                                   rtol=0, atol=1e-9 if isothermal else 1e-7, err_msg=name)
    return net0, net1


@pytest.mark.parametrize("isothermal,t_c", [(True, 25.0), (False, 40.0)], ids=["25C", "40C-fit"])
def test_basis_swap_reproduces_the_unswapped_speciation(oracle, isothermal, t_c):
    """CO3-- in place of HCO3- as a primary species of the synthetic
    database: every complex, the swapped-out HCO3- and each mineral's Q/K
    come out as in the database's own basis."""
    db = dbm.read_database(_synthetic()[0])
    net0, net1 = _swap_case(db, ["H+", "Ca++", "HCO3-", "Mg++"], ["OH-", "CO3--", "CaHCO3+", "MgCO3(aq)"],
                            ["H+", "Ca++", "CO3--", "Mg++"], ["OH-", "HCO3-", "CaHCO3+", "MgCO3(aq)"],
                            {"Calcite": dict(rate=1e-8), "Dolomite": dict(rate=1e-9)}, t_c, oracle, isothermal)
    # the swapped-out species' reaction: HCO3- = CO3-- + H+ (water-free)
    k = net1.secondary.index("HCO3-")
    st = {net1.primary[net1.sec_spec[k, j]]: net1.sec_stoich[k, j] for j in range(net1.sec_nspec[k])}
    assert st == {"CO3--": 1.0, "H+": 1.0}
    # the charge and size of the swapped-in primary are the complex's
    assert net1.pri_Z[net1.primary.index("CO3--")] == -2.0


def test_basis_swap_needs_the_swapped_out_species():
    db = dbm.read_database(_synthetic()[0])
    with pytest.raises(ValueError):
        dbm.build_network(db, ["H+", "Ca++", "CO3--", "Mg++"], ["OH-", "CaHCO3+", "MgCO3(aq)"])
    with pytest.raises(ValueError):
        dbm.build_network(db, ["H+", "Ca++", "CO3--", "Mg++"])


@pytest.mark.skipif(not BATCH or not os.path.isdir(BATCH),
                    reason="PFGPU_REFERENCE_ROOT does not name the reference tree")
@pytest.mark.parametrize("isothermal,t_c", [(True, 25.0), (False, 45.0)], ids=["25C", "45C-fit"])
def test_basis_swap_hanford_co2(oracle, isothermal, t_c):
    """CO2(aq) in place of HCO3- with the reference's hanford.dat, where
    CO2(aq) is a complex (database/hanford.dat:429)."""
    db = dbm.read_database(os.path.join(REF, "database", "hanford.dat"))
    _swap_case(db, ["H+", "HCO3-", "Ca++"], ["OH-", "CO3--", "CO2(aq)", "CaHCO3+", "CaCO3(aq)"],
               ["H+", "CO2(aq)", "Ca++"], ["OH-", "CO3--", "HCO3-", "CaHCO3+", "CaCO3(aq)"],
               {"Calcite": dict(rate=1e-6)}, t_c, oracle, isothermal)
