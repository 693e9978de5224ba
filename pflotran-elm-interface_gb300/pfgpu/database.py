"""PFLOTRAN thermodynamic database (.dat) reader and the basis set-up that
turns a chemistry block into a ReactionNetwork.

Database format (DatabaseRead, src/pflotran/reaction_database.F90:26-811):

    'temperature points' n  T_1 ... T_n                              (C)
    'name' a0 Z MW                        primary species, until 'null'
    'name' k (nu 'species')*k logK*n a0 Z MW     aqueous complexes, until 'null'
    'name' Vm k (nu 'species')*k logK*n MW       gases, until 'null'
    'name' Vm k (nu 'species')*k logK*n MW       minerals (Vm in cm^3/mol), until 'null'

    'name' k (nu 'species')*k logK*n Z MW     surface complexes, until 'null'
                                          (one species is the site, '>...')

(tokens are whitespace-separated, names quoted; Fortran 'd' exponents
accepted; a logK of 500 marks a temperature with no data).  Later sections
are not read.

Basis set-up (the subset of BasisInit, reaction_database.F90:812-4040, that
this engine needs): primary species that are not basis species of the
database are swapped in (the change of basis of BasisInit, :1063-1450: the
reactions of the swapped-in primaries and of the secondaries form a linear
system whose inverse writes every secondary -- the swapped-out basis species
included -- in the new basis, logK at every database temperature; mineral
reactions then have each secondary substituted, BasisSubSpeciesInMineralRxn,
reaction_database_aux.F90:494-586); water leaves the species list of every
reaction and its coefficient is kept apart (eqcplxh2ostoich,
kinmnrlh2ostoich), entering ln Q times ln a_H2O, which is 0 unless the
ACTIVITY_H2O option (use_activity_h2o) computes it; logK at the reference temperature
follows ReactionInitializeLogK (reaction_aux.F90:1236-1281: the database
column when the run is isothermal at a database temperature, else the fit);
the five-term temperature fit follows ReactionFitLogKCoef
(reaction_aux.F90:1159-1232: normal equations over the temperatures with
data, solved with the Crout LU of utility.F90:597-735); Debye-Hueckel A, B,
Bdot are interpolated linearly in the table of reaction_database.F90:931-1022.
"""
from __future__ import annotations

import math
import os
import shlex
from dataclasses import dataclass, field

import numpy as np

from .network import ReactionNetwork, default_options

MISSING_LOGK = 500.0

# Debye-Hueckel A, B, Bdot at 0, 25, 60, 100, 150, 200, 250, 300 C
# (reaction_database.F90:931-1022; physical data)
_DH_T = (0.0, 25.0, 60.0, 100.0, 150.0, 200.0, 250.0, 300.0)
_DH_A = (0.4939, 0.5114, 0.5465, 0.5995, 0.6855, 0.7994, 0.9593, 1.2180)
_DH_B = (0.3253, 0.3288, 0.3346, 0.3421, 0.3525, 0.3639, 0.3766, 0.3925)
_DH_BDOT = (0.0374, 0.0410, 0.0440, 0.0460, 0.0470, 0.0470, 0.0340, 0.0000)


def _num(tok: str) -> float:
    return float(tok.lower().replace("d", "e"))


@dataclass
class Reaction:
    stoich: list            # [(species, nu)], in database order, water included
    logK: list              # one per database temperature
    a0: float = 0.0
    Z: float = 0.0
    molar_vol_cm3: float = 0.0
    molar_weight: float = 0.0   # g/mol (gases and minerals)


@dataclass
class Database:
    temperatures: list
    primary: dict = field(default_factory=dict)     # name -> (a0, Z, MW)
    secondary: dict = field(default_factory=dict)   # name -> Reaction
    gases: dict = field(default_factory=dict)       # name -> Reaction
    minerals: dict = field(default_factory=dict)    # name -> Reaction
    surface_complexes: dict = field(default_factory=dict)  # name -> Reaction (site included in stoich)


def read_database(source: str) -> Database:
    """Parse a database from a path or from its text."""
    text = open(source).read() if os.path.exists(source) else source
    toks = shlex.split(text)
    if len(toks) < 2 or toks[0] != "temperature points":
        raise ValueError("not a PFLOTRAN database: expected 'temperature points'")
    nt = int(_num(toks[1]))
    temps = [_num(t) for t in toks[2:2 + nt]]
    i = 2 + nt
    db = Database(temperatures=temps)
    def skip_note(i):
        # an optional trailing source note ('pcl-goethite colloid'): a string
        # followed by a string (the next record's name) where a record starts
        # with a name and a number
        if i + 1 < len(toks) and not _is_num(toks[i]) and not _is_num(toks[i + 1]):
            return i + 1
        return i

    # primary species: name a0 Z MW
    while toks[i] != "null":
        db.primary[toks[i]] = (_num(toks[i + 1]), _num(toks[i + 2]), _num(toks[i + 3]))
        i = skip_note(i + 4)
    i += 4  # the 'null' record has the same four fields

    def pairs(i, k):
        st = []
        for _ in range(k):
            st.append((toks[i + 1], _num(toks[i])))
            i += 2
        return st, i

    # aqueous complexes: name k pairs logK*nt a0 Z MW
    while True:
        name = toks[i]
        k = int(_num(toks[i + 1]))
        st, i = pairs(i + 2, k)
        logK = [_num(t) for t in toks[i:i + nt]]
        i += nt
        a0, Z = _num(toks[i]), _num(toks[i + 1])
        i = skip_note(i + 3)
        if name == "null":
            break
        db.secondary[name] = Reaction(st, logK, a0=a0, Z=Z)
    # gases, then minerals: name Vm k pairs logK*nt MW
    for table in (db.gases, db.minerals):
        while i < len(toks):
            name = toks[i]
            vm = _num(toks[i + 1])
            k = int(_num(toks[i + 2]))
            st, i = pairs(i + 3, k)
            logK = [_num(t) for t in toks[i:i + nt]]
            mw = _num(toks[i + nt]) if i + nt < len(toks) else 0.0
            i = skip_note(i + nt + 1)
            if name == "null":
                break
            table[name] = Reaction(st, logK, molar_vol_cm3=vm, molar_weight=mw)
    # surface complexes: name k pairs logK*nt Z MW (the site is one of the
    # species, its name starting with '>')
    while i + 1 < len(toks):
        name = toks[i]
        k = int(_num(toks[i + 1]))
        st, i = pairs(i + 2, k)
        logK = [_num(t) for t in toks[i:i + nt]]
        i += nt
        Z = _num(toks[i]) if i < len(toks) else 0.0
        i += 2
        # an optional trailing source note ('llnl-99'): a string followed by
        # a string (the next record's name) rather than by a count
        if i + 1 < len(toks) and not _is_num(toks[i]) and not _is_num(toks[i + 1]):
            i += 1
        if name == "null":
            break
        db.surface_complexes[name] = Reaction(st, logK, Z=Z)
    return db


def _is_num(tok: str) -> bool:
    try:
        _num(tok)
        return True
    except ValueError:
        return False


# unit factors to m, m^3 and kg
_AREA_LEN = {"m": 1.0, "dm": 1.0e-1, "cm": 1.0e-2, "mm": 1.0e-3}
_BULK_VOL = {"m^3": 1.0, "dm^3": 1.0e-3, "L": 1.0e-3, "cm^3": 1.0e-6, "mm^3": 1.0e-9}
_MASS = {"kg": 1.0, "g": 1.0e-3, "mg": 1.0e-6}


def mineral_surface_area(value, units: str, mineral: Reaction, volfrac, name: str = "mineral"):
    """Specific surface area of a kinetic mineral given in a constraint, in
    the engine's units (m^2 mineral per m^3 bulk, PfCellState.mnrl_area),
    following MineralProcessConstraint (reaction_mineral.F90:590-640).

    units is "<area>/<bulk volume>" (e.g. "cm^2/cm^3", "m^2/m^3") or, when it
    ends in "g", "<area>/<mass of mineral>" (e.g. "cm^2/g", "m^2/kg"): the
    mass-based area becomes m^2 mineral / m^3 mineral through the molar
    weight (g/mol) and molar volume of the database, then m^2 / m^3 bulk
    through the mineral's volume fraction.  value and volfrac may be arrays
    (a per-cell dataset).  The reference's errors are raised as ValueError: a
    molar weight or volume that is zero or the database's 500 marker, or a
    zero volume fraction, with a mass-based area."""
    num, _, den = units.replace(" ", "").partition("/")
    if not num.endswith("^2") or num[:-2] not in _AREA_LEN or not den:
        raise ValueError("%s: unsupported specific surface area units %r" % (name, units))
    area = _AREA_LEN[num[:-2]] ** 2
    per_unit_mass = den.endswith("g")
    if per_unit_mass:
        if den not in _MASS:
            raise ValueError("%s: unsupported specific surface area units %r" % (name, units))
        conv = area / _MASS[den]  # m^2 / kg mineral
        mw, vm = mineral.molar_weight, mineral.molar_vol_cm3 * 1.0e-6
        eps = 1.0e-40
        if mw < eps or mw == MISSING_LOGK:
            raise ValueError("Zero or undefined molar weight for mineral %r prevents specifying its "
                             "specific surface area per mass" % name)
        if vm < eps or mineral.molar_vol_cm3 == MISSING_LOGK:
            raise ValueError("Zero or undefined molar volume for mineral %r prevents specifying its "
                             "specific surface area per mass" % name)
        # m^2/kg * 1e-3 kg/g * g/mol / (m^3/mol) = m^2 mineral / m^3 mineral
        conv = conv * 1.0e-3 * mw / vm
        vf = np.asarray(volfrac, np.float64)
        out = conv * vf
        if np.any(out < 1.0e-40):
            raise ValueError("The zero volume fraction assigned to mineral %r prevents the use of a "
                             "mass-based surface area" % name)
        out = out * np.asarray(value, np.float64)
    else:
        if den not in _BULK_VOL:
            raise ValueError("%s: unsupported specific surface area units %r" % (name, units))
        out = area / _BULK_VOL[den] * np.asarray(value, np.float64)
    return float(out) if np.ndim(out) == 0 else out


def _crout_solve(a, b):
    """Crout LU with implicit pivoting and the substitutions
    (utility.F90:597-735) for the small normal-equation systems of the fit."""
    n = len(b)
    a = [list(map(float, row)) for row in a]
    b = list(map(float, b))
    vv = []
    for i in range(n):
        big = max(abs(x) for x in a[i])
        if big == 0.0:
            raise ZeroDivisionError("singular logK fit")
        vv.append(1.0 / big)
    indx = [0] * n
    for j in range(n):
        for i in range(j):
            s = a[i][j]
            for k in range(i):
                s = s - a[i][k] * a[k][j]
            a[i][j] = s
        big, imax = 0.0, j
        for i in range(j, n):
            s = a[i][j]
            for k in range(j):
                s = s - a[i][k] * a[k][j]
            a[i][j] = s
            dum = vv[i] * abs(s)
            if dum >= big:
                big, imax = dum, i
        if j != imax:
            a[imax], a[j] = a[j], a[imax]
            vv[imax] = vv[j]
        indx[j] = imax
        if a[j][j] == 0.0:
            a[j][j] = 1.0e-20
        if j != n - 1:
            dum = 1.0 / a[j][j]
            for i in range(j + 1, n):
                a[i][j] = a[i][j] * dum
    ii = -1
    for i in range(n):
        ll = indx[i]
        s = b[ll]
        b[ll] = b[i]
        if ii >= 0:
            for j in range(ii, i):
                s = s - a[i][j] * b[j]
        elif s != 0.0:
            ii = i
        b[i] = s
    for i in range(n - 1, -1, -1):
        s = b[i]
        for j in range(i + 1, n):
            s = s - a[i][j] * b[j]
        b[i] = s / a[i][i]
    return b


def fit_logK_coefs(temperatures, logK):
    """The five coefficients c of logK(T) = c1 ln T + c2 + c3 T + c4/T + c5/T^2
    (T in K) fitted over the temperatures whose logK is not 500."""
    rows, ys = [], []
    for t, k in zip(temperatures, logK):
        if abs(k - MISSING_LOGK) < 1.0e-10:
            continue
        tk = t + 273.15
        rows.append((math.log(tk), 1.0, tk, 1.0 / tk, 1.0 / (tk * tk)))
        ys.append(k)
    rhs = [sum(r[j] * y for r, y in zip(rows, ys)) for j in range(5)]
    a = [[sum(r[j] * r[k] for r in rows) for k in range(5)] for j in range(5)]
    return _crout_solve(a, rhs)


def eval_logK(coefs, t_c):
    tk = t_c + 273.15
    return coefs[0] * math.log(tk) + coefs[1] + coefs[2] * tk + coefs[3] / tk + coefs[4] / (tk * tk)


def debye_huckel(t_c: float):
    """(A, B, Bdot) at the reference temperature t_c (C)."""
    if t_c <= 0.01:
        return _DH_A[0], _DH_B[0], _DH_BDOT[0]
    if t_c > 300.0:
        return _DH_A[-1], _DH_B[-1], _DH_BDOT[-1]
    for k in range(1, len(_DH_T)):
        lo, hi = _DH_T[k - 1], _DH_T[k]
        if lo < t_c <= hi:
            w = (t_c - lo) / (hi - lo)
            return tuple(v[k - 1] + w * (v[k] - v[k - 1]) for v in (_DH_A, _DH_B, _DH_BDOT))
    raise AssertionError("unreachable")


def _reference_logK(db: Database, rxn: Reaction, coefs, t_ref: float, isothermal: bool):
    if isothermal:
        for k, t in enumerate(db.temperatures):
            if abs(t - t_ref) < 1.0e-10:
                return rxn.logK[k]
    return eval_logK(coefs, t_ref)


def _drop_water(stoich, primary):
    """The reaction's primary-species coefficients; water is left out (see
    _water)."""
    out = {}
    for sp, nu in stoich:
        if sp == "H2O":
            continue
        if sp not in primary:
            raise KeyError("species %s is not a primary species of this network (no basis swapping)" % sp)
        out[sp] = out.get(sp, 0.0) + nu
    return out


def _water(stoich):
    """The reaction's water coefficient (eqcplxh2ostoich / kinmnrlh2ostoich)."""
    return sum(nu for sp, nu in stoich if sp == "H2O")


def _lu_inverse(a):
    """Inverse by LUDecomposition and one LUBackSubstitution per unit vector
    (the reference's sec_matrix_inverse, reaction_database.F90:1316-1326),
    through the same Crout restatement as the logK fit."""
    n = len(a)
    inv = np.zeros((n, n))
    for k in range(n):
        e = [0.0] * n
        e[k] = 1.0
        inv[:, k] = _crout_solve(a, e)
    return inv


def swap_basis(db: Database, primary, secondary):
    """The change of basis of BasisInit (reaction_database.F90:1063-1450).
    primary: the new basis (database basis species and/or complexes);
    secondary: the complexes of the network, which must include every basis
    species of the database that the new basis leaves out and that some
    kept reaction uses.  Returns (reactions, minerals_fn): reactions maps each
    secondary to a Reaction in [H2O] + primary (stoichiometry with
    |nu| > 1e-40, logK per database temperature); minerals_fn(Reaction)
    rewrites a mineral's reaction in the new basis."""
    new_basis = ["H2O"] + list(primary)
    bidx = {sp: k for k, sp in enumerate(new_basis)}
    sidx = {sp: k for k, sp in enumerate(secondary)}
    rows = []  # the species with a database reaction: swapped-in primaries, then secondaries
    for p in primary:
        if p in db.secondary:
            rows.append(db.secondary[p])
        elif p not in db.primary:
            raise KeyError("%s is neither a basis species nor a complex of the database" % p)
    for sp in secondary:
        if sp in db.secondary:
            rows.append(db.secondary[sp])
        elif sp not in db.primary:
            raise KeyError("%s is neither a basis species nor a complex of the database" % sp)
    nsec = len(secondary)
    if len(rows) != nsec:
        raise ValueError("the new basis leaves %d reactions for %d secondary species (a swapped-out basis "
                         "species must be listed as a secondary)" % (len(rows), nsec))
    names = [p for p in primary if p in db.secondary] + [sp for sp in secondary if sp in db.secondary]
    nt = len(db.temperatures)
    P = np.zeros((nsec, len(new_basis)))
    S = np.zeros((nsec, nsec))
    L = np.zeros((nsec, nt))
    for r, (name, rxn) in enumerate(zip(names, rows)):
        L[r] = rxn.logK
        if name in bidx:
            P[r, bidx[name]] = -1.0
        else:
            S[r, sidx[name]] = -1.0
        for sp, nu in rxn.stoich:
            if sp in bidx:
                P[r, bidx[sp]] = nu
            elif sp in sidx:
                S[r, sidx[sp]] = nu
            else:
                raise KeyError("%s (in the reaction of %s) is neither in the new basis nor a secondary" % (sp, name))
    Sinv = _lu_inverse(S)
    stoich = -(Sinv @ P)
    logK = np.zeros((nsec, nt))
    missing = np.abs(L - MISSING_LOGK) < 1.0e-10
    for j in range(nsec):
        for t in range(nt):
            logK[j, t] = logK[j, t] - float(np.dot(Sinv[j], L[:, t]))
            # a combination that takes in a temperature without data has
            # none either (the literal combination would carry 500 into the
            # fit as if it were data)
            if np.any(missing[np.abs(Sinv[j]) > 0.0, t]):
                logK[j, t] = MISSING_LOGK
    out = {}
    for j, sp in enumerate(secondary):
        st = [(new_basis[c], float(stoich[j, c])) for c in range(len(new_basis)) if abs(stoich[j, c]) > 1.0e-40]
        if sp in db.secondary:
            a0, Z = db.secondary[sp].a0, db.secondary[sp].Z
        else:
            a0, Z = db.primary[sp][0], db.primary[sp][1]
        out[sp] = Reaction(st, list(logK[j]), a0=a0, Z=Z)

    def mineral(rxn: Reaction) -> Reaction:
        """Each secondary of the mineral's reaction replaced by its reaction
        in the new basis, logK += coefficient * the secondary's logK
        (BasisSubSpeciesInMineralRxn; coefficients below 1e-10 dropped)."""
        st = list(rxn.stoich)
        lk = list(rxn.logK)
        for sp in secondary:
            scale = None
            keep = []
            for name, nu in st:
                if name == sp:
                    scale = nu
                else:
                    keep.append([name, nu])
            if scale is None:
                continue
            for name, nu in out[sp].stoich:
                for item in keep:
                    if item[0] == name:
                        item[1] = item[1] + scale * nu
                        break
                else:
                    keep.append([name, scale * nu])
            st = [(name, nu) for name, nu in keep if abs(nu) > 1.0e-10]
            lk = [MISSING_LOGK if (abs(a - MISSING_LOGK) < 1.0e-10 or abs(b - MISSING_LOGK) < 1.0e-10)
                  else a + scale * b for a, b in zip(lk, out[sp].logK)]
        return Reaction(st, lk, a0=rxn.a0, Z=rxn.Z, molar_vol_cm3=rxn.molar_vol_cm3, molar_weight=rxn.molar_weight)

    return out, mineral


def build_network(db: Database, primary, secondary=None, minerals=None, options=None,
                  reference_temperature: float = 25.0) -> ReactionNetwork:
    """ReactionNetwork of `primary` (basis species of the database), the
    complexes `secondary` (None: every complex made of the primaries and
    water, in database order) and the kinetic minerals `minerals`, a dict
    name -> rate parameters {rate (mol/m^2/s), [activation_energy,
    affinity_threshold, rate_limiter, irreversible, min_scale_factor,
    Temkin_const, affinity_power]}.  options: solver options
    (default_options()); isothermal runs take logK at the reference
    temperature, others the temperature fits."""
    options = dict(options) if options is not None else default_options()
    isothermal = bool(options.get("isothermal", 1))
    pset = set(primary)
    for p in primary:
        if p not in db.primary and p not in db.secondary:
            raise KeyError("%s is neither a basis species nor a complex of the database" % p)
    swap = any(p not in db.primary for p in primary)
    if swap:
        if secondary is None:
            raise ValueError("a swapped basis needs its secondary species listed")
        swapped, swap_mineral = swap_basis(db, primary, secondary)
        sec_rxns = [(name, swapped[name]) for name in secondary]
    else:
        if secondary is None:
            secondary = [name for name, r in db.secondary.items()
                         if all(sp in pset or sp == "H2O" for sp, _ in r.stoich)]
        sec_rxns = [(name, db.secondary[name]) for name in secondary]
    secs = []
    for name, r in sec_rxns:
        coefs = fit_logK_coefs(db.temperatures, r.logK)
        secs.append(dict(name=name, stoich=_drop_water(r.stoich, pset), h2o=_water(r.stoich),
                         logK=_reference_logK(db, r, coefs, reference_temperature, isothermal),
                         logKcoef=coefs, Z=r.Z, a0=r.a0))
    mins = []
    for name, par in (minerals or {}).items():
        r = swap_mineral(db.minerals[name]) if swap else db.minerals[name]
        coefs = fit_logK_coefs(db.temperatures, r.logK)
        m = dict(name=name, stoich=_drop_water(r.stoich, pset), h2o=_water(r.stoich),
                 logK=_reference_logK(db, r, coefs, reference_temperature, isothermal),
                 logKcoef=coefs, molar_vol=r.molar_vol_cm3 * 1.0e-6)
        m.update(par)
        if "rate" not in m:
            raise KeyError("mineral %s: a rate constant is required" % name)
        mins.append(m)
    def z_a0(p):  # a swapped-in primary keeps its complex's charge and size
        return (db.primary[p][1], db.primary[p][0]) if p in db.primary else (db.secondary[p].Z, db.secondary[p].a0)
    return ReactionNetwork.build(list(primary), [z_a0(p)[0] for p in primary], [z_a0(p)[1] for p in primary], secs,
                                 mins, debye=debye_huckel(reference_temperature), options=options)


def constraint_reaction(db: Database, primary, name: str, kind: str = "mineral",
                        reference_temperature: float = 25.0, isothermal: bool = True) -> dict:
    """The reaction of a MINERAL or GAS constraint row (any mineral or gas of
    the database, kinetic or not) in the network's primaries, water dropped:
    dict(spec=[primary indices], stoich=[...], logK=logK at the reference
    temperature, logKcoef=the five-term fit, or None when isothermal), for
    ReactionEngine.equilibrate(..., reactions={component: ...})."""
    table = db.minerals if kind == "mineral" else db.gases
    if kind not in ("mineral", "gas"):
        raise ValueError("kind must be 'mineral' or 'gas'")
    r = table[name]
    pset = set(primary)
    nu = _drop_water(r.stoich, pset)
    index = {p: k for k, p in enumerate(primary)}
    coefs = fit_logK_coefs(db.temperatures, r.logK)
    return dict(spec=[index[sp] for sp in nu], stoich=[nu[sp] for sp in nu],
                logK=_reference_logK(db, r, coefs, reference_temperature, isothermal),
                logKcoef=None if isothermal else coefs)

