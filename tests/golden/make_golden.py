"""Generate the known-answer fixtures in tests/golden/ from the reference's own
regression decks, thermodynamic databases and gold files.

Runs only where the reference tree is mounted: pass its root as argv[1] or in
PFGPU_REFERENCE_ROOT.  The tests read the JSON this writes and never the
reference tree itself.

Sources (paths within fmyuan/pflotran-elm-interface):
  regression_tests/ascem/batch/<deck>.in              chemistry block, constraint, times
  regression_tests/ascem/batch/{calcite,carbonate,ca-carbonate}.dat  database
  regression_tests/ascem/batch/<deck>.regression.gold  expected values
  regression_tests/ascem/batch/batch.cfg:20-27         tolerances (1e-12 absolute)
  src/pflotran/unittests/test_eos_water.pf:146-157     IFC67 density pin
"""
import json
import os
import re
import shlex
import sys

ROOT = os.environ.get("PFGPU_REFERENCE_ROOT", "")
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                "pflotran-elm-interface_gb300"))
BATCH = os.path.join(ROOT, "regression_tests", "ascem", "batch")
OUT = os.path.dirname(os.path.abspath(__file__))

DECKS = ["carbonate-unit-activity", "carbonate-debye-huckel-activity",
         "ca-carbonate-unit-activity", "ca-carbonate-debye-huckel-activity",
         "calcite-kinetics", "calcite-kinetics-volume-fractions", "calcite-area-per-mass",
         "surface-complexation-1"]

TIME_UNITS = {"s": 1.0, "sec": 1.0, "min": 60.0, "h": 3600.0, "hr": 3600.0,
              "d": 86400.0, "day": 86400.0, "w": 7 * 86400.0,
              "mo": 365.0 / 12.0 * 86400.0, "y": 365.0 * 86400.0, "yr": 365.0 * 86400.0}


def fnum(s):
    return float(s.lower().replace("d", "e"))


def read_dat(path):
    """The database through the package's reader (pfgpu.database), in the
    dictionaries this script uses."""
    from pfgpu.database import read_database
    db = read_database(path)
    primary = {k: dict(a0=v[0], Z=v[1]) for k, v in db.primary.items()}
    secondary = {k: dict(stoich=r.stoich, logK=r.logK, a0=r.a0, Z=r.Z) for k, r in db.secondary.items()}
    minerals = {k: dict(stoich=r.stoich, logK=r.logK, molar_vol_cm3=r.molar_vol_cm3) for k, r in db.minerals.items()}
    return db.temperatures, primary, secondary, minerals


def block(lines, start):
    out = []
    for ln in lines[start + 1:]:
        s = ln.strip()
        if s == "/" or s.upper() == "END":
            break
        if s:
            out.append(s)
    return out


def read_deck(path):
    raw = [ln.split("#")[0].split("!")[0].rstrip() for ln in open(path)]
    lines = [ln for ln in raw]
    up = [ln.strip().upper() for ln in lines]
    deck = {}
    i = up.index("PRIMARY_SPECIES")
    deck["primary"] = block(lines, i)
    i = up.index("SECONDARY_SPECIES")
    deck["secondary"] = block(lines, i)
    deck["minerals"] = block(lines, up.index("MINERALS")) if "MINERALS" in up else []
    deck["rates"] = {}
    if "MINERAL_KINETICS" in up:
        j = up.index("MINERAL_KINETICS") + 1
        while up[j] != "/":
            name = lines[j].strip()
            k = j + 1
            while up[k] != "/":
                m = re.match(r"RATE_CONSTANT\s+(\S+)\s*(\S*)", lines[k].strip(), re.I)
                if m:
                    v = fnum(m.group(1))
                    unit = m.group(2)
                    if unit == "mol/cm^2-sec":
                        v *= 1.0e4
                    deck["rates"][name] = v
                k += 1
            j = k + 1
    chem = " ".join(up[up.index("CHEMISTRY"):])
    deck["database"] = re.search(r"DATABASE\s+(\S+)", " ".join(lines)).group(1)
    deck["log_formulation"] = "LOG_FORMULATION" in chem
    m = re.search(r"ACTIVITY_COEFFICIENTS\s+(\w+)", chem)
    deck["act_coef"] = m.group(1) if m and m.group(1) in ("TIMESTEP", "NEWTON_ITERATION", "OFF") else "OFF"
    ci = [k for k, s in enumerate(up) if s.startswith("CONSTRAINT INITIAL")][0]
    k = up.index("CONCENTRATIONS", ci)
    deck["constraint"] = {}
    for s in block(lines, k):
        parts = s.split()
        deck["constraint"][parts[0]] = (parts[2].upper(), fnum(parts[1]))
    deck["mineral_init"] = {}
    if "MINERALS" in up[ci:]:
        k = up.index("MINERALS", ci)
        for s in block(lines, k):
            p = s.split()
            area = fnum(p[2])
            unit = p[3] if len(p) > 3 else "m^2/m^3"
            if unit == "cm^2/cm^3":
                area *= 100.0
            elif unit != "m^2/m^3":
                # converted in main() with the database's molar weight/volume
                deck.setdefault("area_units", {})[p[0]] = unit
            deck["mineral_init"][p[0]] = (fnum(p[1]), area)
    if "SURFACE_COMPLEXATION_RXN" in up:
        j = up.index("SURFACE_COMPLEXATION_RXN")
        site = [lines[k].split() for k in range(j, len(up)) if up[k].startswith("SITE ")][0]
        deck["surface"] = dict(site=site[1], site_density=fnum(site[2]),
                               complexes=block(lines, up.index("COMPLEXES", j)))
    deck["porosity"] = fnum(re.search(r"POROSITY\s+(\S+)", " ".join(lines)).group(1))
    for key in ("FINAL_TIME", "INITIAL_TIMESTEP_SIZE", "MAXIMUM_TIMESTEP_SIZE"):
        m = re.search(key + r"\s+(\S+)\s+(\S+)", " ".join(lines))
        deck[key.lower()] = fnum(m.group(1)) * TIME_UNITS[m.group(2)]
    return deck


def read_gold(path):
    gold = {}
    txt = open(path).read().splitlines()
    for i, ln in enumerate(txt):
        m = re.match(r"-- (\w+): (.+) --", ln)
        if m and m.group(1) != "SOLUTION" and m.group(1) != "DISCRETE":
            gold[m.group(2)] = float(txt[i + 1].split()[1])
        if m and m.group(1) == "SOLUTION":
            for ln2 in txt[i + 1:]:
                mm = re.match(r"\s+(Time Steps|Newton Iterations):\s+(\d+)", ln2)
                if mm:
                    gold[mm.group(1)] = int(mm.group(2))
    return gold


def main():
    tref_index = None
    fixtures = {}
    for name in DECKS:
        deck = read_deck(os.path.join(BATCH, name + ".in"))
        temps, pri, sec, mins = read_dat(os.path.join(BATCH, deck["database"].lstrip("./")))
        tref_index = temps.index(25.0)
        primary = deck["primary"]
        fx = dict(
            deck=name,
            source="regression_tests/ascem/batch/%s.in" % name,
            primary=primary,
            pri_Z=[pri[s]["Z"] for s in primary],
            pri_a0=[pri[s]["a0"] for s in primary],
            secondaries=[dict(name=s, stoich={sp: nu for sp, nu in sec[s]["stoich"] if sp != "H2O"},
                              logK=sec[s]["logK"][tref_index], Z=sec[s]["Z"], a0=sec[s]["a0"])
                         for s in deck["secondary"]],
            minerals=[dict(name=m, stoich={sp: nu for sp, nu in mins[m]["stoich"] if sp != "H2O"},
                           logK=mins[m]["logK"][tref_index], rate=deck["rates"][m],
                           molar_vol=mins[m]["molar_vol_cm3"] * 1.0e-6)
                      for m in deck["minerals"]],
            log_formulation=deck["log_formulation"],
            act_coef=deck["act_coef"],
            constraint=deck["constraint"],
            mineral_init=deck["mineral_init"],
            porosity=deck["porosity"],
            final_time=deck["final_time"],
            dt=deck["maximum_timestep_size"],
            gold=read_gold(os.path.join(BATCH, name + ".regression.gold")),
            tolerance_abs=1.0e-12,
        )
        if deck.get("surface"):
            # equilibrium surface complexation on a fixed site density
            # (SURFACE_COMPLEXATION_RXN ... SITE name density, NULL_SURFACE)
            from pfgpu.database import read_database
            db = read_database(os.path.join(BATCH, deck["database"].lstrip("./")))
            sf = deck["surface"]
            cplx = []
            for cname in sf["complexes"]:
                r = db.surface_complexes[cname]
                cplx.append(dict(name=cname, logK=r.logK[tref_index], Z=r.Z,
                                 free_site_stoich=sum(nu for sp, nu in r.stoich if sp == sf["site"]),
                                 stoich={sp: nu for sp, nu in r.stoich if sp != sf["site"] and sp != "H2O"}))
            fx["surface_complexation"] = dict(site=sf["site"], site_density=sf["site_density"], complexes=cplx)
        if deck.get("area_units"):
            # specific surface area per mass of mineral (MineralProcessConstraint,
            # reaction_mineral.F90:590-640) through the package's conversion
            from pfgpu.database import mineral_surface_area, read_database
            db = read_database(os.path.join(BATCH, deck["database"].lstrip("./")))
            fx["mineral_area_input"] = {}
            for m, unit in deck["area_units"].items():
                vf, raw = deck["mineral_init"][m]
                fx["mineral_area_input"][m] = [raw, unit]
                fx["mineral_init"][m] = (vf, mineral_surface_area(raw, unit, db.minerals[m], vf, m))
        fixtures[name] = fx
    # IFC67 pin: src/pflotran/unittests/test_eos_water.pf
    pf = open(os.path.join(ROOT, "src", "pflotran", "unittests", "test_eos_water.pf")).read()
    m = re.search(r"998\.\d+", pf)
    fixtures["_eos_water_pin"] = dict(source="src/pflotran/unittests/test_eos_water.pf",
                                      t=20.0, p=101325.0, density=float(m.group(0)))
    with open(os.path.join(OUT, "kat_batch.json"), "w") as f:
        json.dump(fixtures, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(OUT, "kat_batch.json"))


if __name__ == "__main__":
    if len(sys.argv) > 1:
        ROOT = sys.argv[1]
        BATCH = os.path.join(ROOT, "regression_tests", "ascem", "batch")
    if not ROOT:
        sys.exit("usage: make_golden.py <root of the reference tree>  (or set PFGPU_REFERENCE_ROOT)")
    main()
