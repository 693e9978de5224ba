"""Known-answer-test drivers shared by the oracle and GPU tests.

A KAT fixture (tests/golden/kat_batch.json, made by make_golden.py from the
reference's regression decks) describes one single-cell batch problem.  The
drivers reproduce the reference's sequence for it:

  constraint equilibration          reaction.F90:1328-2115
  initial auxvars: RTotal, then (activity on) 2x [RActivityCoefficients, RTotal]
                                    condition_control.F90:1638-1649
  per time step (GIRT single cell, no transport):
    fixed accumulation: RTotal at c   reactive_transport.F90:931-1043
    TIMESTEP activity update          pm_rt.F90:531-537
    Newton to convergence on (A(c)-A_k)/dt + R(c) = 0
    RTotal at the solution; RUpdateKineticState   pm_rt.F90:1177-1223
"""
import json
import math
import os

import numpy as np

from pfgpu import abi
from pfgpu.network import CellState, ReactionNetwork, default_options, tight_options

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "kat_batch.json")))
CON = {"T": 1, "F": 2, "PH": 3, "P": 3, "Z": 4, "CHG": 4, "L": 5}


def kat_names(kind=None):
    names = [k for k in KAT if not k.startswith("_")]
    if kind == "surface":
        return [k for k in names if "surface_complexation" in KAT[k]]
    names = [k for k in names if "surface_complexation" not in KAT[k]]
    if kind == "speciation":
        return [k for k in names if KAT[k]["gold"].get("Time Steps", 0) == 0]
    if kind == "kinetics":
        return [k for k in names if KAT[k]["gold"].get("Time Steps", 0) > 0]
    return names


def network(fx, tight=True):
    freq = {"OFF": abi.PF_ACT_COEF_OFF, "TIMESTEP": abi.PF_ACT_COEF_TIMESTEP,
            "NEWTON_ITERATION": abi.PF_ACT_COEF_NEWTON_ITER}[fx["act_coef"]]
    mk = tight_options if tight else default_options
    opts = mk(act_coef_update_frequency=freq, use_log_formulation=int(fx["log_formulation"]))
    return ReactionNetwork.build(fx["primary"], fx["pri_Z"], fx["pri_a0"], fx["secondaries"],
                                 fx["minerals"], options=opts)


def initial_state(fx, net, oracle, density):
    st = CellState.empty(net, 1)
    st.a["porosity"][:] = fx["porosity"]
    st.a["den_kg"][:] = density
    for m, mname in enumerate(net.minerals):
        vf, area = fx["mineral_init"][mname]
        st.a["mnrl_volfrac"][m] = vf
        st.a["mnrl_area"][m] = area
    ctype = [CON[fx["constraint"][s][0]] for s in net.primary]
    cconc = np.array([[fx["constraint"][s][1]] for s in net.primary])
    # constraints equilibrate with the default (not tight) tolerances
    eq_net = net.with_options(max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12)
    rc, its = oracle.equilibrate(eq_net, st, ctype, cconc)
    assert rc == 0 and its[0] > 0, (rc, its)
    # The constraint is equilibrated once on the constraint coupler's own
    # auxvar (patch.F90:5331); cells take only its free-ion molarity
    # (basis_molarity, reaction.F90:2104-2106) and start from a fresh auxvar
    # with unit activity coefficients (condition_control.F90:1470-1475).
    basis_molarity = st.a["pri_molal"] * density / 1000.0
    st.a["pri_molal"][:] = basis_molarity / density * 1000.0
    st.a["pri_act_coef"][:] = 1.0
    st.a["sec_act_coef"][:] = 1.0
    st.a["sec_molal"][:] = 0.0
    oracle.update_auxvars(net, st, update_act=False)
    if net.options["act_coef_update_frequency"] != abi.PF_ACT_COEF_OFF:
        oracle.update_auxvars(net, st, update_act=True)
        oracle.update_auxvars(net, st, update_act=True)
    return st


def step_times(fx):
    t, out = 0.0, []
    while t < fx["final_time"] * (1 - 1e-14):
        dt = min(fx["dt"], fx["final_time"] - t)
        out.append(dt)
        t += dt
    return out


def run_kinetics(fx, net, st, react, aux, act, kin):
    """Time-step loop; react/aux/act/kin are callables (oracle or GPU)."""
    for dt in step_times(fx):
        aux(st, False)
        if net.options["act_coef_update_frequency"] == abi.PF_ACT_COEF_TIMESTEP:
            act(st)
        react(st, dt)
        kin(st, dt)
    return st


def outputs(fx, net, st):
    out = {}
    h = net.h_ion_id
    out["pH"] = -math.log10(st.a["pri_molal"][h, 0] * st.a["pri_act_coef"][h, 0])
    for k, s in enumerate(net.primary):
        out["Total " + s] = st.a["total"][k, 0]
        out["Gamma " + s] = st.a["pri_act_coef"][k, 0]
    for m, s in enumerate(net.minerals):
        out[s + " VF"] = st.a["mnrl_volfrac"][m, 0]
        out[s + " Rate"] = st.a["mnrl_rate"][m, 0]
    return out
