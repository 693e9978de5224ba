"""Host-side reaction network and per-cell state.

`ReactionNetwork` is the flattened counterpart of PFLOTRAN's reaction_rt_type
(src/pflotran/reaction_aux.F90:123-311) restricted to what the per-cell hot
path reads: aqueous complexes (eqcplxspecid/eqcplxstoich/eqcplx_logK, Z, a0),
kinetic minerals (kinmnrlspecid/kinmnrlstoich/kinmnrl_logK, TST constants,
reaction_mineral_aux.F90:82-138), the Debye-Hueckel constants and the
CHEMISTRY-block options.  `CellState` is the structure-of-arrays form of
rt_auxvar/global_auxvar/material_auxvar.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def default_options(**kw) -> dict:
    """ReactionCreate defaults (src/pflotran/reaction_aux.F90:391-393, 427-432,
    533-537) with LOG_FORMULATION and ACTIVITY_COEFFICIENTS TIMESTEP on, the
    settings of the operator-split decks."""
    o = dict(
        use_log_formulation=1,
        act_coef_update_frequency=abi.PF_ACT_COEF_TIMESTEP,
        act_coef_update_algorithm=abi.PF_ACT_COEF_ALGO_LAG,
        maximum_reaction_cuts=10,
        maximum_reaction_iterations=20,
        use_total_as_guess=0,
        isothermal=1,
        fork_literal_rsolve=0,
        max_dlnC_rreact=5.0,
        max_relative_change_tolerance=1e-6,
        max_residual_tolerance=1e-12,
        max_rel_residual_tolerance=1e-8,
        use_activity_h2o=0,
    )
    o.update(kw)
    return o


def tight_options(**kw) -> dict:
    """Tolerances four orders tighter than the defaults: the Newton solves run
    until the relative update is below 1e-10, so the returned iterate is
    within ~1e-10 of the root (quadratic convergence puts it far closer);
    separates arithmetic error from stopping-rule noise.  (Tighter than this,
    the update of a component whose total cancels to 1e-12 of its terms
    stays at rounding noise and never passes the test.)"""
    return default_options(max_relative_change_tolerance=1e-10,
                           max_residual_tolerance=1e-300,
                           max_rel_residual_tolerance=1e-300,
                           maximum_reaction_iterations=60, **kw)


def _ptr(a, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return C.cast(a.ctypes.data, C.POINTER(ctype))


@dataclass
class ReactionNetwork:
    primary: list
    secondary: list = field(default_factory=list)
    minerals: list = field(default_factory=list)
    pri_Z: np.ndarray = None
    pri_a0: np.ndarray = None
    # secondary complexes
    sec_nspec: np.ndarray = None
    sec_spec: np.ndarray = None
    sec_stoich: np.ndarray = None
    sec_logK: np.ndarray = None
    sec_logKcoef: np.ndarray = None
    sec_Z: np.ndarray = None
    sec_a0: np.ndarray = None
    # kinetic minerals
    mnrl_nspec: np.ndarray = None
    mnrl_spec: np.ndarray = None
    mnrl_stoich: np.ndarray = None
    mnrl_logK: np.ndarray = None
    mnrl_logKcoef: np.ndarray = None
    mnrl_rate_constant: np.ndarray = None
    mnrl_activation_energy: np.ndarray = None
    mnrl_molar_vol: np.ndarray = None
    mnrl_affinity_threshold: np.ndarray = None
    mnrl_rate_limiter: np.ndarray = None
    mnrl_irreversible: np.ndarray = None
    mnrl_min_scale_factor: np.ndarray = None
    mnrl_Temkin_const: np.ndarray = None
    mnrl_affinity_power: np.ndarray = None
    # water in the reactions (eqcplxh2ostoich, kinmnrlh2ostoich; None: none)
    sec_h2o_stoich: np.ndarray = None
    mnrl_h2o_stoich: np.ndarray = None
    debyeA: float = 0.5114
    debyeB: float = 0.3288
    debyeBdot: float = 0.0410
    options: dict = field(default_factory=default_options)
    # equilibrium sorption (None: none): dict(surface=[dict(site_density,
    # [surface ('null', 'mineral', 'rock')], [mineral], complexes=[dict(name,
    # stoich={primary: nu}, free_site_stoich, logK, [logKcoef], [h2o_stoich])])]
    # (equilibrium surface complexation, one entry per site), kd=[dict(species, type ('linear',
    # 'langmuir', 'freundlich'), coeff, [b], [n], [mineral])], kd_units
    # ('kg/m3 bulk' or 'mL/g soil'), soil_particle_density, ionx=[dict(
    # cations=[(name, k), ...] (the first is the reference cation), cec,
    # [mineral])])
    sorption: dict = None
    # kinetic-mineral rate prefactors (None: none): {mineral name: [dict(rate,
    # [activation_energy], species=[dict(name (primary or secondary), [alpha],
    # [beta], [atten_coef])])]}, the PREFACTOR blocks of the mineral's kinetics
    prefactors: dict = None

    @property
    def has_prefactors(self):
        return bool(self.prefactors) and any(len(v) for v in self.prefactors.values())

    @property
    def nkd(self):
        return len((self.sorption or {}).get("kd", ()))

    @property
    def nionx(self):
        return len((self.sorption or {}).get("ionx", ()))

    @property
    def nsrfcplx_rxn(self):
        return len((self.sorption or {}).get("surface", ()))

    @property
    def nsrfcplx(self):
        return sum(len(r["complexes"]) for r in (self.sorption or {}).get("surface", ()))

    @property
    def has_sorption(self):
        return self.nkd + self.nionx + self.nsrfcplx_rxn > 0

    @property
    def ncomp(self):
        return len(self.primary)

    @property
    def nsec(self):
        return len(self.secondary)

    @property
    def nmnrl(self):
        return len(self.minerals)

    @property
    def h_ion_id(self):
        return self.primary.index("H+") if "H+" in self.primary else -1

    @staticmethod
    def build(primary, pri_Z, pri_a0, secondaries, minerals=(), debye=(0.5114, 0.3288, 0.0410),
              options=None):
        """primary: names; secondaries: list of dicts {name, stoich:{species:nu}, logK, Z, a0,
        [logKcoef]}; minerals: list of dicts {name, stoich, logK, rate (mol/m^2/s), molar_vol
        (m^3/mol), [logKcoef, activation_energy, affinity_threshold, rate_limiter, irreversible]}.
        """
        n = len(primary)
        idx = {s: i for i, s in enumerate(primary)}

        def flatten(rxns):
            m = len(rxns)
            stride = max([len(r["stoich"]) for r in rxns] + [1])
            nspec = np.zeros(m, np.int32)
            spec = np.zeros((m, stride), np.int32)
            sto = np.zeros((m, stride), np.float64)
            for i, r in enumerate(rxns):
                items = list(r["stoich"].items())
                nspec[i] = len(items)
                for s, (name, nu) in enumerate(items):
                    spec[i, s] = idx[name] if isinstance(name, str) else int(name)
                    sto[i, s] = nu
            return nspec, spec, sto

        net = ReactionNetwork(primary=list(primary))
        net.pri_Z = np.asarray(pri_Z, np.float64)
        net.pri_a0 = np.asarray(pri_a0, np.float64)
        net.secondary = [r["name"] for r in secondaries]
        net.sec_nspec, net.sec_spec, net.sec_stoich = flatten(secondaries)
        net.sec_logK = np.array([r["logK"] for r in secondaries], np.float64)
        net.sec_Z = np.array([r["Z"] for r in secondaries], np.float64)
        net.sec_a0 = np.array([r["a0"] for r in secondaries], np.float64)
        if any(r.get("h2o", 0.0) for r in secondaries):
            net.sec_h2o_stoich = np.array([r.get("h2o", 0.0) for r in secondaries], np.float64)
        if secondaries and all("logKcoef" in r for r in secondaries):
            net.sec_logKcoef = np.array([r["logKcoef"] for r in secondaries], np.float64)
        mins = list(minerals)
        net.minerals = [r["name"] for r in mins]
        net.mnrl_nspec, net.mnrl_spec, net.mnrl_stoich = flatten(mins)
        nm = len(mins)
        net.mnrl_logK = np.array([r["logK"] for r in mins], np.float64)
        net.mnrl_rate_constant = np.array([r["rate"] for r in mins], np.float64)
        net.mnrl_molar_vol = np.array([r["molar_vol"] for r in mins], np.float64)
        net.mnrl_activation_energy = np.array([r.get("activation_energy", 0.0) for r in mins],
                                              np.float64)
        net.mnrl_affinity_threshold = np.array([r.get("affinity_threshold", 0.0) for r in mins],
                                               np.float64)
        net.mnrl_rate_limiter = np.array([r.get("rate_limiter", 0.0) for r in mins], np.float64)
        net.mnrl_irreversible = np.array([r.get("irreversible", 0) for r in mins], np.int32)
        if any(r.get("h2o", 0.0) for r in mins):
            net.mnrl_h2o_stoich = np.array([r.get("h2o", 0.0) for r in mins], np.float64)
        if mins and all("logKcoef" in r for r in mins):
            net.mnrl_logKcoef = np.array([r["logKcoef"] for r in mins], np.float64)
        for key in ("min_scale_factor", "Temkin_const", "affinity_power"):
            if any(key in r for r in mins):
                setattr(net, "mnrl_" + key,
                        np.array([r.get(key, 1.0) for r in mins], np.float64))
        if nm == 0:
            for k in ("mnrl_logK", "mnrl_rate_constant", "mnrl_molar_vol",
                      "mnrl_activation_energy", "mnrl_affinity_threshold", "mnrl_rate_limiter"):
                setattr(net, k, np.zeros(0, np.float64))
            net.mnrl_irreversible = np.zeros(0, np.int32)
        net.debyeA, net.debyeB, net.debyeBdot = debye
        net.options = options if options is not None else default_options()
        assert net.pri_Z.shape == (n,)
        return net

    def with_options(self, **kw):
        import copy
        other = copy.copy(self)
        other.options = dict(self.options)
        other.options.update(kw)
        return other

    def desc(self) -> abi.PfNetworkDesc:
        """PfNetworkDesc pointing into this object's arrays (keep self alive)."""
        self._keep = []

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a

        d = abi.PfNetworkDesc()
        d.ncomp, d.nsec, d.nmnrl = self.ncomp, self.nsec, self.nmnrl
        d.sec_stride = int(self.sec_spec.shape[1]) if self.nsec else 1
        d.mnrl_stride = int(self.mnrl_spec.shape[1]) if self.nmnrl else 1
        d.h_ion_id = self.h_ion_id
        i32, f64 = np.int32, np.float64
        d.sec_nspec = _ptr(arr(self.sec_nspec, i32), C.c_int32)
        d.sec_spec = _ptr(arr(self.sec_spec, i32), C.c_int32)
        d.sec_stoich = _ptr(arr(self.sec_stoich, f64), C.c_double)
        d.sec_logK = _ptr(arr(self.sec_logK, f64), C.c_double)
        d.sec_logKcoef = _ptr(arr(self.sec_logKcoef, f64), C.c_double)
        d.pri_Z = _ptr(arr(self.pri_Z, f64), C.c_double)
        d.pri_a0 = _ptr(arr(self.pri_a0, f64), C.c_double)
        d.sec_Z = _ptr(arr(self.sec_Z, f64), C.c_double)
        d.sec_a0 = _ptr(arr(self.sec_a0, f64), C.c_double)
        d.mnrl_nspec = _ptr(arr(self.mnrl_nspec, i32), C.c_int32)
        d.mnrl_spec = _ptr(arr(self.mnrl_spec, i32), C.c_int32)
        d.mnrl_stoich = _ptr(arr(self.mnrl_stoich, f64), C.c_double)
        d.mnrl_logK = _ptr(arr(self.mnrl_logK, f64), C.c_double)
        d.mnrl_logKcoef = _ptr(arr(self.mnrl_logKcoef, f64), C.c_double)
        d.mnrl_rate_constant = _ptr(arr(self.mnrl_rate_constant, f64), C.c_double)
        d.mnrl_activation_energy = _ptr(arr(self.mnrl_activation_energy, f64), C.c_double)
        d.mnrl_molar_vol = _ptr(arr(self.mnrl_molar_vol, f64), C.c_double)
        d.mnrl_affinity_threshold = _ptr(arr(self.mnrl_affinity_threshold, f64), C.c_double)
        d.mnrl_rate_limiter = _ptr(arr(self.mnrl_rate_limiter, f64), C.c_double)
        d.mnrl_irreversible = _ptr(arr(self.mnrl_irreversible, i32), C.c_int32)
        d.mnrl_min_scale_factor = _ptr(arr(self.mnrl_min_scale_factor, f64), C.c_double)
        d.mnrl_Temkin_const = _ptr(arr(self.mnrl_Temkin_const, f64), C.c_double)
        d.mnrl_affinity_power = _ptr(arr(self.mnrl_affinity_power, f64), C.c_double)
        d.debyeA, d.debyeB, d.debyeBdot = self.debyeA, self.debyeB, self.debyeBdot
        d.sec_h2o_stoich = _ptr(arr(self.sec_h2o_stoich, f64), C.c_double)
        d.mnrl_h2o_stoich = _ptr(arr(self.mnrl_h2o_stoich, f64), C.c_double)
        d.opts = self.options_struct()
        if self.has_sorption:
            self._sorb = self._sorption_desc(arr)
            d.sorption = C.pointer(self._sorb)
        if self.has_prefactors:
            self._pref = self._prefactor_desc(arr)
            d.prefactors = C.pointer(self._pref)
        return d

    def _prefactor_desc(self, arr) -> abi.PfPrefactorDesc:
        MP, MS = abi.PF_MAX_PREFACTORS, abi.PF_MAX_PREFACTOR_SPECIES
        nm = self.nmnrl
        pidx = {s: i for i, s in enumerate(self.primary)}
        sidx = {s: i for i, s in enumerate(self.secondary)}
        i32, f64 = np.int32, np.float64
        cnt = np.zeros(nm, i32)
        rate, ea = np.zeros((nm, MP), f64), np.zeros((nm, MP), f64)
        nsp = np.zeros((nm, MP), i32)
        spec = np.zeros((nm, MP, MS), i32)
        alpha, beta, atten = (np.zeros((nm, MP, MS), f64) for _ in range(3))
        for name, prefs in self.prefactors.items():
            m = self.minerals.index(name)
            if len(prefs) > MP:
                raise ValueError("mineral %s: more than %d prefactors" % (name, MP))
            cnt[m] = len(prefs)
            for p, pr in enumerate(prefs):
                rate[m, p] = pr["rate"]
                ea[m, p] = pr.get("activation_energy", 0.0)
                sps = list(pr.get("species", ()))
                if len(sps) > MS:
                    raise ValueError("mineral %s: more than %d prefactor species" % (name, MS))
                nsp[m, p] = len(sps)
                for k, sp in enumerate(sps):
                    nm_ = sp["name"]
                    spec[m, p, k] = pidx[nm_] if nm_ in pidx else -(sidx[nm_] + 1)
                    alpha[m, p, k] = sp.get("alpha", 0.0)
                    beta[m, p, k] = sp.get("beta", 0.0)
                    atten[m, p, k] = sp.get("atten_coef", 0.0)
        pd = abi.PfPrefactorDesc()
        pd.num_prefactors = _ptr(arr(cnt, i32), C.c_int32)
        pd.rate = _ptr(arr(rate, f64), C.c_double)
        pd.activation_energy = _ptr(arr(ea, f64), C.c_double)
        pd.nspec = _ptr(arr(nsp, i32), C.c_int32)
        pd.spec = _ptr(arr(spec, i32), C.c_int32)
        pd.alpha = _ptr(arr(alpha, f64), C.c_double)
        pd.beta = _ptr(arr(beta, f64), C.c_double)
        pd.atten_coef = _ptr(arr(atten, f64), C.c_double)
        return pd

    def _sorption_desc(self, arr) -> abi.PfSorptionDesc:
        sp = self.sorption
        idx = {s: i for i, s in enumerate(self.primary)}
        mins = {m: i for i, m in enumerate(self.minerals)}
        i32, f64 = np.int32, np.float64
        kinds = {"linear": abi.PF_SORPTION_LINEAR, "langmuir": abi.PF_SORPTION_LANGMUIR,
                 "freundlich": abi.PF_SORPTION_FREUNDLICH}
        sd = abi.PfSorptionDesc()
        kd = list(sp.get("kd", ()))
        sd.nkd = len(kd)
        sd.kd_units = {"kg/m3 bulk": abi.PF_KD_UNIT_KG_M3_BULK,
                       "mL/g soil": abi.PF_KD_UNIT_MLW_GSOIL}[sp.get("kd_units", "kg/m3 bulk")]
        sd.soil_particle_density = float(sp.get("soil_particle_density", 2650.0))
        if kd:
            sd.kd_spec = _ptr(arr([idx[r["species"]] for r in kd], i32), C.c_int32)
            sd.kd_type = _ptr(arr([kinds[r.get("type", "linear")] for r in kd], i32), C.c_int32)
            sd.kd_coeff = _ptr(arr([r["coeff"] for r in kd], f64), C.c_double)
            sd.kd_langmuir_b = _ptr(arr([r.get("b", 0.0) for r in kd], f64), C.c_double)
            sd.kd_freundlich_n = _ptr(arr([r.get("n", 1.0) for r in kd], f64), C.c_double)
            sd.kd_mineral = _ptr(arr([mins[r["mineral"]] if r.get("mineral") else -1 for r in kd], i32),
                                 C.c_int32)
        ix = list(sp.get("ionx", ()))
        sd.nionx = len(ix)
        if ix:
            stride = max(len(r["cations"]) for r in ix)
            cat = np.zeros((len(ix), stride), i32)
            kk = np.zeros((len(ix), stride), f64)
            for i, r in enumerate(ix):
                for j, (name, k) in enumerate(r["cations"]):
                    cat[i, j], kk[i, j] = idx[name], k
            sd.ionx_stride = stride
            sd.ionx_ncation = _ptr(arr([len(r["cations"]) for r in ix], i32), C.c_int32)
            sd.ionx_cation = _ptr(arr(cat, i32), C.c_int32)
            sd.ionx_k = _ptr(arr(kk, f64), C.c_double)
            sd.ionx_cec = _ptr(arr([r["cec"] for r in ix], f64), C.c_double)
            sd.ionx_mineral = _ptr(arr([mins[r["mineral"]] if r.get("mineral") else -1 for r in ix], i32),
                                   C.c_int32)
        sx = list(sp.get("surface", ()))
        sd.nsrfcplx_rxn = len(sx)
        if sx:
            cplx = [c for r in sx for c in r["complexes"]]
            sd.nsrfcplx = len(cplx)
            stride = max(1, max(len(c["stoich"]) for c in cplx))
            spec = np.zeros((len(cplx), stride), i32)
            nu = np.zeros((len(cplx), stride), f64)
            for k, c in enumerate(cplx):
                for p, (name, v) in enumerate(c["stoich"].items()):
                    spec[k, p], nu[k, p] = idx[name], v
            ptr = np.cumsum([0] + [len(r["complexes"]) for r in sx])
            stype = {"null": abi.PF_SURF_NULL, "mineral": abi.PF_SURF_MINERAL, "rock": abi.PF_SURF_ROCK}
            sd.srfcplx_rxn_ptr = _ptr(arr(ptr, i32), C.c_int32)
            sd.srfcplx_surf_type = _ptr(arr([stype[r.get("surface", "null")] for r in sx], i32), C.c_int32)
            sd.srfcplx_mineral = _ptr(arr([mins[r["mineral"]] if r.get("mineral") else -1 for r in sx], i32),
                                      C.c_int32)
            sd.srfcplx_site_density = _ptr(arr([r["site_density"] for r in sx], f64), C.c_double)
            sd.srfcplx_stride = stride
            sd.srfcplx_nspec = _ptr(arr([len(c["stoich"]) for c in cplx], i32), C.c_int32)
            sd.srfcplx_spec = _ptr(arr(spec, i32), C.c_int32)
            sd.srfcplx_stoich = _ptr(arr(nu, f64), C.c_double)
            sd.srfcplx_free_site_stoich = _ptr(arr([c.get("free_site_stoich", 1.0) for c in cplx], f64), C.c_double)
            sd.srfcplx_logK = _ptr(arr([c["logK"] for c in cplx], f64), C.c_double)
            if all(c.get("logKcoef") is not None for c in cplx):
                sd.srfcplx_logKcoef = _ptr(arr([c["logKcoef"] for c in cplx], f64), C.c_double)
            if any(c.get("h2o_stoich", 0.0) for c in cplx):
                sd.srfcplx_h2o_stoich = _ptr(arr([c.get("h2o_stoich", 0.0) for c in cplx], f64), C.c_double)
        return sd

    def options_struct(self) -> abi.PfOptions:
        o = abi.PfOptions()
        for k, _ in abi.PfOptions._fields_:
            setattr(o, k, self.options[k])
        return o


# ---------------------------------------------------------------- cell state
STATE_FIELDS = {
    # name: (rows, dtype)  rows: 'n' ncomp, 's' nsec, 'm' nmnrl, 1 scalar
    "total": ("n", np.float64), "pri_molal": ("n", np.float64),
    "pri_act_coef": ("n", np.float64), "sec_act_coef": ("s", np.float64),
    "sec_molal": ("s", np.float64), "mnrl_volfrac": ("m", np.float64),
    "mnrl_area": ("m", np.float64), "mnrl_rate": ("m", np.float64),
    "porosity": (1, np.float64), "saturation": (1, np.float64),
    "den_kg": (1, np.float64), "volume": (1, np.float64),
    "temperature": (1, np.float64), "dt_cell": (1, np.float64),
    "status": (1, np.int32), "newton_its": (1, np.int32), "num_substeps": (1, np.int32),
    # networks with sorption only
    "total_sorb": ("n", np.float64), "ionx_ref_sorbed": ("x", np.float64),
    # networks with the water activity option only
    "ln_act_h2o": (1, np.float64),
    # networks with surface complexation only
    "srfcplx_free_site": ("r", np.float64), "srfcplx_conc": ("c", np.float64),
}
OPTIONAL_FIELDS = ("dt_cell",)
SORPTION_FIELDS = ("total_sorb", "ionx_ref_sorbed")
SURFACE_FIELDS = ("srfcplx_free_site", "srfcplx_conc")
H2O_FIELDS = ("ln_act_h2o",)


def _rows(net, r):
    return {"n": net.ncomp, "s": net.nsec, "m": net.nmnrl, "x": net.nionx, "r": net.nsrfcplx_rxn,
            "c": net.nsrfcplx}.get(r, r)


class CellState:
    """SoA per-cell state. Arrays are numpy (host) or torch tensors (device),
    shaped (rows, ncells) so that value(k, cell) = a[k*ncells+cell]."""

    def __init__(self, net: ReactionNetwork, arrays: dict):
        self.net = net
        self.a = dict(arrays)
        self.ncells = int(self.a["porosity"].shape[-1])

    @staticmethod
    def empty(net, ncells, with_dt=False):
        a = {}
        for k, (r, dt) in STATE_FIELDS.items():
            if k in OPTIONAL_FIELDS and not with_dt:
                continue
            if k in SORPTION_FIELDS and not net.has_sorption:
                continue
            if k in SURFACE_FIELDS and not net.nsrfcplx_rxn:
                continue
            if k in H2O_FIELDS and not net.options.get("use_activity_h2o"):
                continue
            rows = _rows(net, r)
            a[k] = np.zeros((rows, ncells), dt) if r != 1 else np.zeros(ncells, dt)
        if net.has_sorption:
            a["ionx_ref_sorbed"][:] = 1.0e-9  # reactive_transport_aux.F90:282
        if net.nsrfcplx_rxn:
            a["srfcplx_free_site"][:] = 1.0e-9  # srfcplxrxn_free_site_conc's initial value
        a["pri_act_coef"][:] = 1.0
        a["sec_act_coef"][:] = 1.0
        a["saturation"][:] = 1.0
        a["volume"][:] = 1.0
        a["temperature"][:] = 25.0
        return CellState(net, a)

    def copy(self):
        out = {}
        for k, v in self.a.items():
            out[k] = v.copy() if isinstance(v, np.ndarray) else v.clone()
        return CellState(self.net, out)

    def to(self, device):
        import torch
        out = {}
        for k, v in self.a.items():
            t = v if not isinstance(v, np.ndarray) else torch.from_numpy(np.ascontiguousarray(v))
            out[k] = t.to(device).contiguous()
        return CellState(self.net, out)

    def numpy(self):
        out = {}
        for k, v in self.a.items():
            out[k] = v if isinstance(v, np.ndarray) else v.detach().cpu().numpy()
        return CellState(self.net, out)

    def subset(self, idx):
        out = {}
        for k, v in self.a.items():
            if isinstance(v, np.ndarray):
                out[k] = np.ascontiguousarray(v[..., idx])
            else:
                out[k] = v[..., idx].contiguous()
        return CellState(self.net, out)

    def struct(self, where: str | None = None, net: ReactionNetwork | None = None) -> abi.PfCellState:
        """The PfCellState of these arrays, after checking each one against
        the field table: its dtype, rows x ncells elements (rows of `net`,
        default this state's network) and C-contiguous storage.  where =
        "device": every array a CUDA tensor, all on one device; "host": every
        array a numpy array; None: either.  A buffer of the wrong type or
        length would be read past its end by the kernels, so a mismatch is a
        ValueError naming the field.  Missing fields stay NULL pointers, which
        the library refuses where the network needs them."""
        net = net or self.net
        s = abi.PfCellState()
        s.ncells = self.ncells
        device = None
        for k, (r, dt) in STATE_FIELDS.items():
            v = self.a.get(k)
            ct = C.c_int32 if dt == np.int32 else C.c_double
            if v is None:
                setattr(s, k, C.cast(None, C.POINTER(ct)))
                continue
            want = _rows(net, r) * self.ncells
            if isinstance(v, np.ndarray):
                if where == "device":
                    raise ValueError("state field %r is a host array; this call needs CUDA tensors" % k)
                if v.dtype != dt or not v.flags.c_contiguous or v.size != want:
                    raise ValueError("state field %r: need a C-contiguous %s array of %d values, got %s %s%s"
                                     % (k, np.dtype(dt).name, want, v.dtype, v.shape,
                                        "" if v.flags.c_contiguous else " (not contiguous)"))
                addr = v.ctypes.data
            else:
                tname = "torch." + np.dtype(dt).name
                if str(v.dtype) != tname or not v.is_contiguous() or v.numel() != want:
                    raise ValueError("state field %r: need a contiguous %s tensor of %d values, got %s %s%s"
                                     % (k, tname, want, v.dtype, tuple(v.shape),
                                        "" if v.is_contiguous() else " (not contiguous)"))
                if where == "host":
                    raise ValueError("state field %r is a tensor; this call needs host numpy arrays" % k)
                if where == "device":
                    if not v.is_cuda:
                        raise ValueError("state field %r is on %s; this call needs CUDA tensors" % (k, v.device))
                    if device is not None and v.device != device:
                        raise ValueError("state field %r is on %s, others on %s" % (k, v.device, device))
                    device = v.device
                addr = v.data_ptr()
            setattr(s, k, C.cast(addr, C.POINTER(ct)))
        return s
