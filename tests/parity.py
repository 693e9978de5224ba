"""Per-cell comparison of an operator-split step against the oracle.

Quantities and their scales (FP64 throughout; REL = 1e-10):
  pri_molal, sec_molal   relative to the oracle's value
  total                  relative to the component's gross scale
                         den*(m_k + sum_i |nu_ik| s_i) (totals cancel)
  mnrl_rate              relative to the rate's gross scale
                         |I| (1 + p QK/|1 - QK|), QK = (Q/K)^(1/sigma): the
                         rate is k A sign(1-QK) |1-QK|^p, so an error d in
                         ln Q moves it by p |I| QK/|1-QK| d; near equilibrium
                         (QK -> 1) the affinity cancels and only this gross
                         scale is meaningful (the same reason totals use one)
  mnrl_volfrac           relative to |volfrac| + gross rate * V_m * dt
  status, num_substeps   exact (they define the path)

A cell that failed (status != 0: dt cut maximum_reaction_cuts times) is
compared on its status, path and totals only: RStep restores its totals, and
its molalities and rates are whatever the last non-converged Newton iterate
held -- the reference's time loop discards them (the whole step is cut and
repeated, pmc_subsurface_osrt.F90:381-396), and two factorisations of the
same non-converging iteration drift apart by rounding.

Cells are classified by their Newton path against the oracle's:
  path-identical   same Newton iteration count, substep count and status
                   (single-RReact cells, cells with dt cuts, failed cells)
  flip             any of the three differs: a stopping test or a dt cut
                   decided by rounding
The oracle run on inputs one ulp away (totals up, totals down, initial
molalities up) measures how often the reference algorithm itself flips or
moves a path-identical cell by more than REL ("outliers": its stopping tests
|r| < 1e-12 and ||r||/||r0|| < 1e-8 are absolute, so an iterate can pass them
far from the root in weakly constrained species, and where it lands depends
on the rounding of earlier iterates).

The report (REPORT, printed at the end of the session by conftest) holds per
case: cells by class, flips and outliers of the GPU and of the oracle
against itself, max error per quantity over the compared cells, the GPU's
and the oracle's own max error over flipped cells, Newton counts.
"""
import numpy as np

REL = 1.0e-10
LOG_TO_LN = 2.30258509299
REPORT = {}


def gross_total(net, st):
    """den*(m_k + sum_i |nu_ik| s_i): the scale of total_k before cancellation."""
    g = st.a["pri_molal"].copy()
    for i in range(net.nsec):
        for s in range(net.sec_nspec[i]):
            g[net.sec_spec[i, s]] += abs(net.sec_stoich[i, s]) * st.a["sec_molal"][i]
    return g * st.a["den_kg"] * 1e-3


def mineral_qk(net, st):
    """(Q/K)^(1/sigma) per mineral and cell at st's molalities, activity
    coefficients and temperature (RKineticMineral, reaction_mineral.F90:
    766-782, Temkin constant sigma; logK(T) by ReactionInterpolateLogK)."""
    nm, N = net.nmnrl, st.ncells
    la = np.log(st.a["pri_molal"] * st.a["pri_act_coef"])
    tk = (st.a["temperature"] if "temperature" in st.a else np.full(N, 25.0)) + 273.15
    out = np.empty((nm, N))
    for m in range(nm):
        if net.options.get("isothermal", 1) or net.mnrl_logKcoef is None:
            logK = np.full(N, net.mnrl_logK[m])
        else:
            c = net.mnrl_logKcoef[m]
            logK = c[0] * np.log(tk) + c[1] + c[2] * tk + c[3] / tk + c[4] / (tk * tk)
        lnq = -logK * LOG_TO_LN
        for k in range(net.mnrl_nspec[m]):
            lnq = lnq + net.mnrl_stoich[m, k] * la[net.mnrl_spec[m, k]]
        if net.mnrl_h2o_stoich is not None and "ln_act_h2o" in st.a:
            lnq = lnq + net.mnrl_h2o_stoich[m] * st.a["ln_act_h2o"]
        sigma = net.mnrl_Temkin_const[m] if net.mnrl_Temkin_const is not None else 1.0
        out[m] = np.exp(lnq / sigma)
    return out


def gross_rate(net, st):
    if not net.nmnrl:
        return np.zeros((0, st.ncells))
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        qk = mineral_qk(net, st)
        p = (net.mnrl_affinity_power if net.mnrl_affinity_power is not None else np.ones(net.nmnrl))[:, None]
        amp = np.where(np.abs(1.0 - qk) > 0, p * qk / np.abs(1.0 - qk), np.inf)
        g = np.abs(st.a["mnrl_rate"]) * (1.0 + amp)
    return np.where(np.isfinite(g), g, np.abs(st.a["mnrl_rate"]))


def _dt_cells(st, dt):
    return st.a["dt_cell"] if "dt_cell" in st.a else np.full(st.ncells, float(dt))


def cell_errors(net, ref, got, dt):
    """Per-quantity, per-cell maximum relative difference (dict of arrays of
    ncells) under the scales above."""
    def r(a, b, scale):
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.abs(a - b) / scale
        # equal values (including equal infinities) agree, and so do NaNs in
        # the same place (a cell the reference leaves NaN, e.g. a failed
        # activity iteration, reaction.F90:4420-4431)
        e = np.where((a == b) | (np.isnan(a) & np.isnan(b)), 0.0, e)
        return np.nan_to_num(e, nan=np.inf).reshape(-1, ref.ncells).max(axis=0)
    e = {"pri_molal": r(got.a["pri_molal"], ref.a["pri_molal"], np.abs(ref.a["pri_molal"]))}
    if net.nsec:
        e["sec_molal"] = r(got.a["sec_molal"], ref.a["sec_molal"], np.maximum(np.abs(ref.a["sec_molal"]), 1e-300))
    e["total"] = r(got.a["total"], ref.a["total"], np.maximum(gross_total(net, ref), 1e-300))
    if net.nmnrl:
        gr = np.maximum(gross_rate(net, ref), 1e-30)
        e["mnrl_rate"] = r(got.a["mnrl_rate"], ref.a["mnrl_rate"], gr)
        vs = np.abs(ref.a["mnrl_volfrac"]) + gr * net.mnrl_molar_vol[:, None] * _dt_cells(ref, dt)[None, :]
        e["mnrl_volfrac"] = r(got.a["mnrl_volfrac"], ref.a["mnrl_volfrac"], np.maximum(vs, 1e-30))
    # failed in both: status, path and the restored totals only
    failed = (ref.a["status"] != 0) & (got.a["status"] != 0)
    for k in e:
        if k != "total":
            e[k] = np.where(failed, 0.0, e[k])
    return e


def max_err(e):
    m = None
    for v in e.values():
        m = v if m is None else np.maximum(m, v)
    return m


def same_path(ref, got, its=True):
    p = (ref.a["num_substeps"] == got.a["num_substeps"]) & (ref.a["status"] == got.a["status"])
    if its:
        p &= ref.a["newton_its"] == got.a["newton_its"]
    return p


def summarise(net, ref, got, dt, its=True):
    """(path mask, per-quantity errors, per-cell max error)."""
    p = same_path(ref, got, its)
    e = cell_errors(net, ref, got, dt)
    return p, e, max_err(e)


def compare(net, ref, got, dt, label, self_runs=(), its=True):
    """Compares got with ref; self_runs: the oracle on one-ulp-perturbed
    inputs.  its=False: the path is the substep count and status only (the
    converged-tolerance runs, where the Newton count does not change the
    result beyond REL).  Returns the report entry; the caller asserts."""
    p, e, m = summarise(net, ref, got, dt, its)
    flips = ~p
    outl = p & (m >= REL)
    ok = p & ~outl
    s_flips = s_out = None
    s_flip_err = None
    if self_runs:
        sf = np.zeros(ref.ncells, bool)
        so = np.zeros(ref.ncells, bool)
        s_flip_err = 0.0
        for s in self_runs:
            sp, _, sm = summarise(net, ref, s, dt, its)
            sf |= ~sp
            so |= sp & (sm >= REL)
            if (~sp).any():
                s_flip_err = max(s_flip_err, float(sm[~sp].max()))
        s_flips, s_out = int(sf.sum()), int((so & ~sf).sum())
    sub = ref.a["num_substeps"]
    stt = ref.a["status"]
    cls = {"single": (sub == 1) & (stt == 0), "cut": (sub > 1) & (stt == 0), "failed": stt != 0}
    entry = dict(
        cells=int(ref.ncells), compared=int(p.sum()), flips=int(flips.sum()), outliers=int(outl.sum()),
        outliers_by_class={k: int((outl & v).sum()) for k, v in
                           {"single": (ref.a["num_substeps"] == 1) & (ref.a["status"] == 0),
                            "cut": (ref.a["num_substeps"] > 1) & (ref.a["status"] == 0),
                            "failed": ref.a["status"] != 0}.items()},
        oracle_self_flips=s_flips, oracle_self_outliers=s_out,
        compared_by_class={k: int((p & v).sum()) for k, v in cls.items()},
        cells_by_class={k: int(v.sum()) for k, v in cls.items()},
        max_rel_err={k: (float(v[ok].max()) if ok.any() else 0.0) for k, v in e.items()},
        max_rel_err_cut_cells=(float(m[ok & cls["cut"]].max()) if (ok & cls["cut"]).any() else None),
        flip_max_err_gpu=(float(m[flips].max()) if flips.any() else None),
        flip_max_err_oracle_self=s_flip_err,
        failed_ref=int((stt != 0).sum()), failed_gpu=int((got.a["status"] != 0).sum()),
        its_mean=float(ref.a["newton_its"].mean()) if ref.ncells else 0.0,
        its_max=int(ref.a["newton_its"].max()) if ref.ncells else 0,
        substeps_max=int(sub.max()) if ref.ncells else 0)
    REPORT[label] = entry
    return entry, ok


def check(entry, label, min_compared=0):
    """The common assertions: flips and outliers within twice the oracle's
    own one-ulp counts plus max(2, 1 %) of the cells; every compared
    quantity below REL on the non-outlier path-identical cells."""
    slack = max(2, 0.01 * entry["cells"])
    assert entry["compared"] >= min_compared, (label, entry["compared"], min_compared)
    if entry["oracle_self_flips"] is not None:
        assert entry["flips"] <= 2 * entry["oracle_self_flips"] + slack, (label, entry)
        assert entry["outliers"] <= 2 * entry["oracle_self_outliers"] + slack, (label, entry)
    for k, v in entry["max_rel_err"].items():
        assert v < REL, (label, k, v, entry)


def format_report():
    lines = ["parity report (GPU vs oracle; flips/outliers: GPU | oracle one-ulp self; errors on compared cells)"]
    for k in sorted(REPORT):
        r = REPORT[k]
        errs = " ".join("%s %.1e" % (q, v) for q, v in r["max_rel_err"].items())
        ob = r["outliers_by_class"]
        lines.append("  %-34s cells %6d compared %6d (single %d, cut %d, failed %d) flips %d|%s outliers %d|%s "
                     "(%d/%d/%d) its mean %.1f max %d | %s | flip err gpu %s oracle %s" % (
                         k, r["cells"], r["compared"], r["compared_by_class"]["single"],
                         r["compared_by_class"]["cut"], r["compared_by_class"]["failed"], r["flips"],
                         r["oracle_self_flips"], r["outliers"], r["oracle_self_outliers"], ob["single"], ob["cut"],
                         ob["failed"], r["its_mean"],
                         r["its_max"], errs,
                         "%.1e" % r["flip_max_err_gpu"] if r["flip_max_err_gpu"] is not None else "-",
                         "%.1e" % r["flip_max_err_oracle_self"] if r["flip_max_err_oracle_self"] else "-"))
    return lines
