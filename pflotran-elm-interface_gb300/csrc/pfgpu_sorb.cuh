// pfgpu_sorb.cuh -- equilibrium sorption of one cell, shared by the kernels.
//
// RTotalSorb (src/pflotran/reaction.F90:4783-4832) without dynamic K_D:
// surface complexation (RTotalSorbEqSurfCplx1), ion exchange (RTotalSorbEqIonx, :4906-5140,
// the "#if 1" Newton on the reference cation's K_D when the cations' charges
// differ, the closed form when they are all equal) and then the K_D
// isotherms (RTotalSorbKD, reaction_isotherm.F90:273-359).
#pragma once

#include "pfgpu_common.cuh"

namespace pfgpu {

// The per-cell surface-complexation state a kernel passes to total_sorb:
// the free-site warm start and the complexes' output (one value per
// reaction / complex, `stride` apart; conc may be null), the cell's
// temperature (logK of the complexes in non-isothermal runs) and ln a_H2O.
struct SurfCell {
  double* free_site;
  double* conc;
  int64_t stride;
  double temp;
  double lnaw;
};

__device__ __forceinline__ SurfCell surf_cell(const DevNet& net, const PfCellState& st, int64_t cell) {
  SurfCell s;
  s.free_site = (net.nsrx > 0 && st.srfcplx_free_site) ? st.srfcplx_free_site + cell : nullptr;
  s.conc = (net.nsrx > 0 && st.srfcplx_conc) ? st.srfcplx_conc + cell : nullptr;
  s.stride = st.ncells;
  s.temp = st.temperature ? st.temperature[cell] : 25.0;
  s.lnaw = cell_lnaw(net, st, cell);
  return s;
}

// RTotalSorbEqSurfCplx1 (reaction_surf_complex.F90:641-900) for every
// surface complexation reaction: the free-site concentration S_x from the
// site balance (Newton on S_x when a complex holds more than one site,
// relative change 1e-12, damping 0.5 after 1000 iterations, :743-799;
// otherwise the closed form), the complexes S_k, the sorbed totals and
// their derivative with the free site's response dS_x/dm (:803-893).
template <class Mol, class Gam, class VF, class AddS, class AddDS>
__device__ void total_sorb_srfcplx(const DevNet& net, const Tables& T, Mol mol, Gam gam, VF volfrac,
                                   double porosity, const SurfCell& sc, AddS add_S, AddDS add_dS) {
  const bool tdep = !net.o.isothermal && (net.flags & NETF_SX_LOGKCOEF);
  const bool h2o = water_on(net);
  double la[PF_MAX_NCOMP];  // ln a of the primaries (:686-687)
  for (int j = 0; j < net.n; ++j) la[j] = log(mol(j)) + log(gam(j));
  for (int r = 0; r < net.nsrx; ++r) {
    const int k0 = T.sx_begin(r), k1 = T.sx_end(r);
    double site;
    if (T.sx_type(r) == PF_SURF_MINERAL) site = T.sx_dens(r) * volfrac(T.sx_min(r));
    else if (T.sx_type(r) == PF_SURF_ROCK) site = T.sx_dens(r) * net.soil_density * (1.0 - porosity);
    else site = T.sx_dens(r);
    if (sc.conc)
      for (int k = k0; k < k1; ++k) sc.conc[k * sc.stride] = 0.0;
    if (site < 1.0e-40) {  // :728-737
      if (sc.free_site) sc.free_site[r * sc.stride] = 0.0;
      continue;
    }
    double S[PF_MAX_NSRFCPLX];
    double free_site = fmax(sc.free_site ? sc.free_site[r * sc.stride] : 1.0e-9, 1.0e-40);
    bool one_more = false;
    int its = 0;
    double damping = 1.0;
    for (;;) {
      its = its + 1;
      double total = free_site;
      const double ln_free = log(free_site);
      for (int k = k0; k < k1; ++k) {
        double lnQK = -(tdep ? interp_logK(T.sx_logKcoef(k), sc.temp) : T.sx_logK(k)) * LOG_TO_LN;
        if (h2o) lnQK = add_h2o(lnQK, T.sx_h2o(k), sc.lnaw);
        lnQK = lnQK + T.sx_nuf(k) * ln_free;
        for (int p = T.sx_cbegin(k); p < T.sx_cend(k); ++p) {
          const int j = T.sx_spec(p);
          lnQK = lnQK + T.sx_nu(p) * la[j];
        }
        S[k - k0] = exp(lnQK);
        total = total + T.sx_nuf(k) * S[k - k0];
      }
      if (one_more) break;
      if (T.sx_flag(r)) {
        const double res = site - total;
        double dres = 1.0;
        for (int k = k0; k < k1; ++k) dres = dres + T.sx_nuf(k) * S[k - k0] / free_site;
        const double dfree = res / dres;
        if (its > 1000) damping = 0.5;
        free_site = free_site + damping * dfree;
        if (fabs(dfree / free_site) < 1.0e-12) one_more = true;
      } else {
        total = total / free_site;
        free_site = site / total;
        one_more = true;
      }
    }
    if (sc.free_site) sc.free_site[r * sc.stride] = free_site;
    if (sc.conc)
      for (int k = k0; k < k1; ++k) sc.conc[k * sc.stride] = S[k - k0];
    // dS_x/dm_j (:803-824), in registers
    double dSx[PF_MAX_NCOMP];
    for (int j = 0; j < net.n; ++j) dSx[j] = 0.0;
    double den = 0.0;
    for (int k = k0; k < k1; ++k) {
      for (int p = T.sx_cbegin(k); p < T.sx_cend(k); ++p)
        dSx[T.sx_spec(p)] = dSx[T.sx_spec(p)] + T.sx_nu(p) * T.sx_nuf(k) * S[k - k0];
      den = den + T.sx_nuf(k) * T.sx_nuf(k) * S[k - k0];
    }
    den = den / free_site;
    den = den + 1.0;
    for (int j = 0; j < net.n; ++j) dSx[j] = (-dSx[j] / den) / mol(j);
    // sorbed totals and derivative (:846-893)
    for (int k = k0; k < k1; ++k) {
      const int p0 = T.sx_cbegin(k), p1 = T.sx_cend(k);
      for (int p = p0; p < p1; ++p) add_S(T.sx_spec(p), T.sx_nu(p) * S[k - k0]);
      const double nui_Si_over_Sx = T.sx_nuf(k) * S[k - k0] / free_site;
      for (int q = p0; q < p1; ++q) {
        const int jc = T.sx_spec(q);
        const double t = T.sx_nu(q) * S[k - k0] / mol(jc) + nui_Si_over_Sx * dSx[jc];
        for (int p = p0; p < p1; ++p) add_dS(T.sx_spec(p), jc, T.sx_nu(p) * t);
      }
    }
  }
}

// Inputs come through callables so that each kernel keeps its own storage:
// mol(j) and gam(j) (molality and activity coefficient of primary j),
// volfrac(m) (kinetic-mineral volume fraction).  ionx_ref points at the
// cell's first warm-start value (eqionx_ref_cation_sorbed_conc), one per
// ion-exchange reaction ref_stride apart; it is updated in place as the
// reference updates rt_auxvar.  Results go to add_S(j, v) (total_sorb_eq,
// mol/m^3 bulk) and add_dS(i, j, v) (dtotal_sorb_eq(i,j), kg water/m^3
// bulk).  Returns false when the ion-exchange Newton passes 20000
// iterations (the reference's ierror, :4981-4986).
template <class Mol, class Gam, class VF, class AddS, class AddDS>
__device__ bool total_sorb(const DevNet& net, const Tables& T, Mol mol, Gam gam, VF volfrac, double porosity,
                           double den_kg, double* ionx_ref, int64_t ref_stride, AddS add_S, AddDS add_dS,
                           const SurfCell& sc) {
  if (net.nsrx > 0) total_sorb_srfcplx(net, T, mol, gam, volfrac, porosity, sc, add_S, add_dS);
  for (int r = 0; r < net.nionx; ++r) {
    const int b = T.ix_begin(r), nc = T.ix_end(r) - b;
    const int mi = T.ix_min(r);
    const double omega = mi >= 0 ? fmax(T.ix_cec(r) * volfrac(mi), 1.0e-40) : T.ix_cec(r);
    double X[PF_MAX_IONX_CATIONS];
    if (T.ix_zflag(r)) {
      const int ic = T.ix_cat(b);
      const double ref_conc = mol(ic) * gam(ic);
      const double ref_Z = T.pri_Z(ic);
      const double ref_k = T.ix_k(b);
      double ref_X = ref_Z * ionx_ref[r * ref_stride] / omega;
      bool one_more = false;
      double KDj = ref_X / (ref_k * ref_conc);
      int it = 0;
      for (;;) {
        it = it + 1;
        if (it > 20000) return false;
        ref_X = KDj * (ref_k * ref_conc);
        X[0] = ref_X;
        double total = ref_X, dres = 0.0;
        for (int j = 1; j < nc; ++j) {
          const int jc = T.ix_cat(b + j);
          X[j] = T.ix_k(b + j) * mol(jc) * gam(jc) * pow(KDj, T.pri_Z(jc) / ref_Z);
          total = total + X[j];
          dres = dres + X[j] / KDj * T.pri_Z(jc);
        }
        dres = dres / ref_Z + (ref_k * ref_conc);
        const double res = 1.0 - total;
        if (one_more) break;
        const double delta = res / dres;
        KDj = KDj + delta;
        KDj = fmax(KDj, 1.0e-40);
        if (fabs(delta / KDj) < 1.0e-12) one_more = true;
      }
      ionx_ref[r * ref_stride] = ref_X * omega / ref_Z;
    } else {
      double sumkm = 0.0;
      for (int j = 0; j < nc; ++j) {
        const int jc = T.ix_cat(b + j);
        X[j] = mol(jc) * gam(jc) * T.ix_k(b + j);
        sumkm = sumkm + X[j];
      }
      for (int j = 0; j < nc; ++j) X[j] = X[j] / sumkm;
    }
    double sumZX = 0.0;
    for (int i = 0; i < nc; ++i) sumZX = sumZX + T.pri_Z(T.ix_cat(b + i)) * X[i];
    for (int i = 0; i < nc; ++i) {
      const int ic = T.ix_cat(b + i);
      const double t1 = X[i] * omega / T.pri_Z(ic);
      add_S(ic, t1);
      const double t2 = T.pri_Z(ic) / sumZX;
      for (int j = 0; j < nc; ++j) {
        const int jc = T.ix_cat(b + j);
        add_dS(ic, jc, i == j ? t1 * (1.0 - (t2 * X[j])) / mol(jc) : (-t1) * t2 * X[j] / mol(jc));
      }
    }
  }
  for (int r = 0; r < net.nkd; ++r) {
    const int ic = T.kd_spec(r);
    const double m = mol(ic);
    double kd = net.kd_units == PF_KD_UNIT_MLW_GSOIL
                    ? T.kd_coeff(r) * den_kg * (1.0 - porosity) * net.soil_density * 1.0e-3
                    : T.kd_coeff(r);
    const int mi = T.kd_min(r);
    if (mi >= 0) kd = kd * volfrac(mi);
    double res = 0.0, dres = 0.0;
    const int ty = T.kd_type(r);
    if (ty == PF_SORPTION_LINEAR) {
      res = kd * m;
      dres = kd;
    } else if (ty == PF_SORPTION_LANGMUIR) {
      const double t = kd * m;
      res = t * T.kd_b(r) / (1.0 + t);
      dres = res / m - res / (1.0 + t) * t / m;
    } else if (ty == PF_SORPTION_FREUNDLICH) {
      const double on = 1.0 / T.kd_n(r);
      res = kd * pow(m, on);
      dres = res / m * on;
    }
    add_S(ic, res);
    add_dS(ic, ic, dres);
  }
  return true;
}

}  // namespace pfgpu
