// pfgpu_sorb.cuh -- equilibrium sorption of one cell, shared by the kernels.
//
// RTotalSorb (src/pflotran/reaction.F90:4783-4832) without surface
// complexation or dynamic K_D: ion exchange (RTotalSorbEqIonx, :4906-5140,
// the "#if 1" Newton on the reference cation's K_D when the cations' charges
// differ, the closed form when they are all equal) and then the K_D
// isotherms (RTotalSorbKD, reaction_isotherm.F90:273-359).
#pragma once

#include "pfgpu_common.cuh"

namespace pfgpu {

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
                           double den_kg, double* ionx_ref, int64_t ref_stride, AddS add_S, AddDS add_dS) {
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
