// oracle_capi.cpp -- C entry points of the CPU oracle (TEST INFRASTRUCTURE).
//
// Wraps the restatement in rxn_oracle.hpp for ctypes: each entry point takes
// the same PfNetworkDesc / PfCellState (host pointers, SoA layout
// value(k,cell) = a[k*ncells+cell]) as the GPU library, loops over cells
// (OpenMP when nthreads > 1) and writes results back in place.
#include "rxn_oracle.hpp"

#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace oracle;

namespace {

inline void gather(const Net& net, const PfCellState* s, int64_t i, Cell& c) {
  const int64_t N = s->ncells;
  for (int k = 0; k < net.n; ++k) {
    c.total[k] = s->total[k * N + i];
    c.pri_molal[k] = s->pri_molal[k * N + i];
    c.pri_act_coef[k] = s->pri_act_coef[k * N + i];
  }
  for (int k = 0; k < net.ns; ++k) {
    c.sec_act_coef[k] = s->sec_act_coef[k * N + i];
    c.sec_molal[k] = s->sec_molal[k * N + i];
  }
  for (int k = 0; k < net.nm; ++k) {
    c.mnrl_volfrac[k] = s->mnrl_volfrac[k * N + i];
    c.mnrl_area[k] = s->mnrl_area[k * N + i];
    c.mnrl_rate[k] = s->mnrl_rate[k * N + i];
  }
  c.porosity = s->porosity[i];
  c.sat = s->saturation[i];
  c.den_kg = s->den_kg[i];
  c.volume = s->volume[i];
  c.temp = s->temperature ? s->temperature[i] : 25.0;
  // rt_auxvar%ln_act_h2o: RTAuxVarInit's 0 unless the water activity option
  // computes it
  c.ln_act_h2o = (net.o.use_activity_h2o && s->ln_act_h2o) ? s->ln_act_h2o[i] : 0.0;
  c.ierror = 0;
  for (int k = 0; k < net.n; ++k) c.total_sorb[k] = s->total_sorb ? s->total_sorb[k * N + i] : 0.0;
  const int nionx = net.sorb ? net.sorb->nionx : 0;
  for (int k = 0; k < nionx; ++k) c.ionx_ref[k] = s->ionx_ref_sorbed ? s->ionx_ref_sorbed[k * N + i] : 1.0e-9;
  const int nsrx = net.sorb ? net.sorb->nsrfcplx_rxn : 0, nsc = net.sorb ? net.sorb->nsrfcplx : 0;
  for (int k = 0; k < nsrx; ++k) c.srf_free[k] = s->srfcplx_free_site ? s->srfcplx_free_site[k * N + i] : 1.0e-9;
  for (int k = 0; k < nsc; ++k) c.srf_conc[k] = s->srfcplx_conc ? s->srfcplx_conc[k * N + i] : 0.0;
  set_logK(net, c);
}

inline void scatter(const Net& net, const PfCellState* s, int64_t i, const Cell& c) {
  const int64_t N = s->ncells;
  for (int k = 0; k < net.n; ++k) {
    s->total[k * N + i] = c.total[k];
    s->pri_molal[k * N + i] = c.pri_molal[k];
    s->pri_act_coef[k * N + i] = c.pri_act_coef[k];
  }
  for (int k = 0; k < net.ns; ++k) {
    s->sec_act_coef[k * N + i] = c.sec_act_coef[k];
    s->sec_molal[k * N + i] = c.sec_molal[k];
  }
  for (int k = 0; k < net.nm; ++k) {
    s->mnrl_volfrac[k * N + i] = c.mnrl_volfrac[k];
    s->mnrl_area[k * N + i] = c.mnrl_area[k];
    s->mnrl_rate[k * N + i] = c.mnrl_rate[k];
  }
  if (s->total_sorb)
    for (int k = 0; k < net.n; ++k) s->total_sorb[k * N + i] = c.total_sorb[k];
  if (s->ionx_ref_sorbed && net.sorb)
    for (int k = 0; k < net.sorb->nionx; ++k) s->ionx_ref_sorbed[k * N + i] = c.ionx_ref[k];
  if (s->ln_act_h2o) s->ln_act_h2o[i] = c.ln_act_h2o;
  if (s->srfcplx_free_site && net.sorb)
    for (int k = 0; k < net.sorb->nsrfcplx_rxn; ++k) s->srfcplx_free_site[k * N + i] = c.srf_free[k];
  if (s->srfcplx_conc && net.sorb)
    for (int k = 0; k < net.sorb->nsrfcplx; ++k) s->srfcplx_conc[k * N + i] = c.srf_conc[k];
}

// Rate prefactors: counts and ids in range; a primary prefactor species that
// follows a secondary one in the same mineral may not see a count above the
// mineral's own (the reference would read past the mineral's species list).
int check_prefactors(const PfNetworkDesc* d) {
  const PfPrefactorDesc* pf = d->prefactors;
  if (!pf) return PF_OK;
  if (!pf->num_prefactors || !pf->rate || !pf->activation_energy || !pf->nspec || !pf->spec || !pf->alpha ||
      !pf->beta || !pf->atten_coef)
    return PF_ERR_INVALID;
  for (int m = 0; m < d->nmnrl; ++m) {
    const int np = pf->num_prefactors[m];
    if (np < 0 || np > PF_MAX_PREFACTORS) return PF_ERR_INVALID;
    int cnt = d->mnrl_nspec[m];
    for (int p = 0; p < np; ++p) {
      const int ns = pf->nspec[m * PF_MAX_PREFACTORS + p];
      if (ns < 0 || ns > PF_MAX_PREFACTOR_SPECIES) return PF_ERR_INVALID;
      for (int k = 0; k < ns; ++k) {
        const int id = pf->spec[(m * PF_MAX_PREFACTORS + p) * PF_MAX_PREFACTOR_SPECIES + k];
        if (id >= d->ncomp || -id - 1 >= d->nsec) return PF_ERR_INVALID;
        if (id < 0) cnt = d->sec_nspec[-id - 1];
        else if (cnt > d->mnrl_nspec[m]) return PF_ERR_UNSUPPORTED;
      }
    }
  }
  return PF_OK;
}

int check(const PfNetworkDesc* d, const PfCellState* s) {
  if (!d || !s) return PF_ERR_INVALID;
  if (d->ncomp < 1 || d->ncomp > MAXN || d->nsec < 0 || d->nsec > MAXS || d->nmnrl < 0 ||
      d->nmnrl > MAXM)
    return PF_ERR_TOO_LARGE;
  return check_prefactors(d);
}

template <class F>
void for_cells(int64_t n, int nthreads, F&& f) {
#ifdef _OPENMP
  if (nthreads > 1) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
#endif
  (void)nthreads;
  for (int64_t i = 0; i < n; ++i) f(i);
}

}  // namespace

extern "C" {

// RStep for every cell (the pmc_subsurface_osrt.F90:349-378 loop body).
int oracle_rstep(const PfNetworkDesc* d, const PfCellState* s, double dt, int nthreads) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  int64_t failed = 0;
  for_cells(s->ncells, nthreads, [&](int64_t i) {
    Cell c;
    gather(net, s, i, c);
    double guess[MAXN];
    for (int k = 0; k < net.n; ++k) guess[k] = c.pri_molal[k];
    double dti = s->dt_cell ? s->dt_cell[i] : dt;
    StepResult r = rstep(net, c, guess, dti);
    scatter(net, s, i, c);
    if (s->status) s->status[i] = r.ierror ? PF_CELL_TOO_MANY_CUTS : PF_CELL_OK;
    if (s->newton_its) s->newton_its[i] = r.num_iterations;
    if (s->num_substeps) s->num_substeps[i] = r.num_sub_steps;
    if (r.ierror) {
#ifdef _OPENMP
#pragma omp atomic
#endif
      failed++;
    }
  });
  return failed ? PF_CELL_FAILURES : PF_OK;
}

// RReact alone (no flooring, no sub-stepping): one implicit step solved from
// guess = pri_molal.  Used to emulate a converged single-cell implicit step.
int oracle_rreact(const PfNetworkDesc* d, const PfCellState* s, double dt, int nthreads) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  int64_t failed = 0;
  for_cells(s->ncells, nthreads, [&](int64_t i) {
    Cell c;
    gather(net, s, i, c);
    double guess[MAXN];
    for (int k = 0; k < net.n; ++k) guess[k] = c.pri_molal[k];
    int its = 0;
    int ierr = rreact(net, c, guess, dt, &its);
    scatter(net, s, i, c);
    if (s->status) s->status[i] = ierr;
    if (s->newton_its) s->newton_its[i] = its;
    if (ierr) {
#ifdef _OPENMP
#pragma omp atomic
#endif
      failed++;
    }
  });
  return failed ? PF_CELL_FAILURES : PF_OK;
}

// implicit_step for every cell (the converged single-cell GIRT step).
int oracle_implicit_step(const PfNetworkDesc* d, const PfCellState* s, double dt, double rel_tol,
                         int max_its) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  int failed = 0;
  for (int64_t i = 0; i < s->ncells; ++i) {
    Cell c;
    gather(net, s, i, c);
    int its = 0;
    int ierr = implicit_step(net, c, dt, rel_tol, max_its, &its);
    scatter(net, s, i, c);
    if (s->status) s->status[i] = ierr;
    if (s->newton_its) s->newton_its[i] = its;
    failed += ierr;
  }
  return failed ? PF_CELL_FAILURES : PF_OK;
}

int oracle_update_kinetic_state(const PfNetworkDesc* d, const PfCellState* s, double dt) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  for (int64_t i = 0; i < s->ncells; ++i) {
    Cell c;
    gather(net, s, i, c);
    update_kinetic_state(net, c, dt);
    scatter(net, s, i, c);
  }
  return PF_OK;
}

// RTUpdateAuxVars for cells (reactive_transport.F90:3625-3660).
int oracle_update_auxvars(const PfNetworkDesc* d, const PfCellState* s, int update_act, int nthreads) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  for_cells(s->ncells, nthreads, [&](int64_t i) {
    Cell c;
    gather(net, s, i, c);
    if (update_act) activity_coefficients(net, c);
    total(net, c);
    scatter(net, s, i, c);
  });
  return PF_OK;
}

// RTUpdateActivityCoefficients for cells (reactive_transport.F90:3441-3521).
int oracle_update_activity_coefs(const PfNetworkDesc* d, const PfCellState* s, int nthreads) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  for_cells(s->ncells, nthreads, [&](int64_t i) {
    Cell c;
    gather(net, s, i, c);
    activity_coefficients(net, c);
    scatter(net, s, i, c);
  });
  return PF_OK;
}

// ReactionEquilibrateConstraint subset for every cell; ctype[ncomp] shared,
// cconc[k*ncells+i] per cell.  iterations[i] = count or -1 on failure.
int oracle_equilibrate(const PfNetworkDesc* d, const PfCellState* s, const int32_t* ctype,
                       const PfConstraintReaction* creact, const double* cconc, int use_prev_soln_as_guess,
                       int32_t* iterations, int nthreads) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  int64_t failed = 0;
  const int64_t N = s->ncells;
  for_cells(N, nthreads, [&](int64_t i) {
    Cell c;
    gather(net, s, i, c);
    int ct[MAXN];
    double cc[MAXN];
    for (int k = 0; k < net.n; ++k) { ct[k] = ctype[k]; cc[k] = cconc[k * N + i]; }
    int its = equilibrate_constraint(net, c, ct, cc, use_prev_soln_as_guess != 0, creact);
    scatter(net, s, i, c);
    if (iterations) iterations[i] = its;
    if (its < 0) {
#ifdef _OPENMP
#pragma omp atomic
#endif
      failed++;
    }
  });
  return failed ? PF_CELL_FAILURES : PF_OK;
}

double oracle_ifc67_density(double t, double p) { return ifc67_density(t, p); }

// Global-implicit residual + BAIJ Jacobian of a structured grid (see
// girt_assemble).  grid_i = {nx, ny, nz}, grid_d = {dx, dy, dz, D_m,
// tortuosity, dispersivity}.
int oracle_girt_assemble(const PfNetworkDesc* d, const PfCellState* s, const int32_t* grid_i,
                         const double* grid_d, const double* qx, const double* qy, const double* qz,
                         const double* fixed_total, const double* fixed_sorb, double dt,
                         const int32_t* rowptr, const int32_t* colidx, double* r, double* values,
                         int numerical_derivatives) {
  int rc = check(d, s);
  if (rc) return rc;
  Net net(d);
  GirtGrid g{grid_i[0], grid_i[1], grid_i[2], grid_d[0], grid_d[1], grid_d[2], qx, qy, qz,
             grid_d[3], grid_d[4], grid_d[5]};
  const int64_t N = s->ncells;
  if ((int64_t)g.nx * g.ny * g.nz != N) return PF_ERR_INVALID;
  if (net.sorb && !fixed_sorb) return PF_ERR_INVALID;
  std::vector<Cell> cells(N);
  for (int64_t i = 0; i < N; ++i) gather(net, s, i, cells[i]);
  std::vector<int> rp(N + 1), ci(rowptr[N]);
  for (int64_t i = 0; i <= N; ++i) rp[i] = rowptr[i];
  for (int64_t b = 0; b < rowptr[N]; ++b) ci[b] = colidx[b];
  girt_assemble(net, cells.data(), g, fixed_total, fixed_sorb, dt, rp.data(), ci.data(), r, values,
                numerical_derivatives != 0);
  for (int64_t i = 0; i < N; ++i) scatter(net, s, i, cells[i]);
  return PF_OK;
}

// Operator-split transport matrix on a structured grid (see
// transport_matrix); grid_i = {nx, ny, nz}, grid_d = {dx, dy, dz, D_m,
// tortuosity, dispersivity}; porosity/saturation/volume per cell.
int oracle_transport_matrix(const int32_t* grid_i, const double* grid_d, const double* qx, const double* qy,
                            const double* qz, const double* porosity, const double* saturation,
                            const double* volume, double dt, const int32_t* rowptr, const int32_t* colidx,
                            double* values) {
  GirtGrid g{grid_i[0], grid_i[1], grid_i[2], grid_d[0], grid_d[1], grid_d[2], qx, qy, qz,
             grid_d[3], grid_d[4], grid_d[5]};
  const int64_t N = (int64_t)g.nx * g.ny * g.nz;
  std::vector<Cell> cells(N);
  for (int64_t i = 0; i < N; ++i) {
    cells[i].porosity = porosity[i];
    cells[i].sat = saturation[i];
    cells[i].volume = volume[i];
  }
  std::vector<int> rp(N + 1), ci(rowptr[N]);
  for (int64_t i = 0; i <= N; ++i) rp[i] = rowptr[i];
  for (int64_t b = 0; b < rowptr[N]; ++b) ci[b] = colidx[b];
  transport_matrix(cells.data(), g, dt, rp.data(), ci.data(), values);
  return PF_OK;
}

// Boundary and source terms of the operator-split transport system (see
// transport_bc_terms): bc_type[6], bc_q / bc_total as 6 pointers each (NULL
// where a face has none), bc_sat[6]; sources as arrays of nsrc; outputs
// diag_add[N] and rhs_add[ncomp][N].
int oracle_transport_bc_terms(const int32_t* grid_i, const double* grid_d, const double* porosity,
                              const double* saturation, const double* volume, int32_t ncomp, const int32_t* bc_type,
                              const double* const* bc_q, const double* const* bc_total, const double* bc_sat,
                              int32_t nsrc, const int32_t* src_cell, const int32_t* src_type, const double* src_q,
                              const double* src_total, double* diag_add, double* rhs_add) {
  GirtGrid g{grid_i[0], grid_i[1], grid_i[2], grid_d[0], grid_d[1], grid_d[2], nullptr, nullptr, nullptr,
             grid_d[3], grid_d[4], grid_d[5]};
  const int64_t N = (int64_t)g.nx * g.ny * g.nz;
  std::vector<Cell> cells(N);
  for (int64_t i = 0; i < N; ++i) {
    cells[i].porosity = porosity[i];
    cells[i].sat = saturation[i];
    cells[i].volume = volume[i];
  }
  TransportBC bc{};
  for (int f = 0; f < 6; ++f) {
    bc.type[f] = bc_type[f];
    bc.q[f] = bc_q[f];
    bc.total[f] = bc_total[f];
    bc.sat[f] = bc_sat[f];
    if (bc.type[f] != 0 && !bc.total[f]) return PF_ERR_INVALID;
  }
  TransportSrc src{nsrc, src_cell, src_type, src_q, src_total};
  for (int s = 0; s < nsrc; ++s)
    if (src_cell[s] < 0 || src_cell[s] >= N) return PF_ERR_INVALID;
  transport_bc_terms(cells.data(), g, ncomp, bc, src, diag_add, rhs_add);
  return PF_OK;
}

}  // extern "C"
