/*
 * osrt_shim.c -- what the Fortran shim does, in C, for the tests.
 *
 * PFLOTRAN keeps each cell's chemistry in derived types (rt_auxvar,
 * global_auxvar, material_auxvar; reactive_transport_aux.F90:21-74,
 * global_aux.F90:11-35, material_aux.F90:53-77), one record per cell, and
 * its operator-split loop calls RStep once per cell
 * (pmc_subsurface_osrt.F90:346-378).  The drop-in replacement gathers the
 * records into the engine's component-major arrays, makes one
 * pf_rstep_host call, and scatters the results back into the records --
 * the body of pfgpu_osrt_react in include/pfgpu_mod.F90.  This file does
 * exactly that over an array of ShimCell records (the per-cell fields the
 * step reads or writes, laid out as one record per cell), so that a GPU
 * test can drive the library the way the Fortran caller would, through the
 * C ABI alone.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pfgpu.h"

typedef struct ShimCell {
  /* rt_auxvar */
  double total[PF_MAX_NCOMP];
  double pri_molal[PF_MAX_NCOMP];
  double pri_act_coef[PF_MAX_NCOMP];
  double sec_act_coef[PF_MAX_NSEC];
  double sec_molal[PF_MAX_NSEC];
  double mnrl_volfrac[PF_MAX_NMNRL];
  double mnrl_area[PF_MAX_NMNRL];
  double mnrl_rate[PF_MAX_NMNRL];
  /* material_auxvar and global_auxvar */
  double porosity, saturation, den_kg, volume, temperature;
  /* RStep's outputs: ierror, num_iterations, num_timesteps */
  int32_t status, newton_its, num_substeps, pad;
} ShimCell;

size_t shim_cell_size(void) { return sizeof(ShimCell); }

/* byte offsets of the members, in declaration order (for the test's numpy dtype) */
size_t shim_cell_offset(int32_t k) {
  static const size_t off[] = {
      offsetof(ShimCell, total), offsetof(ShimCell, pri_molal), offsetof(ShimCell, pri_act_coef),
      offsetof(ShimCell, sec_act_coef), offsetof(ShimCell, sec_molal), offsetof(ShimCell, mnrl_volfrac),
      offsetof(ShimCell, mnrl_area), offsetof(ShimCell, mnrl_rate), offsetof(ShimCell, porosity),
      offsetof(ShimCell, saturation), offsetof(ShimCell, den_kg), offsetof(ShimCell, volume),
      offsetof(ShimCell, temperature), offsetof(ShimCell, status), offsetof(ShimCell, newton_its),
      offsetof(ShimCell, num_substeps)};
  return (k >= 0 && k < (int32_t)(sizeof(off) / sizeof(off[0]))) ? off[k] : (size_t)-1;
}

/* One operator-split reaction step over ncells records: gather, one
 * pf_rstep_host call, scatter.  *rstep_error as the reference's loop sets
 * it (1 when any cell failed), *sum_its accumulates the Newton iterations.
 * Returns the library's status, or PF_ERR_INVALID on a bad argument. */
int32_t shim_osrt_react(PfNetwork* net, ShimCell* cells, int64_t ncells, int32_t ncomp, int32_t nsec,
                        int32_t nmnrl, double dt, int32_t* rstep_error, int64_t* sum_its) {
  if (!net || (!cells && ncells) || ncells < 0 || ncomp < 1 || ncomp > PF_MAX_NCOMP || nsec < 0 ||
      nsec > PF_MAX_NSEC || nmnrl < 0 || nmnrl > PF_MAX_NMNRL || !rstep_error || !sum_its)
    return PF_ERR_INVALID;
  const size_t N = (size_t)ncells;
  /* contiguous temporaries, component-major: a[k*N + cell] */
  const size_t nd = N * (3 * (size_t)ncomp + 2 * (size_t)nsec + 3 * (size_t)nmnrl + 5);
  double* buf = (double*)malloc((nd ? nd : 1) * sizeof(double));
  int32_t* ibuf = (int32_t*)malloc((3 * N ? 3 * N : 1) * sizeof(int32_t));
  if (!buf || !ibuf) {
    free(buf);
    free(ibuf);
    return PF_ERR_INVALID;
  }
  double* p = buf;
  double* total = p; p += N * ncomp;
  double* pri = p; p += N * ncomp;
  double* pac = p; p += N * ncomp;
  double* sac = p; p += N * nsec;
  double* sm = p; p += N * nsec;
  double* vf = p; p += N * nmnrl;
  double* area = p; p += N * nmnrl;
  double* rate = p; p += N * nmnrl;
  double* por = p; p += N;
  double* sat = p; p += N;
  double* den = p; p += N;
  double* vol = p; p += N;
  double* temp = p;
  int32_t* status = ibuf;
  int32_t* its = ibuf + N;
  int32_t* nsub = ibuf + 2 * N;
  /* gather: the per-cell reads of the reference's loop (guess = pri_molal) */
  for (size_t c = 0; c < N; ++c) {
    const ShimCell* r = &cells[c];
    for (int k = 0; k < ncomp; ++k) {
      total[k * N + c] = r->total[k];
      pri[k * N + c] = r->pri_molal[k];
      pac[k * N + c] = r->pri_act_coef[k];
    }
    for (int k = 0; k < nsec; ++k) {
      sac[k * N + c] = r->sec_act_coef[k];
      sm[k * N + c] = r->sec_molal[k];
    }
    for (int k = 0; k < nmnrl; ++k) {
      vf[k * N + c] = r->mnrl_volfrac[k];
      area[k * N + c] = r->mnrl_area[k];
      rate[k * N + c] = 0.0;
    }
    por[c] = r->porosity;
    sat[c] = r->saturation;
    den[c] = r->den_kg;
    vol[c] = r->volume;
    temp[c] = r->temperature;
  }
  PfCellState st;
  memset(&st, 0, sizeof(st));
  st.ncells = ncells;
  st.total = total;
  st.pri_molal = pri;
  st.pri_act_coef = pac;
  st.sec_act_coef = nsec ? sac : NULL;
  st.sec_molal = nsec ? sm : NULL;
  st.mnrl_volfrac = nmnrl ? vf : NULL;
  st.mnrl_area = nmnrl ? area : NULL;
  st.mnrl_rate = nmnrl ? rate : NULL;
  st.porosity = por;
  st.saturation = sat;
  st.den_kg = den;
  st.volume = vol;
  st.temperature = temp;
  st.status = status;
  st.newton_its = its;
  st.num_substeps = nsub;
  PfStepStats stats;
  const int32_t rc = pf_rstep_host(net, &st, dt, PF_KERNEL_BATCHED, &stats);
  if (rc == PF_OK || rc == PF_CELL_FAILURES) {
    /* scatter: what the reference's loop leaves in the auxvars */
    for (size_t c = 0; c < N; ++c) {
      ShimCell* r = &cells[c];
      for (int k = 0; k < ncomp; ++k) {
        r->total[k] = total[k * N + c];
        r->pri_molal[k] = pri[k * N + c];
        r->pri_act_coef[k] = pac[k * N + c];
      }
      for (int k = 0; k < nsec; ++k) {
        r->sec_act_coef[k] = sac[k * N + c];
        r->sec_molal[k] = sm[k * N + c];
      }
      for (int k = 0; k < nmnrl; ++k) {
        r->mnrl_volfrac[k] = vf[k * N + c];
        r->mnrl_rate[k] = rate[k * N + c];
      }
      r->status = status[c];
      r->newton_its = its[c];
      r->num_substeps = nsub[c];
    }
    *rstep_error = stats.failed_cells > 0 ? 1 : 0;
    *sum_its += stats.newton_iterations;
  }
  free(buf);
  free(ibuf);
  return rc;
}
