// oracle_count.cpp -- the oracle's RStep with counted arithmetic.
//
// TEST INFRASTRUCTURE ONLY (see flop_real.hpp).  The restatement in
// rxn_oracle.hpp is compiled here with double -> Real; the C ABI struct
// definitions are included first so that they keep their plain doubles.
// oracle_count_rstep runs RStep for each cell of a state (single thread) and
// returns the flops and transcendental calls per cell together with the
// Newton iterations, so the per-iteration work of the reference algorithm
// can be compared with the analytic model (pfgpu/flops.py).
#include <cstdint>
#include <vector>

#include "../include/pfgpu.h"
#include "flop_real.hpp"

#define double Real
#include "rxn_oracle.hpp"
#undef double

using oracle::Cell;
using oracle::Net;

extern "C" {

// For every cell: flops[cell], transcendentals[cell], its[cell] of one RStep;
// the state is advanced as oracle_rstep advances it.
int oracle_count_rstep(const PfNetworkDesc* d, const PfCellState* s, double dt, int64_t* flops,
                       int64_t* transcendentals, int32_t* its) {
  if (!d || !s) return PF_ERR_INVALID;
  Net net(d);
  const int64_t N = s->ncells;
  for (int64_t i = 0; i < N; ++i) {
    Cell c{};
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
      c.mnrl_rate[k] = 0.0;
    }
    c.porosity = s->porosity[i];
    c.sat = s->saturation[i];
    c.den_kg = s->den_kg[i];
    c.volume = s->volume[i];
    c.temp = s->temperature ? s->temperature[i] : 25.0;
    c.ln_act_h2o = 0.0;
    c.ierror = 0;
    oracle::set_logK(net, c);  // per-cell logK(T): part of the cell's work
    flopcount::counters() = flopcount::Counters{};
    Real guess[oracle::MAXN];
    for (int k = 0; k < net.n; ++k) guess[k] = c.pri_molal[k];
    const double tdt = s->dt_cell ? s->dt_cell[i] : dt;
    oracle::StepResult r = oracle::rstep(net, c, guess, Real(tdt));
    flops[i] = flopcount::counters().flops;
    transcendentals[i] = flopcount::counters().transcendentals;
    its[i] = r.num_iterations;
    for (int k = 0; k < net.n; ++k) {
      s->total[k * N + i] = c.total[k].v;
      s->pri_molal[k * N + i] = c.pri_molal[k].v;
      s->pri_act_coef[k * N + i] = c.pri_act_coef[k].v;
    }
    for (int k = 0; k < net.ns; ++k) {
      s->sec_act_coef[k * N + i] = c.sec_act_coef[k].v;
      s->sec_molal[k * N + i] = c.sec_molal[k].v;
    }
    for (int k = 0; k < net.nm; ++k) {
      s->mnrl_volfrac[k * N + i] = c.mnrl_volfrac[k].v;
      s->mnrl_rate[k * N + i] = c.mnrl_rate[k].v;
    }
    if (s->status) s->status[i] = r.ierror ? PF_CELL_TOO_MANY_CUTS : PF_CELL_OK;
    if (s->newton_its) s->newton_its[i] = r.num_iterations;
    if (s->num_substeps) s->num_substeps[i] = r.num_sub_steps;
  }
  return PF_OK;
}

}  // extern "C"
