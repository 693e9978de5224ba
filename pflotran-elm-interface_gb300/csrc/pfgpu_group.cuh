// pfgpu_group.cuh -- the group-per-cell step kernel template (see
// pfgpu_group.cu for the design); instantiated per group size in
// pfgpu_group_g{2,4,8}.cu.
#pragma once
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"
#include "pfgpu_prefactor.cuh"
#include "pfgpu_sorb.cuh"

namespace pfgpu {
namespace group {

constexpr unsigned FULL = 0xffffffffu;
constexpr long long TMA_WAIT_LIMIT = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

enum Phase : int { NEED = 0, START = 1, ITER = 2, DONE = 3, BACK = 4 };

// per-cell workspace (doubles): J n*n | power table 4n | s ns | Ksec' ns |
// Kmin' nm | volfrac nm | rate nm | Im nm | dIm/dlnQ nm | x n |
// pivot scales n | rhs n; the adjoint adds Tbar n | lambda n | nu.Tbar nm |
// area gradient nm; then ints: pivot order n | remaining rows n
// The size is padded to G (mod 16) doubles: shared memory serves a warp's
// 8-byte accesses 16 lanes at a time, and the groups of a half-warp then
// start G bank pairs apart, so G consecutive doubles per group (the
// column-split rank-1 update) never collide.
__host__ __device__ inline int ws_doubles(const DevNet& net, bool adj, int G) {
  const int base = net.n * net.n + 7 * net.n + 2 * net.ns + 5 * net.nm + (adj ? 2 * net.n + 2 * net.nm : 0);
  const int g = G % 16;
  return base + ((g - base % 16) + 16) % 16;
}

__device__ __forceinline__ double dh_ln_gamma(double z, double a0, double sI, double I, const DevNet& net) {
  return fabs(z) > 1.0e-10 ? (-z * z * sI * net.A / (1.0 + a0 * net.B * sI) + net.Bdot * I) * LOG_TO_LN : 0.0;
}

template <int G>
__device__ __forceinline__ double gsum(double v, unsigned mask) {
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off, G);
  return v;
}
template <int G>
__device__ __forceinline__ unsigned long long gmax(unsigned long long v, unsigned mask) {
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(mask, v, off, G);
    v = o > v ? o : v;
  }
  return v;
}

// Staging of a network's tables into the block's shared memory: one bulk
// TMA copy of each packed block (the prefixes the group kernel reads), on an
// mbarrier whose phase `parity` completes the copy; a bounded wait (never a
// hang): on a timeout the launch-level error flag is set and every thread of
// the block returns false together.  `init` initialises the barrier (the
// first staging of a launch); a later staging into the same memory must
// follow a __syncthreads() after the last reads of the previous tables.
__device__ __forceinline__ bool stage_tables(const DevNet& net, unsigned char* smem, uint64_t* bar, uint32_t parity,
                                             bool init, unsigned long long* counters) {
  const int tid = threadIdx.x;
  const uint32_t ibytes = (uint32_t)(net.ent_staged ? net.int_words_grp : net.int_words_core) * 4u;
  const uint32_t dbytes = (uint32_t)(net.ent_staged ? net.dbl_words_grp : net.dbl_words_core) * 8u;
  int32_t* sI = reinterpret_cast<int32_t*>(smem);
  double* sD = reinterpret_cast<double*>(smem + ibytes);
  if (init) {
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
  }
  if (tid == 0) {
    // the block's earlier generic-proxy accesses to this memory come before
    // the async-proxy writes of the copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(ibytes + dbytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sI)),
                 "l"(net.ints), "r"(ibytes), "r"(smem_u32(bar))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sD)),
                 "l"(net.dbls), "r"(dbytes), "r"(smem_u32(bar))
                 : "memory");
  }
  uint32_t done = 0;
  long long spins = 0;
  while (!done && spins < TMA_WAIT_LIMIT) {
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    ++spins;
  }
  if (__syncthreads_or(!done)) {
    if (tid == 0) atomicOr(&counters[2], 1ull);
    return false;
  }
  return true;
}

// Equilibrium sorption of one cell inside a group's evaluation (RTotalSorb
// in RTAuxVarCompute with RAccumulationSorb[Derivative], reaction.F90:
// 3861-3865, 3904-3909), run by one lane of the group: the sorbed totals to
// the state and, times V/dt, to the residual rhs[] and the full rows of the
// log-form Jacobian J (column j scaled by m_j).  m[], gam[]: molalities and
// activity coefficients by species; vf[]: mineral volume fractions.  Out of
// line so that networks without sorption keep the kernel's registers.
// Returns false when the ion-exchange Newton fails (the reference's ierror).
__device__ __forceinline__ bool group_sorb(const DevNet& net, const Tables& T, const PfCellState& st, long long cell,
                                        const double* m, const double* gam, const double* vf, double den_k,
                                        double v_t, double* J, double* rhs) {
  const SoA soa{st.ncells};
  const int n = net.n;
  for (int j = 0; j < n; ++j) st.total_sorb[soa.at(j, cell)] = 0.0;
  return total_sorb(
      net, T, [&](int j) { return m[j]; }, [&](int j) { return gam[j]; }, [&](int k) { return vf[k]; },
      st.porosity[cell], den_k, st.ionx_ref_sorbed ? st.ionx_ref_sorbed + cell : nullptr, st.ncells,
      [&](int j, double v) {
        st.total_sorb[soa.at(j, cell)] += v;
        rhs[j] = fma(v_t, v, rhs[j]);
      },
      [&](int i, int j, double v) { J[i * n + j] = fma(v_t * v, m[j], J[i * n + j]); }, surf_cell(net, st, cell));
}

// Kinetic-mineral rate prefactors (RKineticMineral, reaction_mineral.F90:
// 820-858, derivative 976-1070) inside a group's evaluation, out of line so
// that networks without them keep the kernel's registers.  TG: the network's
// tables in global memory (the prefactor tables are not among the staged
// ones); a[], sv[]: activities and complexes' molalities by species.
static __device__ __noinline__ double group_pref_rate(const Tables& TG, const PfCellState& st, long long cell, int m,
                                               const double* a, const double* sv, double temp) {
  const SoA soa{st.ncells};
  double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
  return prefactor_rate(
      TG, m, [&](int j) { return log(a[j]); },
      [&](int i) { return log(sv[i]) + log(st.sec_act_coef[soa.at(i, cell)]); }, temp, pref, lnps);
}

// The prefactor part of the log-form Jacobian of every active mineral with
// prefactors, added to the full rows J (column j scaled by m_j), by one lane
// of the group.  m[], gam[]: molalities and activity coefficients by
// species; Ks[]: the complexes' K/gamma of the set-up pre-pass; Im[]: the
// minerals' volume-scaled rates of this evaluation (0: inactive).
static __device__ __noinline__ void group_pref_jacobian(const DevNet& net, const Tables& TG, const PfCellState& st,
                                                 long long cell, const double* a, const double* sv,
                                                 const double* m, const double* gam, const double* Ks,
                                                 const double* Im, double temp, double* J) {
  const SoA soa{st.ncells};
  const int n = net.n;
  auto ln_act = [&](int j) { return log(a[j]); };
  auto ln_sec_act = [&](int i) { return log(sv[i]) + log(st.sec_act_coef[soa.at(i, cell)]); };
  for (int k = 0; k < net.nm; ++k) {
    if (TG.pf_cnt(k) == 0 || Im[k] == 0.0) continue;
    double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
    const double sum = prefactor_rate(TG, k, ln_act, ln_sec_act, temp, pref, lnps);
    prefactor_derivative(
        TG, k, Im[k], sum, pref, lnps, ln_act, ln_sec_act, [&](int j) { return gam[j]; },
        [&](int i) { return st.sec_act_coef[soa.at(i, cell)]; }, [&](int j) { return log(m[j]); },
        [&](int i) { return log(Ks[i]) + log(st.sec_act_coef[soa.at(i, cell)]); }, temp,
        [&](int r, int c, double v) { J[r * n + c] = fma(v, m[c], J[r * n + c]); });
  }
}

// The step for the cells of one network's work queue, by the block's warps,
// with the network's tables already staged at the start of smem.  A warp
// returns when the queue is empty and its cells are done.
template <int G, int R, bool ADJ>
__device__ __forceinline__ void group_body(const DevNet& net, const GroupTabs& gt, const PfCellState& st,
                                           double dt_uniform, const double* __restrict__ scratch,
                                           unsigned long long* queue, unsigned long long* counters,
                                           const PfAdjointArgs& adj, double* __restrict__ adj_store,
                                           unsigned char* smem, int threads, int adj_pass = 0) {
  const int tid = threadIdx.x;
  const int lane_id = tid & 31;
  const uint32_t ibytes = (uint32_t)(net.ent_staged ? net.int_words_grp : net.int_words_core) * 4u;
  const uint32_t dbytes = (uint32_t)(net.ent_staged ? net.dbl_words_grp : net.dbl_words_core) * 8u;
  const int32_t* sI = reinterpret_cast<const int32_t*>(smem);
  const double* sD = reinterpret_cast<const double*>(smem + ibytes);
  const Tables T{sI, sD, &net};

  const int n = net.n, ns = net.ns, nm = net.nm;
  const int gi = lane_id / G, r = lane_id % G;
  const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << (gi * G));
  const int cells_per_block = threads / G;  // the threads taking part (whole warps)
  const int slot = tid / G;
  const int WS = ws_doubles(net, ADJ, G);
  double* wsbase = reinterpret_cast<double*>(smem + ibytes + dbytes);
  double* J = wsbase + (size_t)slot * WS;
  double* pw = J + n * n;
  double* sv = pw + 4 * n;
  double* Ks = sv + ns;
  double* Km = Ks + ns;
  double* vfm = Km + nm;
  double* ratem = vfm + nm;
  double* mIm = ratem + nm;
  double* mf = mIm + nm;
  double* xs = mf + nm;
  double* vvs = xs + n;      // implicit-pivot scales, then 1/pivot
  double* rhsv = vvs + n;    // residual / right-hand side, eliminated in place
  double* tb = rhsv + n;     // ADJ: Tbar of every species
  double* lamv = tb + n;     // ADJ: lambda of every species
  double* nuT = lamv + n;    // ADJ: nu_m . Tbar per mineral
  double* garea = nuT + nm;  // ADJ: dL/dln area of this cell per mineral
  int* piv = reinterpret_cast<int*>(wsbase + (size_t)cells_per_block * WS) + slot * 2 * n;
  int* rows = piv + n;

  const SoA soa{st.ncells};
  const PfOptions o = net.o;
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  const bool newton_iter_act = o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER;
  const bool has_sorb = !ADJ && has_sorption(net);  // the adjoint refuses sorption
  const bool has_pf = !ADJ && (net.flags & NETF_PREFACTOR);  // and rate prefactors
  const Tables TG{net.ints, net.dbls, &net};
  const unsigned neg_mask = (unsigned)net.neg_mask;
  const int64_t ncells = st.ncells;
  const double* sc_sec = scratch;
  const double* sc_min = scratch + (size_t)ns * ncells;
  const double* sc_lnc = scratch + (size_t)(ns + nm) * ncells;

  // group state (identical in every lane of the group)
  int phase = NEED;
  long long cell = -1;
  double psv = 0, den_L = 0, den_k = 0, volume = 0, target = 0, cum = 0, dt = 0, inv_dt = 0, r0 = 0;
  double sqI = 0.0, lgI = 0.0;
  bool dry = false, zero_step = false;
  // factorisation: LDL^T of the symmetric positive definite log-form
  // Jacobian; the pivoted LU on the rare trip where a pivot of LDL^T is not
  // positive (the evaluation is then redone, its count unchanged), and
  // always when activity coefficients follow each Newton iteration (a redone
  // evaluation would see this evaluation's complexes)
  bool use_lu = false, redo = false;
  int its = 0, its_total = 0, nsub = 0, num_cuts = 0, n_const = 0;
  // own species / rows i = r + G*t
  double c[R], lnc[R], g[R], tot[R], fixed[R], init_tot[R], guess[R], lnguess[R], small_val[R];
  unsigned small_mask = 0;  // bit t: own species t was floored
  unsigned long long my_its = 0, my_fail = 0, my_maxits = 0, my_maxsub = 0;
  // adjoint: running dL/dT of the own species, direct dL/dT0 of floored
  // ones, the substep being walked back, per-lane parameter accumulators
  // (own complexes s = r + G*q, own minerals m = r + G*q)
  constexpr int QS = ADJ ? (PF_MAX_NSEC + G - 1) / G : 1;
  constexpr int QM = ADJ ? (PF_MAX_NMNRL + G - 1) / G : 1;
  double Tbar[R], gdir[R];
  double gK[QS], gKm[QM], glnk[QM];
  double loss_acc = 0.0;
  int sb = 0;
  bool back_done = false, back_fail = false;
  if constexpr (ADJ) {
    for (int q = 0; q < QS; ++q) gK[q] = 0.0;
    for (int q = 0; q < QM; ++q) { gKm[q] = 0.0; glnk[q] = 0.0; }
  }
#pragma unroll
  for (int t = 0; t < R; ++t) {
    Tbar[t] = gdir[t] = 0.0;
    c[t] = lnc[t] = g[t] = tot[t] = fixed[t] = init_tot[t] = guess[t] = lnguess[t] = small_val[t] = 0.0;
  }

  for (;;) {
    // ------------------------------------------------- work-queue refill
    const unsigned need = __ballot_sync(FULL, r == 0 && phase == NEED);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane_id == leader) base = atomicAdd(queue, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      const long long q = (long long)(base + __popc(need & ((1u << (gi * G)) - 1u)));
      if (phase == NEED) {
        phase = (q < ncells) ? START : DONE;
        if (phase == START) {
          cell = st.cell_order ? (long long)st.cell_order[q] : q;
          const double por = st.porosity[cell], sat = st.saturation[cell];
          den_k = st.den_kg[cell];
          volume = st.volume[cell];
          dry = sat < RT_MIN_SATURATION;
          psv = por * sat * 1000.0 * volume;
          den_L = den_k * 1.0e-3;
          small_mask = 0;
#pragma unroll
          for (int t = 0; t < R; ++t) {
            const int i = r + G * t;
            if (i < n) {
              double tv = st.total[soa.at(i, cell)];
              if (tv <= 1.0e-40) {  // RStep floor (reaction.F90:3618-3624)
                small_mask |= 1u << t;
                small_val[t] = tv;
                tv = 1.0e-40;
              }
              tot[t] = tv;
              guess[t] = o.use_total_as_guess ? tv : st.pri_molal[soa.at(i, cell)];
              lnguess[t] = sc_lnc[soa.at(i, cell)];
              g[t] = st.pri_act_coef[soa.at(i, cell)];
              c[t] = guess[t];
            }
          }
          for (int s = r; s < ns; s += G) {
            Ks[s] = sc_sec[soa.at(s, cell)];
            // the complexes' molalities live in sv for the whole cell (the
            // last evaluation's, as rt_auxvar holds them); written back once
            sv[s] = st.sec_molal[soa.at(s, cell)];
          }
          for (int m = r; m < nm; m += G) {
            Km[m] = sc_min[soa.at(m, cell)];
            vfm[m] = st.mnrl_volfrac[soa.at(m, cell)];
            ratem[m] = 0.0;
          }
          target = st.dt_cell ? st.dt_cell[cell] : dt_uniform;
          cum = 0.0;
          dt = target;
          its_total = 0;
          nsub = 0;
          num_cuts = 0;
          n_const = 0;
          zero_step = !(cum < target);
          if constexpr (ADJ) {
            if (adj_pass == 2) {
              // backward pass of a two-pass adjoint: the forward pass left the
              // cell's dL/dT(final) in dL_dtotal0 and, in adj_status, its
              // substep count and floored species (bit 30 set), or the final
              // status of a cell without a backward pass
              zero_step = false;
              const int seed = adj.adj_status[cell];
              if (!(seed & (1 << 30))) {
                phase = NEED;
              } else {
                const unsigned fmask = (unsigned)seed & 0xffffffu;
                nsub = (seed >> 24) & 31;
                small_mask = 0;
#pragma unroll
                for (int t = 0; t < R; ++t) {
                  const int i = r + G * t;
                  if (i >= n) continue;
                  const double gj = adj.dL_dtotal0[soa.at(i, cell)];
                  const bool fl = (fmask >> i) & 1u;
                  if (fl) small_mask |= 1u << t;
                  gdir[t] = fl ? gj : 0.0;
                  Tbar[t] = fl ? 0.0 : gj;
                  tb[i] = Tbar[t];
                }
                for (int m = r; m < nm; m += G) garea[m] = 0.0;
                sb = nsub - 1;
#pragma unroll
                for (int t = 0; t < R; ++t) {
                  const int i = r + G * t;
                  if (i < n) c[t] = adj_store[((size_t)sb * (n + 1) + i) * ncells + cell];
                }
                inv_dt = 1.0 / adj_store[((size_t)sb * (n + 1) + n) * ncells + cell];
                phase = BACK;
              }
            }
          }
        }
      }
    }
    if (__all_sync(FULL, phase == DONE)) break;

    bool finish_cell = false, cell_failed = false;
    if (zero_step) {
      finish_cell = true;
      zero_step = false;
      phase = NEED;
    }

    if (phase == START) {
#pragma unroll
      for (int t = 0; t < R; ++t) {
        fixed[t] = dry ? 0.0 : psv * tot[t];
        init_tot[t] = tot[t];
        c[t] = guess[t];
        lnc[t] = lnguess[t];
        // RAccumulationSorb into the fixed accumulation (reaction.F90:
        // 3836-3839): the sorbed total of the last evaluation
        const int i = r + G * t;
        if (has_sorb && i < n) fixed[t] = fma(st.total_sorb[soa.at(i, cell)], volume, fixed[t]);
      }
      its = 0;
      r0 = 0.0;
      inv_dt = 1.0 / dt;
      phase = ITER;
    }

    // ---------------------------------------------------------- Newton trip
    // (a backward trip, BACK, shares the evaluation and the factorisation)
    if (phase == ITER || (ADJ && phase == BACK)) {
      const bool back = ADJ && phase == BACK;
      if (!back && !redo) its += 1;
      redo = false;
      // LDL^T needs the symmetric log-form Jacobian: the sorption derivative
      // (the reference's surface complexation term is not symmetric) goes
      // into the full rows of the pivoted LU
      const bool ldl = !use_lu && !newton_iter_act && !has_sorb && !has_pf;
      if (newton_iter_act) {
        // RActivityCoefficients LAG from this iterate and the previous
        // evaluation's sec_molal (reaction.F90:4553-4612)
        double Ip = 0.0;
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const int i = r + G * t;
          if (i < n) Ip = Ip + c[t] * T.pri_Z(i) * T.pri_Z(i);
        }
        for (int s = r; s < ns; s += G) {
          const double z = T.sec_Z(s);
          Ip = Ip + sv[s] * z * z;
        }
        const double I = 0.5 * gsum<G>(Ip, gmask);
        sqI = sqrt(I);
        lgI = I;
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const int i = r + G * t;
          if (i < n) g[t] = exp(dh_ln_gamma(T.pri_Z(i), T.pri_a0(i), sqI, I, net));
        }
      }
      // ---- power table of the own species
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int i = r + G * t;
        if (i < n) {
          const double a = c[t] * g[t];
          pw[i] = a;
          pw[n + i] = a * a;
          xs[i] = c[t];  // molality by species for the entry assembly (xs is free until the solve)
          if (has_sorb || has_pf) vvs[i] = g[t];  // activity coefficient by species (free until the solve)
          if (neg_mask & (1u << i)) {
            const double ia = 1.0 / a;
            pw[2 * n + i] = ia;
            pw[3 * n + i] = ia * ia;
          }
        }
      }
      __syncwarp(gmask);
      const double a_acc = dry ? 1.0 : psv * inv_dt * den_L;
      // ---- the complexes dealt to the lanes longest list first (RTotalAqueous
      // in product form)
      for (int k = r; k < ns; k += G) {
        const int s = gt.s_perm[k];
        double v = newton_iter_act ? exp(Ks[s] - dh_ln_gamma(T.sec_Z(s), T.sec_a0(s), sqI, lgI, net)) : Ks[s];
        for (int p = T.sec_begin(s); p < T.sec_end(s); ++p) {
          const int pe = T.sec_pidx(p);
          v *= (pe >= 0) ? pw[pe] : exp(T.sec_nu(p) * log(pw[T.sec_idx(p)]));
        }
        sv[s] = v;
      }
      // ---- kinetic minerals m = r, r+G, ... (reaction_mineral.F90:647-1078)
      const double temp_c = st.temperature ? st.temperature[cell] : 25.0;
      if (has_pf) __syncwarp(gmask);  // the prefactors read other lanes' complexes
      for (int m = r; m < nm; m += G) {
        const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
        double Imv = 0.0, fv = 0.0, rv = 0.0;
        double QK = Km[m];
        for (int p = b; p < e; ++p) {
          const int pe = T.mnrl_pidx(p);
          QK *= (pe >= 0) ? pw[pe] : exp(T.mnrl_nu(p) * log(pw[T.mnrl_idx(p)]));
        }
        double aff;
        if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
        else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
        else aff = 1.0 - QK;
        const double sign_ = fsign1(aff);
        const bool active = (vfm[m] > 0 || sign_ < 0.0) && !(T.irreversible(m) == 1 && sign_ < 0.0) &&
                            !(T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m));
        if (active) {
          const double rl = T.limiter(m);
          if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
          double k;
          if (has_pf && TG.pf_cnt(m) > 0) {
            k = group_pref_rate(TG, st, cell, m, pw, sv, temp_c);
          } else {
            double arr = 1.0;
            if (T.ea(m) > 0.0)
              arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp_c + 273.15)));
            k = T.rate(m) * arr;
          }
          double Im_const = -st.mnrl_area[soa.at(m, cell)];
          if (has_msf) Im_const = Im_const / T.msf(m);
          double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * k : Im_const * sign_ * fabs(aff) * k;
          rv = Im;
          if (!dry) {
            Im_const = Im_const * volume;
            Im = Im * volume;
            double dIm_dQK = has_pw ? -Im * T.power(m) / fabs(aff) : -Im_const * k;
            if (has_tk)
              dIm_dQK = dIm_dQK * (1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m))) / QK * (1.0 - aff);
            else if (has_msf)
              dIm_dQK = dIm_dQK * (1.0 / T.msf(m)) / QK * (1.0 - aff);
            double ft = dIm_dQK * QK;
            if (rl > 0.0) {
              const double den = 1.0 + (1.0 - aff) / rl;
              ft = ft * (1.0 + QK / rl / den) / den;
            }
            Imv = Im;
            // the reference's den*1e-3 on dQK/dm (:944-947); the adjoint
            // takes the true derivative
            fv = back ? ft : ft * den_k * 1.0e-3;
          }
        }
        if (!back) ratem[m] = rv;
        mIm[m] = Imv;
        mf[m] = fv;
        if constexpr (ADJ) {
          if (back) {
            double acc = 0.0;
            for (int p = b; p < e; ++p) acc = fma(T.mnrl_nu(p), tb[T.mnrl_idx(p)], acc);
            nuT[m] = acc;
          }
        }
      }
      __syncwarp(gmask);
      // ---- own rows: totals, residual, Jacobian row (log formulation),
      // from the tables staged in shared memory
      const double b_tot = den_L / a_acc;
      double dot_p = 0.0;
      unsigned long long mx_p = 0;
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int i = r + G * t;
        if (i >= n) continue;
        double* Jr = J + i * n;
        // the pivoted LU (fallback) assembles full rows here; LDL^T assembles
        // the lower triangle entry by entry below
        if (!ldl)
          for (int j = 0; j < n; ++j) Jr[j] = 0.0;
        double Sa = 0.0;
        if (ldl) {
          for (int q = gt.sp_ptr[i]; q < gt.sp_ptr[i + 1]; ++q) Sa = fma(gt.sp_nu[q], sv[gt.sp_s[q]], Sa);
          Sa = a_acc * Sa;
        } else {
          for (int q = gt.sp_ptr[i]; q < gt.sp_ptr[i + 1]; ++q) {
            const int s = gt.sp_s[q];
            const double sa = a_acc * sv[s];
            const double nui = T.sec_nu(gt.sp_p[q]);
            Sa = fma(nui, sa, Sa);
            const double co = nui * sa;
            for (int p = T.sec_begin(s); p < T.sec_end(s); ++p) {
              const int j = T.sec_idx(p);
              Jr[j] = fma(T.sec_nu(p), co, Jr[j]);
            }
          }
        }
        double rr;
        if (!back) {
          tot[t] = fma(b_tot, Sa, den_L * c[t]);
          rr = dry ? 0.0 : fma(a_acc, c[t], Sa) - fixed[t] * inv_dt;
        } else {
          rr = 0.0;  // backward solve J u = B Tbar
        }
        if (!ldl) Jr[i] = fma(a_acc, c[t], Jr[i]);
        for (int q = gt.mp_ptr[i]; q < gt.mp_ptr[i + 1]; ++q) {
          const int m = gt.mp_m[q];
          const double nui = gt.mp_nu[q];
          if (back) rr = fma(nui * mf[m], nuT[m], rr);
          else if (!dry) rr = fma(nui, mIm[m], rr);
          if (ldl) continue;
          const double co = nui * mf[m];
          for (int p = T.mnrl_begin(m); p < T.mnrl_end(m); ++p) {
            const int j = T.mnrl_idx(p);
            Jr[j] = fma(T.mnrl_nu(p), co, Jr[j]);
          }
        }
        if (dry && !ldl)
          for (int j = 0; j < n; ++j) Jr[j] = (i == j) ? c[t] : 0.0;
        rhsv[i] = rr;
        dot_p = fma(rr, rr, dot_p);
        mx_p = max(mx_p, absbits(rr));
      }
      if (ldl) {
        // ---- lower triangle entry by entry, dealt round-robin to the lanes:
        // J_ij = a_acc (m_i d_ij + sum_s nu_si nu_sj s_s) + sum_m nu_mi nu_mj f_m
        // from the per-entry lists of complexes and minerals (one store per entry)
        const int ne = n * (n + 1) / 2;
        const Tables TE = net.ent_staged ? T : Tables{net.ints, net.dbls, &net};
        for (int e = r; e < ne; e += G) {
          const int f = TE.ent_ij(e);
          const int i = f / n, j = f - i * n;
          double acc = 0.0;
          for (int q = TE.ent_begin(e); q < TE.ent_end(e); ++q) acc = fma(TE.ent_cf(q), sv[TE.ent_sc(q)], acc);
          if (i == j) acc = acc + xs[i];
          double v = a_acc * acc;
          for (int q = TE.ent_mbegin(e); q < TE.ent_mend(e); ++q) v = fma(TE.ent_mcf(q), mf[TE.ent_mm(q)], v);
          if (dry) v = (i == j) ? xs[i] : 0.0;
          J[f] = v;
        }
      }
      // ---- rate prefactors: their part of the Jacobian, one lane of the
      // group, into the full rows (the rates above already carry them)
      if (has_pf && !back && !dry) {
        __syncwarp(gmask);
        if (r == 0) group_pref_jacobian(net, TG, st, cell, pw, sv, xs, vvs, Ks, mIm, temp_c, J);
        __syncwarp(gmask);
      }
      // ---- equilibrium sorption: one lane of the group, into the full rows
      // and the residual; the residual norms are taken again
      bool sorb_fail = false;
      if (has_sorb && !back) {
        __syncwarp(gmask);
        int bad = 0;
        if (r == 0) bad = !group_sorb(net, T, st, cell, xs, vvs, vfm, den_k, volume * inv_dt, J, rhsv);
        sorb_fail = __shfl_sync(gmask, bad, gi * G) != 0;
        __syncwarp(gmask);
        dot_p = 0.0;
        mx_p = 0;
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const int i = r + G * t;
          if (i >= n) continue;
          const double rr = rhsv[i];
          dot_p = fma(rr, rr, dot_p);
          mx_p = max(mx_p, absbits(rr));
        }
      }
      // ---- convergence tests on the residual (reaction.F90:3946-3953)
      const double two_norm = sqrt(gsum<G>(dot_p, gmask));
      const unsigned long long mxb = gmax<G>(mx_p, gmask);
      if (!back && its == 1) r0 = two_norm;
      int react_end = -1;
      if (back) {
        // falls through to the factorisation below
      } else if (sorb_fail) {
        react_end = 1;  // RTAuxVarCompute's ierror: no total restore (reaction.F90:3861-3865)
      } else if (its > o.maximum_reaction_iterations) {
#pragma unroll
        for (int t = 0; t < R; ++t) tot[t] = init_tot[t];
        react_end = 1;
      } else if (__longlong_as_double((long long)mxb) < o.max_residual_tolerance ||
                 two_norm < o.max_rel_residual_tolerance * r0) {
        react_end = 0;
      }
      if (back || react_end < 0) {
        __syncwarp(gmask);
        bool solved = false;
        if (ldl) {
          // ---- LDL^T, right-looking over the lower triangle; the forward
          // solve L y = rhs rides along; D^-1 in vvs, L below the diagonal
          bool fail = false;
          for (int k = 0; k < n; ++k) {
            const double dk = J[k * n + k];
            if (!(dk > 0.0) || absbits(dk) >= 0x7ff0000000000000ull) {  // same value in every lane
              fail = true;
              break;
            }
            const double inv = 1.0 / dk;
            const int i0 = k + 1 + ((r - (k + 1)) % G + G) % G;  // first own row below k
            // column k: keep the unscaled values (xs is free until the
            // solve), store l_ik = a_ik / d_k, forward-eliminate the rhs
            const double yk = rhsv[k];
            for (int i = i0; i < n; i += G) {
              const double a = J[i * n + k];
              xs[i] = a;
              const double l = a * inv;
              J[i * n + k] = l;
              rhsv[i] = fma(-l, yk, rhsv[i]);
            }
            if (r == k % G) vvs[k] = inv;
            __syncwarp(gmask);
            // trailing update a_ij -= l_ik a_jk over the (n-k-1)(n-k)/2
            // entries k < j <= i, dealt round-robin to the lanes (rows of
            // unequal length would leave lanes idle)
            {
              int i = k + 1, j = k + 1 + r;  // entry r of the row-major triangle
              while (i < n && j > i) { j -= i - k; i += 1; }
              while (i < n) {
                J[i * n + j] = fma(-J[i * n + k], xs[j], J[i * n + j]);
                j += G;
                while (i < n && j > i) { j -= i - k; i += 1; }
              }
            }
            __syncwarp(gmask);
          }
          if (fail) {
            use_lu = true;  // factorise this evaluation again with pivoting
            redo = true;
          } else {
            // D^-1, then the backward solve L^T x = z by columns
            for (int i = r; i < n; i += G) rhsv[i] = rhsv[i] * vvs[i];
            __syncwarp(gmask);
            for (int k = n - 1; k >= 0; --k) {
              const double xk = rhsv[k];
              if (r == 0) xs[k] = xk;
              for (int i = r; i < k; i += G) rhsv[i] = fma(-J[k * n + i], xk, rhsv[i]);
              __syncwarp(gmask);
            }
            solved = true;
          }
        } else {
        use_lu = false;
        // ---- implicit-pivot scales (utility.F90:621-644), rows over the lanes
        bool bad = false;
        for (int i = r; i < n; i += G) {
          unsigned long long am = 0;
          for (int j = 0; j < n; ++j) am = max(am, absbits(J[i * n + j]));
          if (am == 0ull || am > 0x7ff0000000000000ull) bad = true;
          vvs[i] = 1.0 / __longlong_as_double((long long)am);
          rows[i] = i;
        }
        if (__any_sync(gmask, bad)) {
          if (back) back_fail = true;
          else react_end = 1;  // singular: no total restore (reaction.F90:3963-3966)
        } else {
          __syncwarp(gmask);
          // ---- right-looking elimination over the remaining rows (compact
          // list), rhs alongside; work split by (row, column) pairs
          int nrem = n;
          for (int k = 0; k < n; ++k) {
            unsigned long long key = 0;
            int prow = -1, ppos = -1;
            for (int e = r; e < nrem; e += G) {
              const int i = rows[e];
              const unsigned long long dum = absbits(vvs[i] * J[i * n + k]);
              if (dum > key || (dum == key && i > prow)) { key = dum; prow = i; ppos = e; }
            }
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1) {
              const unsigned long long ok = __shfl_xor_sync(gmask, key, off, G);
              const int orow = __shfl_xor_sync(gmask, prow, off, G);
              const int opos = __shfl_xor_sync(gmask, ppos, off, G);
              if (ok > key || (ok == key && orow > prow)) { key = ok; prow = orow; ppos = opos; }
            }
            double a = J[prow * n + k];
            if (absbits(a) == 0ull) a = 1.0e-20;
            const double rp = 1.0 / a;
            const double bp = rhsv[prow];
            __syncwarp(gmask);
            if (r == 0) {
              J[prow * n + k] = a;
              vvs[prow] = rp;  // holds 1/pivot from here on
              piv[k] = prow;
              rows[ppos] = rows[nrem - 1];
            }
            nrem -= 1;
            __syncwarp(gmask);
            for (int e = r; e < nrem; e += G) {
              const int i = rows[e];
              const double l = J[i * n + k] * rp;
              J[i * n + k] = l;
              rhsv[i] = fma(-l, bp, rhsv[i]);
            }
            __syncwarp(gmask);
            // rank-1 update of the remaining rows, columns split over the lanes
            const double* Jp = J + prow * n;
            for (int e = 0; e < nrem; ++e) {
              double* Ji = J + rows[e] * n;
              const double l = Ji[k];
              for (int j = k + 1 + r; j < n; j += G) Ji[j] = fma(-l, Jp[j], Ji[j]);
            }
            __syncwarp(gmask);
          }
          // ---- back substitution by columns: x_k = (rhs_p - sum_{j>k} U_pj x_j)/U_pk
          for (int k = n - 1; k >= 0; --k) {
            const int prow = piv[k];
            const double xk = rhsv[prow] * vvs[prow];
            if (r == 0) xs[k] = xk;
            for (int kk = r; kk < k; kk += G) {
              const int i = piv[kk];
              rhsv[i] = fma(-J[i * n + k], xk, rhsv[i]);
            }
            __syncwarp(gmask);
          }
          solved = true;
        }
        }
        if (solved) {
          __syncwarp(gmask);
          if constexpr (ADJ) {
            if (back) {
              // u = x; lambda = (Tbar - u)/(psv/dt); theta_bar += (dT/dtheta)^T u
              // - (dR/dtheta)^T lambda; Tbar(previous substep) = Tbar - u
              const double ipd = den_L / a_acc;
#pragma unroll
              for (int t = 0; t < R; ++t) {
                const int i = r + G * t;
                if (i < n) lamv[i] = (Tbar[t] - xs[i]) * ipd;
              }
              __syncwarp(gmask);
              for (int s2 = r, q = 0; s2 < ns; s2 += G, ++q) {
                double acc = 0.0;
                for (int p = T.sec_begin(s2); p < T.sec_end(s2); ++p) acc = fma(T.sec_nu(p), xs[T.sec_idx(p)], acc);
                gK[q] = fma(acc, -LOG_TO_LN * den_L * sv[s2], gK[q]);
              }
              for (int m = r, q = 0; m < nm; m += G, ++q) {
                if (mIm[m] == 0.0 && mf[m] == 0.0) continue;
                double lam = 0.0;
                for (int p = T.mnrl_begin(m); p < T.mnrl_end(m); ++p)
                  lam = fma(T.mnrl_nu(p), lamv[T.mnrl_idx(p)], lam);
                gKm[q] = fma(LOG_TO_LN * mf[m], lam, gKm[q]);
                glnk[q] = fma(-mIm[m], lam, glnk[q]);
                garea[m] = fma(-mIm[m], lam, garea[m]);
              }
#pragma unroll
              for (int t = 0; t < R; ++t) {
                const int i = r + G * t;
                if (i < n) {
                  Tbar[t] = Tbar[t] - xs[i];
                  tb[i] = Tbar[t];
                }
              }
              sb -= 1;
              if (sb >= 0) {
#pragma unroll
                for (int t = 0; t < R; ++t) {
                  const int i = r + G * t;
                  if (i < n) c[t] = adj_store[((size_t)sb * (n + 1) + i) * ncells + cell];
                }
                inv_dt = 1.0 / adj_store[((size_t)sb * (n + 1) + n) * ncells + cell];
              } else {
                back_done = true;
              }
              __syncwarp(gmask);
            }
          }
          if (!back) {
            // ---- update of the own species (reaction.F90:3993-4046)
            const double tol = o.max_relative_change_tolerance;
            bool small = true;
            double nc[R], u[R];
#pragma unroll
            for (int t = 0; t < R; ++t) {
              const int i = r + G * t;
              if (i < n) {
                u[t] = o.fork_literal_rsolve ? 0.0 : xs[i];
                u[t] = fmin(fmax(u[t], -o.max_dlnC_rreact), o.max_dlnC_rreact);
                nc[t] = c[t] * exp(-u[t]);
                small = small && (absbits(nc[t] - c[t]) < absbits(tol * c[t]));
              }
            }
            if (__all_sync(gmask, small)) {
              react_end = 0;
            } else {
#pragma unroll
              for (int t = 0; t < R; ++t) {
                const int i = r + G * t;
                if (i < n) {
                  lnc[t] = lnc[t] - u[t];
                  c[t] = nc[t];
                }
              }
            }
          }
        }
      }
      // ---- RStep bookkeeping (reaction.F90:3650-3718)
      if (!back && react_end >= 0) {
        its_total += its;
        if (react_end == 1) {
          num_cuts = num_cuts + 1;
          if (num_cuts > o.maximum_reaction_cuts) {
            finish_cell = true;
            cell_failed = true;
          } else {
            dt = 0.5 * dt;
            n_const = 0;
            phase = START;
          }
        } else {
          for (int m = r; m < nm; m += G) {  // MineralUpdateKineticState
            const double v = vfm[m] + ratem[m] * T.molar_vol(m) * dt;
            vfm[m] = v < 0.0 ? 0.0 : v;
          }
          if (ADJ || adj_pass == 1) {
            // the adjoint's substep store: the converged iterate and dt
            if (nsub < PF_ADJ_MAX_SUBSTEPS) {
#pragma unroll
              for (int t = 0; t < R; ++t) {
                const int i = r + G * t;
                if (i < n) adj_store[((size_t)nsub * (n + 1) + i) * ncells + cell] = c[t];
              }
              if (r == 0) adj_store[((size_t)nsub * (n + 1) + n) * ncells + cell] = dt;
            }
          }
          cum = cum + dt;
          nsub += 1;
          n_const += 1;
#pragma unroll
          for (int t = 0; t < R; ++t) {
            guess[t] = c[t];
            lnguess[t] = lnc[t];
          }
          if (n_const >= 4) {
            num_cuts = num_cuts - 1;
            dt = fmin(2.0 * dt, target - cum);
          }
          if (cum >= target) finish_cell = true;
          else phase = START;
        }
      }
    }

    if constexpr (ADJ) {
      // end of a backward pass: per-cell gradients
      if (phase == BACK && (back_done || back_fail)) {
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const int i = r + G * t;
          if (i < n)
            adj.dL_dtotal0[soa.at(i, cell)] = back_fail ? 0.0 : ((small_mask & (1u << t)) ? gdir[t] : Tbar[t]);
        }
        for (int m = r; m < nm; m += G) adj.dL_dlnarea[soa.at(m, cell)] = back_fail ? 0.0 : garea[m];
        if (r == 0 && adj.adj_status) adj.adj_status[cell] = back_fail ? 3 : 0;
        back_done = back_fail = false;
        phase = NEED;
      }
    }

    // ---------------------------------------------------- cell write-back
    if (finish_cell) {
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int i = r + G * t;
        if (i < n) {
          double tv = tot[t];
          if (!cell_failed && (small_mask & (1u << t))) tv = small_val[t];
          st.total[soa.at(i, cell)] = tv;
          st.pri_molal[soa.at(i, cell)] = c[t];
          if (newton_iter_act) st.pri_act_coef[soa.at(i, cell)] = g[t];
        }
      }
      for (int s = r; s < ns; s += G) st.sec_molal[soa.at(s, cell)] = sv[s];
      if (newton_iter_act)
        for (int s = r; s < ns; s += G)
          st.sec_act_coef[soa.at(s, cell)] = exp(dh_ln_gamma(T.sec_Z(s), T.sec_a0(s), sqI, lgI, net));
      for (int m = r; m < nm; m += G) {
        st.mnrl_volfrac[soa.at(m, cell)] = vfm[m];
        st.mnrl_rate[soa.at(m, cell)] = ratem[m];
      }
      if (r == 0) {
        if (st.status) st.status[cell] = cell_failed ? PF_CELL_TOO_MANY_CUTS : PF_CELL_OK;
        if (st.newton_its) st.newton_its[cell] = its_total;
        if (st.num_substeps) st.num_substeps[cell] = nsub;
        my_its += (unsigned long long)its_total;
        my_fail += cell_failed ? 1ull : 0ull;
        my_maxits = max(my_maxits, (unsigned long long)its_total);
        my_maxsub = max(my_maxsub, (unsigned long long)nsub);
      }
      phase = NEED;
      if (ADJ || adj_pass == 1) {
        // loss contribution and dL/dT(final); start the backward pass (or,
        // in the forward pass of a two-pass adjoint, leave its seed)
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const int i = r + G * t;
          if (i >= n) continue;
          const double tv = (!cell_failed && (small_mask & (1u << t))) ? small_val[t] : tot[t];
          double gj;
          if (adj.weight) {
            const double w = adj.weight[soa.at(i, cell)], d = tv - adj.target[soa.at(i, cell)];
            loss_acc = fma(w * d, d, loss_acc);
            gj = 2.0 * w * d;
          } else {
            gj = adj.dL_dtotal[soa.at(i, cell)];
          }
          // a floored component's final total is its restored input
          // (reaction.F90:3721-3725): dL/dT0 directly, no path through m
          const bool fl = small_mask & (1u << t);
          gdir[t] = fl ? gj : 0.0;
          Tbar[t] = fl ? 0.0 : gj;
          if constexpr (ADJ) tb[i] = Tbar[t];  // (the forward kernel's workspace has no tb)
        }
        if constexpr (ADJ)
          for (int m = r; m < nm; m += G) garea[m] = 0.0;
        const int astat = cell_failed ? 1 : (nsub > PF_ADJ_MAX_SUBSTEPS ? 2 : 0);
        if (astat != 0 || dry || nsub == 0) {
#pragma unroll
          for (int t = 0; t < R; ++t) {
            const int i = r + G * t;
            if (i < n) adj.dL_dtotal0[soa.at(i, cell)] = (astat == 0) ? gdir[t] : 0.0;
          }
          for (int m = r; m < nm; m += G) adj.dL_dlnarea[soa.at(m, cell)] = 0.0;
          if (r == 0 && adj.adj_status) adj.adj_status[cell] = astat;
        } else if (adj_pass == 1) {
          // forward pass of a two-pass adjoint: dL/dT(final) and the seed of
          // the backward pass (substeps, floored species of the group)
          unsigned fm = 0;
#pragma unroll
          for (int t = 0; t < R; ++t) {
            const int i = r + G * t;
            if (i >= n) continue;
            adj.dL_dtotal0[soa.at(i, cell)] = gdir[t] + Tbar[t];  // one of the two is zero
            if (small_mask & (1u << t)) fm |= 1u << i;
          }
#pragma unroll
          for (int off = 1; off < G; off <<= 1) fm |= __shfl_xor_sync(gmask, fm, off);
          if (r == 0) adj.adj_status[cell] = (1 << 30) | (nsub << 24) | (int)fm;
        } else if constexpr (ADJ) {
          sb = nsub - 1;
#pragma unroll
          for (int t = 0; t < R; ++t) {
            const int i = r + G * t;
            if (i < n) c[t] = adj_store[((size_t)sb * (n + 1) + i) * ncells + cell];
          }
          inv_dt = 1.0 / adj_store[((size_t)sb * (n + 1) + n) * ncells + cell];
          phase = BACK;
        }
        __syncwarp(gmask);
      }
    }
  }
  if constexpr (ADJ) {
    // parameter gradients and the loss: sum the groups of the warp (lanes
    // r, r+G, ... hold the same parameters), one atomic per parameter
    auto across = [&](double v) {
#pragma unroll
      for (int off = 16; off >= G; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
      return v;
    };
    for (int q = 0; q < (ns + G - 1) / G; ++q) {
      const double v = across(gK[q]);
      const int s2 = r + G * q;
      if (gi == 0 && s2 < ns && v != 0.0) atomicAdd(&adj.dL_dlogK_sec[s2], v);
    }
    for (int q = 0; q < (nm + G - 1) / G; ++q) {
      const double a = across(gKm[q]), b = across(glnk[q]);
      const int m = r + G * q;
      if (gi == 0 && m < nm) {
        if (a != 0.0) atomicAdd(&adj.dL_dlogK_mnrl[m], a);
        if (b != 0.0) atomicAdd(&adj.dL_dlnk[m], b);
      }
    }
    double l = loss_acc;
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(FULL, l, off);
    if (lane_id == 0 && adj.loss && l != 0.0) atomicAdd(adj.loss, l);
  } else if (adj_pass == 1) {
    double l = loss_acc;
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(FULL, l, off);
    if (lane_id == 0 && adj.loss && l != 0.0) atomicAdd(adj.loss, l);
  }
  if (counters) {
    for (int off = 16; off > 0; off >>= 1) {
      my_its += __shfl_down_sync(FULL, my_its, off);
      my_fail += __shfl_down_sync(FULL, my_fail, off);
      my_maxits = max(my_maxits, __shfl_down_sync(FULL, my_maxits, off));
      my_maxsub = max(my_maxsub, __shfl_down_sync(FULL, my_maxsub, off));
    }
    if (lane_id == 0) {
      atomicAdd(&counters[0], my_its);
      if (my_fail) atomicAdd(&counters[1], my_fail);
      atomicMax(&counters[3], my_maxits);
      atomicMax(&counters[4], my_maxsub);
    }
  }
}

template <int G, int R, bool ADJ>
__global__ void __launch_bounds__(256, 1)
rstep_group_kernel(DevNet net, GroupTabs gt, PfCellState st, double dt_uniform, const double* __restrict__ scratch,
                   unsigned long long* queue, unsigned long long* counters, PfAdjointArgs adj,
                   double* __restrict__ adj_store, int adj_pass) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t tma_bar;
  if (!stage_tables(net, smem, &tma_bar, 0u, true, counters)) return;
  group_body<G, R, ADJ>(net, gt, st, dt_uniform, scratch, queue, counters, adj, adj_store, smem, (int)blockDim.x,
                        adj_pass);
}

// The adjoint runs in two passes when it has a status array to carry the
// seeds: every cell's forward solve first, by the forward kernel with the
// substep store, the loss and the seeds switched on (adj_pass 1), then every
// cell's backward pass by the adjoint kernel (adj_pass 2, the queue
// restarted).  The forward Newton trips in the adjoint instantiation ran at
// 13 of 32 lanes per instruction against 22 in the forward kernel (ncu), in
// one pass or two; its backward trips alone run at 24.
template <int G, int R>
int launch_k(const DevNet& net, const GroupTabs& gt, const PfCellState& st, double dt, size_t smem, int grid,
             int tpb, const double* scratch, unsigned long long* queue, unsigned long long* counters,
             const PfAdjointArgs* adj, double* adj_store, cudaStream_t stream) {
  if (adj) {
    auto k = rstep_group_kernel<G, R, true>;
    cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    if (!adj->adj_status) {
      k<<<grid, tpb, smem, stream>>>(net, gt, st, dt, scratch, queue, counters, *adj, adj_store, 0);
    } else {
      auto kf = rstep_group_kernel<G, R, false>;
      err = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err != cudaSuccess) return (int)err;
      kf<<<grid, tpb, smem, stream>>>(net, gt, st, dt, scratch, queue, counters, *adj, adj_store, 1);
      err = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), stream);
      if (err != cudaSuccess) return (int)err;
      k<<<grid, tpb, smem, stream>>>(net, gt, st, dt, scratch, queue, counters, *adj, adj_store, 2);
    }
  } else {
    auto k = rstep_group_kernel<G, R, false>;
    cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    k<<<grid, tpb, smem, stream>>>(net, gt, st, dt, scratch, queue, counters, PfAdjointArgs{}, nullptr, 0);
  }
  return (int)cudaGetLastError();
}

}  // namespace group
}  // namespace pfgpu
