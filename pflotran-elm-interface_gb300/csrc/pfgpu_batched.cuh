// pfgpu_batched.cuh -- batched persistent operator-split reaction kernel.
//
// Same step as RStep/RReact (src/pflotran/reaction.F90:3564-4055) per cell,
// organised for GB300's FP64 pipe (1/64 of the FP32 rate, so the count of
// FP64 instructions per Newton trip and the fraction of active lanes decide
// the throughput):
//
//   * one lane per cell, ncomp a compile-time constant, so the n-indexed
//     loops unroll and c, ln c, gamma and totals live in registers;
//   * persistent grid with a device work queue: a lane whose cell finished
//     takes the next one at the top of the following Newton trip (warp-
//     aggregated atomicAdd; the queue index only grows, so the loop is
//     bounded).  An optional cell order (longest first, from the previous
//     step's iteration counts) removes the tail of slow cells;
//   * everything a cell needs once -- logK(T), 1/gamma of every complex,
//     ln of the initial guess -- is computed by a convergent pre-pass
//     (cell_setup_kernel) into scratch, so the refill of one lane costs the
//     warp loads, not transcendentals;
//   * reaction tables staged once per block into shared memory by a bulk TMA
//     copy (cp.async.bulk + mbarrier, bounded wait);
//   * speciation in product form: for integer stoichiometry nu in {+-1,+-2}
//     s_i = exp(-logK_i ln10)/gamma_i * prod_j (m_j gamma_j)^nu_ij is
//     exp(lnQK)/gamma_i of RTotalAqueous (reaction.F90:4711-4718) without the
//     exp: a per-lane table of a, a^2, 1/a, 1/a^2 turns every factor into one
//     multiply (other coefficients fall back to exp(nu ln a));
//   * d total/d m (reaction.F90:4731-4744) is sum_i nu_ik nu_ij s_i / m_j; in
//     the log formulation RSolve multiplies column j by m_j (:5494-5499), so
//     the log-space Jacobian is a*(delta_kj m_j + G_kj) with the symmetric
//     G = sum_i s_i nu_i nu_i^T, accumulated on one triangle and mirrored;
//   * the Crout LU's implicit pivot scaling (utility.F90:621-666) makes the
//     pivot sequence invariant under RSolve's row normalisation (:5486-5492),
//     which is folded away; magnitude comparisons use the integer order of
//     IEEE bit patterns, keeping them off the FP64 pipe;
//   * RReact's closing RTAuxVarCompute (:4052) and MineralUpdateKineticState's
//     rate evaluation (reaction_mineral.F90:1490) happen at the iterate of the
//     last evaluation, so both reuse it.
#pragma once
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"
#include "pfgpu_sorb.cuh"

namespace pfgpu {
namespace batched {

constexpr unsigned FULL = 0xffffffffu;
constexpr long long TMA_WAIT_LIMIT = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

enum Phase : int { NEED = 0, START = 1, ITER = 2, DONE = 3, BACK = 4 };

template <int N, bool JS>
struct Lane {
  // thread-strided shared-memory vectors: element e of this lane at base[e*stride]
  double* base;
  int stride;
  double* Jl;  // local-memory Jacobian when !JS
  __device__ __forceinline__ double& J(int i, int j) {
    if constexpr (JS) return base[(i * N + j) * stride];
    else return Jl[i * N + j];
  }
  __device__ __forceinline__ double& Jf(int flat) {
    if constexpr (JS) return base[flat * stride];
    else return Jl[flat];
  }
  static constexpr int OFF = JS ? N * N : 0;
  // power table a, a^2, 1/a, 1/a^2 (live in the evaluation) shares storage
  // with the pivot scales VV (live in the factorisation)
  __device__ __forceinline__ double& P(int e) { return base[(OFF + e) * stride]; }
  __device__ __forceinline__ double& VV(int j) { return base[(OFF + j) * stride]; }
  __device__ __forceinline__ double& S(int j) { return base[(OFF + 4 * N + j) * stride]; }
  __device__ __forceinline__ double& rhs(int j) { return base[(OFF + 5 * N + j) * stride]; }
  static constexpr int DOUBLES = OFF + 6 * N;
};

// Crout LU with implicit partial pivoting (utility.F90:597-688) and the
// solve (utility.F90:692-735) in place on rhs.  VV(j) holds 1/pivot once row
// j is final.  Returns 1 for a zero row (ierror of LUDecomposition).
template <int N, bool JS>
__device__ __forceinline__ int lu_solve(Lane<N, JS>& L, int* indx, int stride) {
  constexpr int U = (N <= 12) ? N : 1;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    unsigned long long am = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) am = max(am, absbits(L.J(i, j)));
    if (am == 0ull || am > 0x7ff0000000000000ull) return 1;
    L.VV(i) = 1.0 / __longlong_as_double((long long)am);
  }
#pragma unroll U
  for (int j = 0; j < N; ++j) {
#pragma unroll U
    for (int i = 1; i < j; ++i) {
      double sum = L.J(i, j);
#pragma unroll U
      for (int k = 0; k < i; ++k) sum = fma(-L.J(i, k), L.J(k, j), sum);
      L.J(i, j) = sum;
    }
    unsigned long long amax = 0;
    int imax = j;
#pragma unroll U
    for (int i = j; i < N; ++i) {
      double sum = L.J(i, j);
#pragma unroll U
      for (int k = 0; k < j; ++k) sum = fma(-L.J(i, k), L.J(k, j), sum);
      L.J(i, j) = sum;
      const unsigned long long dum = absbits(L.VV(i) * sum);
      if (dum >= amax) { imax = i; amax = dum; }
    }
    // unconditional swap (a no-op when imax == j) keeps the warp converged
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const double a = L.J(imax, k), b = L.J(j, k);
      L.J(imax, k) = b;
      L.J(j, k) = a;
    }
    L.VV(imax) = L.VV(j);
    indx[j * stride] = imax;
    double piv = L.J(j, j);
    if (absbits(piv) == 0ull) { piv = 1.0e-20; L.J(j, j) = piv; }
    const double rp = 1.0 / piv;
    L.VV(j) = rp;
#pragma unroll U
    for (int i = j + 1; i < N; ++i) L.J(i, j) = L.J(i, j) * rp;
  }
#pragma unroll U
  for (int i = 0; i < N; ++i) {
    const int ll = indx[i * stride];
    double sum = L.rhs(ll);
    L.rhs(ll) = L.rhs(i);
#pragma unroll U
    for (int j = 0; j < i; ++j) sum = fma(-L.J(i, j), L.rhs(j), sum);
    L.rhs(i) = sum;
  }
#pragma unroll U
  for (int i = N - 1; i >= 0; --i) {
    double sum = L.rhs(i);
#pragma unroll U
    for (int j = i + 1; j < N; ++j) sum = fma(-L.J(i, j), L.rhs(j), sum);
    L.rhs(i) = sum * L.VV(i);
  }
  return 0;
}

// LDL^T of the symmetric positive definite log-form Jacobian (the upper
// triangle is read: J = U^T D U with U unit upper, stored above the
// diagonal), solving J x = rhs in place; D^-1 in VV.  Half the flops of the
// LU and no pivot search; the solution is that of the pivoted LU up to
// rounding.  Returns 1 when a pivot is not positive and finite (the caller
// then factorises again with the pivoted LU).
template <int N, bool JS>
__device__ __forceinline__ int ldl_solve(Lane<N, JS>& L) {
  constexpr int U = (N <= 12) ? N : 1;
#pragma unroll U
  for (int k = 0; k < N; ++k) {
    const double dk = L.J(k, k);
    if (!(dk > 0.0) || absbits(dk) >= 0x7ff0000000000000ull) return 1;
    const double inv = 1.0 / dk;
#pragma unroll U
    for (int i = k + 1; i < N; ++i) {
      const double t = L.J(k, i) * inv;
#pragma unroll U
      for (int j = i; j < N; ++j) L.J(i, j) = fma(-t, L.J(k, j), L.J(i, j));
    }
    const double yk = L.rhs(k);
#pragma unroll U
    for (int i = k + 1; i < N; ++i) {
      const double u = L.J(k, i) * inv;
      L.J(k, i) = u;
      L.rhs(i) = fma(-u, yk, L.rhs(i));
    }
    L.VV(k) = inv;
  }
#pragma unroll
  for (int k = 0; k < N; ++k) L.rhs(k) = L.rhs(k) * L.VV(k);
#pragma unroll U
  for (int k = N - 1; k >= 0; --k) {
    double xk = L.rhs(k);
#pragma unroll U
    for (int j = k + 1; j < N; ++j) xk = fma(-L.J(k, j), L.rhs(j), xk);
    L.rhs(k) = xk;
  }
  return 0;
}

// Debye-Hueckel ln gamma (the exponent of RActivityCoefficients, LAG form)
__device__ __forceinline__ double dh_ln_gamma(double z, double a0, double sI, double I, const DevNet& net) {
  return fabs(z) > 1.0e-10 ? (-z * z * sI * net.A / (1.0 + a0 * net.B * sI) + net.Bdot * I) * LOG_TO_LN : 0.0;
}

template <int N, bool JS, bool ADJ>
__global__ void __launch_bounds__(256)
rstep_batched_kernel(DevNet net, PfCellState st, double dt_uniform, const double* __restrict__ scratch,
                     unsigned long long* queue, unsigned long long* counters, PfAdjointArgs adj) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t tma_bar;
  const int tid = threadIdx.x;
  const int lane_id = tid & 31;
  const int stride = blockDim.x;
  const uint32_t ibytes = (uint32_t)net.int_words * 4u;  // multiples of 16 (host pads)
  const uint32_t dbytes = (uint32_t)net.dbl_words * 8u;
  int32_t* sI = reinterpret_cast<int32_t*>(smem);
  double* sD = reinterpret_cast<double*>(smem + ibytes);

  // ---- stage the network tables: one bulk TMA copy per block -------------
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tma_bar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&tma_bar)),
                 "r"(ibytes + dbytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sI)),
                 "l"(net.ints), "r"(ibytes), "r"(smem_u32(&tma_bar))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sD)),
                 "l"(net.dbls), "r"(dbytes), "r"(smem_u32(&tma_bar))
                 : "memory");
  }
  {
    uint32_t done = 0;
    long long spins = 0;
    while (!done && spins < TMA_WAIT_LIMIT) {
      asm volatile(
          "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
          : "=r"(done)
          : "r"(smem_u32(&tma_bar)), "r"(0)
          : "memory");
      ++spins;
    }
    // every thread waited on the same barrier; a timeout (never expected)
    // flags the launch and leaves without touching any cell
    if (__syncthreads_or(!done)) {
      if (tid == 0) atomicOr(&counters[2], 1ull);
      return;
    }
  }
  const Tables T{sI, sD, &net};
  double* lane_mem = reinterpret_cast<double*>(smem + ibytes + dbytes) + tid;
  int* indx = reinterpret_cast<int*>(reinterpret_cast<double*>(smem + ibytes + dbytes) +
                                     (size_t)Lane<N, JS>::DOUBLES * stride) + tid;
  double Jlocal[JS ? 1 : N * N];
  Lane<N, JS> L{lane_mem, stride, Jlocal};

  const SoA soa{st.ncells};
  const PfOptions o = net.o;
  const int ns = net.ns, nm = net.nm;
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  const bool logf = o.use_log_formulation != 0;
  const bool newton_iter_act = o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER;
  const unsigned neg_mask = (unsigned)net.neg_mask;
  const bool has_sorb = !ADJ && has_sorption(net);  // the adjoint refuses sorption
  const int64_t ncells = st.ncells;
  const double* sc_sec = scratch;                                  // [ns][ncells]
  const double* sc_min = scratch + (size_t)ns * ncells;            // [nm][ncells]
  const double* sc_lnc = scratch + (size_t)(ns + nm) * ncells;     // [n][ncells]

  // per-lane state
  int phase = NEED;
  long long cell = -1;
  double c[N], lnc[N], g[N], tot[N];
  double fixed[N], init_tot[N], guess[N], lnguess[N], small_val[N];
  double Ksec[PF_MAX_NSEC];
  double Kmin[PF_MAX_NMNRL], rate[PF_MAX_NMNRL], vf[PF_MAX_NMNRL];
  double psv = 0, den_L = 0, den_k = 0, volume = 0, target = 0, cum = 0, dt = 0, inv_dt = 0, r0 = 0;
  double temp = 25.0;
  double sqI = 0.0, lgI = 0.0;  // ionic strength of the last evaluation (NEWTON_ITER activity)
  bool dry = false;
  // LDL^T unless a pivot failed on this evaluation (then it is redone, its
  // count unchanged, with the pivoted LU) or activity coefficients follow
  // each iteration (a redone evaluation would see this one's complexes)
  bool use_lu = false, redo = false;
  // adjoint state (ADJ): converged iterate and dt of every substep, the
  // running dL/dT, direct dL/dT0 of floored components, per-lane gradient
  // accumulators for the network parameters, per-cell area gradient
  constexpr int SMAX = ADJ ? PF_ADJ_MAX_SUBSTEPS : 1;
  constexpr int SADJ = ADJ ? PF_MAX_NSEC : 1;
  constexpr int MADJ = ADJ ? PF_MAX_NMNRL : 1;
  double cst[SMAX][N], dts[SMAX];
  double Tbar[N], gdir[N];
  double sloc[SADJ], mImV[MADJ], mdQ[MADJ];
  double gK[SADJ], gKm[MADJ], glnk[MADJ], garea[MADJ];
  double loss_acc = 0.0;
  int sb = 0;
  if constexpr (ADJ) {
    for (int i = 0; i < ns; ++i) gK[i] = 0.0;
    for (int m = 0; m < nm; ++m) { gKm[m] = 0.0; glnk[m] = 0.0; }
  }
  int its = 0, its_total = 0, nsub = 0, num_cuts = 0, n_const = 0;
  unsigned small_mask = 0;
  bool zero_step = false;
  unsigned long long my_its = 0, my_fail = 0, my_maxits = 0, my_maxsub = 0;

  for (;;) {
    // ---------------------------------------------------- work-queue refill
    const unsigned need = __ballot_sync(FULL, phase == NEED);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane_id == leader) base = atomicAdd(queue, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (phase == NEED) {
        const long long q = (long long)(base + __popc(need & ((1u << lane_id) - 1u)));
        phase = (q < ncells) ? START : DONE;
        if (phase == START) {
          cell = st.cell_order ? (long long)st.cell_order[q] : q;
          // load the cell: pure loads, the transcendentals were done by the pre-pass
          const double por = st.porosity[cell], sat = st.saturation[cell];
          den_k = st.den_kg[cell];
          volume = st.volume[cell];
          temp = st.temperature ? st.temperature[cell] : 25.0;
          dry = sat < RT_MIN_SATURATION;
          psv = por * sat * 1000.0 * volume;
          den_L = den_k * 1.0e-3;
          small_mask = 0;
#pragma unroll
          for (int j = 0; j < N; ++j) {
            double t = st.total[soa.at(j, cell)];
            if (t <= 1.0e-40) {  // RStep floor (reaction.F90:3618-3624)
              small_mask |= 1u << j;
              small_val[j] = t;
              t = 1.0e-40;
            }
            tot[j] = t;
            guess[j] = o.use_total_as_guess ? t : st.pri_molal[soa.at(j, cell)];
            lnguess[j] = sc_lnc[soa.at(j, cell)];
            g[j] = st.pri_act_coef[soa.at(j, cell)];
          }
          for (int i = 0; i < ns; ++i) Ksec[i] = sc_sec[soa.at(i, cell)];
          for (int m = 0; m < nm; ++m) {
            Kmin[m] = sc_min[soa.at(m, cell)];
            vf[m] = st.mnrl_volfrac[soa.at(m, cell)];
            rate[m] = 0.0;
          }
          target = st.dt_cell ? st.dt_cell[cell] : dt_uniform;
          cum = 0.0;
          dt = target;
          its_total = 0;
          nsub = 0;
          num_cuts = 0;
          n_const = 0;
          zero_step = !(cum < target);  // nothing to integrate: write back as is
#pragma unroll
          for (int j = 0; j < N; ++j) c[j] = guess[j];
        }
      }
    }
    if (__all_sync(FULL, phase == DONE)) break;

    bool finish_cell = false, cell_failed = false;
    bool back_done_flag = false, back_fail_flag = false;
    if (zero_step) {
      finish_cell = true;
      zero_step = false;
      phase = NEED;
    }

    // --------------------------------------------------------- RReact start
    if (phase == START) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        fixed[j] = dry ? 0.0 : psv * tot[j];
        init_tot[j] = tot[j];
        c[j] = guess[j];
        lnc[j] = lnguess[j];
      }
      if (has_sorb) {
        // RAccumulationSorb into the fixed accumulation (reaction.F90:3836-3839):
        // the sorbed total of the last evaluation, as the reference keeps it
#pragma unroll
        for (int j = 0; j < N; ++j) fixed[j] = fma(st.total_sorb[soa.at(j, cell)], volume, fixed[j]);
      }
      its = 0;
      r0 = 0.0;
      inv_dt = 1.0 / dt;
      phase = ITER;
    }

    // ------------------------------------------------------- Newton trip
    if (phase == ITER || (ADJ && phase == BACK)) {
      // A backward trip (adjoint, BACK) shares the evaluation and the
      // factorisation with a forward Newton trip: at the converged iterate of
      // substep sb it solves J^T lambda = (dT/dlnm)^T Tbar with the true
      // Jacobian (J is symmetric in the log formulation), then accumulates
      // the parameter gradients.
      const bool back = ADJ && phase == BACK;
      if (!back && !redo) its += 1;
      redo = false;
      // LDL^T needs the symmetric log-form Jacobian; the reference's surface
      // complexation derivative is not symmetric (its free-site term takes
      // nu_f for nu_f^2 and only the complex's own species), so networks
      // with surface complexes keep the pivoted LU
      const bool ldl = (logf || back || dry) && !use_lu && !newton_iter_act && !(net.nsrx > 0 && !back);
      if (newton_iter_act) {
        // RActivityCoefficients LAG (reaction.F90:4553-4612) from this
        // iterate and the previous evaluation's sec_molal
        double I = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) I = I + c[j] * T.pri_Z(j) * T.pri_Z(j);
        for (int i = 0; i < ns; ++i) {
          const double z = T.sec_Z(i);
          I = I + st.sec_molal[soa.at(i, cell)] * z * z;
        }
        I = 0.5 * I;
        sqI = sqrt(I);
        lgI = I;
#pragma unroll
        for (int j = 0; j < N; ++j) g[j] = exp(dh_ln_gamma(T.pri_Z(j), T.pri_a0(j), sqI, I, net));
      }
      // ---- power table and RTotalAqueous in product form -----------------
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const double a = c[j] * g[j];
        L.P(j) = a;
        L.P(N + j) = a * a;
        if (neg_mask & (1u << j)) {
          const double ia = 1.0 / a;
          L.P(2 * N + j) = ia;
          L.P(3 * N + j) = ia * ia;
        }
        L.S(j) = 0.0;
      }
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) L.J(i, j) = 0.0;
      const double a_acc = dry ? 1.0 : psv * inv_dt * den_L;  // psvd_t * den_kg_per_L
      for (int i = 0; i < ns; ++i) {
        const int b = T.sec_begin(i), e = T.sec_end(i);
        double s = newton_iter_act
                       ? exp(Ksec[i] - dh_ln_gamma(T.sec_Z(i), T.sec_a0(i), sqI, lgI, net))
                       : Ksec[i];
        for (int p = b; p < e; ++p) {
          const int pe = T.sec_pidx(p);
          s *= (pe >= 0) ? L.P(pe) : exp(T.sec_nu(p) * log(L.P(T.sec_idx(p))));
        }
        if (back) {
          if constexpr (ADJ) sloc[i] = s;
        } else {
          st.sec_molal[soa.at(i, cell)] = s;
        }
        const double sa = a_acc * s;
        for (int p = b; p < e; ++p) {
          const int kp = T.sec_idx(p);
          L.S(kp) = fma(T.sec_nu(p), sa, L.S(kp));
        }
        for (int q = T.spair_begin(i); q < T.spair_begin(i + 1); ++q) {
          const int f = T.spair_idx(q);
          L.Jf(f) = fma(T.spair_coef(q), sa, L.Jf(f));
        }
      }
      const double b_tot = den_L / a_acc;
      if (!back) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          tot[j] = fma(b_tot, L.S(j), den_L * c[j]);
          L.rhs(j) = dry ? 0.0 : fma(a_acc, c[j], L.S(j)) - fixed[j] * inv_dt;
        }
      }
      if (dry && !back) {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
          for (int j = 0; j < N; ++j) L.J(i, j) = (i == j) ? (logf ? c[j] : 1.0) : 0.0;
      } else if (logf || back) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          if (!ldl) {  // LDL^T reads the upper triangle only
#pragma unroll
            for (int j = 0; j < i; ++j) L.J(i, j) = L.J(j, i);
          }
          L.J(i, i) = fma(a_acc, c[i], L.J(i, i));
        }
        if (back) {
          // the backward solve is J u = B Tbar with B the minerals' part of
          // J (u = Tbar - (psv/dt) lambda, formed without cancellation);
          // Tbar by species id for the mineral loop goes to S
#pragma unroll
          for (int i = 0; i < N; ++i) {
            L.rhs(i) = 0.0;
            L.S(i) = Tbar[i];
          }
        }
      } else {
        // linear formulation: d/dm_j = column j of G divided by m_j
        double ic[N];
#pragma unroll
        for (int j = 0; j < N; ++j) ic[j] = 1.0 / c[j];
#pragma unroll
        for (int i = 0; i < N; ++i) {
#pragma unroll
          for (int j = 0; j < i; ++j) {
            const double gv = L.J(j, i);
            L.J(i, j) = gv * ic[j];
            L.J(j, i) = gv * ic[i];
          }
          L.J(i, i) = fma(L.J(i, i), ic[i], a_acc);
        }
        // mineral columns below also need 1/m_j by species id: park it in S
#pragma unroll
        for (int j = 0; j < N; ++j) L.S(j) = ic[j];
      }
      // ---- RKineticMineral (reaction_mineral.F90:647-1078) ---------------
      for (int m = 0; m < nm; ++m) {
        const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
        if (!back) rate[m] = 0.0;
        if constexpr (ADJ) { mImV[m] = 0.0; mdQ[m] = 0.0; }
        double QK = Kmin[m];
        for (int p = b; p < e; ++p) {
          const int pe = T.mnrl_pidx(p);
          QK *= (pe >= 0) ? L.P(pe) : exp(T.mnrl_nu(p) * log(L.P(T.mnrl_idx(p))));
        }
        double aff;
        if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
        else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
        else aff = 1.0 - QK;
        const double sign_ = fsign1(aff);
        if (!(vf[m] > 0 || sign_ < 0.0)) continue;
        if (T.irreversible(m) == 1 && sign_ < 0.0) continue;
        if (T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m)) continue;
        const double rl = T.limiter(m);
        if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
        double arr = 1.0;
        if (T.ea(m) > 0.0)
          arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp + 273.15)));
        const double k = T.rate(m) * arr;
        double Im_const = -st.mnrl_area[soa.at(m, cell)];
        if (has_msf) Im_const = Im_const / T.msf(m);
        double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * k : Im_const * sign_ * fabs(aff) * k;
        if (!back) rate[m] = Im;
        if (dry) continue;  // RReaction returns before minerals in a dry cell
        Im_const = Im_const * volume;
        Im = Im * volume;
        double dIm_dQK = has_pw ? -Im * T.power(m) / fabs(aff) : -Im_const * k;
        if (has_tk)
          dIm_dQK = dIm_dQK * (1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m))) / QK * (1.0 - aff);
        else if (has_msf)
          dIm_dQK = dIm_dQK * (1.0 / T.msf(m)) / QK * (1.0 - aff);
        // dIm/dQK * QK with the rate-limiter chain rule: the true d Im / d ln Q
        double ft = dIm_dQK * QK;
        if (rl > 0.0) {
          const double den = 1.0 + (1.0 - aff) / rl;
          ft = ft * (1.0 + QK / rl / den) / den;
        }
        // the reference's Jacobian multiplies dQK/dm by den*1e-3
        // (reaction_mineral.F90:944-947), treating molality as molarity;
        // Newton keeps it (same iterates), the adjoint uses the derivative
        const double f = back ? ft : ft * den_k * 1.0e-3;
        if constexpr (ADJ) {
          mImV[m] = Im;
          mdQ[m] = ft;
        }
        if (!back) {
          for (int p = b; p < e; ++p) L.rhs(T.mnrl_idx(p)) = fma(T.mnrl_nu(p), Im, L.rhs(T.mnrl_idx(p)));
        } else {
          double nuT = 0.0;
          for (int p = b; p < e; ++p) nuT = fma(T.mnrl_nu(p), L.S(T.mnrl_idx(p)), nuT);
          for (int p = b; p < e; ++p)
            L.rhs(T.mnrl_idx(p)) = fma(T.mnrl_nu(p) * f, nuT, L.rhs(T.mnrl_idx(p)));
        }
        // d R / d ln m (log form: the m_q of the column scale cancels 1/m_q)
        for (int q = T.mpair_begin(m); q < T.mpair_begin(m + 1); ++q) {
          const int fl = T.mpair_idx(q);
          const double v = T.mpair_coef(q) * f;
          L.Jf(fl) = fma(v, (logf || back) ? 1.0 : L.S(fl % N), L.Jf(fl));
        }
      }
      // ---- equilibrium sorption: RTotalSorb inside RTAuxVarCompute, with
      // RAccumulationSorb[Derivative] (reaction.F90:3861-3865, 3904-3909).
      // The power table is dead after the minerals: it holds molality and
      // gamma by species for the sorption routine.
      bool sorb_fail = false;
      if (has_sorb && !back) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          L.P(N + j) = c[j];
          L.P(2 * N + j) = g[j];
          st.total_sorb[soa.at(j, cell)] = 0.0;
        }
        const double v_t = volume * inv_dt;
        sorb_fail = !total_sorb(
            net, T, [&](int j) { return L.P(N + j); }, [&](int j) { return L.P(2 * N + j); },
            [&](int m) { return vf[m]; }, st.porosity[cell], den_k,
            st.ionx_ref_sorbed ? st.ionx_ref_sorbed + cell : nullptr, ncells,
            [&](int j, double v) {
              st.total_sorb[soa.at(j, cell)] += v;
              L.rhs(j) = fma(v_t, v, L.rhs(j));
            },
            [&](int i, int j, double v) { L.J(i, j) = fma(v_t * v, logf ? L.P(N + j) : 1.0, L.J(i, j)); },
            surf_cell(net, st, cell));
      }
      // ---- convergence tests on the residual (reaction.F90:3946-3953) -----
      double dot = 0.0;
      unsigned long long mxb = 0;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const double r = L.rhs(j);
        dot = fma(r, r, dot);
        mxb = max(mxb, absbits(r));
      }
      const double two_norm = sqrt(dot);
      if (its == 1) r0 = two_norm;
      int react_end = -1;  // -1: continue, 0: converged, 1: failed
      bool back_done = false, back_fail = false;
      if (back) {
        const int fr = ldl ? ldl_solve<N, JS>(L) : lu_solve<N, JS>(L, indx, stride);
        if (!ldl) use_lu = false;
        if (ldl && fr) {
          use_lu = true;
          redo = true;
        } else if (fr) {
          back_fail = true;
        } else if constexpr (ADJ) {
          // u = rhs; lambda = (Tbar - u)/(psv/dt).  theta_bar += (dT/dtheta)^T u
          // - (dR/dtheta)^T lambda;  Tbar(previous substep) = Tbar - u
          const double pd = a_acc / den_L;
          const double ipd = 1.0 / pd;
#pragma unroll
          for (int j = 0; j < N; ++j) {
            L.S(j) = L.rhs(j);                       // u
            L.rhs(j) = (Tbar[j] - L.rhs(j)) * ipd;   // lambda
          }
          for (int i = 0; i < ns; ++i) {
            double acc = 0.0;
            for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) acc = fma(T.sec_nu(p), L.S(T.sec_idx(p)), acc);
            gK[i] = fma(acc, -LOG_TO_LN * den_L * sloc[i], gK[i]);
          }
          for (int m = 0; m < nm; ++m) {
            if (mImV[m] == 0.0 && mdQ[m] == 0.0) continue;
            double lam = 0.0;
            for (int p = T.mnrl_begin(m); p < T.mnrl_end(m); ++p)
              lam = fma(T.mnrl_nu(p), L.rhs(T.mnrl_idx(p)), lam);
            gKm[m] = fma(LOG_TO_LN * mdQ[m], lam, gKm[m]);
            glnk[m] = fma(-mImV[m], lam, glnk[m]);
            garea[m] = fma(-mImV[m], lam, garea[m]);
          }
#pragma unroll
          for (int j = 0; j < N; ++j) Tbar[j] = Tbar[j] - L.S(j);
          sb -= 1;
          if (sb >= 0) {
#pragma unroll
            for (int j = 0; j < N; ++j) c[j] = cst[sb][j];
            inv_dt = 1.0 / dts[sb];
          } else {
            back_done = true;
          }
        }
      } else if (sorb_fail) {
        react_end = 1;  // RTAuxVarCompute's ierror: no total restore (reaction.F90:3861-3865)
      } else if (its > o.maximum_reaction_iterations) {
#pragma unroll
        for (int j = 0; j < N; ++j) tot[j] = init_tot[j];
        react_end = 1;
      } else if (__longlong_as_double((long long)mxb) < o.max_residual_tolerance ||
                 two_norm < o.max_rel_residual_tolerance * r0) {
        react_end = 0;
      } else {
        const int fr = ldl ? ldl_solve<N, JS>(L) : lu_solve<N, JS>(L, indx, stride);
        if (!ldl) use_lu = false;
        if (ldl && fr) {
          use_lu = true;  // react_end stays -1: the evaluation repeats with the pivoted LU
          redo = true;
        } else if (fr) {
          react_end = 1;  // singular: no total restore (reaction.F90:3963-3966)
        } else {
          const double tol = o.max_relative_change_tolerance;
          bool small = true;
          double nc[N], u[N];
#pragma unroll
          for (int j = 0; j < N; ++j) u[j] = o.fork_literal_rsolve ? 0.0 : L.rhs(j);
          if (logf) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
              u[j] = fmin(fmax(u[j], -o.max_dlnC_rreact), o.max_dlnC_rreact);
              nc[j] = c[j] * exp(-u[j]);
            }
          } else {
            double min_ratio = 1.7976931348623157e308;
#pragma unroll
            for (int j = 0; j < N; ++j)
              if (c[j] <= u[j]) min_ratio = fmin(min_ratio, fabs(c[j] / u[j]));
#pragma unroll
            for (int j = 0; j < N; ++j) nc[j] = c[j] - (min_ratio < 1.0 ? u[j] * min_ratio * 0.99 : u[j]);
          }
#pragma unroll
          for (int j = 0; j < N; ++j) small = small && (absbits(nc[j] - c[j]) < absbits(tol * c[j]));
          if (small) {
            react_end = 0;
          } else {
#pragma unroll
            for (int j = 0; j < N; ++j) {
              lnc[j] = logf ? lnc[j] - u[j] : log(nc[j]);
              c[j] = nc[j];
            }
          }
        }
      }
      back_done_flag = back_done;
      back_fail_flag = back_fail;
      // ------------------------------------------------ RStep bookkeeping
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
          for (int m = 0; m < nm; ++m) {  // MineralUpdateKineticState
            const double v = vf[m] + rate[m] * T.molar_vol(m) * dt;
            vf[m] = v < 0.0 ? 0.0 : v;
          }
          if constexpr (ADJ) {
            if (nsub < SMAX) {
#pragma unroll
              for (int j = 0; j < N; ++j) cst[nsub][j] = c[j];
              dts[nsub] = dt;
            }
          }
          cum = cum + dt;
          nsub += 1;
          n_const += 1;
#pragma unroll
          for (int j = 0; j < N; ++j) {
            guess[j] = c[j];
            lnguess[j] = lnc[j];
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
      if (phase == BACK && (back_done_flag || back_fail_flag)) {
#pragma unroll
        for (int j = 0; j < N; ++j)
          adj.dL_dtotal0[soa.at(j, cell)] =
              back_fail_flag ? 0.0 : ((small_mask & (1u << j)) ? gdir[j] : Tbar[j]);
        for (int m = 0; m < nm; ++m) adj.dL_dlnarea[soa.at(m, cell)] = back_fail_flag ? 0.0 : garea[m];
        if (adj.adj_status) adj.adj_status[cell] = back_fail_flag ? 3 : 0;
        back_done_flag = back_fail_flag = false;
        phase = NEED;
      }
    }

    // ------------------------------------------------------ cell write-back
    if (finish_cell) {
      if (!cell_failed) {
#pragma unroll
        for (int j = 0; j < N; ++j)
          if (small_mask & (1u << j)) tot[j] = small_val[j];
      }
#pragma unroll
      for (int j = 0; j < N; ++j) {
        st.total[soa.at(j, cell)] = tot[j];
        st.pri_molal[soa.at(j, cell)] = c[j];
        if (newton_iter_act) st.pri_act_coef[soa.at(j, cell)] = g[j];
      }
      if (newton_iter_act) {
        // gamma of the complexes at the last evaluation's ionic strength
        for (int i = 0; i < ns; ++i)
          st.sec_act_coef[soa.at(i, cell)] = exp(dh_ln_gamma(T.sec_Z(i), T.sec_a0(i), sqI, lgI, net));
      }
      for (int m = 0; m < nm; ++m) {
        st.mnrl_volfrac[soa.at(m, cell)] = vf[m];
        st.mnrl_rate[soa.at(m, cell)] = rate[m];
      }
      if (st.status) st.status[cell] = cell_failed ? PF_CELL_TOO_MANY_CUTS : PF_CELL_OK;
      if (st.newton_its) st.newton_its[cell] = its_total;
      if (st.num_substeps) st.num_substeps[cell] = nsub;
      my_its += (unsigned long long)its_total;
      my_fail += cell_failed ? 1ull : 0ull;
      my_maxits = max(my_maxits, (unsigned long long)its_total);
      my_maxsub = max(my_maxsub, (unsigned long long)nsub);
      phase = NEED;
      if constexpr (ADJ) {
        // loss contribution and dL/dT(final); start the backward pass
        double gsum = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) {
          double gj;
          if (adj.weight) {
            const double w = adj.weight[soa.at(j, cell)], d = tot[j] - adj.target[soa.at(j, cell)];
            loss_acc = fma(w * d, d, loss_acc);
            gj = 2.0 * w * d;
          } else {
            gj = adj.dL_dtotal[soa.at(j, cell)];
          }
          // a floored component's final total is its restored input
          // (reaction.F90:3721-3725): dL/dT0 directly, no path through m
          const bool fl = small_mask & (1u << j);
          gdir[j] = fl ? gj : 0.0;
          Tbar[j] = fl ? 0.0 : gj;
          gsum += fabs(gj);
        }
        for (int m = 0; m < nm; ++m) garea[m] = 0.0;
        const int astat = cell_failed ? 1 : (nsub > SMAX ? 2 : 0);
        if (astat != 0 || dry || nsub == 0) {
#pragma unroll
          for (int j = 0; j < N; ++j) adj.dL_dtotal0[soa.at(j, cell)] = (astat == 0) ? gdir[j] : 0.0;
          for (int m = 0; m < nm; ++m) adj.dL_dlnarea[soa.at(m, cell)] = 0.0;
          if (adj.adj_status) adj.adj_status[cell] = astat;
        } else {
          (void)gsum;
          sb = nsub - 1;
#pragma unroll
          for (int j = 0; j < N; ++j) c[j] = cst[sb][j];
          inv_dt = 1.0 / dts[sb];
          phase = BACK;
        }
      }
    }
  }
  if constexpr (ADJ) {
    // network-parameter gradients and the loss: warp sums, one atomic each
    auto wsum = [&](double v) {
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
      return v;
    };
    for (int i = 0; i < ns; ++i) {
      const double v = wsum(gK[i]);
      if (lane_id == 0 && v != 0.0) atomicAdd(&adj.dL_dlogK_sec[i], v);
    }
    for (int m = 0; m < nm; ++m) {
      const double a = wsum(gKm[m]), b = wsum(glnk[m]);
      if (lane_id == 0) {
        if (a != 0.0) atomicAdd(&adj.dL_dlogK_mnrl[m], a);
        if (b != 0.0) atomicAdd(&adj.dL_dlnk[m], b);
      }
    }
    const double l = wsum(loss_acc);
    if (lane_id == 0 && adj.loss && l != 0.0) atomicAdd(adj.loss, l);
  }
  if (counters) {
    // warp-level reduction, one atomic per warp
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

}  // namespace batched

template <int N, bool JS, bool ADJ>
int launch_batched_k(const DevNet& net, const PfCellState& st, double dt, size_t smem, int grid, int tpb,
                     const double* scratch, unsigned long long* queue, unsigned long long* counters,
                     const PfAdjointArgs& adj, cudaStream_t stream) {
  auto k = batched::rstep_batched_kernel<N, JS, ADJ>;
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return (int)err;
  k<<<grid, tpb, smem, stream>>>(net, st, dt, scratch, queue, counters, adj);
  return (int)cudaGetLastError();
}

// forward variants (Jacobian in shared or local memory) and adjoint variants
// live in separate translation units so that they compile in parallel
template <int N>
int launch_batched_fwd(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                       int num_sms, const double* scratch, unsigned long long* queue,
                       unsigned long long* counters, cudaStream_t stream) {
  const size_t smem = batched_smem_bytes(net, cfg);
  const int tpb = cfg.threads_per_block;
  const int grid = num_sms * cfg.blocks_per_sm;
  const PfAdjointArgs none{};
  if (cfg.jac_in_shared)
    return launch_batched_k<N, true, false>(net, st, dt, smem, grid, tpb, scratch, queue, counters, none, stream);
  return launch_batched_k<N, false, false>(net, st, dt, smem, grid, tpb, scratch, queue, counters, none, stream);
}

template <int N>
int launch_batched_adj(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                       int num_sms, const double* scratch, unsigned long long* queue,
                       unsigned long long* counters, const PfAdjointArgs& adj, cudaStream_t stream) {
  const size_t smem = batched_smem_bytes(net, cfg);
  const int tpb = cfg.threads_per_block;
  const int grid = num_sms * cfg.blocks_per_sm;
  if (cfg.jac_in_shared)
    return launch_batched_k<N, true, true>(net, st, dt, smem, grid, tpb, scratch, queue, counters, adj, stream);
  return launch_batched_k<N, false, true>(net, st, dt, smem, grid, tpb, scratch, queue, counters, adj, stream);
}

}  // namespace pfgpu
