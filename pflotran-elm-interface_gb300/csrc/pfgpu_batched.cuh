// pfgpu_batched.cuh -- batched persistent operator-split reaction kernel.
//
// Same step as RStep/RReact (src/pflotran/reaction.F90:3564-4055) per cell,
// organised for GB300's FP64 pipe:
//   * one lane per cell, ncomp a compile-time constant (all n-indexed loops
//     unroll; c, ln c, ln gamma and totals live in registers);
//   * persistent grid with a device work queue: a lane whose cell finished
//     takes the next cell at the top of the following Newton trip, so lanes
//     with different Newton/substep counts do not idle (warp-aggregated
//     atomicAdd; the queue index only grows, so the loop is bounded);
//   * reaction tables staged once per block into shared memory with a bulk
//     TMA copy (cp.async.bulk + mbarrier, bounded wait);
//   * per-lane vectors indexed by species id (ln a, secondary sums, rhs,
//     pivot scales) and the Jacobian in shared memory, thread-strided so a
//     warp's accesses are bank-conflict free (the Jacobian can be placed in
//     local memory instead for large ncomp; chosen by the autotuner);
//   * FP64 work reduced without changing the mathematics:
//       - d total/d c (reaction.F90:4731-4744) uses exp(lnQK - ln m_j)/gamma_i
//         = s_i/m_j, and in the log formulation RSolve multiplies column j by
//         m_j (:5494-5499), so the log-space Jacobian column is
//         den*(delta_kj m_j + sum_i nu_ik nu_ij s_i): no per-pair exp, no 1/m;
//       - ln m is carried through the log update (ln m <- ln m - u) instead of
//         re-taking log(m) every evaluation; ln gamma_i and logK(T) fold into
//         one per-cell constant per secondary;
//       - the Crout LU's implicit pivot scaling (utility.F90:621-666) makes the
//         pivot sequence invariant to RSolve's explicit row normalisation
//         (:5486-5492), which is therefore folded away;
//       - RReact's final RTAuxVarCompute (:4052) and MineralUpdateKineticState's
//         rate evaluation (reaction_mineral.F90:1490) are at the iterate of the
//         last evaluation, so both reuse it.
#pragma once
#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

namespace pfgpu {
namespace batched {

constexpr unsigned FULL = 0xffffffffu;
constexpr long long TMA_WAIT_LIMIT = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

enum Phase : int { NEED = 0, START = 1, ITER = 2, DONE = 3 };

template <int N, bool JS>
struct Lane {
  // thread-strided shared-memory vectors: element e of this lane at p[e*stride]
  double* base;
  int stride;
  double* Jl;  // local-memory Jacobian when !JS
  __device__ __forceinline__ double& J(int i, int j) {
    if constexpr (JS) return base[(i * N + j) * stride];
    else return Jl[i * N + j];
  }
  static constexpr int OFF = JS ? N * N : 0;
  __device__ __forceinline__ double& lna(int j) { return base[(OFF + j) * stride]; }
  // S (secondary sums, live during the evaluation) and VV (pivot scales, live
  // during the factorisation) share one slot
  __device__ __forceinline__ double& S(int j) { return base[(OFF + N + j) * stride]; }
  __device__ __forceinline__ double& VV(int j) { return base[(OFF + N + j) * stride]; }
  __device__ __forceinline__ double& rhs(int j) { return base[(OFF + 2 * N + j) * stride]; }
  static constexpr int DOUBLES = OFF + 3 * N;
};

// Crout LU with implicit partial pivoting (utility.F90:597-688) on the lane's
// Jacobian, then the solve (utility.F90:692-735) in place on rhs.  The
// reciprocal of each pivot is kept in VV(j) once row j is final.
template <int N, bool JS>
__device__ __forceinline__ int lu_solve(Lane<N, JS>& L, int* indx, int stride) {
#pragma unroll 1
  for (int i = 0; i < N; ++i) {
    double aamax = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j) aamax = fmax(aamax, fabs(L.J(i, j)));
    if (!(aamax > 0.0)) return 1;
    L.VV(i) = 1.0 / aamax;
  }
#pragma unroll 1
  for (int j = 0; j < N; ++j) {
#pragma unroll 1
    for (int i = 1; i < j; ++i) {
      double sum = L.J(i, j);
      for (int k = 0; k < i; ++k) sum = fma(-L.J(i, k), L.J(k, j), sum);
      L.J(i, j) = sum;
    }
    double aamax = 0.0;
    int imax = j;
#pragma unroll 1
    for (int i = j; i < N; ++i) {
      double sum = L.J(i, j);
      for (int k = 0; k < j; ++k) sum = fma(-L.J(i, k), L.J(k, j), sum);
      L.J(i, j) = sum;
      double dum = L.VV(i) * fabs(sum);
      if (dum >= aamax) { imax = i; aamax = dum; }
    }
    // unconditional swap (a no-op when imax == j) keeps the warp converged
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double a = L.J(imax, k), b = L.J(j, k);
      L.J(imax, k) = b;
      L.J(j, k) = a;
    }
    L.VV(imax) = L.VV(j);
    indx[j * stride] = imax;
    double piv = L.J(j, j);
    if (piv == 0.0) { piv = 1.0e-20; L.J(j, j) = piv; }
    const double rp = 1.0 / piv;
    L.VV(j) = rp;
#pragma unroll 1
    for (int i = j + 1; i < N; ++i) L.J(i, j) = L.J(i, j) * rp;
  }
  // forward substitution with the row interchanges
#pragma unroll 1
  for (int i = 0; i < N; ++i) {
    const int ll = indx[i * stride];
    double sum = L.rhs(ll);
    L.rhs(ll) = L.rhs(i);
    for (int j = 0; j < i; ++j) sum = fma(-L.J(i, j), L.rhs(j), sum);
    L.rhs(i) = sum;
  }
#pragma unroll 1
  for (int i = N - 1; i >= 0; --i) {
    double sum = L.rhs(i);
    for (int j = i + 1; j < N; ++j) sum = fma(-L.J(i, j), L.rhs(j), sum);
    L.rhs(i) = sum * L.VV(i);
  }
  return 0;
}

template <int N, bool JS>
__global__ void __launch_bounds__(256)
rstep_batched_kernel(DevNet net, PfCellState st, double dt_uniform, unsigned long long* queue,
                     unsigned long long* counters) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t tma_bar;
  const int tid = threadIdx.x;
  const int lane_id = tid & 31;
  const int stride = blockDim.x;
  const uint32_t ibytes = (uint32_t)net.int_words * 4u;   // multiple of 16 (host pads)
  const uint32_t dbytes = (uint32_t)net.dbl_words * 8u;   // multiple of 16 (host pads)
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
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(sI)),
        "l"(net.ints), "r"(ibytes), "r"(smem_u32(&tma_bar))
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
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
    // every thread saw the same barrier; a timeout (never expected) flags the
    // launch and leaves without touching any cell
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
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN,
             has_pw = net.flags & NETF_POWER;
  const bool iso = o.isothermal != 0;
  const bool logf = o.use_log_formulation != 0;
  const bool newton_iter_act = o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER;

  // per-lane state
  int phase = NEED;
  long long cell = -1;
  double c[N], lnc[N], lng[N], tot[N];
  double fixed[N], init_tot[N], guess[N], small_val[N];
  double lnKeff[PF_MAX_NSEC];
  double lnKm[PF_MAX_NMNRL], rate[PF_MAX_NMNRL], vf[PF_MAX_NMNRL];
  double psv = 0, den_L = 0, den_k = 0, volume = 0, target = 0, cum = 0, dt = 0, inv_dt = 0, r0 = 0;
  double temp = 25.0;
  bool dry = false;
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
        cell = (long long)(base + __popc(need & ((1u << lane_id) - 1u)));
        phase = (cell < st.ncells) ? START : DONE;
        if (phase == START) {
          // load the cell (gather; rows are component-major)
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
            guess[j] = st.pri_molal[soa.at(j, cell)];
            lng[j] = log(st.pri_act_coef[soa.at(j, cell)]);
          }
          if (o.use_total_as_guess) {
#pragma unroll
            for (int j = 0; j < N; ++j) guess[j] = tot[j];
          }
          const double tk = temp + 273.15;
          const bool tsec = !iso && (net.flags & NETF_SEC_LOGKCOEF);
          const bool tmin = !iso && (net.flags & NETF_MNRL_LOGKCOEF);
          for (int i = 0; i < ns; ++i) {
            const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
            const double g = st.sec_act_coef[soa.at(i, cell)];
            lnKeff[i] = -logK * LOG_TO_LN - (g == 1.0 ? 0.0 : log(g));
          }
          for (int m = 0; m < nm; ++m) {
            const double logK = tmin ? interp_logK(T.mnrl_logKcoef(m), temp) : T.mnrl_logK(m);
            lnKm[m] = -logK * LOG_TO_LN;
            vf[m] = st.mnrl_volfrac[soa.at(m, cell)];
            rate[m] = 0.0;
          }
          (void)tk;
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
        lnc[j] = log(c[j]);
      }
      its = 0;
      r0 = 0.0;
      inv_dt = 1.0 / dt;
      phase = ITER;
    }

    // ------------------------------------------------------- Newton trip
    if (phase == ITER) {
      its += 1;
      if (newton_iter_act) {
        // RActivityCoefficients LAG (reaction.F90:4553-4612) from this
        // iterate's molalities and the previous evaluation's sec_molal
        double I = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) I = I + c[j] * T.pri_Z(j) * T.pri_Z(j);
        for (int i = 0; i < ns; ++i) {
          const double z = T.sec_Z(i);
          I = I + st.sec_molal[soa.at(i, cell)] * z * z;
        }
        I = 0.5 * I;
        const double sI_ = sqrt(I);
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const double z = T.pri_Z(j);
          lng[j] = fabs(z) > 1.0e-10
                       ? (-z * z * sI_ * net.A / (1.0 + T.pri_a0(j) * net.B * sI_) + net.Bdot * I) * LOG_TO_LN
                       : 0.0;
        }
        const bool tsec = !iso && (net.flags & NETF_SEC_LOGKCOEF);
        for (int i = 0; i < ns; ++i) {
          const double z = T.sec_Z(i);
          const double lg = fabs(z) > 1.0e-10
                                ? (-z * z * sI_ * net.A / (1.0 + T.sec_a0(i) * net.B * sI_) + net.Bdot * I) *
                                      LOG_TO_LN
                                : 0.0;
          const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
          lnKeff[i] = -logK * LOG_TO_LN - lg;
        }
      }
      // ---- RTotalAqueous in the factored form ---------------------------
#pragma unroll
      for (int j = 0; j < N; ++j) {
        L.lna(j) = lnc[j] + lng[j];
        L.S(j) = 0.0;
      }
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) L.J(i, j) = 0.0;
      for (int i = 0; i < ns; ++i) {
        const int b = T.sec_begin(i), e = T.sec_end(i);
        double lnQK = lnKeff[i];
        for (int p = b; p < e; ++p) lnQK = fma(T.sec_nu(p), L.lna(T.sec_idx(p)), lnQK);
        const double s = exp(lnQK);
        st.sec_molal[soa.at(i, cell)] = s;
        for (int p = b; p < e; ++p) {
          const int kp = T.sec_idx(p);
          const double t = T.sec_nu(p) * s;
          L.S(kp) = L.S(kp) + t;
          for (int q = b; q < e; ++q) {
            const int kq = T.sec_idx(q);
            L.J(kp, kq) = fma(T.sec_nu(q), t, L.J(kp, kq));
          }
        }
      }
      const double a = psv * inv_dt * den_L;  // psvd_t * den_kg_per_L
#pragma unroll
      for (int j = 0; j < N; ++j) {
        tot[j] = (c[j] + L.S(j)) * den_L;
        L.rhs(j) = dry ? -fixed[j] * inv_dt : (psv * tot[j] - fixed[j]) * inv_dt;
      }
      if (dry) {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
          for (int j = 0; j < N; ++j) L.J(i, j) = (i == j) ? (logf ? c[j] : 1.0) : 0.0;
      } else if (logf) {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
          for (int j = 0; j < N; ++j) L.J(i, j) = (i == j) ? a * (c[j] + L.J(i, j)) : a * L.J(i, j);
      } else {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const double aic = a / c[j];
#pragma unroll
          for (int i = 0; i < N; ++i) L.J(i, j) = (i == j) ? a + aic * L.J(i, j) : aic * L.J(i, j);
        }
      }
      // ---- RKineticMineral (reaction_mineral.F90:647-1078) -----------------
      if (!logf && nm > 0) {
#pragma unroll
        for (int j = 0; j < N; ++j) L.VV(j) = 1.0 / c[j];  // exp(-ln_conc) by species id
      }
      for (int m = 0; m < nm; ++m) {
        const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
        rate[m] = 0.0;
        double lnQK = lnKm[m];
        for (int p = b; p < e; ++p) lnQK = fma(T.mnrl_nu(p), L.lna(T.mnrl_idx(p)), lnQK);
        const double QK = exp(lnQK);
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
        double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * k
                           : Im_const * sign_ * fabs(aff) * k;
        rate[m] = Im;
        if (dry) continue;  // RReaction returns before minerals in a dry cell
        Im_const = Im_const * volume;
        Im = Im * volume;
        double dIm_dQK = has_pw ? -Im * T.power(m) / fabs(aff) : -Im_const * k;
        if (has_tk)
          dIm_dQK = dIm_dQK * (1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m))) / QK * (1.0 - aff);
        else if (has_msf)
          dIm_dQK = dIm_dQK * (1.0 / T.msf(m)) / QK * (1.0 - aff);
        double f = dIm_dQK * QK * den_k * 1.0e-3;
        if (rl > 0.0) {
          const double den = 1.0 + (1.0 - aff) / rl;
          f = f * (1.0 + QK / rl / den) / den;
        }
        for (int p = b; p < e; ++p) {
          const int kp = T.mnrl_idx(p);
          L.rhs(kp) = fma(T.mnrl_nu(p), Im, L.rhs(kp));
          const double t = T.mnrl_nu(p) * f;
          for (int q = b; q < e; ++q) {
            const int kq = T.mnrl_idx(q);
            // log form: the column scale m_q cancels the 1/m_q of dQK/dm_q
            L.J(kp, kq) = logf ? fma(T.mnrl_nu(q), t, L.J(kp, kq))
                               : fma(T.mnrl_nu(q) * t, L.VV(kq), L.J(kp, kq));
          }
        }
      }
      // ---- convergence tests on the residual (reaction.F90:3946-3953) -----
      double dot = 0.0, mx = 0.0;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const double r = L.rhs(j);
        dot = fma(r, r, dot);
        mx = fmax(mx, fabs(r));
      }
      const double two_norm = sqrt(dot);
      if (its == 1) r0 = two_norm;
      int react_end = -1;  // -1: continue, 0: converged, 1: failed
      if (its > o.maximum_reaction_iterations) {
#pragma unroll
        for (int j = 0; j < N; ++j) tot[j] = init_tot[j];
        react_end = 1;
      } else if (mx < o.max_residual_tolerance || two_norm < o.max_rel_residual_tolerance * r0) {
        react_end = 0;
      } else {
        if (lu_solve<N, JS>(L, indx, stride)) {
          react_end = 1;  // singular: no total restore (reaction.F90:3963-3966)
        } else {
          const double tol = o.max_relative_change_tolerance;
          bool small = true;
          double nc[N];
#pragma unroll
          for (int j = 0; j < N; ++j) {
            double u = o.fork_literal_rsolve ? 0.0 : L.rhs(j);
            if (logf) {
              u = fmin(fmax(u, -o.max_dlnC_rreact), o.max_dlnC_rreact);
              nc[j] = c[j] * exp(-u);
              L.rhs(j) = u;
            } else {
              nc[j] = c[j] - u;  // positivity scaling applied below
            }
          }
          if (!logf) {
            double min_ratio = 1.7976931348623157e308;
#pragma unroll
            for (int j = 0; j < N; ++j)
              if (c[j] <= L.rhs(j)) min_ratio = fmin(min_ratio, fabs(c[j] / L.rhs(j)));
            if (min_ratio < 1.0) {
#pragma unroll
              for (int j = 0; j < N; ++j) nc[j] = c[j] - L.rhs(j) * min_ratio * 0.99;
            }
          }
#pragma unroll
          for (int j = 0; j < N; ++j) small = small && (fabs(nc[j] - c[j]) < tol * c[j]);
          if (small) {
            react_end = 0;
          } else {
#pragma unroll
            for (int j = 0; j < N; ++j) {
              lnc[j] = logf ? lnc[j] - L.rhs(j) : log(nc[j]);
              c[j] = nc[j];
            }
          }
        }
      }
      // ------------------------------------------------ RStep bookkeeping
      if (react_end >= 0) {
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
          cum = cum + dt;
          nsub += 1;
          n_const += 1;
#pragma unroll
          for (int j = 0; j < N; ++j) guess[j] = c[j];
          if (n_const >= 4) {
            num_cuts = num_cuts - 1;
            dt = fmin(2.0 * dt, target - cum);
          }
          if (cum >= target) finish_cell = true;
          else phase = START;
        }
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
        if (newton_iter_act) st.pri_act_coef[soa.at(j, cell)] = exp(lng[j]);
      }
      if (newton_iter_act) {
        // sec_act_coef = exp(lnKeff-part); recompute from the last lnKeff
        const bool tsec = !iso && (net.flags & NETF_SEC_LOGKCOEF);
        for (int i = 0; i < ns; ++i) {
          const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
          st.sec_act_coef[soa.at(i, cell)] = exp(-logK * LOG_TO_LN - lnKeff[i]);
        }
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
    }
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

template <int N>
int launch_batched_n(const DevNet& net, const PfCellState& st, double dt, const PfLaunchConfig& cfg,
                     int num_sms, unsigned long long* queue, unsigned long long* counters,
                     cudaStream_t stream) {
  const size_t smem = batched_smem_bytes(net, cfg);
  const int tpb = cfg.threads_per_block;
  const int grid = num_sms * cfg.blocks_per_sm;
  cudaError_t err;
  if (cfg.jac_in_shared) {
    auto k = batched::rstep_batched_kernel<N, true>;
    err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    k<<<grid, tpb, smem, stream>>>(net, st, dt, queue, counters);
  } else {
    auto k = batched::rstep_batched_kernel<N, false>;
    err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    k<<<grid, tpb, smem, stream>>>(net, st, dt, queue, counters);
  }
  return (int)cudaGetLastError();
}

}  // namespace pfgpu
