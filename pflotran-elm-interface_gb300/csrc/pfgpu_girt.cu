// pfgpu_girt.cu -- global-implicit residual and BAIJ Jacobian assembly on a
// structured grid (7-point stencil).
//
// Replaces, for a structured grid with zero-flux outer boundaries, the
// per-Newton-iteration assembly of
//   RTResidualFlux / RTResidualNonFlux  (src/pflotran/reactive_transport.F90:2052-2669)
//   RTJacobianFlux / RTJacobianNonFlux  (:2897-3349, log scaling :2879, :3316-3340)
// with TDispersion/TFluxCoef/TFlux/TFluxDerivative (transport.F90:52-609).
//
// Structure of the Jacobian this exploits: the transport coefficient of a
// connection is the same for every component (one D_m, one phase), so the
// connection's blocks are scalar multiples of one cell's dtotal:
//   block (up, up) += c_up dtot_up      block (up, dn) += c_dn dtot_dn
//   block (dn, dn) -= c_dn dtot_dn      block (dn, up) -= c_up dtot_up
// Every block in block column X is therefore a scalar times dtot_X (times the
// column scaling diag(m_X) in the log formulation), plus, on the diagonal, the
// accumulation and reaction derivatives of X.  The cell that owns column X
// computes dtot_X once and writes the diagonal block and the (Y, X) block of
// every neighbour row Y; nothing is accumulated in memory.
//
// GB300 runs FP64 at ~1.7 lane-operations per clock per SM and a warp
// instruction costs the same pipe time with idle lanes, so all FP64 work is
// one cell per lane:
//   girt_cell_kernel      RTotal (totals, sec_molal), kinetic minerals and
//                         their derivative, dtotal entry by entry, the block
//                         column, and the cell's reaction residual
//   girt_residual_kernel  flux + accumulation terms of the residual row
//                         (needs the neighbours' totals of the first launch)
// With equilibrium sorption the cell kernel also runs RTotalSorb (total_sorb,
// the ion-exchange warm start) and adds dtotal_sorb * V/dt to its diagonal
// block (RAccumulationSorbDerivative, reactive_transport.F90:3183); the
// residual kernel adds (S - S_k) * V/dt (RAccumulationSorb, :1026 and :2412).
// Both are unconditional in the reference, dry cells included.  Minerals with
// rate prefactors take their rate from prefactor_rate, and the cell kernel
// adds the prefactor derivative to its diagonal block the same way.
// Per-thread scratch (molalities, secondary molalities, mineral terms) lives
// in shared memory, interleaved by thread so that accesses are conflict-free.
// The diagonal flux term sums the connection coefficients first
// ((sum_q c_q) dtot rather than sum_q (c_q dtot)); every c_q there is >= 0
// (upwinding), so the two orders differ by rounding only.
#include <vector>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"
#include "pfgpu_prefactor.cuh"
#include "pfgpu_sorb.cuh"

namespace pfgpu {
namespace girt {

struct Geo {
  int nx, ny, nz;
  double dx, dy, dz;
  double diffusion, tortuosity, dispersivity;
  const double* qx;
  const double* qy;
  const double* qz;
};

// doubles of per-thread shared memory: m, 1/m, ln a, totals (n each), the
// secondary molalities (ns), the mineral column terms u (one per mineral CSR
// slot) and the mineral derivative factors (nm)
__host__ __device__ inline int thread_doubles(const DevNet& net) {
  return 4 * net.n + net.ns + net.nnz_m + net.nm;
}

// harmonic_tran_coefs_over_dist (transport.F90:199-225) for a connection at
// the midpoint of equal cells (dist_up = dist_dn = dist/2)
__device__ __forceinline__ double tran_coef(double por_up, double sat_up, double por_dn, double sat_dn, double q,
                                            double dist, const Geo& g) {
  const double dist_up = dist * 0.5, dist_dn = dist - dist_up;
  const double mech = g.dispersivity * fabs(q);
  const double hu = fmax(mech + 1.0 * sat_up * por_up * g.tortuosity * g.diffusion, 1.0e-40);
  const double hd = fmax(mech + 1.0 * sat_dn * por_dn * g.tortuosity * g.diffusion, 1.0e-40);
  return (hu * hd) / (hu * dist_dn + hd * dist_up);
}

// The six connections of cell X in the order the reference's x, y, z
// connection loops reach it (x-, x+, y-, y+, z-, z+): neighbour, whether X is
// the upstream (lower-index) cell, and TFluxCoef's T_up, T_dn (L/s).
struct Conns {
  int ex[6], other[6], up[6];
  double cup[6], cdn[6];
};

__device__ __forceinline__ void connections(const PfCellState& st, const Geo& g, long long X, Conns& c) {
  const long long nxy = (long long)g.nx * g.ny;
  const int i = (int)(X % g.nx), j = (int)((X / g.nx) % g.ny), k = (int)(X / nxy);
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int axis = q >> 1, plus = q & 1;
    const int pos = axis == 0 ? i : (axis == 1 ? j : k);
    const int lim = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    const int ex = plus ? (pos < lim - 1) : (pos > 0);
    c.ex[q] = ex;
    c.up[q] = plus;
    c.other[q] = 0;
    c.cup[q] = c.cdn[q] = 0.0;
    if (!ex) continue;
    const long long s = axis == 0 ? 1 : (axis == 1 ? (long long)g.nx : nxy);
    const long long other = plus ? X + s : X - s;
    c.other[q] = (int)other;
    const int face = plus ? pos : pos - 1;
    double qf, area, dist;
    if (axis == 0) {
      qf = g.qx[((long long)k * g.ny + j) * (g.nx - 1) + face];
      area = g.dy * g.dz;
      dist = g.dx;
    } else if (axis == 1) {
      qf = g.qy[((long long)k * (g.ny - 1) + face) * g.nx + i];
      area = g.dx * g.dz;
      dist = g.dy;
    } else {
      qf = g.qz[((long long)face * g.ny + j) * g.nx + i];
      area = g.dx * g.dy;
      dist = g.dz;
    }
    const long long cu = plus ? X : other, cd = plus ? other : X;
    const double pu = st.porosity[cu], su = st.saturation[cu], pdn = st.porosity[cd], sdn = st.saturation[cd];
    if (!(sdn < RT_MIN_SATURATION) && !(su < RT_MIN_SATURATION)) {
      const double tr = tran_coef(pu, su, pdn, sdn, qf, dist, g);
      double a, b;
      if (qf > 0.0) { a = tr + qf; b = -tr; }
      else { a = tr; b = -tr + qf; }
      c.cup[q] = a * area * 1000.0;
      c.cdn[q] = b * area * 1000.0;
    }
  }
}

__device__ __forceinline__ int find_block(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                                          long long row, long long col) {
  for (int b = rowptr[row]; b < rowptr[row + 1]; ++b)
    if (colidx[b] == (int)col) return b;
  return -1;
}

// Rate prefactors (the girt_cell_kernel<true> instantiation only).  P: the thread's scratch (m at P[j*bd], ln a at
// P[o_lna + j*bd], complexes at P[o_s + i*bd]).
__device__ __noinline__ double pref_rate(const Tables& T, const PfCellState& st, long long X, const double* P,
                                         int bd, int o_lna, int o_s, double temp, int m) {
  const SoA soa{st.ncells};
  double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
  return prefactor_rate(
      T, m, [&](int j) { return P[o_lna + j * bd]; },
      [&](int i) { return log(P[o_s + i * bd]) + log(st.sec_act_coef[soa.at(i, X)]); }, temp, pref, lnps);
}

// adds the prefactor part of the reaction Jacobian of the minerals in mask
// to the diagonal block D (column-major, columns scaled by m when logf)
__device__ __noinline__ void pref_jacobian(const DevNet& net, const Tables& T, const PfCellState& st, long long X,
                                           const double* P, int bd, int o_lna, int o_s, double temp,
                                           double volume, bool logf, bool tsec, unsigned mask, double* D) {
  const SoA soa{st.ncells};
  const int n = net.n;
  auto ln_act = [&](int j) { return P[o_lna + j * bd]; };
  auto ln_sec_act = [&](int i) { return log(P[o_s + i * bd]) + log(st.sec_act_coef[soa.at(i, X)]); };
  for (int m = 0; m < net.nm; ++m) {
    if (!((mask >> m) & 1u)) continue;
    double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
    const double sum = prefactor_rate(T, m, ln_act, ln_sec_act, temp, pref, lnps);
    prefactor_derivative(
        T, m, st.mnrl_rate[soa.at(m, X)] * volume, sum, pref, lnps, ln_act, ln_sec_act,
        [&](int j) { return st.pri_act_coef[soa.at(j, X)]; }, [&](int i) { return st.sec_act_coef[soa.at(i, X)]; },
        [&](int j) { return log(P[j * bd]); },
        [&](int i) {
          return add_h2o(-(tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i)) * LOG_TO_LN, T.sec_h2o(i),
                         cell_lnaw(net, st, X));
        },
        temp,
        [&](int r, int c, double v) { D[c * n + r] = fma(v, logf ? P[c * bd] : 1.0, D[c * n + r]); });
  }
}

// The mineral part of RReaction's residual for one cell (RKineticMineral
// without the derivative, reaction_mineral.F90:647-913), at primary ln
// activities lna[] and complexes' ln activities ln_sec_act(i): the same
// arithmetic as the cell kernel's mineral loop.
template <class LnSecAct>
__device__ void mineral_residual(const DevNet& net, const Tables& T, const PfCellState& st, long long X,
                                 const double* lna, LnSecAct ln_sec_act, double temp, double volume, double* Res) {
  const SoA soa{st.ncells};
  const bool tmin = !net.o.isothermal && (net.flags & NETF_MNRL_LOGKCOEF);
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  for (int m = 0; m < net.nm; ++m) {
    const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
    const double logK = tmin ? interp_logK(T.mnrl_logKcoef(m), temp) : T.mnrl_logK(m);
    double lnQK = -logK * LOG_TO_LN;
    if (water_on(net)) lnQK = add_h2o(lnQK, T.mnrl_h2o(m), cell_lnaw(net, st, X));
    for (int p = b; p < e; ++p) lnQK = lnQK + T.mnrl_nu(p) * lna[T.mnrl_idx(p)];
    const double QK = exp(lnQK);
    double aff;
    if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
    else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
    else aff = 1.0 - QK;
    const double sign_ = fsign1(aff);
    const double vf = st.mnrl_volfrac[soa.at(m, X)];
    const bool active = (vf > 0 || sign_ < 0.0) && !(T.irreversible(m) == 1 && sign_ < 0.0) &&
                        !(T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m));
    if (!active) continue;
    const double rl = T.limiter(m);
    if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
    double kr;
    if ((net.flags & NETF_PREFACTOR) && T.pf_cnt(m) > 0) {
      double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
      kr = prefactor_rate(T, m, [&](int j) { return lna[j]; }, ln_sec_act, temp, pref, lnps);
    } else {
      double arr = 1.0;
      if (T.ea(m) > 0.0) arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp + 273.15)));
      kr = T.rate(m) * arr;
    }
    double Im_const = -st.mnrl_area[soa.at(m, X)];
    if (has_msf) Im_const = Im_const / T.msf(m);
    double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * kr : Im_const * sign_ * fabs(aff) * kr;
    Im = Im * volume;
    for (int p = b; p < e; ++p) Res[T.mnrl_idx(p)] = Res[T.mnrl_idx(p)] + T.mnrl_nu(p) * Im;
  }
}

// The reaction part of the diagonal block by forward differences
// (RReactionDerivative's numerical branch, reaction.F90:4176-4230): each
// primary molality raised by 1e-5 of itself, RTotal's complexes at the
// raised value, the mineral residual again; columns below 1e-40 in magnitude
// zeroed, then added to D in the column scaling.
__device__ __noinline__ void numerical_reaction_jacobian(const DevNet& net, const Tables& T, const PfCellState& st,
                                                         long long X, const double* P, int bd, int o_lna, int o_s,
                                                         double temp, double volume, bool logf, bool tsec,
                                                         double* D) {
  const SoA soa{st.ncells};
  const int n = net.n;
  double lna[PF_MAX_NCOMP], res0[PF_MAX_NCOMP], res1[PF_MAX_NCOMP];
  for (int j = 0; j < n; ++j) {
    lna[j] = P[o_lna + j * bd];
    res0[j] = 0.0;
  }
  mineral_residual(
      net, T, st, X, lna, [&](int i) { return log(P[o_s + i * bd]) + log(st.sec_act_coef[soa.at(i, X)]); }, temp,
      volume, res0);
  for (int jc = 0; jc < n; ++jc) {
    const double m0 = P[jc * bd];
    const double pert = m0 * 1.0e-5;  // perturbation_tolerance, reaction.F90:41
    const double saved = lna[jc];
    lna[jc] = log(m0 + pert) + log(st.pri_act_coef[soa.at(jc, X)]);
    for (int i = 0; i < n; ++i) res1[i] = 0.0;
    auto ln_sec_act = [&](int i) {  // RTotal of the perturbed copy, complex i
      double lnQK = -(tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i)) * LOG_TO_LN;
      if (water_on(net)) lnQK = add_h2o(lnQK, T.sec_h2o(i), cell_lnaw(net, st, X));
      for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) lnQK = lnQK + T.sec_nu(p) * lna[T.sec_idx(p)];
      const double g = st.sec_act_coef[soa.at(i, X)];
      return log(exp(lnQK) / g) + log(g);
    };
    mineral_residual(net, T, st, X, lna, ln_sec_act, temp, volume, res1);
    lna[jc] = saved;
    const double mc = logf ? m0 : 1.0;
    for (int ic = 0; ic < n; ++ic) {
      double J = (res1[ic] - res0[ic]) / pert;
      if (fabs(J) < 1.0e-40) J = 0.0;
      D[jc * n + ic] = fma(J, mc, D[jc * n + ic]);
    }
  }
}

// HAS_PF: rate prefactors; NUMJAC: the reaction Jacobian by forward
// differences (instantiated with HAS_PF, whose rate code it needs)
template <bool HAS_PF, bool NUMJAC>
__global__ void __launch_bounds__(128) girt_cell_kernel(DevNet net, GirtTabs gt, PfCellState st, Geo g, double dt,
                                                        const int32_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ colidx, double* __restrict__ r,
                                                        double* __restrict__ values, int vec2) {
  extern __shared__ double smem[];
  const long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= st.ncells) return;
  const int bd = blockDim.x;
  double* P = smem + threadIdx.x;  // this thread's scratch: P[k * bd]
  const int n = net.n, nn = n * n, ns = net.ns, nm = net.nm;
  const int o_ic = n * bd, o_lna = 2 * n * bd, o_t = 3 * n * bd, o_s = 4 * n * bd, o_u = (4 * n + ns) * bd,
            o_G = (4 * n + ns + net.nnz_m) * bd;
  const Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  const bool logf = net.o.use_log_formulation != 0;
  const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
  const bool tmin = !net.o.isothermal && (net.flags & NETF_MNRL_LOGKCOEF);
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  constexpr bool has_pf = HAS_PF;  // rate prefactors: a separate instantiation
  unsigned pf_active = 0;  // minerals whose prefactor derivative is due
  const double temp = st.temperature ? st.temperature[X] : 25.0;
  const bool has_h2o = water_on(net);
  const double lnaw = cell_lnaw(net, st, X);
  const double den_k = st.den_kg[X], den_L = den_k * 1.0e-3;
  const double por = st.porosity[X], sat = st.saturation[X], volume = st.volume[X];
  const bool dry = sat < RT_MIN_SATURATION;
  // ---- RTotalAqueous (reaction.F90:4665-4759)
  for (int jj = 0; jj < n; ++jj) {
    const double m = st.pri_molal[soa.at(jj, X)];
    P[jj * bd] = m;
    P[o_ic + jj * bd] = 1.0 / m;
    P[o_lna + jj * bd] = log(m) + log(st.pri_act_coef[soa.at(jj, X)]);
  }
  for (int jj = 0; jj < n; ++jj) P[o_t + jj * bd] = P[jj * bd];  // total = m, then += nu s
  for (int i = 0; i < ns; ++i) {
    const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
    double lnQK = -logK * LOG_TO_LN;
    if (has_h2o) lnQK = add_h2o(lnQK, T.sec_h2o(i), lnaw);
    const int b = T.sec_begin(i), e = T.sec_end(i);
    for (int p = b; p < e; ++p) lnQK = lnQK + T.sec_nu(p) * P[o_lna + T.sec_idx(p) * bd];
    const double sv = exp(lnQK) / st.sec_act_coef[soa.at(i, X)];
    P[o_s + i * bd] = sv;
    st.sec_molal[soa.at(i, X)] = sv;
  }
  // totals in the reference's order: per component, the secondaries ascending
  for (int i = 0; i < ns; ++i) {
    const double sv = P[o_s + i * bd];
    for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) {
      const int a = o_t + T.sec_idx(p) * bd;
      P[a] = P[a] + T.sec_nu(p) * sv;
    }
  }
  for (int jj = 0; jj < n; ++jj) st.total[soa.at(jj, X)] = P[o_t + jj * bd] * den_L;
  // ---- RKineticMineral (reaction_mineral.F90:647-1078): rates, reaction
  // residual (into r, finished by girt_residual_kernel), derivative factors
  for (int jj = 0; jj < n; ++jj) r[X * n + jj] = 0.0;
  for (int m = 0; m < nm; ++m) {
    const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
    double Gm = 0.0, QK = 0.0;
    bool active = false;
    if (!dry) {
      const double logK = tmin ? interp_logK(T.mnrl_logKcoef(m), temp) : T.mnrl_logK(m);
      double lnQK = -logK * LOG_TO_LN;
      if (has_h2o) lnQK = add_h2o(lnQK, T.mnrl_h2o(m), lnaw);
      for (int p = b; p < e; ++p) lnQK = lnQK + T.mnrl_nu(p) * P[o_lna + T.mnrl_idx(p) * bd];
      QK = exp(lnQK);
      double aff;
      if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
      else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
      else aff = 1.0 - QK;
      const double sign_ = fsign1(aff);
      const double vf = st.mnrl_volfrac[soa.at(m, X)];
      active = (vf > 0 || sign_ < 0.0) && !(T.irreversible(m) == 1 && sign_ < 0.0) &&
               !(T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m));
      double rate_out = 0.0;
      if (active) {
        const double rl = T.limiter(m);
        if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
        double kr;
        if (has_pf && T.pf_cnt(m) > 0) {
          kr = pref_rate(T, st, X, P, bd, o_lna, o_s, temp, m);
          pf_active |= 1u << m;
        } else {
          double arr = 1.0;
          if (T.ea(m) > 0.0)
            arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp + 273.15)));
          kr = T.rate(m) * arr;
        }
        double Im_const = -st.mnrl_area[soa.at(m, X)];
        if (has_msf) Im_const = Im_const / T.msf(m);
        double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * kr : Im_const * sign_ * fabs(aff) * kr;
        rate_out = Im;
        Im_const = Im_const * volume;
        Im = Im * volume;
        for (int p = b; p < e; ++p) r[X * n + T.mnrl_idx(p)] = r[X * n + T.mnrl_idx(p)] + T.mnrl_nu(p) * Im;
        double dIm_dQK = has_pw ? -Im * T.power(m) / fabs(aff) : -Im_const * kr;
        if (has_tk)
          dIm_dQK = dIm_dQK * (1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m))) / QK * (1.0 - aff);
        else if (has_msf)
          dIm_dQK = dIm_dQK * (1.0 / T.msf(m)) / QK * (1.0 - aff);
        if (rl > 0.0) {
          const double den = 1.0 + (1.0 - aff) / rl;
          Gm = dIm_dQK * (1.0 + QK / rl / den) / den;
        } else {
          Gm = dIm_dQK;
        }
      }
      st.mnrl_rate[soa.at(m, X)] = rate_out;
    }
    P[o_G + m * bd] = Gm;
    // dQK/dm_j (the reference's den*1e-3 factor included, :944-947)
    for (int p = b; p < e; ++p)
      P[o_u + p * bd] = active ? T.mnrl_nu(p) * QK * P[o_ic + T.mnrl_idx(p) * bd] * den_k * 1.0e-3 : 0.0;
  }
  // ---- block column X
  Conns c;
  connections(st, g, X, c);
  int blk[6];
  double sc[6];
  double csum = 0.0;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    blk[q] = c.ex[q] ? find_block(rowptr, colidx, c.other[q], X) : -1;
    sc[q] = c.up[q] ? -c.cup[q] : c.cdn[q];  // block (Y, X) = sc * dtot_X
    if (c.ex[q]) csum = csum + (c.up[q] ? c.cup[q] : -c.cdn[q]);
  }
  const int dblk = find_block(rowptr, colidx, X, X);
  const double psvd_t = por * sat * 1000.0 * volume / dt;
  const double cdiag = csum + psvd_t;
  auto entry = [&](int fe, double& vdiag, double& e) {
    const int col = fe / n, row = fe - col * n;
    const int f = row * n + col;
    double acc = 0.0;
    for (int q = gt.e_sec_ptr[f]; q < gt.e_sec_ptr[f + 1]; ++q)
      acc = fma(gt.e_sec_nr[q], P[o_s + gt.e_sec_p[q] * bd], acc);
    const double d = ((row == col ? 1.0 : 0.0) + acc * P[o_ic + col * bd]) * den_L;
    double jr = 0.0;
    if (!NUMJAC)
      for (int q = gt.e_mn_ptr[f]; q < gt.e_mn_ptr[f + 1]; ++q)
        jr = fma(gt.e_mn_nr[q] * P[o_G + gt.e_mn_m[q] * bd], P[o_u + gt.e_mn_p[q] * bd], jr);
    if (fabs(jr) < 1.0e-40) jr = 0.0;  // reaction.F90:4232-4237
    const double mc = logf ? P[col * bd] : 1.0;
    const double v = dry ? fma(d, csum, (row == col) ? 1.0 : 0.0) : fma(d, cdiag, jr);
    vdiag = v * mc;
    e = d * mc;
  };
  if (vec2) {
    for (int fe = 0; fe < nn; fe += 2) {
      double v0, e0, v1, e1;
      entry(fe, v0, e0);
      entry(fe + 1, v1, e1);
      if (dblk >= 0) *reinterpret_cast<double2*>(values + (size_t)dblk * nn + fe) = make_double2(v0, v1);
#pragma unroll
      for (int q = 0; q < 6; ++q)
        if (blk[q] >= 0)
          *reinterpret_cast<double2*>(values + (size_t)blk[q] * nn + fe) = make_double2(sc[q] * e0, sc[q] * e1);
    }
  } else {
    for (int fe = 0; fe < nn; ++fe) {
      double v0, e0;
      entry(fe, v0, e0);
      if (dblk >= 0) values[(size_t)dblk * nn + fe] = v0;
#pragma unroll
      for (int q = 0; q < 6; ++q)
        if (blk[q] >= 0) values[(size_t)blk[q] * nn + fe] = sc[q] * e0;
    }
  }
  // ---- rate-prefactor part of the reaction Jacobian (its residual part is in
  // the rates above), added to the diagonal block in the column scaling
  if (NUMJAC && !dry && dblk >= 0)
    numerical_reaction_jacobian(net, T, st, X, P, bd, o_lna, o_s, temp, volume, logf, tsec,
                                values + (size_t)dblk * nn);
  else if (has_pf && pf_active && dblk >= 0)
    pref_jacobian(net, T, st, X, P, bd, o_lna, o_s, temp, volume, logf, tsec, pf_active,
                  values + (size_t)dblk * nn);
  // ---- equilibrium sorption (RTotalSorb in RTUpdateAuxVars; a failed
  // ion-exchange solve leaves the last iterate, the reference's
  // message-and-continue).  Only this thread writes its diagonal block.
  if (has_sorption(net) && dblk >= 0) {
    for (int jj = 0; jj < n; ++jj) st.total_sorb[soa.at(jj, X)] = 0.0;
    double* D = values + (size_t)dblk * nn;
    const double v_t = volume / dt;
    total_sorb(
        net, T, [&](int j) { return P[j * bd]; }, [&](int j) { return st.pri_act_coef[soa.at(j, X)]; },
        [&](int m) { return st.mnrl_volfrac[soa.at(m, X)]; }, por, den_k,
        st.ionx_ref_sorbed ? st.ionx_ref_sorbed + X : nullptr, st.ncells,
        [&](int j, double v) { st.total_sorb[soa.at(j, X)] += v; },
        [&](int i, int j, double v) { D[j * n + i] = fma(v * v_t, logf ? P[j * bd] : 1.0, D[j * n + i]); },
        surf_cell(net, st, X));
  }
}

// residual row of cell X: connections (reference order), fixed and current
// accumulation, then the reaction part the cell kernel left in r
__global__ void __launch_bounds__(128) girt_residual_kernel(DevNet net, PfCellState st, Geo g,
                                                            const double* __restrict__ total_k,
                                                            const double* __restrict__ sorb_k, double dt,
                                                            double* __restrict__ r) {
  const long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= st.ncells) return;
  const long long N = st.ncells;
  const int n = net.n;
  Conns c;
  connections(st, g, X, c);
  const double sat = st.saturation[X];
  const bool dry = sat < RT_MIN_SATURATION;
  const double psv = st.porosity[X] * sat * 1000.0 * st.volume[X];
  const bool sorb = has_sorption(net);
  for (int row = 0; row < n; ++row) {
    const double tx = st.total[(size_t)row * N + X];
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      if (!c.ex[q]) continue;
      const double ty = st.total[(size_t)row * N + c.other[q]];
      const double tu = c.up[q] ? tx : ty, td = c.up[q] ? ty : tx;
      const double res = c.cup[q] * tu + c.cdn[q] * td;
      v = c.up[q] ? v + res : v - res;
    }
    double accum_k = dry ? 0.0 : psv * total_k[(size_t)row * N + X];
    double accum = dry ? 0.0 : psv * tx;
    if (sorb) {
      accum_k = accum_k + sorb_k[(size_t)row * N + X] * st.volume[X];
      accum = accum + st.total_sorb[(size_t)row * N + X] * st.volume[X];
    }
    v = v - accum_k / dt;
    v = v + accum / dt;
    if (!dry) v = v + r[X * n + row];
    r[X * n + row] = v;
  }
}

}  // namespace girt

int girt_build_tables(const DevNet& net, const int32_t* I, const double* D, void** d_buf, GirtTabs* out) {
  const int n = net.n, nn = n * n;
  std::vector<std::vector<int32_t>> sp(nn), mp(nn), mm(nn);
  std::vector<std::vector<double>> snr(nn), mnr(nn);
  for (int i = 0; i < net.ns; ++i) {
    const int b = I[net.o_sec_ptr + i], e = I[net.o_sec_ptr + i + 1];
    for (int pc = b; pc < e; ++pc)
      for (int pr = b; pr < e; ++pr) {
        const int f = I[net.o_sec_idx + pr] * n + I[net.o_sec_idx + pc];
        sp[f].push_back(i);
        snr[f].push_back(D[net.o_sec_nu + pr] * D[net.o_sec_nu + pc]);
      }
  }
  for (int m = 0; m < net.nm; ++m) {
    const int b = I[net.o_mnrl_ptr + m], e = I[net.o_mnrl_ptr + m + 1];
    for (int pc = b; pc < e; ++pc)
      for (int pr = b; pr < e; ++pr) {
        const int f = I[net.o_mnrl_idx + pr] * n + I[net.o_mnrl_idx + pc];
        mp[f].push_back(pc);
        mm[f].push_back(m);
        mnr[f].push_back(D[net.o_mnrl_nu + pr]);
      }
  }
  std::vector<int32_t> ints;
  std::vector<double> dbls;
  auto csr = [&](const std::vector<std::vector<int32_t>>& rows, int* o_ptr, int* o_idx) {
    *o_ptr = (int)ints.size();
    int c = 0;
    for (auto& rw : rows) { ints.push_back(c); c += (int)rw.size(); }
    ints.push_back(c);
    *o_idx = (int)ints.size();
    for (auto& rw : rows) ints.insert(ints.end(), rw.begin(), rw.end());
  };
  auto flat = [&](const std::vector<std::vector<int32_t>>& rows) {
    const int o = (int)ints.size();
    for (auto& rw : rows) ints.insert(ints.end(), rw.begin(), rw.end());
    return o;
  };
  auto flatd = [&](const std::vector<std::vector<double>>& rows) {
    const int o = (int)dbls.size();
    for (auto& rw : rows) dbls.insert(dbls.end(), rw.begin(), rw.end());
    return o;
  };
  int o_esp, o_esi, o_emp, o_emi;
  csr(sp, &o_esp, &o_esi);
  csr(mp, &o_emp, &o_emi);
  const int o_emm = flat(mm);
  const int d_esnr = flatd(snr), d_emnr = flatd(mnr);
  if (dbls.empty()) dbls.push_back(0.0);
  const size_t ib = (ints.size() * 4 + 15) & ~size_t(15);
  void* buf = nullptr;
  if (cudaMalloc(&buf, ib + dbls.size() * 8) != cudaSuccess) return PF_ERR_CUDA;
  if (cudaMemcpy(buf, ints.data(), ints.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy((char*)buf + ib, dbls.data(), dbls.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(buf);
    return PF_ERR_CUDA;
  }
  const int32_t* di = (const int32_t*)buf;
  const double* dd = (const double*)((char*)buf + ib);
  out->e_sec_ptr = di + o_esp;
  out->e_sec_p = di + o_esi;
  out->e_sec_nr = dd + d_esnr;
  out->e_mn_ptr = di + o_emp;
  out->e_mn_p = di + o_emi;
  out->e_mn_m = di + o_emm;
  out->e_mn_nr = dd + d_emnr;
  *d_buf = buf;
  return PF_OK;
}

// threads per block of the cell kernel and its shared memory
size_t girt_smem_bytes(const DevNet& net, int* threads_per_block) {
  const size_t tbytes = (size_t)girt::thread_doubles(net) * sizeof(double);
  int tpb = 128;
  while (tpb > 32 && tpb * tbytes > 72u * 1024u) tpb -= 32;
  if (threads_per_block) *threads_per_block = tpb;
  return tpb * tbytes;
}

int launch_girt_assemble(const DevNet& net, const GirtTabs& gt, const PfCellState& st, const PfGirtArgs& a,
                         int num_sms, cudaStream_t s) {
  (void)num_sms;
  if (st.ncells == 0) return PF_OK;
  girt::Geo g{a.nx, a.ny, a.nz, a.dx, a.dy, a.dz, a.diffusion_coefficient, a.tortuosity, a.dispersivity,
              a.qx, a.qy, a.qz};
  int tpb = 32;
  const size_t smem = girt_smem_bytes(net, &tpb);
  if (smem > 227u * 1024u) return PF_ERR_TOO_LARGE;
  auto k = a.numerical_derivatives ? girt::girt_cell_kernel<true, true>
           : (net.flags & NETF_PREFACTOR) ? girt::girt_cell_kernel<true, false>
                                          : girt::girt_cell_kernel<false, false>;
  if (smem > 48u * 1024u &&
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return PF_ERR_CUDA;
  // 16-byte stores when every block starts on a 16-byte boundary
  const int vec2 = ((net.n * net.n) % 2 == 0) && (((uintptr_t)a.values & 15) == 0);
  const long long blocks = (st.ncells + tpb - 1) / tpb;
  k<<<(unsigned)blocks, tpb, smem, s>>>(net, gt, st, g, a.dt, a.rowptr, a.colidx, a.residual, a.values, vec2);
  if (cudaGetLastError() != cudaSuccess) return PF_ERR_CUDA;
  const long long rblocks = (st.ncells + 127) / 128;
  girt::girt_residual_kernel<<<(unsigned)rblocks, 128, 0, s>>>(net, st, g, a.total_k, a.total_sorb_k, a.dt,
                                                                a.residual);
  return cudaGetLastError() == cudaSuccess ? PF_OK : PF_ERR_CUDA;
}

}  // namespace pfgpu

using namespace pfgpu;

extern "C" int32_t pf_girt_pattern(int32_t nx, int32_t ny, int32_t nz, int32_t* rowptr, int32_t* colidx) {
  if (nx < 1 || ny < 1 || nz < 1) return PF_ERR_INVALID;
  const long long N = (long long)nx * ny * nz, nxy = (long long)nx * ny;
  if (N > 0x7fffffffll / 7) return PF_ERR_TOO_LARGE;
  long long b = 0;
  for (long long X = 0; X < N; ++X) {
    const int i = (int)(X % nx), j = (int)((X / nx) % ny), k = (int)(X / nxy);
    if (rowptr) rowptr[X] = (int32_t)b;
    long long cand[7] = {k > 0 ? X - nxy : -1, j > 0 ? X - nx : -1, i > 0 ? X - 1 : -1, X,
                         i < nx - 1 ? X + 1 : -1, j < ny - 1 ? X + nx : -1, k < nz - 1 ? X + nxy : -1};
    for (int q = 0; q < 7; ++q)
      if (cand[q] >= 0) {
        if (colidx) colidx[b] = (int32_t)cand[q];
        ++b;
      }
  }
  if (rowptr) rowptr[N] = (int32_t)b;
  return (int32_t)b;
}
