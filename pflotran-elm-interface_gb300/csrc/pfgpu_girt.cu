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
// GB300 runs FP64 at ~2 lane-operations per clock per SM and a warp
// instruction costs the same pipe time with idle lanes, so all FP64 work is
// one cell per lane, and the count of FP64 operations per cell sets the
// speed:
//   girt_cell_kernel      RTotal (totals, sec_molal), kinetic minerals and
//                         their derivative, dtotal, the block column, and the
//                         cell's reaction residual
//   girt_residual_kernel  flux + accumulation terms of the residual row
//                         (needs the neighbours' totals of the first launch)
// The cell kernel's arithmetic:
//   * speciation in product form: s_i = K_i prod_j a_j^nu_ij / gamma_i with
//     K_i = exp(-logK_i ln 10) computed once per block (isothermal, no water
//     term) and every factor one multiply from a power table of a, a^2, 1/a,
//     1/a^2 -- no transcendental per complex or per species;
//   * d total/d m_c = den (delta_rc + sum_i nu_ri nu_ci s_i / m_c); the log
//     formulation scales column c by m_c, which cancels the division:
//     den (delta_rc m_c + sum_i nu_ri nu_ci s_i) is symmetric, so the sum is
//     accumulated once per complex on the packed lower triangle, and so is
//     the kinetic minerals' part sum_m nu_rm nu_cm dIm/dQK QK den 1e-3;
//   * the blocks are written as whole 32-byte sectors (four doubles per
//     store; BAIJ blocks of n*n % 4 == 0 doubles start on 32-byte
//     boundaries).
// With equilibrium sorption the cell kernel also runs RTotalSorb (total_sorb,
// the ion-exchange warm start) and adds dtotal_sorb * V/dt to its diagonal
// block (RAccumulationSorbDerivative, reactive_transport.F90:3183); the
// residual kernel adds (S - S_k) * V/dt (RAccumulationSorb, :1026 and :2412).
// Both are unconditional in the reference, dry cells included.  Minerals with
// rate prefactors take their rate from prefactor_rate, and the cell kernel
// adds the prefactor derivative to its diagonal block the same way.
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

// Shared memory of a block of the cell kernel:
//   block part   K (ns + nm doubles, isothermal networks without water:
//                exp(-logK ln 10) of every complex and kinetic mineral), then,
//                when they fit, copies of the network's tables and of the
//                assembly tables (read there instead of global memory)
//   thread part  per-thread scratch, interleaved by thread (element e of a
//                thread at P[e * bd], bd = threads per block, so that a warp's
//                accesses to one element fall in distinct banks):
//     pa  [2n]        a = m gamma and 1/a of the species that need it (their
//                     squares are one more multiply); 1/m afterwards (linear
//                     formulation)
//     E   [n(n+1)/2]  packed lower triangle of sum_i nu_ri nu_ci s_i, turned
//                     into d total/d m times the column scaling (log form)
//     T   [n]         totals (mol/kg water); then GQ [nm] = dIm/dQK * QK *
//                     den_kg * 1e-3 of each kinetic mineral
//     lna [n]         ln a (rate prefactors and numerical derivatives only)
struct Layout {
  int pa, E, T, GQ, lna, per_thread;
};
__host__ __device__ inline Layout layout(const DevNet& net, bool with_lna, bool e_in_smem = true) {
  const int n = net.n;
  Layout L;
  L.pa = 0;
  L.E = 2 * n;
  L.T = L.E + (e_in_smem ? n * (n + 1) / 2 : 0);
  L.GQ = L.T;
  L.lna = L.T + (n > net.nm ? n : net.nm);
  L.per_thread = L.lna + (with_lna ? n : 0);
  return L;
}
// bytes of the block part: K, then the staged tables (each 16-byte padded)
__host__ __device__ inline size_t pad16(size_t b) { return (b + 15) & ~size_t(15); }
__host__ __device__ inline size_t block_k_bytes(const DevNet& net) { return pad16((size_t)(net.ns + net.nm) * 8); }
__host__ __device__ inline size_t block_table_bytes(const DevNet& net, const GirtTabs& gt) {
  return pad16((size_t)net.int_words * 4) + pad16((size_t)net.dbl_words * 8) + (size_t)gt.ibytes + (size_t)gt.dbytes;
}

// packed index of the symmetric entry (r, c)
__device__ __forceinline__ int sym_index(int r, int c) {
  const int hi = r > c ? r : c, lo = r > c ? c : r;
  return hi * (hi + 1) / 2 + lo;
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

// What the rate-prefactor and forward-difference helpers read of one cell:
// m and the activity coefficients from the state, ln a from the thread's
// scratch, the complexes' molalities as written by this launch.
struct CellView {
  const PfCellState* st;
  long long X;
  const double* lna;  // the thread's ln a, element j at lna[j * bd]
  int bd;
  __device__ __forceinline__ int64_t at(int k) const { return (int64_t)k * st->ncells + X; }
  __device__ __forceinline__ double m(int j) const { return st->pri_molal[at(j)]; }
  __device__ __forceinline__ double ln_act(int j) const { return lna[j * bd]; }
  __device__ __forceinline__ double ln_sec_act(int i) const {
    return log(st->sec_molal[at(i)]) + log(st->sec_act_coef[at(i)]);
  }
};

// Rate prefactors (instantiations with HAS_LNA only)
__device__ __noinline__ double pref_rate(const Tables& T, const CellView& cv, double temp, int m) {
  double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
  return prefactor_rate(
      T, m, [&](int j) { return cv.ln_act(j); }, [&](int i) { return cv.ln_sec_act(i); }, temp, pref, lnps);
}

// adds the prefactor part of the reaction Jacobian of the minerals in mask
// to the diagonal block D (column-major, columns scaled by m when logf)
__device__ __noinline__ void pref_jacobian(const DevNet& net, const Tables& T, const CellView& cv, double temp,
                                           double volume, bool logf, bool tsec, unsigned mask, double* D) {
  const PfCellState& st = *cv.st;
  const int n = net.n;
  auto ln_act = [&](int j) { return cv.ln_act(j); };
  auto ln_sec_act = [&](int i) { return cv.ln_sec_act(i); };
  for (int m = 0; m < net.nm; ++m) {
    if (!((mask >> m) & 1u)) continue;
    double pref[PF_MAX_PREFACTORS], lnps[PF_MAX_PREFACTORS][PF_MAX_PREFACTOR_SPECIES];
    const double sum = prefactor_rate(T, m, ln_act, ln_sec_act, temp, pref, lnps);
    prefactor_derivative(
        T, m, st.mnrl_rate[cv.at(m)] * volume, sum, pref, lnps, ln_act, ln_sec_act,
        [&](int j) { return st.pri_act_coef[cv.at(j)]; }, [&](int i) { return st.sec_act_coef[cv.at(i)]; },
        [&](int j) { return log(cv.m(j)); },
        [&](int i) {
          return add_h2o(-(tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i)) * LOG_TO_LN, T.sec_h2o(i),
                         cell_lnaw(net, st, cv.X));
        },
        temp,
        [&](int r, int c, double v) { D[c * n + r] = fma(v, logf ? cv.m(c) : 1.0, D[c * n + r]); });
  }
}

// The mineral part of RReaction's residual for one cell (RKineticMineral
// without the derivative, reaction_mineral.F90:647-913), at primary ln
// activities lna[] and complexes' ln activities ln_sec_act(i): the same
// arithmetic as the cell kernel's mineral loop, with ln Q/K summed as the
// reference sums it.
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
__device__ __noinline__ void numerical_reaction_jacobian(const DevNet& net, const Tables& T, const CellView& cv,
                                                         double temp, double volume, bool logf, bool tsec,
                                                         double* D) {
  const PfCellState& st = *cv.st;
  const long long X = cv.X;
  const int n = net.n;
  double lna[PF_MAX_NCOMP], res0[PF_MAX_NCOMP], res1[PF_MAX_NCOMP];
  for (int j = 0; j < n; ++j) {
    lna[j] = cv.ln_act(j);
    res0[j] = 0.0;
  }
  // RTotal of the copy at lna[], complex i, as the reference's RTotal forms
  // it (both residuals from the same formula, so that their difference is
  // the perturbation's alone)
  auto ln_sec_act = [&](int i) {
    double lnQK = -(tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i)) * LOG_TO_LN;
    if (water_on(net)) lnQK = add_h2o(lnQK, T.sec_h2o(i), cell_lnaw(net, st, X));
    for (int p = T.sec_begin(i); p < T.sec_end(i); ++p) lnQK = lnQK + T.sec_nu(p) * lna[T.sec_idx(p)];
    const double g = st.sec_act_coef[cv.at(i)];
    return log(exp(lnQK) / g) + log(g);
  };
  mineral_residual(net, T, st, X, lna, ln_sec_act, temp, volume, res0);
  for (int jc = 0; jc < n; ++jc) {
    const double m0 = cv.m(jc);
    const double pert = m0 * 1.0e-5;  // perturbation_tolerance, reaction.F90:41
    const double saved = lna[jc];
    lna[jc] = log(m0 + pert) + log(st.pri_act_coef[cv.at(jc)]);
    for (int i = 0; i < n; ++i) res1[i] = 0.0;
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

// 32-byte store of four doubles (dst 32-byte aligned): one whole sector
__device__ __forceinline__ void st_sector(double* dst, double a, double b, double c, double d) {
  asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(dst), "d"(a), "d"(b), "d"(c), "d"(d) : "memory");
}

// Kernel of one cell per thread.  HAS_PF: rate prefactors; NUMJAC: the
// reaction Jacobian by forward differences (instantiated with HAS_PF, whose
// rate code it needs).  vec: doubles per store of the block writes (4: every
// block starts on a 32-byte boundary and n*n % 4 == 0; 2: 16 bytes; 1).
// staged: the tables are copied into the block's shared memory.  kmode: 0
// without a K cache, 1 computing the per-cell K of the reactions into kcache,
// 2 reading them from it.
template <bool HAS_PF, bool NUMJAC>
__device__ __forceinline__ void girt_cell(const DevNet& net, const GirtTabs& gt, const PfCellState& st, const Geo& g,
                                          double dt, const int32_t* __restrict__ rowptr,
                                          const int32_t* __restrict__ colidx, double* __restrict__ r,
                                          double* __restrict__ values, int vec, int staged,
                                          double* __restrict__ kcache, int kmode, double* __restrict__ Eg) {
  constexpr bool HAS_LNA = HAS_PF || NUMJAC;
  extern __shared__ __align__(16) unsigned char sraw[];
  const int bd = blockDim.x;
  const Layout Lo = layout(net, HAS_LNA, Eg == nullptr);
  double* const Kc = reinterpret_cast<double*>(sraw);
  size_t off = block_k_bytes(net);
  const int32_t* sI = net.ints;
  const double* sD = net.dbls;
  const unsigned char* gbase = reinterpret_cast<const unsigned char*>(gt.buf);
  if (staged) {
    int32_t* dI = reinterpret_cast<int32_t*>(sraw + off);
    for (int k = threadIdx.x; k < net.int_words; k += bd) dI[k] = net.ints[k];
    off += pad16((size_t)net.int_words * 4);
    double* dD = reinterpret_cast<double*>(sraw + off);
    for (int k = threadIdx.x; k < net.dbl_words; k += bd) dD[k] = net.dbls[k];
    off += pad16((size_t)net.dbl_words * 8);
    const int gw = (gt.ibytes + gt.dbytes) / 8;  // both parts are 8-byte multiples
    double* dG = reinterpret_cast<double*>(sraw + off);
    for (int k = threadIdx.x; k < gw; k += bd) dG[k] = reinterpret_cast<const double*>(gt.buf)[k];
    sI = dI;
    sD = dD;
    gbase = sraw + off;
    off += (size_t)gt.ibytes + gt.dbytes;
  }
  const int32_t* gI = reinterpret_cast<const int32_t*>(gbase);
  const double* gD = reinterpret_cast<const double*>(gbase + gt.ibytes);
  const int32_t* __restrict__ s_pair_ptr = gI + gt.o_spp;
  const int32_t* __restrict__ s_pair_k = gI + gt.o_spk;
  const double* __restrict__ s_pair_c = gD + gt.d_spc;
  const int32_t* __restrict__ m_ent_ptr = gI + gt.o_mep;
  const int32_t* __restrict__ m_ent_m = gI + gt.o_mem;
  const double* __restrict__ m_ent_c = gD + gt.d_mec;
  const Tables T{sI, sD, &net};
  const int n = net.n, nn = n * n, ns = net.ns, nm = net.nm;
  const bool has_h2o = water_on(net);
  const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
  const bool tmin = !net.o.isothermal && (net.flags & NETF_MNRL_LOGKCOEF);
  const bool kc_sec = !tsec && !has_h2o, kc_mn = !tmin && !has_h2o;
  if (kmode != 2)
    for (int k = threadIdx.x; k < ns + nm; k += bd) {
      if (k < ns ? kc_sec : kc_mn)
        Kc[k] = exp(-(k < ns ? net.dbls[net.o_sec_logK + k] : net.dbls[net.o_mnrl_logK + k - ns]) * LOG_TO_LN);
    }
  __syncthreads();
  const long long X = (long long)blockIdx.x * bd + threadIdx.x;
  if (X >= st.ncells) return;
  double* P = reinterpret_cast<double*>(sraw + off) + threadIdx.x;  // element e at P[e * bd]
  const SoA soa{st.ncells};
  const bool logf = net.o.use_log_formulation != 0;
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  unsigned pf_active = 0;  // minerals whose prefactor derivative is due
  const double temp = st.temperature ? st.temperature[X] : 25.0;
  const double lnaw = cell_lnaw(net, st, X);
  const double den_k = st.den_kg[X], den_L = den_k * 1.0e-3;
  const double por = st.porosity[X], sat = st.saturation[X], volume = st.volume[X];
  const bool dry = sat < RT_MIN_SATURATION;
  const unsigned neg = (unsigned)net.neg_mask;
  // K of complex i (divided by its activity coefficient) and of mineral m:
  // the block's table, or logK at the cell's temperature (ln T and 1/T once
  // per cell) with the water term; cached per cell when kmode != 0
  const LogKAtT logk_t(temp);
  auto k_sec = [&](int i) {
    if (kmode == 2) return kcache[soa.at(i, X)];
    double K;
    if (kc_sec) {
      K = Kc[i];
    } else {
      const double logK = tsec ? logk_t(T.sec_logKcoef(i)) : T.sec_logK(i);
      K = exp(add_h2o(-logK * LOG_TO_LN, T.sec_h2o(i), lnaw));
    }
    K = K / st.sec_act_coef[soa.at(i, X)];
    if (kmode == 1) kcache[soa.at(i, X)] = K;
    return K;
  };
  auto k_mn = [&](int m) {
    if (kmode == 2) return kcache[soa.at(ns + m, X)];
    double K;
    if (kc_mn) {
      K = Kc[ns + m];
    } else {
      const double logK = tmin ? logk_t(T.mnrl_logKcoef(m)) : T.mnrl_logK(m);
      K = exp(add_h2o(-logK * LOG_TO_LN, T.mnrl_h2o(m), lnaw));
    }
    if (kmode == 1) kcache[soa.at(ns + m, X)] = K;
    return K;
  };
  // ---- RTotalAqueous (reaction.F90:4665-4759) in product form: s_i =
  // (K_i / gamma_i) prod_j a_j^nu_ij, each factor one or two multiplies from
  // a and 1/a for nu in {+-1, +-2} (exp(nu ln a) otherwise); the reference's
  // exp(ln K + sum nu ln a) / gamma_i to rounding
  for (int j = 0; j < n; ++j) {
    const double m = st.pri_molal[soa.at(j, X)], gam = st.pri_act_coef[soa.at(j, X)];
    const double a = m * gam;
    P[(Lo.pa + j) * bd] = a;
    if ((neg >> j) & 1u) P[(Lo.pa + n + j) * bd] = 1.0 / a;
    P[(Lo.T + j) * bd] = m;  // total = m, then += nu s
    if constexpr (HAS_LNA) P[(Lo.lna + j) * bd] = log(m) + log(gam);
  }
  const int nsym = n * (n + 1) / 2;
  // the packed sum: in the thread's shared scratch, or (Eg) in global memory,
  // [entry][cell], when the shared scratch would cap the resident warps
  auto Eref = [&](int k) -> double& { return Eg ? Eg[(size_t)k * st.ncells + X] : P[(Lo.E + k) * bd]; };
  for (int k = 0; k < nsym; ++k) Eref(k) = 0.0;
  // factor a_j^nu from its power-table code (0: a, 1: a^2, 2: 1/a, 3: 1/a^2)
  auto factor = [&](int pe, double nu, int j) {
    if (pe >= 0) {
      const int code = pe / n;
      const double b = P[(Lo.pa + (code >= 2 ? n : 0) + j) * bd];
      return (code & 1) ? b * b : b;
    }
    const double la = HAS_LNA ? P[(Lo.lna + j) * bd] : log(P[(Lo.pa + j) * bd]);
    return exp(nu * la);
  };
  for (int i = 0; i < ns; ++i) {
    double s = k_sec(i);
    const int b = T.sec_begin(i), e = T.sec_end(i);
    for (int p = b; p < e; ++p) s *= factor(T.sec_pidx(p), T.sec_nu(p), T.sec_idx(p));
    st.sec_molal[soa.at(i, X)] = s;
    // totals in the reference's order: per component, the complexes ascending
    for (int p = b; p < e; ++p) {
      const int a = (Lo.T + T.sec_idx(p)) * bd;
      P[a] = P[a] + T.sec_nu(p) * s;
    }
    // sum_i nu_ri nu_ci s_i, complexes ascending as the reference's entries
    for (int q = s_pair_ptr[i]; q < s_pair_ptr[i + 1]; ++q) {
      double& a = Eref(s_pair_k[q]);
      a = fma(s_pair_c[q], s, a);
    }
  }
  for (int j = 0; j < n; ++j) st.total[soa.at(j, X)] = P[(Lo.T + j) * bd] * den_L;
  // ---- RKineticMineral (reaction_mineral.F90:647-1078): rates, reaction
  // residual (into r, finished by girt_residual_kernel), derivative factors
  // (GQ takes the place of the totals)
  for (int j = 0; j < n; ++j) r[X * n + j] = 0.0;
  const CellView cv{&st, X, P + Lo.lna * bd, bd};
  for (int m = 0; m < nm; ++m) {
    const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
    double GQ = 0.0;
    if (!dry) {
      double QK = k_mn(m);
      for (int p = b; p < e; ++p) QK *= factor(T.mnrl_pidx(p), T.mnrl_nu(p), T.mnrl_idx(p));
      double aff;
      if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
      else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
      else aff = 1.0 - QK;
      const double sign_ = fsign1(aff);
      const double vf = st.mnrl_volfrac[soa.at(m, X)];
      const bool active = (vf > 0 || sign_ < 0.0) && !(T.irreversible(m) == 1 && sign_ < 0.0) &&
                          !(T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m));
      double rate_out = 0.0;
      if (active) {
        const double rl = T.limiter(m);
        if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
        double kr;
        if (HAS_PF && T.pf_cnt(m) > 0) {
          kr = pref_rate(T, cv, temp, m);
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
        double Gm;
        if (rl > 0.0) {
          const double den = 1.0 + (1.0 - aff) / rl;
          Gm = dIm_dQK * (1.0 + QK / rl / den) / den;
        } else {
          Gm = dIm_dQK;
        }
        // d rate_r/d m_c = nu_r Gm nu_c QK / m_c den_kg 1e-3 (:944-947, :1062-1071)
        GQ = Gm * QK * den_k * 1.0e-3;
      }
      st.mnrl_rate[soa.at(m, X)] = rate_out;
    } else if (kmode == 1) {
      k_mn(m);  // the cache holds every cell's K
    }
    P[(Lo.GQ + m) * bd] = GQ;
  }
  // ---- d total/d m in the column scaling: log formulation
  // den (delta_rc m_c + sum_i nu_ri nu_ci s_i), symmetric; the linear one
  // divides the sum by m_c per column at the write, from 1/m in pa
  if (logf) {
    for (int hi = 0, k = 0; hi < n; ++hi)
      for (int lo = 0; lo <= hi; ++lo, ++k) {
        double& a = Eref(k);
        a = (lo == hi ? a + st.pri_molal[soa.at(hi, X)] : a) * den_L;
      }
  } else {
    for (int j = 0; j < n; ++j) {
      const double im = 1.0 / st.pri_molal[soa.at(j, X)];
      P[(Lo.pa + j) * bd] = im;
      P[(Lo.pa + n + j) * bd] = den_L * im;
    }
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
  // entry fe of the column-major block: e = d total/d m in the column scaling,
  // v = the diagonal block's value
  auto entry = [&](int fe, double& v, double& e) {
    const int col = fe / n, row = fe - col * n;
    const double E = Eref(sym_index(row, col));
    const double im = logf ? 0.0 : P[(Lo.pa + col) * bd];
    e = logf ? E : fma(E, P[(Lo.pa + n + col) * bd], row == col ? den_L : 0.0);
    if (dry) {
      v = fma(csum, e, row == col ? (logf ? st.pri_molal[soa.at(col, X)] : 1.0) : 0.0);
      return;
    }
    double jl = 0.0;
    if (!NUMJAC) {
      const int f = row * n + col;
      const int qb = m_ent_ptr[f], qe = m_ent_ptr[f + 1];
      if (qb < qe) {
        for (int q = qb; q < qe; ++q) jl = fma(m_ent_c[q], P[(Lo.GQ + m_ent_m[q]) * bd], jl);
        // the reference zeroes |d R/d m| < 1e-40 before the column scaling
        // (reaction.F90:4232-4237)
        if (logf) {
          if (fabs(jl) < 1.0e-40 * st.pri_molal[soa.at(col, X)]) jl = 0.0;
        } else {
          jl = jl * im;
          if (fabs(jl) < 1.0e-40) jl = 0.0;
        }
      }
    }
    v = fma(cdiag, e, jl);
  };
  if (vec == 4) {
    for (int fe = 0; fe < nn; fe += 4) {
      double v[4], e[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) entry(fe + u, v[u], e[u]);
      if (dblk >= 0) st_sector(values + (size_t)dblk * nn + fe, v[0], v[1], v[2], v[3]);
#pragma unroll
      for (int q = 0; q < 6; ++q)
        if (blk[q] >= 0)
          st_sector(values + (size_t)blk[q] * nn + fe, sc[q] * e[0], sc[q] * e[1], sc[q] * e[2], sc[q] * e[3]);
    }
  } else if (vec == 2) {
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
  if constexpr (HAS_LNA) {
    if (NUMJAC && !dry && dblk >= 0)
      numerical_reaction_jacobian(net, T, cv, temp, volume, logf, tsec, values + (size_t)dblk * nn);
    else if (HAS_PF && pf_active && dblk >= 0)
      pref_jacobian(net, T, cv, temp, volume, logf, tsec, pf_active, values + (size_t)dblk * nn);
  }
  // ---- equilibrium sorption (RTotalSorb in RTUpdateAuxVars; a failed
  // ion-exchange solve leaves the last iterate, the reference's
  // message-and-continue).  Only this thread writes its diagonal block.
  if (has_sorption(net) && dblk >= 0) {
    for (int jj = 0; jj < n; ++jj) st.total_sorb[soa.at(jj, X)] = 0.0;
    double* D = values + (size_t)dblk * nn;
    const double v_t = volume / dt;
    total_sorb(
        net, T, [&](int j) { return st.pri_molal[soa.at(j, X)]; }, [&](int j) { return st.pri_act_coef[soa.at(j, X)]; },
        [&](int m) { return st.mnrl_volfrac[soa.at(m, X)]; }, por, den_k,
        st.ionx_ref_sorbed ? st.ionx_ref_sorbed + X : nullptr, st.ncells,
        [&](int j, double v) { st.total_sorb[soa.at(j, X)] += v; },
        [&](int i, int j, double v) {
          D[j * n + i] = fma(v * v_t, logf ? st.pri_molal[soa.at(j, X)] : 1.0, D[j * n + i]);
        },
        surf_cell(net, st, X));
  }
}

#define PF_GIRT_CELL_ARGS                                                                                           \
  DevNet net, GirtTabs gt, PfCellState st, Geo g, double dt, const int32_t* __restrict__ rowptr,                   \
      const int32_t* __restrict__ colidx, double* __restrict__ r, double* __restrict__ values, int vec, int staged, \
      double* __restrict__ kcache, int kmode, double* __restrict__ Eg
template <bool HAS_PF, bool NUMJAC>
__global__ void __launch_bounds__(128, 5) girt_cell_kernel(PF_GIRT_CELL_ARGS) {
  girt_cell<HAS_PF, NUMJAC>(net, gt, st, g, dt, rowptr, colidx, r, values, vec, staged, kcache, kmode, Eg);
}
#undef PF_GIRT_CELL_ARGS

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
  // per complex: its reaction's species pairs (p <= q in the reaction's list)
  std::vector<int32_t> sp_ptr{0}, sp_k;
  std::vector<double> sp_c;
  for (int i = 0; i < net.ns; ++i) {
    const int b = I[net.o_sec_ptr + i], e = I[net.o_sec_ptr + i + 1];
    for (int p = b; p < e; ++p)
      for (int q = p; q < e; ++q) {
        const int r = I[net.o_sec_idx + p], c = I[net.o_sec_idx + q];
        const int hi = r > c ? r : c, lo = r > c ? c : r;
        sp_k.push_back(hi * (hi + 1) / 2 + lo);
        sp_c.push_back(D[net.o_sec_nu + p] * D[net.o_sec_nu + q]);
      }
    sp_ptr.push_back((int32_t)sp_k.size());
  }
  // per flat entry row*n+col: the minerals whose reaction holds both species
  std::vector<std::vector<int32_t>> em(nn);
  std::vector<std::vector<double>> ec(nn);
  for (int m = 0; m < net.nm; ++m) {
    const int b = I[net.o_mnrl_ptr + m], e = I[net.o_mnrl_ptr + m + 1];
    for (int pr = b; pr < e; ++pr)
      for (int pc = b; pc < e; ++pc) {
        const int f = I[net.o_mnrl_idx + pr] * n + I[net.o_mnrl_idx + pc];
        em[f].push_back(m);
        ec[f].push_back(D[net.o_mnrl_nu + pr] * D[net.o_mnrl_nu + pc]);
      }
  }
  std::vector<int32_t> ints;
  std::vector<double> dbls;
  out->o_spp = (int)ints.size();
  ints.insert(ints.end(), sp_ptr.begin(), sp_ptr.end());
  out->o_spk = (int)ints.size();
  ints.insert(ints.end(), sp_k.begin(), sp_k.end());
  out->o_mep = (int)ints.size();
  int cnt = 0;
  for (auto& rw : em) { ints.push_back(cnt); cnt += (int)rw.size(); }
  ints.push_back(cnt);
  out->o_mem = (int)ints.size();
  for (auto& rw : em) ints.insert(ints.end(), rw.begin(), rw.end());
  out->d_spc = (int)dbls.size();
  dbls.insert(dbls.end(), sp_c.begin(), sp_c.end());
  out->d_mec = (int)dbls.size();
  for (auto& rw : ec) dbls.insert(dbls.end(), rw.begin(), rw.end());
  if (dbls.empty()) dbls.push_back(0.0);
  while (ints.size() % 4) ints.push_back(0);  // the doubles start on a 16-byte boundary
  const size_t ib = ints.size() * 4;
  void* buf = nullptr;
  if (cudaMalloc(&buf, ib + dbls.size() * 8) != cudaSuccess) return PF_ERR_CUDA;
  if (cudaMemcpy(buf, ints.data(), ib, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy((char*)buf + ib, dbls.data(), dbls.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(buf);
    return PF_ERR_CUDA;
  }
  out->buf = buf;
  out->ibytes = (int)ib;
  out->dbytes = (int)(dbls.size() * 8);
  *d_buf = buf;
  return PF_OK;
}

// threads per block of the cell kernel, whether the tables are staged in
// shared memory, and the dynamic shared memory: the block size (a multiple
// of 32, at most 128) that keeps the most warps resident, staging the tables
// when that costs no warps
size_t girt_smem_bytes(const DevNet& net, const GirtTabs& gt, bool with_lna, bool e_in_smem, int* threads_per_block,
                       int* staged) {
  const size_t tbytes = (size_t)girt::layout(net, with_lna, e_in_smem).per_thread * sizeof(double);
  const size_t kbytes = girt::block_k_bytes(net), tab = girt::block_table_bytes(net, gt);
  const size_t sm_bytes = 228u * 1024u, per_block_reserved = 1024u;
  int best = 0, best_warps = -1, best_staged = 0;
  for (int st = 1; st >= 0; --st) {
    for (int tpb = 32; tpb <= 128; tpb += 32) {
      const size_t b = tpb * tbytes + kbytes + (st ? tab : 0);
      if (b > 227u * 1024u) break;
      int blocks = (int)(sm_bytes / (b + per_block_reserved));
      if (blocks > 32) blocks = 32;
      const int warps = blocks * tpb / 32 > 48 ? 48 : blocks * tpb / 32;
      if (warps > best_warps || (warps == best_warps && st == best_staged)) {
        best_warps = warps;
        best = tpb;
        best_staged = st;
      }
    }
  }
  if (best == 0) return (size_t)-1;
  if (threads_per_block) *threads_per_block = best;
  if (staged) *staged = best_staged;
  return best * tbytes + kbytes + (best_staged ? tab : 0);
}

int launch_girt_assemble(const DevNet& net, const GirtTabs& gt, const PfCellState& st, const PfGirtArgs& a,
                         int num_sms, cudaStream_t s, double* e_scratch) {
  (void)num_sms;
  if (st.ncells == 0) return PF_OK;
  girt::Geo g{a.nx, a.ny, a.nz, a.dx, a.dy, a.dz, a.diffusion_coefficient, a.tortuosity, a.dispersivity,
              a.qx, a.qy, a.qz};
  const bool pf = (net.flags & NETF_PREFACTOR) != 0;
  const bool with_lna = pf || a.numerical_derivatives;
  const int nn = net.n * net.n;
  const uintptr_t va = (uintptr_t)a.values;
  auto k = a.numerical_derivatives ? girt::girt_cell_kernel<true, true>
           : pf                    ? girt::girt_cell_kernel<true, false>
                                   : girt::girt_cell_kernel<false, false>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
    return PF_ERR_CUDA;
  // the block size and table staging that keep the most warps resident, the
  // kernel's registers included (occupancy calculator); staging on a tie
  const bool e_smem = e_scratch == nullptr;
  const size_t tbytes = (size_t)girt::layout(net, with_lna, e_smem).per_thread * sizeof(double);
  const size_t kbytes = girt::block_k_bytes(net), tab = girt::block_table_bytes(net, gt);
  int tpb = 0, staged = 0, best_warps = 0;
  size_t smem = 0;
  for (int stg = 1; stg >= 0; --stg)
    for (int t = 32; t <= 128; t += 32) {
      const size_t b = t * tbytes + kbytes + (stg ? tab : 0);
      if (b > 227u * 1024u) continue;
      int nb = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, t, b) != cudaSuccess) return PF_ERR_CUDA;
      if (nb * t / 32 > best_warps) {
        best_warps = nb * t / 32;
        tpb = t;
        staged = stg;
        smem = b;
      }
    }
  if (tpb == 0) return PF_ERR_TOO_LARGE;
  // whole-sector stores when every block starts on a 32-byte boundary
  const int vec = (nn % 4 == 0 && (va & 31) == 0) ? 4 : ((nn % 2 == 0 && (va & 15) == 0) ? 2 : 1);
  const int kmode = a.k_cache ? (a.k_cache_valid ? 2 : 1) : 0;
  const long long blocks = (st.ncells + tpb - 1) / tpb;
  k<<<(unsigned)blocks, tpb, smem, s>>>(net, gt, st, g, a.dt, a.rowptr, a.colidx, a.residual, a.values, vec, staged,
                                        a.k_cache, kmode, e_scratch);
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
