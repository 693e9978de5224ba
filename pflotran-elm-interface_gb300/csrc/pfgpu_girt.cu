// pfgpu_girt.cu -- global-implicit residual and BAIJ Jacobian assembly on a
// structured grid (7-point stencil).
//
// Replaces, for the interior of a structured grid with zero-flux outer
// boundaries, the per-Newton-iteration assembly of
//   RTResidualFlux / RTResidualNonFlux  (src/pflotran/reactive_transport.F90:2052-2669)
//   RTJacobianFlux / RTJacobianNonFlux  (:2897-3349, log scaling :2879, :3316-3340)
// with TDispersion/TFluxCoef/TFlux/TFluxDerivative (transport.F90:52-609).
//
// Two kernels:
//   girt_cell_kernel   one thread per cell: RTotal (totals, dtotal), the
//                      reaction residual and RReactionDerivative block -> scratch
//                      (FP64-bound; the same per-cell chemistry as a Newton
//                      evaluation)
//   girt_row_kernel    one warp per block row: every entry of the row's (up to)
//                      seven ncomp x ncomp blocks and the row's residual, written
//                      as consecutive doubles (coalesced stores of the
//                      PETSc SeqBAIJ layout: blocks in ascending column order,
//                      each block column-major).
// Contributions are summed in the reference's order: connections x, then y,
// then z (each cell sees its lower-index connection first), then
// accumulation, then reaction; the log formulation scales block columns by the
// column cell's free-ion molalities last (MatDiagonalScaleLocal).
#include <vector>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

namespace pfgpu {
namespace girt {

constexpr int NM = PF_MAX_NCOMP;

struct Geo {
  int nx, ny, nz;
  double dx, dy, dz;
  double diffusion, tortuosity, dispersivity;
  const double* qx;
  const double* qy;
  const double* qz;
};

// per-cell scratch layout (doubles, cell-major): tot[n] dtot[n*n] jrxn[n*n] rrxn[n]
__host__ __device__ inline int scratch_stride(int n) { return 2 * n + 2 * n * n; }

__global__ void __launch_bounds__(128) girt_cell_kernel(DevNet net, PfCellState st, double* __restrict__ sc) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= st.ncells) return;
  const Tables T{net.ints, net.dbls, &net};
  const SoA soa{st.ncells};
  const int n = net.n, ns = net.ns, nm = net.nm;
  const int stride = scratch_stride(n);
  double* out = sc + (size_t)cell * stride;
  double* tot = out;
  double* dtot = out + n;
  double* jrxn = out + n + n * n;
  double* rrxn = out + n + 2 * n * n;
  const double temp = st.temperature ? st.temperature[cell] : 25.0;
  const bool tsec = !net.o.isothermal && (net.flags & NETF_SEC_LOGKCOEF);
  const bool tmin = !net.o.isothermal && (net.flags & NETF_MNRL_LOGKCOEF);
  const double den_k = st.den_kg[cell], den_L = den_k * 1.0e-3;
  double c[NM], lnc[NM], lna[NM], ic[NM], t[NM], D[NM * NM];
  for (int j = 0; j < n; ++j) {
    c[j] = st.pri_molal[soa.at(j, cell)];
    lnc[j] = log(c[j]);
    lna[j] = lnc[j] + log(st.pri_act_coef[soa.at(j, cell)]);
    ic[j] = 1.0 / c[j];
    t[j] = c[j];
    for (int k = 0; k < n; ++k) D[j * NM + k] = (j == k) ? 1.0 : 0.0;
  }
  // RTotalAqueous (reaction.F90:4665-4759); exp(lnQK - ln m_j)/gamma = s/m_j
  for (int i = 0; i < ns; ++i) {
    const double logK = tsec ? interp_logK(T.sec_logKcoef(i), temp) : T.sec_logK(i);
    double lnQK = -logK * LOG_TO_LN;
    const int b = T.sec_begin(i), e = T.sec_end(i);
    for (int p = b; p < e; ++p) lnQK = lnQK + T.sec_nu(p) * lna[T.sec_idx(p)];
    const double s = exp(lnQK) / st.sec_act_coef[soa.at(i, cell)];
    st.sec_molal[soa.at(i, cell)] = s;
    for (int p = b; p < e; ++p) t[T.sec_idx(p)] += T.sec_nu(p) * s;
    for (int pj = b; pj < e; ++pj) {
      const int jc = T.sec_idx(pj);
      const double tr = T.sec_nu(pj) * s * ic[jc];
      for (int pi = b; pi < e; ++pi) D[T.sec_idx(pi) * NM + jc] += T.sec_nu(pi) * tr;
    }
  }
  for (int j = 0; j < n; ++j) {
    tot[j] = t[j] * den_L;
    st.total[soa.at(j, cell)] = tot[j];
    for (int k = 0; k < n; ++k) dtot[j * n + k] = D[j * NM + k] * den_L;
  }
  // RReaction / RReactionDerivative (reaction.F90:4059-4240): kinetic minerals
  double R[NM];
  for (int j = 0; j < n; ++j) {
    R[j] = 0.0;
    for (int k = 0; k < n; ++k) D[j * NM + k] = 0.0;
  }
  const double sat = st.saturation[cell], volume = st.volume[cell];
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  if (!(sat < RT_MIN_SATURATION)) {
    for (int m = 0; m < nm; ++m) {
      st.mnrl_rate[soa.at(m, cell)] = 0.0;
    }
    for (int m = 0; m < nm; ++m) {
      const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
      const double logK = tmin ? interp_logK(T.mnrl_logKcoef(m), temp) : T.mnrl_logK(m);
      double lnQK = -logK * LOG_TO_LN;
      for (int p = b; p < e; ++p) lnQK = lnQK + T.mnrl_nu(p) * lna[T.mnrl_idx(p)];
      const double QK = exp(lnQK);
      double aff;
      if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
      else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
      else aff = 1.0 - QK;
      const double sign_ = fsign1(aff);
      const double vf = st.mnrl_volfrac[soa.at(m, cell)];
      if (!(vf > 0 || sign_ < 0.0)) continue;
      if (T.irreversible(m) == 1 && sign_ < 0.0) continue;
      if (T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m)) continue;
      const double rl = T.limiter(m);
      if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
      double arr = 1.0;
      if (T.ea(m) > 0.0) arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp + 273.15)));
      const double k = T.rate(m) * arr;
      double Im_const = -st.mnrl_area[soa.at(m, cell)];
      if (has_msf) Im_const = Im_const / T.msf(m);
      double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * k : Im_const * sign_ * fabs(aff) * k;
      st.mnrl_rate[soa.at(m, cell)] = Im;
      Im_const = Im_const * volume;
      Im = Im * volume;
      for (int p = b; p < e; ++p) R[T.mnrl_idx(p)] += T.mnrl_nu(p) * Im;
      double dIm_dQK = has_pw ? -Im * T.power(m) / fabs(aff) : -Im_const * k;
      if (has_tk) dIm_dQK = dIm_dQK * (1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m))) / QK * (1.0 - aff);
      else if (has_msf) dIm_dQK = dIm_dQK * (1.0 / T.msf(m)) / QK * (1.0 - aff);
      const double den = 1.0 + (1.0 - aff) / rl;
      for (int pj = b; pj < e; ++pj) {
        const int jc = T.mnrl_idx(pj);
        const double dQK_dmj = T.mnrl_nu(pj) * QK * ic[jc] * den_k * 1.0e-3;
        for (int pi = b; pi < e; ++pi) {
          const int icp = T.mnrl_idx(pi);
          if (rl <= 0.0) D[icp * NM + jc] += T.mnrl_nu(pi) * dIm_dQK * dQK_dmj;
          else D[icp * NM + jc] += T.mnrl_nu(pi) * dIm_dQK * (1.0 + QK / rl / den) * dQK_dmj / den;
        }
      }
    }
  }
  for (int j = 0; j < n; ++j) {
    rrxn[j] = R[j];
    for (int k = 0; k < n; ++k) {
      const double v = D[j * NM + k];
      jrxn[j * n + k] = fabs(v) < 1.0e-40 ? 0.0 : v;  // reaction.F90:4232-4237
    }
  }
}

// harmonic_tran_coefs_over_dist (transport.F90:199-225) for a connection at
// the midpoint of equal cells (dist_up = dist_dn = dist/2)
__device__ __forceinline__ double tran_coef(double por_up, double sat_up, double por_dn, double sat_dn, double q,
                                            double dist, const Geo& g) {
  if (sat_up < RT_MIN_SATURATION || sat_dn < RT_MIN_SATURATION) return 0.0;
  const double dist_up = dist * 0.5, dist_dn = dist - dist_up;
  const double mech = g.dispersivity * fabs(q);
  const double hu = fmax(mech + 1.0 * sat_up * por_up * g.tortuosity * g.diffusion, 1.0e-40);
  const double hd = fmax(mech + 1.0 * sat_dn * por_dn * g.tortuosity * g.diffusion, 1.0e-40);
  return (hu * hd) / (hu * dist_dn + hd * dist_up);
}

struct Conn {
  long long other;  // neighbour cell
  double cup, cdn;  // T_up, T_dn (component independent), L/s
  int self_is_up;
};

__global__ void __launch_bounds__(256) girt_row_kernel(DevNet net, PfCellState st, Geo g, const double* __restrict__ sc,
                                                       const double* __restrict__ total_k, double dt,
                                                       const int32_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ colidx, double* __restrict__ r,
                                                       double* __restrict__ values) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const int n = net.n, nn = n * n;
  const int stride = scratch_stride(n);
  const long long N = st.ncells;
  const long long nxy = (long long)g.nx * g.ny;
  const bool logf = net.o.use_log_formulation != 0;
  for (long long X = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); X < N; X += warps) {
    const int i = (int)(X % g.nx), j = (int)((X / g.nx) % g.ny), k = (int)(X / nxy);
    const double por = st.porosity[X], sat = st.saturation[X];
    // the cell's connections in the reference's order: x-, x+, y-, y+, z-, z+
    Conn cs[6];
    int nc = 0;
    auto add = [&](bool exists, long long other, double q, double area, double dist, int self_up) {
      if (!exists) return;
      const long long up = self_up ? X : other, dn = self_up ? other : X;
      const double pu = st.porosity[up], su = st.saturation[up], pdn = st.porosity[dn], sdn = st.saturation[dn];
      double cup = 0.0, cdn = 0.0;
      if (!(sdn < RT_MIN_SATURATION) && !(su < RT_MIN_SATURATION)) {
        const double tr = tran_coef(pu, su, pdn, sdn, q, dist, g);
        if (q > 0.0) { cup = tr + q; cdn = -tr; }
        else { cup = tr; cdn = -tr + q; }
        cup = cup * area * 1000.0;
        cdn = cdn * area * 1000.0;
      }
      cs[nc++] = Conn{other, cup, cdn, self_up};
    };
    add(i > 0, X - 1, i > 0 ? g.qx[((long long)k * g.ny + j) * (g.nx - 1) + (i - 1)] : 0.0, g.dy * g.dz, g.dx, 0);
    add(i < g.nx - 1, X + 1, i < g.nx - 1 ? g.qx[((long long)k * g.ny + j) * (g.nx - 1) + i] : 0.0, g.dy * g.dz, g.dx, 1);
    add(j > 0, X - g.nx, j > 0 ? g.qy[((long long)k * (g.ny - 1) + (j - 1)) * g.nx + i] : 0.0, g.dx * g.dz, g.dy, 0);
    add(j < g.ny - 1, X + g.nx, j < g.ny - 1 ? g.qy[((long long)k * (g.ny - 1) + j) * g.nx + i] : 0.0, g.dx * g.dz,
        g.dy, 1);
    add(k > 0, X - nxy, k > 0 ? g.qz[((long long)(k - 1) * g.ny + j) * g.nx + i] : 0.0, g.dx * g.dy, g.dz, 0);
    add(k < g.nz - 1, X + nxy, k < g.nz - 1 ? g.qz[((long long)k * g.ny + j) * g.nx + i] : 0.0, g.dx * g.dy, g.dz,
        1);
    const double* sx = sc + (size_t)X * stride;
    const double* dtot_x = sx + n;
    const double psv = por * sat * 1000.0 * st.volume[X];
    const double psvd_t = psv / dt;
    const bool dry = sat < RT_MIN_SATURATION;
    // ---- residual ----------------------------------------------------------
    for (int row = lane; row < n; row += 32) {
      double v = 0.0;
      for (int q = 0; q < nc; ++q) {
        const double* so = sc + (size_t)cs[q].other * stride;
        const double tu = cs[q].self_is_up ? sx[row] : so[row];
        const double td = cs[q].self_is_up ? so[row] : sx[row];
        const double res = cs[q].cup * tu + cs[q].cdn * td;
        v = cs[q].self_is_up ? v + res : v - res;
      }
      const double accum_k = dry ? 0.0 : psv * total_k[(size_t)row * N + X];
      v = v - accum_k / dt;
      v = v + (dry ? 0.0 : psv * sx[row]) / dt;
      if (!dry) v = v + sx[n + 2 * nn + row];
      r[X * n + row] = v;
    }
    // ---- blocks ------------------------------------------------------------
    const int b0 = rowptr[X], nb = rowptr[X + 1] - b0;
    for (int e = lane; e < nb * nn; e += 32) {
      const int bi = e / nn, fe = e - bi * nn;
      const int col = fe / n, row = fe - col * n;
      const long long Y = colidx[b0 + bi];
      double v;
      if (Y == X) {
        v = 0.0;
        for (int q = 0; q < nc; ++q) {
          const double d = dtot_x[row * n + col];
          v = cs[q].self_is_up ? v + d * cs[q].cup : v + (-(d * cs[q].cdn));
        }
        v = v + (dry ? ((row == col) ? 1.0 : 0.0) : dtot_x[row * n + col] * psvd_t);
        if (!dry) v = v + sx[n + nn + row * n + col];
        if (logf) v = v * st.pri_molal[(size_t)col * N + X];
      } else {
        int q = 0;
        while (q < nc && cs[q].other != Y) ++q;
        if (q < nc) {  // a block column outside the stencil stays zero
          const double* dtot_y = sc + (size_t)Y * stride + n;
          const double d = dtot_y[row * n + col];
          v = cs[q].self_is_up ? d * cs[q].cdn : -(d * cs[q].cup);
          if (logf) v = v * st.pri_molal[(size_t)col * N + Y];
        } else {
          v = 0.0;
        }
      }
      values[(size_t)(b0 + bi) * nn + fe] = v;
    }
  }
}

}  // namespace girt
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

extern "C" int32_t pf_girt_assemble_impl(const DevNet* net, const PfCellState* st, const PfGirtArgs* a, double* scratch,
                                         void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int tpb = 128;
  const int64_t blocks = (st->ncells + tpb - 1) / tpb;
  girt::girt_cell_kernel<<<blocks, tpb, 0, s>>>(*net, *st, scratch);
  if (cudaGetLastError() != cudaSuccess) return PF_ERR_CUDA;
  girt::Geo g{a->nx, a->ny, a->nz, a->dx, a->dy, a->dz, a->diffusion_coefficient, a->tortuosity,
              a->dispersivity, a->qx, a->qy, a->qz};
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int rblocks = sms * 8;
  girt::girt_row_kernel<<<rblocks, 256, 0, s>>>(*net, *st, g, scratch, a->total_k, a->dt, a->rowptr, a->colidx,
                                                a->residual, a->values);
  return cudaGetLastError() == cudaSuccess ? PF_OK : PF_ERR_CUDA;
}

extern "C" size_t pf_girt_scratch_doubles(int32_t n, int64_t ncells) {
  return (size_t)girt::scratch_stride(n) * (size_t)ncells;
}
