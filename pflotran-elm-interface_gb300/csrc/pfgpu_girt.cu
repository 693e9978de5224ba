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
// accumulation and reaction derivatives of X.  One warp owns one cell X and
// writes its whole block column -- the diagonal block and the (Y, X) block of
// every neighbour row Y -- each block as ncomp^2 consecutive doubles, so all
// matrix stores are coalesced and nothing is scattered or accumulated in
// memory.
//
// Two launches per assembly:
//   update_auxvars_kernel (pfgpu_aux.cu)  thread per cell: RTotal -> total,
//                                         sec_molal (RTUpdateAuxVars)
//   girt_column_kernel                    warp per cell: dtotal from sec_molal
//                                         (no exp), kinetic-mineral rates and
//                                         derivatives, the cell's residual row
//                                         and its block column.
// The diagonal flux term sums the connection coefficients first
// ((sum_q c_q) dtot rather than sum_q (c_q dtot)); every c_q there is >= 0
// (upwinding), so the two orders differ by rounding only.
#include <vector>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

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

// doubles of per-warp shared memory: m, 1/m, ln a (n each), the secondary
// column terms t (one per secondary CSR slot), the mineral column terms u (one
// per mineral CSR slot), and per mineral the derivative factor and the rate
__host__ __device__ inline int warp_doubles(const DevNet& net) {
  return (3 * net.n + net.nnz_s + net.nnz_m + 2 * net.nm + 1) & ~1;
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

__global__ void __launch_bounds__(256) girt_column_kernel(DevNet net, GirtTabs gt, PfCellState st, Geo g,
                                                          const double* __restrict__ total_k, double dt,
                                                          const int32_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ colidx,
                                                          double* __restrict__ r, double* __restrict__ values) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const int n = net.n, nn = n * n, ns = net.ns, nm = net.nm;
  double* W = smem + (threadIdx.x >> 5) * warp_doubles(net);
  double* sm_m = W;
  double* sm_ic = W + n;
  double* sm_lna = W + 2 * n;
  double* t = W + 3 * n;
  double* u = t + net.nnz_s;
  double* G = u + net.nnz_m;
  double* Imv = G + nm;
  const Tables T{net.ints, net.dbls, &net};
  const long long N = st.ncells;
  const long long nxy = (long long)g.nx * g.ny;
  const bool logf = net.o.use_log_formulation != 0;
  const bool tmin = !net.o.isothermal && (net.flags & NETF_MNRL_LOGKCOEF);
  const bool has_msf = net.flags & NETF_MSF, has_tk = net.flags & NETF_TEMKIN, has_pw = net.flags & NETF_POWER;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long X = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); X < N; X += warps) {
    const int i = (int)(X % g.nx), j = (int)((X / g.nx) % g.ny), k = (int)(X / nxy);
    const double por = st.porosity[X], sat = st.saturation[X];
    const bool dry = sat < RT_MIN_SATURATION;
    // ---- connections: lane q < 6 takes x-, x+, y-, y+, z-, z+ (the order in
    // which the reference's x, y, z connection loops reach this cell) and
    // lane 6 finds the diagonal block
    int ex = 0, other = 0, up = 0, blk = -1;
    double cup = 0.0, cdn = 0.0;
    if (lane < 6) {
      const int axis = lane >> 1, plus = lane & 1;
      const int pos = axis == 0 ? i : (axis == 1 ? j : k);
      const int lim = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
      ex = plus ? (pos < lim - 1) : (pos > 0);
      if (ex) {
        const long long s = axis == 0 ? 1 : (axis == 1 ? (long long)g.nx : nxy);
        other = (int)(plus ? X + s : X - s);
        up = plus;  // the lower-index cell is upstream of the connection
        const int face = plus ? pos : pos - 1;
        double q, area, dist;
        if (axis == 0) {
          q = g.qx[((long long)k * g.ny + j) * (g.nx - 1) + face];
          area = g.dy * g.dz;
          dist = g.dx;
        } else if (axis == 1) {
          q = g.qy[((long long)k * (g.ny - 1) + face) * g.nx + i];
          area = g.dx * g.dz;
          dist = g.dy;
        } else {
          q = g.qz[((long long)face * g.ny + j) * g.nx + i];
          area = g.dx * g.dy;
          dist = g.dz;
        }
        const long long cu = up ? X : other, cd = up ? other : X;
        const double pu = st.porosity[cu], su = st.saturation[cu], pdn = st.porosity[cd], sdn = st.saturation[cd];
        if (!(sdn < RT_MIN_SATURATION) && !(su < RT_MIN_SATURATION)) {
          const double tr = tran_coef(pu, su, pdn, sdn, q, dist, g);
          if (q > 0.0) { cup = tr + q; cdn = -tr; }
          else { cup = tr; cdn = -tr + q; }
          cup = cup * area * 1000.0;
          cdn = cdn * area * 1000.0;
        }
        for (int b = rowptr[other]; b < rowptr[other + 1]; ++b)
          if (colidx[b] == (int)X) { blk = b; break; }
      }
    } else if (lane == 6) {
      for (int b = rowptr[X]; b < rowptr[X + 1]; ++b)
        if (colidx[b] == (int)X) { blk = b; break; }
    }
    // ---- species and secondary column terms t_p = nu_p s_i / m_species(p)
    for (int jj = lane; jj < n; jj += 32) {
      const double m = st.pri_molal[(size_t)jj * N + X];
      sm_m[jj] = m;
      sm_ic[jj] = 1.0 / m;
      sm_lna[jj] = log(m) + log(st.pri_act_coef[(size_t)jj * N + X]);
    }
    __syncwarp();
    for (int s = lane; s < ns; s += 32) {
      const double sv = st.sec_molal[(size_t)s * N + X];
      for (int p = T.sec_begin(s); p < T.sec_end(s); ++p) t[p] = T.sec_nu(p) * (sv * sm_ic[T.sec_idx(p)]);
    }
    // ---- RKineticMineral (reaction_mineral.F90:647-1078), lane m
    const double den_k = st.den_kg[X], den_L = den_k * 1.0e-3;
    const double temp = st.temperature ? st.temperature[X] : 25.0;
    const double volume = st.volume[X];
    for (int m = lane; m < nm; m += 32) {
      const int b = T.mnrl_begin(m), e = T.mnrl_end(m);
      double Gm = 0.0, Im_v = 0.0, QK = 0.0, rate_out = 0.0;
      bool active = false;
      if (!dry) {
        const double logK = tmin ? interp_logK(T.mnrl_logKcoef(m), temp) : T.mnrl_logK(m);
        double lnQK = -logK * LOG_TO_LN;
        for (int p = b; p < e; ++p) lnQK = lnQK + T.mnrl_nu(p) * sm_lna[T.mnrl_idx(p)];
        QK = exp(lnQK);
        double aff;
        if (has_tk) aff = 1.0 - pow(QK, 1.0 / (has_msf ? T.msf(m) * T.temkin(m) : T.temkin(m)));
        else if (has_msf) aff = 1.0 - pow(QK, 1.0 / T.msf(m));
        else aff = 1.0 - QK;
        const double sign_ = fsign1(aff);
        const double vf = st.mnrl_volfrac[(size_t)m * N + X];
        active = (vf > 0 || sign_ < 0.0) && !(T.irreversible(m) == 1 && sign_ < 0.0) &&
                 !(T.thresh(m) > 0.0 && sign_ < 0.0 && QK < T.thresh(m));
        if (active) {
          const double rl = T.limiter(m);
          if (rl > 0.0) aff = aff / (1.0 + (1.0 - aff) / rl);
          double arr = 1.0;
          if (T.ea(m) > 0.0)
            arr = exp(T.ea(m) / IDEAL_GAS_CONSTANT * (1.0 / (25.0 + 273.15) - 1.0 / (temp + 273.15)));
          const double kr = T.rate(m) * arr;
          double Im_const = -st.mnrl_area[(size_t)m * N + X];
          if (has_msf) Im_const = Im_const / T.msf(m);
          double Im = has_pw ? Im_const * sign_ * pow(fabs(aff), T.power(m)) * kr : Im_const * sign_ * fabs(aff) * kr;
          rate_out = Im;
          Im_const = Im_const * volume;
          Im = Im * volume;
          Im_v = Im;
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
        st.mnrl_rate[(size_t)m * N + X] = rate_out;
      }
      G[m] = Gm;
      Imv[m] = Im_v;
      // dQK/dm_j (the reference's den*1e-3 factor included, :944-947)
      for (int p = b; p < e; ++p)
        u[p] = active ? T.mnrl_nu(p) * QK * sm_ic[T.mnrl_idx(p)] * den_k * 1.0e-3 : 0.0;
    }
    // ---- broadcast the connections
    int c_ex[6], c_other[6], c_up[6], c_blk[6];
    double c_cup[6], c_cdn[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      c_ex[q] = __shfl_sync(0xffffffffu, ex, q);
      c_other[q] = __shfl_sync(0xffffffffu, other, q);
      c_up[q] = __shfl_sync(0xffffffffu, up, q);
      c_blk[q] = __shfl_sync(0xffffffffu, blk, q);
      c_cup[q] = __shfl_sync(0xffffffffu, cup, q);
      c_cdn[q] = __shfl_sync(0xffffffffu, cdn, q);
    }
    const int dblk = __shfl_sync(0xffffffffu, blk, 6);
    __syncwarp();
    const double psv = por * sat * 1000.0 * volume;
    const double psvd_t = psv / dt;
    // ---- residual row (lane = component)
    for (int row = lane; row < n; row += 32) {
      const double tx = st.total[(size_t)row * N + X];
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        if (!c_ex[q]) continue;
        const double ty = st.total[(size_t)row * N + c_other[q]];
        const double tu = c_up[q] ? tx : ty, td = c_up[q] ? ty : tx;
        const double res = c_cup[q] * tu + c_cdn[q] * td;
        v = c_up[q] ? v + res : v - res;
      }
      const double accum_k = dry ? 0.0 : psv * total_k[(size_t)row * N + X];
      v = v - accum_k / dt;
      v = v + (dry ? 0.0 : psv * tx) / dt;
      if (!dry) {
        double R = 0.0;
        for (int q = gt.r_mn_ptr[row]; q < gt.r_mn_ptr[row + 1]; ++q) R = R + gt.r_mn_nu[q] * Imv[gt.r_mn_m[q]];
        v = v + R;
      }
      r[X * n + row] = v;
    }
    // ---- block column X
    double csum = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q)
      if (c_ex[q]) csum = csum + (c_up[q] ? c_cup[q] : -c_cdn[q]);
    for (int fe = lane; fe < nn; fe += 32) {
      const int col = fe / n, row = fe - col * n;
      const int f = row * n + col;
      double d = (row == col) ? 1.0 : 0.0;
      for (int q = gt.e_sec_ptr[f]; q < gt.e_sec_ptr[f + 1]; ++q) d = fma(gt.e_sec_nr[q], t[gt.e_sec_p[q]], d);
      d = d * den_L;
      double jr = 0.0;
      for (int q = gt.e_mn_ptr[f]; q < gt.e_mn_ptr[f + 1]; ++q)
        jr = fma(gt.e_mn_nr[q] * G[gt.e_mn_m[q]], u[gt.e_mn_p[q]], jr);
      if (fabs(jr) < 1.0e-40) jr = 0.0;  // reaction.F90:4232-4237
      const double mc = logf ? sm_m[col] : 1.0;
      double v = d * csum;
      v = v + (dry ? ((row == col) ? 1.0 : 0.0) : d * psvd_t);
      if (!dry) v = v + jr;
      if (dblk >= 0) values[(size_t)dblk * nn + fe] = v * mc;
      const double E = d * mc;
#pragma unroll
      for (int q = 0; q < 6; ++q)
        if (c_ex[q] && c_blk[q] >= 0) values[(size_t)c_blk[q] * nn + fe] = (c_up[q] ? -c_cup[q] : c_cdn[q]) * E;
    }
    __syncwarp();
  }
}

}  // namespace girt

int girt_build_tables(const DevNet& net, const int32_t* I, const double* D, void** d_buf, GirtTabs* out) {
  const int n = net.n, nn = n * n;
  std::vector<std::vector<int32_t>> sp(nn), mp(nn), mm(nn), rm(n);
  std::vector<std::vector<double>> snr(nn), mnr(nn), rnu(n);
  for (int i = 0; i < net.ns; ++i) {
    const int b = I[net.o_sec_ptr + i], e = I[net.o_sec_ptr + i + 1];
    for (int pc = b; pc < e; ++pc)
      for (int pr = b; pr < e; ++pr) {
        const int f = I[net.o_sec_idx + pr] * n + I[net.o_sec_idx + pc];
        sp[f].push_back(pc);
        snr[f].push_back(D[net.o_sec_nu + pr]);
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
    for (int p = b; p < e; ++p) {
      rm[I[net.o_mnrl_idx + p]].push_back(m);
      rnu[I[net.o_mnrl_idx + p]].push_back(D[net.o_mnrl_nu + p]);
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
  int o_esp, o_esi, o_emp, o_emi, o_rmp, o_rmi;
  csr(sp, &o_esp, &o_esi);
  csr(mp, &o_emp, &o_emi);
  const int o_emm = flat(mm);
  csr(rm, &o_rmp, &o_rmi);
  const int d_esnr = flatd(snr), d_emnr = flatd(mnr), d_rmnu = flatd(rnu);
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
  out->r_mn_ptr = di + o_rmp;
  out->r_mn_m = di + o_rmi;
  out->r_mn_nu = dd + d_rmnu;
  *d_buf = buf;
  return PF_OK;
}

size_t girt_smem_bytes(const DevNet& net, int* warps_per_block) {
  const size_t wbytes = (size_t)girt::warp_doubles(net) * sizeof(double);
  int wpb = 8;
  while (wpb > 1 && wpb * wbytes > 96u * 1024u) wpb /= 2;
  if (warps_per_block) *warps_per_block = wpb;
  return wpb * wbytes;
}

int launch_girt_assemble(const DevNet& net, const GirtTabs& gt, const PfCellState& st, const PfGirtArgs& a,
                         int num_sms, cudaStream_t s) {
  if (st.ncells == 0) return PF_OK;
  if (launch_update_auxvars(net, st, 0, s) != 0) return PF_ERR_CUDA;  // RTUpdateAuxVars: total, sec_molal
  girt::Geo g{a.nx, a.ny, a.nz, a.dx, a.dy, a.dz, a.diffusion_coefficient, a.tortuosity, a.dispersivity,
              a.qx, a.qy, a.qz};
  int wpb = 1;
  const size_t smem = girt_smem_bytes(net, &wpb);
  if (smem > 227u * 1024u) return PF_ERR_TOO_LARGE;
  auto k = girt::girt_column_kernel;
  if (smem > 48u * 1024u &&
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return PF_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32 * wpb, smem) != cudaSuccess || per_sm < 1)
    return PF_ERR_CUDA;
  const long long need = (st.ncells + wpb - 1) / wpb;
  const long long cap = (long long)num_sms * per_sm;
  const long long grid = need < cap ? need : cap;
  k<<<(unsigned)grid, 32 * wpb, smem, s>>>(net, gt, st, g, a.total_k, a.dt, a.rowptr, a.colidx, a.residual,
                                           a.values);
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
