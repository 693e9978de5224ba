// pfgpu_transport.cu -- the transport half of the operator-split step.
//
// Replaces, for a structured grid with zero-flux outer boundaries and no
// sources, the transport solve of PMCSubsurfaceOSRTStepDT
// (src/pflotran/pmc_subsurface_osrt.F90:259-330): the fixed accumulation
// psv*T_k (psv = porosity*saturation*1000*volume), the scalar transport matrix
// of RTCalculateTransportMatrix (reactive_transport.F90:1469-1703: per
// internal connection TFluxCoef's T_up / T_dn, transport.F90:495-565, added at
// (up,up), (up,dn) and negated at (dn,dn), (dn,up); psv/dt on the diagonal),
// the right-hand side psv*T_k/dt (RTCalculateRHS_t1 without boundary or
// source terms), and one linear solve per component (the reference's
// KSPSolve loop over idof), all components sharing the matrix.
//
// GPU form: the matrix is never assembled.  A coefficient pass stores per
// cell the diagonal and the six face coefficients (the same harmonic-mean
// dispersion and upwinding as the global-implicit assembly); every component
// is then solved at once by Jacobi-preconditioned BiCGStab, the n systems
// advancing in lock step with their own scalars (kept on the device) and
// frozen one by one as they converge.  One iteration is two 7-point stencil
// products and a few vector updates over n x ncells doubles: HBM-bound.
// Dot products are two-stage (per-block partials, then a fixed-order sum), so
// results do not depend on scheduling.
#include <cmath>
#include <new>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

namespace pfgpu {
namespace tr {

constexpr int TPB = 256;
constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs worth of partial sums per dot product

struct Grid {
  int nx, ny, nz;
  long long N, nxy;
};

// coefficient layout [7][N]: 0 diag, 1 x-, 2 x+, 3 y-, 4 y+, 5 z-, 6 z+
// (off-diagonals are the coefficient of the neighbour's value in this row)
__global__ void coef_kernel(Grid g, double dx, double dy, double dz, const double* __restrict__ qx,
                            const double* __restrict__ qy, const double* __restrict__ qz, double diffusion,
                            double tortuosity, double dispersivity, const double* __restrict__ por,
                            const double* __restrict__ sat, const double* __restrict__ vol, double dt,
                            double* __restrict__ A, double* __restrict__ inv_diag) {
  const long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= g.N) return;
  const int i = (int)(X % g.nx), j = (int)((X / g.nx) % g.ny), k = (int)(X / g.nxy);
  const double psv = por[X] * sat[X] * 1000.0 * vol[X];
  double diag = 0.0, off[6] = {0, 0, 0, 0, 0, 0};
  // connections in the reference's order (x, y, z); this cell is the
  // upstream (lower-index) end of the + connection, downstream of the -
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int axis = q >> 1, plus = q & 1;
    const int pos = axis == 0 ? i : (axis == 1 ? j : k);
    const int lim = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    if (plus ? !(pos < lim - 1) : !(pos > 0)) continue;
    const long long s = axis == 0 ? 1 : (axis == 1 ? (long long)g.nx : g.nxy);
    const long long other = plus ? X + s : X - s;
    const int face = plus ? pos : pos - 1;
    double qf, area, dist;
    if (axis == 0) {
      qf = qx[((long long)k * g.ny + j) * (g.nx - 1) + face];
      area = dy * dz;
      dist = dx;
    } else if (axis == 1) {
      qf = qy[((long long)k * (g.ny - 1) + face) * g.nx + i];
      area = dx * dz;
      dist = dy;
    } else {
      qf = qz[((long long)face * g.ny + j) * g.nx + i];
      area = dx * dy;
      dist = dz;
    }
    const long long cu = plus ? X : other, cd = plus ? other : X;
    const double su = sat[cu], sd = sat[cd];
    if (sd < RT_MIN_SATURATION || su < RT_MIN_SATURATION) continue;  // TFluxCoef: no flux
    // harmonic_tran_coefs_over_dist (transport.F90:199-225), dist_up = dist_dn = dist/2
    const double dist_up = dist * 0.5, dist_dn = dist - dist_up;
    const double mech = dispersivity * fabs(qf);
    const double hu = fmax(mech + 1.0 * su * por[cu] * tortuosity * diffusion, 1.0e-40);
    const double hd = fmax(mech + 1.0 * sd * por[cd] * tortuosity * diffusion, 1.0e-40);
    const double tr = (hu * hd) / (hu * dist_dn + hd * dist_up);
    double cup, cdn;
    if (qf > 0.0) { cup = tr + qf; cdn = -tr; }
    else { cup = tr; cdn = -tr + qf; }
    cup = cup * area * 1000.0;
    cdn = cdn * area * 1000.0;
    if (plus) {  // this row is 'up': +T_up on the diagonal, +T_dn at the neighbour
      diag = diag + cup;
      off[q] = cdn;
    } else {     // this row is 'dn': -T_dn on the diagonal, -T_up at the neighbour
      diag = diag + (-cdn);
      off[q] = -cup;
    }
  }
  diag = diag + psv / dt;
  // a cell with neither storage nor connections (dry: saturation below
  // rt_min_saturation) has an empty row; it becomes an identity row whose
  // right-hand side is its own total, so the cell keeps its totals
  if (diag == 0.0) diag = 1.0;
  A[X] = diag;
#pragma unroll
  for (int q = 0; q < 6; ++q) A[(size_t)(q + 1) * g.N + X] = off[q];
  inv_diag[X] = 1.0 / diag;
}

// (A invD x) at cell X: the 7-point product of the right-preconditioned operator
__device__ __forceinline__ double stencil(const Grid& g, const double* __restrict__ A, const double* __restrict__ invD,
                                          const double* __restrict__ x, long long X) {
  const int i = (int)(X % g.nx), j = (int)((X / g.nx) % g.ny), k = (int)(X / g.nxy);
  double v = A[X] * (invD[X] * x[X]);
  if (i > 0) v = fma(A[g.N + X], invD[X - 1] * x[X - 1], v);
  if (i < g.nx - 1) v = fma(A[2 * g.N + X], invD[X + 1] * x[X + 1], v);
  if (j > 0) v = fma(A[3 * g.N + X], invD[X - g.nx] * x[X - g.nx], v);
  if (j < g.ny - 1) v = fma(A[4 * g.N + X], invD[X + g.nx] * x[X + g.nx], v);
  if (k > 0) v = fma(A[5 * g.N + X], invD[X - g.nxy] * x[X - g.nxy], v);
  if (k < g.nz - 1) v = fma(A[6 * g.N + X], invD[X + g.nxy] * x[X + g.nxy], v);
  return v;
}

template <int NW>
__device__ __forceinline__ void block_partials(double (&v)[NW], double* __restrict__ partials, int c, int ncomp) {
  // block-wide sums of NW values, written to partials[(w*ncomp + c)*gridDim + block]
  __shared__ double sh[NW][TPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    double s = v[w];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) sh[w][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      double s = 0.0;
      for (int k = 0; k < TPB / 32; ++k) s += sh[w][k];
      partials[((size_t)w * ncomp + c) * gridDim.x + blockIdx.x] = s;
    }
  }
  __syncthreads();
}

// the per-component scalars live in one device array S[field][c]
enum Scalar { RHO = 0, ALPHA, OMEGA, BETA, BNORM2, RNORM2, ACTIVE, NSCALAR };

__global__ void spmv_dot_kernel(Grid g, const double* __restrict__ A, const double* __restrict__ invD,
                                const double* __restrict__ x, const double* __restrict__ w, double* __restrict__ y,
                                const double* __restrict__ S, int ncomp, double* __restrict__ partials) {
  const int c = blockIdx.y;
  const bool active = S[ACTIVE * ncomp + c] != 0.0;
  const double* xc = x + (size_t)c * g.N;
  const double* wc = w + (size_t)c * g.N;
  double* yc = y + (size_t)c * g.N;
  double acc[1] = {0.0};
  if (active) {
    for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < g.N; X += (long long)gridDim.x * blockDim.x) {
      const double v = stencil(g, A, invD, xc, X);
      yc[X] = v;
      acc[0] = fma(wc[X], v, acc[0]);
    }
  }
  block_partials<1>(acc, partials, c, ncomp);
}

// t = A invD s, partial dots (t.s, t.t)
__global__ void spmv_dot2_kernel(Grid g, const double* __restrict__ A, const double* __restrict__ invD,
                                 const double* __restrict__ s, double* __restrict__ t, const double* __restrict__ S,
                                 int ncomp, double* __restrict__ partials) {
  const int c = blockIdx.y;
  const bool active = S[ACTIVE * ncomp + c] != 0.0;
  const double* sc = s + (size_t)c * g.N;
  double* tc = t + (size_t)c * g.N;
  double acc[2] = {0.0, 0.0};
  if (active) {
    for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < g.N; X += (long long)gridDim.x * blockDim.x) {
      const double v = stencil(g, A, invD, sc, X);
      tc[X] = v;
      acc[0] = fma(v, sc[X], acc[0]);
      acc[1] = fma(v, v, acc[1]);
    }
  }
  block_partials<2>(acc, partials, c, ncomp);
}

// s = r - alpha v (active components)
__global__ void axpy_s_kernel(long long N, const double* __restrict__ r, const double* __restrict__ v,
                              double* __restrict__ s, const double* __restrict__ S, int ncomp) {
  const int c = blockIdx.y;
  if (S[ACTIVE * ncomp + c] == 0.0) return;
  const double alpha = S[ALPHA * ncomp + c];
  const size_t o = (size_t)c * N;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x)
    s[o + X] = fma(-alpha, v[o + X], r[o + X]);
}

// x += invD (alpha p + omega s); r = s - omega t; partial dots (r0.r, r.r)
__global__ void update_xr_kernel(long long N, const double* __restrict__ invD, double* __restrict__ x,
                                 double* __restrict__ r, const double* __restrict__ p, const double* __restrict__ s,
                                 const double* __restrict__ t, const double* __restrict__ r0,
                                 const double* __restrict__ S, int ncomp, double* __restrict__ partials) {
  const int c = blockIdx.y;
  const bool active = S[ACTIVE * ncomp + c] != 0.0;
  double acc[2] = {0.0, 0.0};
  if (active) {
    const double alpha = S[ALPHA * ncomp + c], omega = S[OMEGA * ncomp + c];
    const size_t o = (size_t)c * N;
    for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x) {
      const double sv = s[o + X];
      x[o + X] = fma(invD[X], fma(alpha, p[o + X], omega * sv), x[o + X]);
      const double rv = fma(-omega, t[o + X], sv);
      r[o + X] = rv;
      acc[0] = fma(r0[o + X], rv, acc[0]);
      acc[1] = fma(rv, rv, acc[1]);
    }
  }
  block_partials<2>(acc, partials, c, ncomp);
}

// p = r + beta (p - omega v)
__global__ void update_p_kernel(long long N, double* __restrict__ p, const double* __restrict__ r,
                                const double* __restrict__ v, const double* __restrict__ S, int ncomp) {
  const int c = blockIdx.y;
  if (S[ACTIVE * ncomp + c] == 0.0) return;
  const double beta = S[BETA * ncomp + c], omega = S[OMEGA * ncomp + c];
  const size_t o = (size_t)c * N;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x)
    p[o + X] = fma(beta, fma(-omega, v[o + X], p[o + X]), r[o + X]);
}

// initial state: x0 = 0, b = psv T / dt, r = r0 = p = b (right Jacobi
// preconditioning: BiCGStab on A invD for y = D x, with x itself updated by
// invD times the y increments); partial sums of b.b
__global__ void init_kernel(long long N, const double* __restrict__ A, const double* __restrict__ total,
                            const double* __restrict__ por,
                            const double* __restrict__ sat, const double* __restrict__ vol, double dt,
                            double* __restrict__ x, double* __restrict__ r, double* __restrict__ r0,
                            double* __restrict__ p, int ncomp, double* __restrict__ partials) {
  const int c = blockIdx.y;
  const size_t o = (size_t)c * N;
  double acc[1] = {0.0};
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x) {
    const double psv = por[X] * sat[X] * 1000.0 * vol[X];
    // identity rows (see coef_kernel) carry the cell's own total
    const bool ident = psv == 0.0 && A[X] == 1.0 && A[N + X] == 0.0 && A[2 * N + X] == 0.0 &&
                       A[3 * N + X] == 0.0 && A[4 * N + X] == 0.0 && A[5 * N + X] == 0.0 && A[6 * N + X] == 0.0;
    const double b = ident ? total[o + X] : psv * total[o + X] / dt;
    x[o + X] = 0.0;
    r[o + X] = b;
    r0[o + X] = b;
    p[o + X] = b;
    acc[0] = fma(b, b, acc[0]);
  }
  block_partials<1>(acc, partials, c, ncomp);
}

// fixed-order sums of the partials, then the BiCGStab scalar recurrences;
// one thread per component.  stage: 0 init, 1 alpha, 2 omega, 3 rho/beta
__global__ void scalar_kernel(int stage, int nparts, const double* __restrict__ partials, double* __restrict__ S,
                              int ncomp, double rtol2) {
  const int c = threadIdx.x;
  if (c >= ncomp) return;
  auto sum = [&](int w) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += partials[((size_t)w * ncomp + c) * nparts + b];
    return s;
  };
  if (stage == 0) {
    const double bb = sum(0);
    S[RHO * ncomp + c] = bb;
    S[BNORM2 * ncomp + c] = bb;
    S[RNORM2 * ncomp + c] = bb;
    S[ALPHA * ncomp + c] = 0.0;
    S[OMEGA * ncomp + c] = 0.0;
    S[BETA * ncomp + c] = 0.0;
    S[ACTIVE * ncomp + c] = bb > 0.0 ? 1.0 : 0.0;  // b = 0: x = 0 is the solution
    return;
  }
  if (S[ACTIVE * ncomp + c] == 0.0) return;
  if (stage == 1) {
    const double r0v = sum(0);
    if (r0v == 0.0) { S[ACTIVE * ncomp + c] = 0.0; S[ALPHA * ncomp + c] = 0.0; return; }  // breakdown
    S[ALPHA * ncomp + c] = S[RHO * ncomp + c] / r0v;
  } else if (stage == 2) {
    const double ts = sum(0), tt = sum(1);
    S[OMEGA * ncomp + c] = tt > 0.0 ? ts / tt : 0.0;
  } else {
    const double rho_new = sum(0), rr = sum(1);
    const double rho = S[RHO * ncomp + c], omega = S[OMEGA * ncomp + c];
    S[RNORM2 * ncomp + c] = rr;
    S[BETA * ncomp + c] = (rho != 0.0 && omega != 0.0) ? (rho_new / rho) * (S[ALPHA * ncomp + c] / omega) : 0.0;
    S[RHO * ncomp + c] = rho_new;
    if (rr <= rtol2 * S[BNORM2 * ncomp + c] || omega == 0.0 || rho_new == 0.0) S[ACTIVE * ncomp + c] = 0.0;
  }
}

// the solution back into the totals
__global__ void finish_kernel(long long N, const double* __restrict__ x, double* __restrict__ total) {
  const int c = blockIdx.y;
  const size_t o = (size_t)c * N;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x)
    total[o + X] = x[o + X];
}

}  // namespace tr
}  // namespace pfgpu

using namespace pfgpu;

struct PfTransport {
  int nx = 0, ny = 0, nz = 0, ncomp = 0;
  long long N = 0;
  double* buf = nullptr;     // A[7N] invD[N] x r r0 p v s t [n N each] partials S
  double* h_scalars = nullptr;  // pinned copy of S for the convergence check
  size_t bytes = 0;
};

extern "C" int32_t pf_transport_create(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp, PfTransport** out) {
  if (!out || nx < 1 || ny < 1 || nz < 1 || ncomp < 1 || ncomp > PF_MAX_NCOMP) return PF_ERR_INVALID;
  *out = nullptr;
  PfTransport* t = new (std::nothrow) PfTransport();
  if (!t) return PF_ERR_INVALID;
  t->nx = nx; t->ny = ny; t->nz = nz; t->ncomp = ncomp;
  t->N = (long long)nx * ny * nz;
  const size_t vec = (size_t)ncomp * (size_t)t->N;
  const size_t doubles = 8 * (size_t)t->N + 7 * vec + 2 * (size_t)tr::RED_BLOCKS * ncomp + tr::NSCALAR * ncomp;
  t->bytes = doubles * sizeof(double);
  if (cudaMalloc(&t->buf, t->bytes) != cudaSuccess ||
      cudaMallocHost(&t->h_scalars, tr::NSCALAR * ncomp * sizeof(double)) != cudaSuccess) {
    if (t->buf) cudaFree(t->buf);
    delete t;
    return PF_ERR_CUDA;
  }
  *out = t;
  return PF_OK;
}

extern "C" int32_t pf_transport_destroy(PfTransport* t) {
  if (!t) return PF_ERR_INVALID;
  if (t->buf) cudaFree(t->buf);
  if (t->h_scalars) cudaFreeHost(t->h_scalars);
  delete t;
  return PF_OK;
}

extern "C" int32_t pf_transport_step(PfTransport* t, const PfTransportArgs* a, void* stream, PfTransportStats* stats) {
  using namespace tr;
  if (!t || !a) return PF_ERR_INVALID;
  if (a->nx != t->nx || a->ny != t->ny || a->nz != t->nz || a->ncomp != t->ncomp) return PF_ERR_INVALID;
  if (!(a->dt > 0.0) || !(a->dx > 0.0) || !(a->dy > 0.0) || !(a->dz > 0.0) || !a->total || !a->porosity ||
      !a->saturation || !a->volume || a->max_iterations < 1 || !(a->rtol > 0.0))
    return PF_ERR_INVALID;
  if ((t->nx > 1 && !a->qx) || (t->ny > 1 && !a->qy) || (t->nz > 1 && !a->qz)) return PF_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const long long N = t->N;
  const int n = t->ncomp;
  const size_t vec = (size_t)n * (size_t)N;
  double* A = t->buf;
  double* invD = A + 7 * N;
  double* x = invD + N;
  double* r = x + vec;
  double* r0 = r + vec;
  double* p = r0 + vec;
  double* v = p + vec;
  double* sv = v + vec;
  double* tv = sv + vec;
  double* partials = tv + vec;
  double* S = partials + 2 * (size_t)RED_BLOCKS * n;
  Grid g{t->nx, t->ny, t->nz, N, (long long)t->nx * t->ny};
  const unsigned cblocks = (unsigned)((N + TPB - 1) / TPB);
  coef_kernel<<<cblocks, TPB, 0, s>>>(g, a->dx, a->dy, a->dz, a->qx, a->qy, a->qz, a->diffusion_coefficient,
                                      a->tortuosity, a->dispersivity, a->porosity, a->saturation, a->volume, a->dt,
                                      A, invD);
  const long long want = (N + TPB - 1) / TPB;
  const dim3 grid((unsigned)(want < RED_BLOCKS ? want : RED_BLOCKS), (unsigned)n);
  const int nparts = (int)grid.x;
  const double rtol2 = a->rtol * a->rtol;
  init_kernel<<<grid, TPB, 0, s>>>(N, A, a->total, a->porosity, a->saturation, a->volume, a->dt, x, r, r0, p, n,
                                   partials);
  scalar_kernel<<<1, 32, 0, s>>>(0, nparts, partials, S, n, rtol2);
  if (cudaGetLastError() != cudaSuccess) return PF_ERR_CUDA;
  int it = 0;
  bool done = false;
  const int check_every = 4;
  while (it < a->max_iterations && !done) {
    spmv_dot_kernel<<<grid, TPB, 0, s>>>(g, A, invD, p, r0, v, S, n, partials);       // v = A invD p, r0.v
    scalar_kernel<<<1, 32, 0, s>>>(1, nparts, partials, S, n, rtol2);                  // alpha
    axpy_s_kernel<<<grid, TPB, 0, s>>>(N, r, v, sv, S, n);                              // s = r - alpha v
    spmv_dot2_kernel<<<grid, TPB, 0, s>>>(g, A, invD, sv, tv, S, n, partials);         // t = A invD s
    scalar_kernel<<<1, 32, 0, s>>>(2, nparts, partials, S, n, rtol2);                  // omega
    update_xr_kernel<<<grid, TPB, 0, s>>>(N, invD, x, r, p, sv, tv, r0, S, n, partials);
    scalar_kernel<<<1, 32, 0, s>>>(3, nparts, partials, S, n, rtol2);                  // rho, beta, test
    update_p_kernel<<<grid, TPB, 0, s>>>(N, p, r, v, S, n);
    ++it;
    if (it % check_every == 0 || it == a->max_iterations) {
      if (cudaMemcpyAsync(t->h_scalars, S, NSCALAR * n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return PF_ERR_CUDA;
      done = true;
      for (int c = 0; c < n; ++c) done = done && t->h_scalars[ACTIVE * n + c] == 0.0;
    }
  }
  finish_kernel<<<grid, TPB, 0, s>>>(N, x, a->total);
  if (cudaGetLastError() != cudaSuccess) return PF_ERR_CUDA;
  if (cudaMemcpyAsync(t->h_scalars, S, NSCALAR * n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PF_ERR_CUDA;
  double worst = 0.0;
  bool conv = true;
  for (int c = 0; c < n; ++c) {
    const double bb = t->h_scalars[BNORM2 * n + c], rr = t->h_scalars[RNORM2 * n + c];
    const double rel = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    worst = rel > worst ? rel : worst;
    conv = conv && !(rel > a->rtol);
  }
  if (stats) {
    stats->iterations = it;
    stats->max_rel_residual = worst;
    stats->converged = conv ? 1 : 0;
  }
  return conv ? PF_OK : PF_CELL_FAILURES;
}
