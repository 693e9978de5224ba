// pfgpu_transport.cu -- the transport half of the operator-split step.
//
// Replaces, for a structured grid, the transport solve of
// PMCSubsurfaceOSRTStepDT (src/pflotran/pmc_subsurface_osrt.F90:259-330):
// the fixed accumulation psv*T_k (psv = porosity*saturation*1000*volume), the
// scalar transport matrix of RTCalculateTransportMatrix
// (reactive_transport.F90:1469-1703: per internal connection TFluxCoef's
// T_up / T_dn, transport.F90:495-565, added at (up,up), (up,dn) and negated at
// (dn,dn), (dn,up); per boundary connection -T_dn on the cell's diagonal;
// psv/dt on the diagonal; extraction sources' coefficient on the diagonal),
// the right-hand side psv*T_k/dt plus the inflowing boundary and injection
// terms of RTCalculateRHS_t1 (:1239-1465), and one linear solve per
// component (the reference's KSPSolve loop over idof), all components
// sharing the matrix.  Boundary faces carry a condition type, the face Darcy
// fluxes and the boundary totals; TDispersionBC (transport.F90:236-374) gives
// the boundary dispersion over half the cell width with the boundary's
// saturation.  The right-hand side's boundary and source part is one FP64
// vector [ncomp][N] written by the coefficient pass and the (sequential,
// deterministic) source pass; without boundaries or sources it is not used.
//
// GPU form.  The matrix is never assembled: a coefficient pass stores per
// cell the diagonal and the six face coefficients (the same harmonic-mean
// dispersion and upwinding as the global-implicit assembly).  On GB300 the
// FP64 pipe, not HBM, bounds a Krylov solve (a 7-point product is ~9 FP64
// operations per 24 bytes; GB300 delivers one FP64 operation per ~13 bytes of
// HBM bandwidth), so the solve is mixed-precision iterative refinement
// (Wilkinson's, with a Krylov inner solver as in GMRES-IR):
//   r = b - A x                      FP64, all components
//   solve (A D^-1) y = r to ~1e-5    FP32 Jacobi-right-preconditioned
//                                    BiCGStab, all components in lock step
//   x += D^-1 y                      FP64
// until ||b - A x|| <= rtol ||b|| in FP64 for every component; x starts at
// T_k.  The FP32 inner iterations run at the FP32 rate on half the bytes;
// the answer is the FP64 one.  Dot products are two-stage (per-block
// partials, then a fixed-order sum in FP64), so results do not depend on
// scheduling.
#include <cmath>
#include <cstring>
#include <new>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

namespace pfgpu {
namespace tr {

constexpr int TPB = 256;
constexpr int RED_BLOCKS = 304;  // at most this many blocks (partial sums) per component (chunk)
constexpr int SPMV_CELLS = 1;    // cells per thread and pass in the stencil products
constexpr int VEC_PAD = 64;      // floats added to each vector's stride (not a power of two)
constexpr int CH = 4;            // components per stencil pass
constexpr double INNER_RTOL = 3.0e-6;  // inner reduction per cycle (floor)
constexpr double INNER_SAFETY = 0.3;    // last cycle: solve to 0.3 rtol ||b|| / ||r||
constexpr int INNER_MAX = 60;    // inner iterations per refinement cycle
constexpr int OUTER_MAX = 30;

struct Grid {
  int nx, ny, nz;
  long long N, nxy;
  long long Np;  // stride of the solver's own vectors: N rounded up to 64, plus padding
};

// per-component scalars, one device array S[field][c]
enum Scalar { RHO = 0, ALPHA, OMEGA, BETA, BNORM2, RNORM2, ACTIVE, ORES2, RHS2, RSCALE, ITOL2,
              ITS, REFS, CYC, MAXCYC,  // counters: inner iterations, cycles, per cycle
              NSCALAR };

__device__ __forceinline__ void cell_ijk(const Grid& g, long long X, int& i, int& j, int& k) {
  const unsigned ux = (unsigned)X, unx = (unsigned)g.nx, uny = (unsigned)g.ny;
  const unsigned row = ux / unx;
  i = (int)(ux - row * unx);
  j = (int)(row % uny);
  k = (int)(row / uny);
}

// A[8][N] FP64: 0 diag, 1 x-, 2 x+, 3 y-, 4 y+, 5 z-, 6 z+ (the coefficient of
// the neighbour's value in this row; 0 where there is none), 7 the right-hand
// side's scale (b = A[7] T_k)
// boundary conditions as the coefficient pass reads them
struct BcDev {
  int type[6];
  const double* q[6];
  const double* total[6];
  double sat[6];
  int ncomp;
  double* bb;  // [ncomp][N] right-hand side additions, nullptr: no boundary or source terms
};

__global__ void coef_kernel(Grid g, double dx, double dy, double dz, const double* __restrict__ qx,
                            const double* __restrict__ qy, const double* __restrict__ qz, double diffusion,
                            double tortuosity, double dispersivity, const double* __restrict__ por,
                            const double* __restrict__ sat, const double* __restrict__ vol, double dt,
                            double* __restrict__ A, double* __restrict__ inv_diag, BcDev bc) {
  const long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= g.N) return;
  int i, j, k;
  cell_ijk(g, X, i, j, k);
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
    const long long st = axis == 0 ? 1 : (axis == 1 ? (long long)g.nx : g.nxy);
    const long long other = plus ? X + st : X - st;
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
  // boundary connections (RTCalculateTransportMatrix :1596-1627 and
  // RTCalculateRHS_t1 :1337-1370): the boundary is the upstream end, q > 0
  // flows into the domain
  if (bc.bb) {
    for (int c = 0; c < bc.ncomp; ++c) bc.bb[(size_t)c * g.N + X] = 0.0;
#pragma unroll 1
    for (int f = 0; f < 6; ++f) {
      if (bc.type[f] == PF_BC_ZERO_FLUX) continue;
      const int axis = f >> 1, plus = f & 1;
      const int pos = axis == 0 ? i : (axis == 1 ? j : k);
      const int lim = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
      if (plus ? pos != lim - 1 : pos != 0) continue;
      const long long na = axis == 0 ? g.ny : g.nx;
      const long long nf = na * (axis == 2 ? g.ny : g.nz);
      const long long fi = axis == 0 ? (j + na * k) : (axis == 1 ? (i + na * k) : (i + na * j));
      const double area = axis == 0 ? dy * dz : (axis == 1 ? dx * dz : dx * dy);
      const double dist0 = 0.5 * (axis == 0 ? dx : (axis == 1 ? dy : dz));
      const double qb = bc.q[f] ? bc.q[f][fi] : 0.0;
      const double sdn = sat[X];
      // TDispersionBC: Dirichlet (and Dirichlet-zero-gradient where the flux
      // enters) disperses against the boundary water over dist0
      double tr = 0.0;
      if (!(bc.sat[f] < RT_MIN_SATURATION) && !(sdn < RT_MIN_SATURATION) &&
          (bc.type[f] == PF_BC_DIRICHLET || (bc.type[f] == PF_BC_DIRICHLET_ZERO_GRADIENT && !(qb < 0.0)))) {
        const double hd = fmax(dispersivity * fabs(qb) + 1.0 * bc.sat[f] * por[X] * tortuosity * diffusion, 1.0e-40);
        tr = hd / dist0;
      }
      // TFluxCoefBC -> TFluxCoef without the upwind saturation check
      double tup = 0.0, tdn = 0.0;
      if (!(sdn < RT_MIN_SATURATION)) {
        if (qb > 0.0) { tup = tr + qb; tdn = -tr; }
        else { tup = tr; tdn = -tr + qb; }
        tup = tup * area * 1000.0;
        tdn = tdn * area * 1000.0;
      }
      diag = diag + (-tdn);
      if (tup != 0.0)
        for (int c = 0; c < bc.ncomp; ++c)
          bc.bb[(size_t)c * g.N + X] = fma(tup, bc.total[f][(size_t)c * nf + fi], bc.bb[(size_t)c * g.N + X]);
    }
  }
  const double storage = psv / dt;
  diag = diag + storage;
  // a cell with neither storage nor connections (dry: saturation below
  // rt_min_saturation) has an empty row; it becomes an identity row whose
  // right-hand side is its own total, so the cell keeps its totals
  double bscale = storage;  // b = bscale * T_k
  if (diag == 0.0) {
    diag = 1.0;
    bscale = 1.0;
  }
  A[X] = diag;
#pragma unroll
  for (int q = 0; q < 6; ++q) A[(size_t)(q + 1) * g.N + X] = off[q];
  A[(size_t)7 * g.N + X] = bscale;
  inv_diag[X] = 1.0 / diag;
}

// Sources and sinks, in array order (one block; thread c owns component c
// of the right-hand side, thread 0 also the diagonal): the source loops of
// RTCalculateTransportMatrix (:1651-1690, extraction: T_in on the diagonal
// when positive) and RTCalculateRHS_t1 (:1372-1418, injection: -T_out times
// the source totals) with TSrcSinkCoef (transport.F90:613-673).  An entry
// whose cell lies outside the grid is skipped and counted in *bad.
__global__ void source_kernel(long long N, int ncomp, int nsrc, const int32_t* __restrict__ cell,
                              const int32_t* __restrict__ type, const double* __restrict__ qs,
                              const double* __restrict__ total, const double* __restrict__ sat,
                              double* __restrict__ A, double* __restrict__ inv_diag, double* __restrict__ bb,
                              unsigned* __restrict__ bad) {
  const int c = threadIdx.x;
  for (int e = 0; e < nsrc; ++e) {
    const long long X = cell[e];
    if (X < 0 || X >= N) {
      if (c == 0) atomicAdd(bad, 1u);
      continue;
    }
    const double q = qs[e];
    double tin = 0.0, tout = 0.0;
    if (!(sat[X] < RT_MIN_SATURATION)) {
      if (type[e] == PF_SRC_EQUILIBRIUM) {
        tin = 1.0e-3;
        tout = -1.0 * tin;
      } else if (type[e] == PF_SRC_MASS_RATE) {
        tin = 0.0;
        tout = -1.0;
      } else if (q > 0.0) {
        tout = -1.0 * q * 1000.0;
      } else {
        tin = -1.0 * q * 1000.0;
      }
    }
    if (c == 0 && !(q > 0.0) && tin > 0.0) {
      A[X] = A[X] + tin;
      inv_diag[X] = 1.0 / A[X];
    }
    if (c < ncomp && !(q < 0.0)) bb[(size_t)c * N + X] = bb[(size_t)c * N + X] - tout * total[(size_t)c * nsrc + e];
  }
}

// Ah[6][N] FP32: the off-diagonals of A D^-1 (column q scaled by the
// neighbour's 1/diag); its diagonal is 1
__global__ void scale_kernel(Grid g, const double* __restrict__ A, const double* __restrict__ invD,
                             float* __restrict__ Ah) {
  const long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= g.N) return;
  int i, j, k;
  cell_ijk(g, X, i, j, k);
  const long long step[6] = {-1, 1, -(long long)g.nx, (long long)g.nx, -g.nxy, g.nxy};
  const bool has[6] = {i > 0, i < g.nx - 1, j > 0, j < g.ny - 1, k > 0, k < g.nz - 1};
#pragma unroll
  for (int q = 0; q < 6; ++q)
    Ah[(size_t)q * g.N + X] = has[q] ? (float)(A[(size_t)(q + 1) * g.N + X] * invD[X + step[q]]) : 0.0f;
}

template <int NW, class T>
__device__ __forceinline__ void block_partials(T (&v)[NW], double* __restrict__ partials, int c, int ncomp) {
  // block-wide sums of NW values (accumulated and summed over the warp in
  // T, the warps' sums added in FP64), written to
  // partials[(w*ncomp + c)*gridDim + block].  FP32 shuffles for the inner
  // solve's dot products: FP64 arithmetic runs at 1/64 of the FP32 rate
  __shared__ double sh[NW][TPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    T s = v[w];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) sh[w][wid] = (double)s;
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

template <int NW, class T>
__device__ __forceinline__ void block_partials_chunk(T (&v)[NW][CH], double* __restrict__ partials, int c0,
                                                     int ncomp) {
#pragma unroll
  for (int cc = 0; cc < CH; ++cc) {
    T t[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) t[w] = v[w][cc];
    if (c0 + cc < ncomp) block_partials<NW, T>(t, partials, c0 + cc, ncomp);
  }
}

// Fixed-order sums of one component's partials (one warp: lane l sums
// partials l, l+32, ..., then a fixed shuffle tree) and its scalar updates.
// stage 0: outer residual (ORES2, and BNORM2 on the first call, first=1)
// stage 1: inner start (RHO, RHS2, RNORM2; ACTIVE unless the component is
//          converged in the outer sense; ITOL2: the inner target, no
//          tighter than what brings the outer residual to rtol)
// stage 2: alpha; stage 3: omega; stage 4: rho, beta and the inner test
__device__ __noinline__ void scalar_component(int stage, int first, int nparts, const double* __restrict__ partials,
                                 double* __restrict__ S, int ncomp, double rtol2, double inner_rtol2, int c,
                                 int lane) {
  auto sum = [&](int w) {
    double s = 0.0;
    const double* p = partials + ((size_t)w * ncomp + c) * nparts;
    for (int b = lane; b < nparts; b += 32) s += __ldcg(p + b);  // other blocks' writes: read from L2
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    return __shfl_sync(0xffffffffu, s, 0);
  };
  const bool two = stage == 0 || stage == 3 || stage == 4;
  const double s0 = sum(0);
  const double s1 = two ? sum(1) : 0.0;
  if (lane != 0) return;
  double* Sc = S + c;
  if (stage == 0) {
    Sc[ORES2 * ncomp] = s0;
    Sc[RSCALE * ncomp] = sqrt(s0);
    if (first) {
      Sc[BNORM2 * ncomp] = s1;
      Sc[ITS * ncomp] = 0.0;
      Sc[REFS * ncomp] = 0.0;
      Sc[MAXCYC * ncomp] = 0.0;
    }
    return;
  }
  if (stage == 1) {
    const bool done = Sc[ORES2 * ncomp] <= rtol2 * Sc[BNORM2 * ncomp];
    Sc[RHO * ncomp] = s0;
    Sc[RNORM2 * ncomp] = s0;
    Sc[RHS2 * ncomp] = done ? 0.0 : s0;
    Sc[ALPHA * ncomp] = 0.0;
    Sc[OMEGA * ncomp] = 0.0;
    Sc[BETA * ncomp] = 0.0;
    Sc[ACTIVE * ncomp] = (!done && s0 > 0.0) ? 1.0 : 0.0;
    const double need = INNER_SAFETY * INNER_SAFETY * rtol2 * Sc[BNORM2 * ncomp] / Sc[ORES2 * ncomp];
    Sc[ITOL2 * ncomp] = done ? 0.0 : fmax(inner_rtol2, need);
    Sc[CYC * ncomp] = 0.0;
    if (!done) Sc[REFS * ncomp] += 1.0;
    return;
  }
  if (Sc[ACTIVE * ncomp] == 0.0) return;
  if (stage == 2) {
    Sc[ITS * ncomp] += 1.0;  // an inner iteration of this component starts
    Sc[CYC * ncomp] += 1.0;
    Sc[MAXCYC * ncomp] = fmax(Sc[MAXCYC * ncomp], Sc[CYC * ncomp]);
    if (s0 == 0.0) { Sc[ACTIVE * ncomp] = 0.0; Sc[ALPHA * ncomp] = 0.0; return; }  // breakdown
    Sc[ALPHA * ncomp] = Sc[RHO * ncomp] / s0;
  } else if (stage == 3) {
    Sc[OMEGA * ncomp] = s1 > 0.0 ? s0 / s1 : 0.0;
  } else {
    const double rho_new = s0, rr = s1;
    const double rho = Sc[RHO * ncomp], omega = Sc[OMEGA * ncomp];
    Sc[RNORM2 * ncomp] = rr;
    Sc[BETA * ncomp] = (rho != 0.0 && omega != 0.0) ? (rho_new / rho) * (Sc[ALPHA * ncomp] / omega) : 0.0;
    Sc[RHO * ncomp] = rho_new;
    if (rr <= Sc[ITOL2 * ncomp] * Sc[RHS2 * ncomp] || omega == 0.0 || rho_new == 0.0) Sc[ACTIVE * ncomp] = 0.0;
  }
}


struct Stage {
  int stage, first;
  double rtol2, inner_rtol2;
  unsigned* counter;  // blocks of the current launch that have written their partials
};

// Called by every block after its partials are written: the last block of
// the launch to arrive sums every component's partials (in block order, so
// the result does not depend on which block is last) and makes the scalar
// update, then re-arms the counter.  Replaces a separate scalar launch.
__device__ __forceinline__ void finish_stage(const Stage& st, const double* __restrict__ partials,
                                             double* __restrict__ S, int ncomp) {
  __shared__ unsigned ticket;
  if (threadIdx.x == 0) {
    __threadfence();  // this block's partials before its ticket
    ticket = atomicAdd(st.counter, 1u);
  }
  __syncthreads();
  if (ticket != gridDim.x * gridDim.y - 1u) return;
  __threadfence();  // every block's partials are visible
  const int nwarps = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = wid; c < ncomp; c += nwarps)
    scalar_component(st.stage, st.first, gridDim.x, partials, S, ncomp, st.rtol2, st.inner_rtol2, c, lane);
  if (threadIdx.x == 0) *st.counter = 0u;
}

// The seven cells a row reads: itself and its x-, x+, y-, y+, z-, z+
// neighbours.  Where a neighbour does not exist the row's coefficient is 0
// (coef_kernel, scale_kernel), so the index only has to stay inside the
// array: it is clamped to [0, N-1] and the product adds 0 * (a finite
// value).  No integer division; N < 2^31, so X + nx*ny fits in 32 bits.
__device__ __forceinline__ void nbr_index(const Grid& g, unsigned X, unsigned (&idx)[7]) {
  const unsigned last = (unsigned)g.N - 1u, nx = (unsigned)g.nx, nxy = (unsigned)g.nxy;
  idx[0] = X;
  idx[1] = X > 0u ? X - 1u : 0u;
  idx[2] = min(X + 1u, last);
  idx[3] = X >= nx ? X - nx : 0u;
  idx[4] = min(X + nx, last);
  idx[5] = X >= nxy ? X - nxy : 0u;
  idx[6] = min(X + nxy, last);
}

// number of components in chunk blockIdx.y (CH, or the remainder)
__device__ __forceinline__ int chunk_size(int ncomp) { return min(CH, ncomp - (int)blockIdx.y * CH); }

__device__ __forceinline__ bool chunk_active(const double* __restrict__ S, int ncomp, int c0, int nc) {
  bool any = false;
  for (int cc = 0; cc < nc; ++cc) any = any || S[ACTIVE * ncomp + c0 + cc] != 0.0;
  return any;
}

// ---------------------------------------------------------------- FP64 outer
// r = b - A x with b = B T_k (B = psv/dt, or 1 on identity rows); partials
// ||r||^2 (w = 0) and, on the first call, ||b||^2 (w = 1)
template <int NC>
__device__ __forceinline__ void residual_body(const Grid& g, const double* __restrict__ A,
                                              const double* __restrict__ total_k, const double* __restrict__ bb,
                                              const double* __restrict__ x, double* __restrict__ r64, bool first,
                                              double (&acc)[2][CH]) {
  const size_t o0 = (size_t)blockIdx.y * CH * (size_t)g.Np;  // x, r64
  const size_t t0 = (size_t)blockIdx.y * CH * (size_t)g.N;   // the caller's totals
  for (unsigned X = blockIdx.x * blockDim.x + threadIdx.x; X < (unsigned)g.N; X += gridDim.x * blockDim.x) {
    unsigned idx[7];
    nbr_index(g, X, idx);
    double w[7], xv[NC][7], tk[NC], ba[NC];
    // all loads before the first store (see spmv_body)
#pragma unroll
    for (int q = 0; q < 7; ++q) w[q] = A[(size_t)q * g.N + X];
    const double bs = A[(size_t)7 * g.N + X];
#pragma unroll
    for (int cc = 0; cc < NC; ++cc) {
      const double* xc = x + o0 + (size_t)cc * g.Np;
#pragma unroll
      for (int q = 0; q < 7; ++q) xv[cc][q] = xc[idx[q]];
      tk[cc] = total_k[t0 + (size_t)cc * g.N + X];
      ba[cc] = bb ? bb[t0 + (size_t)cc * g.N + X] : 0.0;  // boundary and source terms
    }
#pragma unroll
    for (int cc = 0; cc < NC; ++cc) {
      const double b = fma(bs, tk[cc], ba[cc]);
      double ax = w[0] * xv[cc][0];
#pragma unroll
      for (int q = 1; q < 7; ++q) ax = fma(w[q], xv[cc][q], ax);
      const double rv = b - ax;
      r64[o0 + (size_t)cc * g.Np + X] = rv;
      acc[0][cc] = fma(rv, rv, acc[0][cc]);
      if (first) acc[1][cc] = fma(b, b, acc[1][cc]);
    }
  }
}

__global__ void __launch_bounds__(TPB) residual_kernel(Grid g, const double* __restrict__ A,
                                                       const double* __restrict__ total_k,
                                                       const double* __restrict__ bb,
                                                       const double* __restrict__ x, double* __restrict__ r64,
                                                       int ncomp, double* __restrict__ partials,
                                                       double* __restrict__ S, Stage st) {
  const int c0 = blockIdx.y * CH, nc = chunk_size(ncomp);
  const bool first = st.first != 0;
  double acc[2][CH] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  switch (nc) {
    case 4: residual_body<4>(g, A, total_k, bb, x, r64, first, acc); break;
    case 3: residual_body<3>(g, A, total_k, bb, x, r64, first, acc); break;
    case 2: residual_body<2>(g, A, total_k, bb, x, r64, first, acc); break;
    default: residual_body<1>(g, A, total_k, bb, x, r64, first, acc); break;
  }
  block_partials_chunk<2, double>(acc, partials, c0, ncomp);
  finish_stage(st, partials, S, ncomp);
}

// x += ||r|| D^-1 y (the inner correction, which solved for r / ||r||) for
// the components that ran
__global__ void update64_kernel(long long N, long long Np, const double* __restrict__ invD,
                                const float* __restrict__ y, double* __restrict__ x, const double* __restrict__ S,
                                int ncomp) {
  const int c = blockIdx.y;
  if (S[RHS2 * ncomp + c] == 0.0) return;  // no inner solve for this component
  const double scale = S[RSCALE * ncomp + c];
  const size_t o = (size_t)c * Np;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x)
    x[o + X] = fma(invD[X] * scale, (double)y[o + X], x[o + X]);
}

// dst[c][X] = src[c][X] for X < N, component c = blockIdx.y, given strides
__global__ void copy_kernel(long long N, long long src_stride, long long dst_stride, const double* __restrict__ src,
                            double* __restrict__ dst) {
  const double* sc = src + (size_t)blockIdx.y * src_stride;
  double* dc = dst + (size_t)blockIdx.y * dst_stride;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < N; X += (long long)gridDim.x * blockDim.x)
    dc[X] = sc[X];
}

// ---------------------------------------------------------------- FP32 inner
// r = r64 / ||r64|| in FP32 (unit norm whatever the totals' magnitude);
// y = 0; r0 = p = r; partial r.r
__global__ void __launch_bounds__(TPB) inner_init_kernel(long long Np, const double* __restrict__ r64, double* __restrict__ S,
                                  float* __restrict__ r, float* __restrict__ r0, float* __restrict__ p,
                                  float* __restrict__ y, int ncomp, double* __restrict__ partials, Stage st) {
  // over the padded length: the padding of r64 is 0, so is that of r, r0, p, y
  const int c = blockIdx.y;
  const size_t o = (size_t)c * Np;
  const double rs = S[RSCALE * ncomp + c];
  const double inv = rs > 0.0 ? 1.0 / rs : 0.0;
  float acc[1] = {0.0f};
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < Np; X += (long long)gridDim.x * blockDim.x) {
    const float rv = (float)(r64[o + X] * inv);
    r[o + X] = rv;
    r0[o + X] = rv;
    p[o + X] = rv;
    y[o + X] = 0.0f;
    acc[0] = fmaf(rv, rv, acc[0]);
  }
  block_partials<1, float>(acc, partials, c, ncomp);
  finish_stage(st, partials, S, ncomp);
}

// y = (A D^-1) x for the chunk's NC components; TWO = false: partial w.y;
// TWO = true: partials (y.x, y.y)
template <int NC, bool TWO>
__device__ __forceinline__ void spmv_body(const Grid& g, const float* __restrict__ Ah, const float* __restrict__ x,
                                          const float* __restrict__ w, float* __restrict__ y,
                                          float (&acc)[2][CH]) {
  // SPMV_CELLS cells per thread and pass (X, X + stride, ...).  Every load
  // of a pass (coefficients, the NC components' seven values, w) is issued
  // before the first store: a store between two loads orders them, and the
  // pass would wait for memory once per component instead of once
  constexpr int U = SPMV_CELLS;
  const size_t o0 = (size_t)blockIdx.y * CH * (size_t)g.Np;
  const unsigned N = (unsigned)g.N, stride = gridDim.x * blockDim.x;
  for (unsigned X0 = blockIdx.x * blockDim.x + threadIdx.x; X0 < N; X0 += U * stride) {
    unsigned idx[U][7];
    float a[U][6], xv[U][NC][7], wv[U][NC];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const unsigned X = X0 + u * stride;
      ok[u] = X < N;
      const unsigned Xc = ok[u] ? X : N - 1u;  // a cell past the end repeats the last (not stored)
      nbr_index(g, Xc, idx[u]);
#pragma unroll
      for (int q = 0; q < 6; ++q) a[u][q] = Ah[(size_t)q * g.N + Xc];
#pragma unroll
      for (int cc = 0; cc < NC; ++cc) {
        const float* xc = x + o0 + (size_t)cc * g.Np;
#pragma unroll
        for (int q = 0; q < 7; ++q) xv[u][cc][q] = xc[idx[u][q]];
        if (!TWO) wv[u][cc] = w[o0 + (size_t)cc * g.Np + Xc];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int cc = 0; cc < NC; ++cc) {
        float v = xv[u][cc][0];
#pragma unroll
        for (int q = 0; q < 6; ++q) v = fmaf(a[u][q], xv[u][cc][q + 1], v);
        if (!ok[u]) continue;
        y[o0 + (size_t)cc * g.Np + idx[u][0]] = v;
        if (TWO) {
          acc[0][cc] = fmaf(v, xv[u][cc][0], acc[0][cc]);
          acc[1][cc] = fmaf(v, v, acc[1][cc]);
        } else {
          acc[0][cc] = fmaf(wv[u][cc], v, acc[0][cc]);
        }
      }
    }
  }
}

template <bool TWO>
__device__ __forceinline__ void spmv_chunk(const Grid& g, const float* __restrict__ Ah, const float* __restrict__ x,
                                           const float* __restrict__ w, float* __restrict__ y,
                                           double* __restrict__ S, int ncomp, double* __restrict__ partials,
                                           const Stage& st) {
  const int c0 = blockIdx.y * CH, nc = chunk_size(ncomp);
  float acc[2][CH] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  // a chunk with no active component skips the product; an active chunk
  // computes all its components (vectors of converged components are not
  // read again, their partials are ignored)
  if (chunk_active(S, ncomp, c0, nc)) {
    switch (nc) {
      case 4: spmv_body<4, TWO>(g, Ah, x, w, y, acc); break;
      case 3: spmv_body<3, TWO>(g, Ah, x, w, y, acc); break;
      case 2: spmv_body<2, TWO>(g, Ah, x, w, y, acc); break;
      default: spmv_body<1, TWO>(g, Ah, x, w, y, acc); break;
    }
  }
  if (TWO) block_partials_chunk<2, float>(acc, partials, c0, ncomp);
  else {
    float a1[1][CH] = {{acc[0][0], acc[0][1], acc[0][2], acc[0][3]}};
    block_partials_chunk<1, float>(a1, partials, c0, ncomp);
  }
  finish_stage(st, partials, S, ncomp);
}

// v = (A D^-1) p, partial r0.v
__global__ void __launch_bounds__(TPB) spmv_dot_kernel(Grid g, const float* __restrict__ Ah,
                                                       const float* __restrict__ x, const float* __restrict__ w,
                                                       float* __restrict__ y, double* __restrict__ S,
                                                       int ncomp, double* __restrict__ partials, Stage st) {
  spmv_chunk<false>(g, Ah, x, w, y, S, ncomp, partials, st);
}

// t = (A D^-1) s, partials (t.s, t.t)
__global__ void __launch_bounds__(TPB) spmv_dot2_kernel(Grid g, const float* __restrict__ Ah,
                                                        const float* __restrict__ s, float* __restrict__ t,
                                                        double* __restrict__ S, int ncomp,
                                                        double* __restrict__ partials, Stage st) {
  spmv_chunk<true>(g, Ah, s, nullptr, t, S, ncomp, partials, st);
}

// The vector updates run over float4 of the padded vectors (Np is a
// multiple of 4 and every vector starts on a 256-byte boundary); the padding
// is 0 in every vector and stays 0 under these updates.

// s = r - alpha v
__global__ void __launch_bounds__(TPB) axpy_s_kernel(long long Np4, const float4* __restrict__ r, const float4* __restrict__ v,
                              float4* __restrict__ s, const double* __restrict__ S, int ncomp) {
  const int c = blockIdx.y;
  if (S[ACTIVE * ncomp + c] == 0.0) return;
  const float alpha = (float)S[ALPHA * ncomp + c];
  const size_t o = (size_t)c * Np4;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < Np4; X += (long long)gridDim.x * blockDim.x) {
    const float4 rv = r[o + X], vv = v[o + X];
    s[o + X] = make_float4(fmaf(-alpha, vv.x, rv.x), fmaf(-alpha, vv.y, rv.y), fmaf(-alpha, vv.z, rv.z),
                           fmaf(-alpha, vv.w, rv.w));
  }
}

// y += alpha p + omega s; r = s - omega t; partials (r0.r, r.r)
__global__ void __launch_bounds__(TPB) update_yr_kernel(long long Np4, float4* __restrict__ y, float4* __restrict__ r,
                                 const float4* __restrict__ p, const float4* __restrict__ s,
                                 const float4* __restrict__ t, const float4* __restrict__ r0,
                                 double* __restrict__ S, int ncomp, double* __restrict__ partials, Stage st) {
  const int c = blockIdx.y;
  const bool active = S[ACTIVE * ncomp + c] != 0.0;
  float acc[2] = {0.0f, 0.0f};
  if (active) {
    const float alpha = (float)S[ALPHA * ncomp + c], omega = (float)S[OMEGA * ncomp + c];
    const size_t o = (size_t)c * Np4;
    for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < Np4; X += (long long)gridDim.x * blockDim.x) {
      const float4 sv = s[o + X], pv = p[o + X], yv = y[o + X], tv = t[o + X], zv = r0[o + X];
      float4 yn, rn;
      yn.x = fmaf(alpha, pv.x, fmaf(omega, sv.x, yv.x));
      yn.y = fmaf(alpha, pv.y, fmaf(omega, sv.y, yv.y));
      yn.z = fmaf(alpha, pv.z, fmaf(omega, sv.z, yv.z));
      yn.w = fmaf(alpha, pv.w, fmaf(omega, sv.w, yv.w));
      rn.x = fmaf(-omega, tv.x, sv.x);
      rn.y = fmaf(-omega, tv.y, sv.y);
      rn.z = fmaf(-omega, tv.z, sv.z);
      rn.w = fmaf(-omega, tv.w, sv.w);
      y[o + X] = yn;
      r[o + X] = rn;
      acc[0] = fmaf(zv.x, rn.x, fmaf(zv.y, rn.y, fmaf(zv.z, rn.z, fmaf(zv.w, rn.w, acc[0]))));
      acc[1] = fmaf(rn.x, rn.x, fmaf(rn.y, rn.y, fmaf(rn.z, rn.z, fmaf(rn.w, rn.w, acc[1]))));
    }
  }
  block_partials<2, float>(acc, partials, c, ncomp);
  finish_stage(st, partials, S, ncomp);
}

// p = r + beta (p - omega v)
__global__ void __launch_bounds__(TPB) update_p_kernel(long long Np4, float4* __restrict__ p, const float4* __restrict__ r,
                                const float4* __restrict__ v, const double* __restrict__ S, int ncomp) {
  const int c = blockIdx.y;
  if (S[ACTIVE * ncomp + c] == 0.0) return;
  const float beta = (float)S[BETA * ncomp + c], omega = (float)S[OMEGA * ncomp + c];
  const size_t o = (size_t)c * Np4;
  for (long long X = (long long)blockIdx.x * blockDim.x + threadIdx.x; X < Np4; X += (long long)gridDim.x * blockDim.x) {
    const float4 pv = p[o + X], rv = r[o + X], vv = v[o + X];
    p[o + X] = make_float4(fmaf(beta, fmaf(-omega, vv.x, pv.x), rv.x), fmaf(beta, fmaf(-omega, vv.y, pv.y), rv.y),
                           fmaf(beta, fmaf(-omega, vv.z, pv.z), rv.z), fmaf(beta, fmaf(-omega, vv.w, pv.w), rv.w));
  }
}

}  // namespace tr
}  // namespace pfgpu

using namespace pfgpu;

struct PfTransport {
  int nx = 0, ny = 0, nz = 0, ncomp = 0;
  long long N = 0, Np = 0;
  void* buf = nullptr;          // see transport_layout
  double* h_scalars = nullptr;  // pinned copy of S for the convergence checks
  size_t bytes = 0;
  // blocks per component (vector kernels) or per component chunk (stencil
  // kernels): one full wave of the kernel's resident blocks
  int gx_res = 1, gx_sp1 = 1, gx_sp2 = 1, gx_vec = 1;
};

namespace {
struct Layout {
  double *A, *invD, *x, *r64, *partials, *S, *bb;
  float *Ah, *r, *r0, *p, *v, *s, *t, *y;
  unsigned *counter, *bad_src;
};

// Work space, every array on a 256-byte boundary: FP64 A[8][N], invD[N],
// x and r64 [ncomp][Np], partials, S, the right-hand side's boundary and
// source terms bb [ncomp][N]; the stage counter and the count of source
// entries outside the grid; FP32 Ah[6][N] and the inner solver's r, r0, p, v,
// s, t, y [ncomp][Np].  With base == nullptr only the size.
size_t transport_layout(char* base, long long N, long long Np, int n, Layout* L) {
  size_t cur = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + cur : nullptr;
    cur += (bytes + 255) & ~(size_t)255;
    return p;
  };
  const size_t vec = (size_t)n * (size_t)Np;
  Layout l;
  l.A = (double*)take(8 * (size_t)N * 8);
  l.invD = (double*)take((size_t)N * 8);
  l.x = (double*)take(vec * 8);
  l.r64 = (double*)take(vec * 8);
  l.partials = (double*)take(2 * (size_t)tr::RED_BLOCKS * n * 8);
  l.S = (double*)take((size_t)tr::NSCALAR * n * 8);
  l.bb = (double*)take((size_t)n * (size_t)N * 8);
  l.counter = (unsigned*)take(4);
  l.bad_src = (unsigned*)take(4);
  l.Ah = (float*)take(6 * (size_t)N * 4);
  l.r = (float*)take(vec * 4);
  l.r0 = (float*)take(vec * 4);
  l.p = (float*)take(vec * 4);
  l.v = (float*)take(vec * 4);
  l.s = (float*)take(vec * 4);
  l.t = (float*)take(vec * 4);
  l.y = (float*)take(vec * 4);
  if (L) *L = l;
  return cur;
}

int wave_blocks(const void* kernel, int parts) {
  int dev = 0, sms = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, tr::TPB, 0) != cudaSuccess || occ < 1)
    return -1;
  const int b = sms * occ / (parts > 0 ? parts : 1);
  return b < 1 ? 1 : (b > tr::RED_BLOCKS ? tr::RED_BLOCKS : b);
}
}  // namespace

extern "C" int32_t pf_transport_create(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp, PfTransport** out) {
  if (!out || nx < 1 || ny < 1 || nz < 1 || ncomp < 1 || ncomp > PF_MAX_NCOMP) return PF_ERR_INVALID;
  *out = nullptr;
  // 32-bit cell indices, with the padded stride
  if ((long long)nx * ny * nz > 0x7fffffffll - 4096) return PF_ERR_TOO_LARGE;
  PfTransport* t = new (std::nothrow) PfTransport();
  if (!t) return PF_ERR_INVALID;
  t->nx = nx; t->ny = ny; t->nz = nz; t->ncomp = ncomp;
  t->N = (long long)nx * ny * nz;
  t->Np = ((t->N + 63) / 64) * 64 + tr::VEC_PAD;
  t->bytes = transport_layout(nullptr, t->N, t->Np, ncomp, nullptr);
  const int chunks = (ncomp + tr::CH - 1) / tr::CH;
  t->gx_res = wave_blocks((const void*)tr::residual_kernel, chunks);
  t->gx_sp1 = wave_blocks((const void*)tr::spmv_dot_kernel, chunks);
  t->gx_sp2 = wave_blocks((const void*)tr::spmv_dot2_kernel, chunks);
  t->gx_vec = wave_blocks((const void*)tr::update_yr_kernel, ncomp);
  if (t->gx_res < 0 || t->gx_sp1 < 0 || t->gx_sp2 < 0 || t->gx_vec < 0 ||
      cudaMalloc(&t->buf, t->bytes) != cudaSuccess ||
      cudaMemset(t->buf, 0, t->bytes) != cudaSuccess ||  // the vectors' padding stays 0
      cudaMallocHost(&t->h_scalars, (tr::NSCALAR * ncomp + 1) * sizeof(double)) != cudaSuccess) {
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

namespace {
// Device counters and residuals of the last solve -> stats (synchronises s).
int32_t read_stats(PfTransport* t, cudaStream_t s, double rtol, PfTransportStats* stats, bool* conv_out) {
  using namespace tr;
  const int n = t->ncomp;
  Layout L;
  transport_layout(static_cast<char*>(t->buf), t->N, t->Np, n, &L);
  if (cudaMemcpyAsync(t->h_scalars, L.S, NSCALAR * n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(t->h_scalars + NSCALAR * n, L.bad_src, sizeof(unsigned), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PF_ERR_CUDA;
  unsigned bad = 0;
  memcpy(&bad, t->h_scalars + NSCALAR * n, sizeof(unsigned));
  if (bad) return PF_ERR_INVALID;  // a source entry named a cell outside the grid
  const double* h = t->h_scalars;
  double worst = 0.0, its = 0.0, refs = 0.0, cyc = 0.0;
  bool conv = true;
  for (int c = 0; c < n; ++c) {
    const double bb = h[BNORM2 * n + c], rr = h[ORES2 * n + c];
    const double rel = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    worst = rel > worst ? rel : worst;
    conv = conv && !(rel > rtol);
    its = fmax(its, h[ITS * n + c]);
    refs = fmax(refs, h[REFS * n + c]);
    cyc = fmax(cyc, h[MAXCYC * n + c]);
  }
  if (stats) {
    stats->iterations = (int32_t)its;
    stats->max_rel_residual = worst;
    stats->converged = conv ? 1 : 0;
    stats->refinements = (int32_t)refs;
    stats->max_cycle_iterations = (int32_t)cyc;
  }
  if (conv_out) *conv_out = conv;
  return PF_OK;
}

int32_t check_args(const PfTransport* t, const PfTransportArgs* a) {
  if (!t || !a) return PF_ERR_INVALID;
  if (a->nx != t->nx || a->ny != t->ny || a->nz != t->nz || a->ncomp != t->ncomp) return PF_ERR_INVALID;
  if (!(a->dt > 0.0) || !(a->dx > 0.0) || !(a->dy > 0.0) || !(a->dz > 0.0) || !a->total || !a->porosity ||
      !a->saturation || !a->volume || a->max_iterations < 1 || !(a->rtol > 0.0))
    return PF_ERR_INVALID;
  if ((t->nx > 1 && !a->qx) || (t->ny > 1 && !a->qy) || (t->nz > 1 && !a->qz)) return PF_ERR_INVALID;
  for (int f = 0; f < 6; ++f) {
    if (a->bc_type[f] < PF_BC_ZERO_FLUX || a->bc_type[f] > PF_BC_ZERO_GRADIENT) return PF_ERR_INVALID;
    if (a->bc_type[f] != PF_BC_ZERO_FLUX && (!a->bc_total[f] || !(a->bc_saturation[f] >= 0.0))) return PF_ERR_INVALID;
  }
  if (a->nsrc < 0 || (a->nsrc > 0 && (!a->src_cell || !a->src_type || !a->src_q || !a->src_total)))
    return PF_ERR_INVALID;
  return PF_OK;
}

// The solve.  fixed_inner == 0: adaptive, the host checks convergence every
// two inner iterations and after every refinement.  fixed_inner > 0: exactly
// fixed_cycles refinement cycles of fixed_inner inner iterations each, no
// host synchronisation (capturable in a CUDA graph); components that have
// converged make the remaining launches no-ops.
int32_t transport_run(PfTransport* t, const PfTransportArgs* a, cudaStream_t s, int fixed_inner, int fixed_cycles) {
  using namespace tr;
  const long long N = t->N, Np = t->Np, Np4 = Np / 4;
  const int n = t->ncomp;
  Layout L;
  transport_layout(static_cast<char*>(t->buf), N, Np, n, &L);
  Grid g{t->nx, t->ny, t->nz, N, (long long)t->nx * t->ny, Np};
  const unsigned cblocks = (unsigned)((N + TPB - 1) / TPB);
  BcDev bc{};
  bool open = a->nsrc > 0;
  for (int f = 0; f < 6; ++f) {
    bc.type[f] = a->bc_type[f];
    bc.q[f] = a->bc_q[f];
    bc.total[f] = a->bc_total[f];
    bc.sat[f] = a->bc_saturation[f];
    open = open || a->bc_type[f] != PF_BC_ZERO_FLUX;
  }
  bc.ncomp = n;
  bc.bb = open ? L.bb : nullptr;
  if (cudaMemsetAsync(L.bad_src, 0, sizeof(unsigned), s) != cudaSuccess) return PF_ERR_CUDA;
  coef_kernel<<<cblocks, TPB, 0, s>>>(g, a->dx, a->dy, a->dz, a->qx, a->qy, a->qz, a->diffusion_coefficient,
                                      a->tortuosity, a->dispersivity, a->porosity, a->saturation, a->volume, a->dt,
                                      L.A, L.invD, bc);
  if (a->nsrc > 0)
    source_kernel<<<1, 32, 0, s>>>(N, n, a->nsrc, a->src_cell, a->src_type, a->src_q, a->src_total, a->saturation,
                                   L.A, L.invD, L.bb, L.bad_src);
  scale_kernel<<<cblocks, TPB, 0, s>>>(g, L.A, L.invD, L.Ah);
  // blocks: one wave, but no more than the cells need
  auto cap = [&](int gx) { return (unsigned)((long long)gx < (long long)cblocks ? gx : (int)cblocks); };
  const unsigned chunks = (unsigned)((n + CH - 1) / CH);
  const dim3 g_res(cap(t->gx_res), chunks), g_sp1(cap(t->gx_sp1), chunks), g_sp2(cap(t->gx_sp2), chunks);
  const dim3 g_vec(cap(t->gx_vec), (unsigned)n);
  const double rtol2 = a->rtol * a->rtol, irtol2 = INNER_RTOL * INNER_RTOL;
  auto stage = [&](int k, int first) { return Stage{k, first, rtol2, irtol2, L.counter}; };
  if (cudaMemsetAsync(L.counter, 0, sizeof(unsigned), s) != cudaSuccess) return PF_ERR_CUDA;
  copy_kernel<<<g_vec, TPB, 0, s>>>(N, N, Np, a->total, L.x);  // x0 = T_k
  auto outer_residual = [&](int first) {
    residual_kernel<<<g_res, TPB, 0, s>>>(g, L.A, a->total, bc.bb, L.x, L.r64, n, L.partials, L.S,
                                          stage(0, first));
  };
  auto fetch = [&]() {
    return cudaMemcpyAsync(t->h_scalars, L.S, NSCALAR * n * sizeof(double), cudaMemcpyDeviceToHost, s) ==
               cudaSuccess &&
           cudaStreamSynchronize(s) == cudaSuccess;
  };
  auto all_done = [&]() {
    for (int c = 0; c < n; ++c)
      if (t->h_scalars[ORES2 * n + c] > rtol2 * t->h_scalars[BNORM2 * n + c]) return false;
    return true;
  };
  float4 *r4 = (float4*)L.r, *p4 = (float4*)L.p, *v4 = (float4*)L.v, *s4 = (float4*)L.s, *t4 = (float4*)L.t,
         *y4 = (float4*)L.y, *z4 = (float4*)L.r0;
  auto inner_iteration = [&]() {
    spmv_dot_kernel<<<g_sp1, TPB, 0, s>>>(g, L.Ah, L.p, L.r0, L.v, L.S, n, L.partials, stage(2, 0));
    axpy_s_kernel<<<g_vec, TPB, 0, s>>>(Np4, r4, v4, s4, L.S, n);
    spmv_dot2_kernel<<<g_sp2, TPB, 0, s>>>(g, L.Ah, L.s, L.t, L.S, n, L.partials, stage(3, 0));
    update_yr_kernel<<<g_vec, TPB, 0, s>>>(Np4, y4, r4, p4, s4, t4, z4, L.S, n, L.partials, stage(4, 0));
    update_p_kernel<<<g_vec, TPB, 0, s>>>(Np4, p4, r4, v4, L.S, n);
  };
  auto cycle_start = [&]() {  // FP32 correction: (A D^-1) y = r / ||r||
    inner_init_kernel<<<g_vec, TPB, 0, s>>>(Np, L.r64, L.S, L.r, L.r0, L.p, L.y, n, L.partials, stage(1, 0));
  };
  auto cycle_end = [&]() {  // FP64: x += ||r|| D^-1 y, new residual
    update64_kernel<<<g_vec, TPB, 0, s>>>(N, Np, L.invD, L.y, L.x, L.S, n);
    outer_residual(0);
  };
  outer_residual(1);
  if (fixed_inner > 0) {
    for (int cyc = 0; cyc < fixed_cycles; ++cyc) {
      cycle_start();
      for (int it = 0; it < fixed_inner; ++it) inner_iteration();
      cycle_end();
    }
    copy_kernel<<<g_vec, TPB, 0, s>>>(N, Np, N, L.x, a->total);
    return cudaGetLastError() == cudaSuccess ? PF_OK : PF_ERR_CUDA;
  }
  if (cudaGetLastError() != cudaSuccess || !fetch()) return PF_ERR_CUDA;
  int inner_total = 0, outer = 0;
  while (!all_done() && inner_total < a->max_iterations && outer < OUTER_MAX) {
    cycle_start();
    int it = 0;
    bool inner_done = false;
    while (!inner_done && it < INNER_MAX && inner_total < a->max_iterations) {
      inner_iteration();
      ++it;
      ++inner_total;
      if (it % 2 == 0) {
        if (!fetch()) return PF_ERR_CUDA;
        inner_done = true;
        for (int c = 0; c < n; ++c) inner_done = inner_done && t->h_scalars[ACTIVE * n + c] == 0.0;
      }
    }
    cycle_end();
    if (cudaGetLastError() != cudaSuccess || !fetch()) return PF_ERR_CUDA;
    ++outer;
  }
  copy_kernel<<<g_vec, TPB, 0, s>>>(N, Np, N, L.x, a->total);
  return cudaGetLastError() == cudaSuccess ? PF_OK : PF_ERR_CUDA;
}
}  // namespace

extern "C" int32_t pf_transport_step(PfTransport* t, const PfTransportArgs* a, void* stream, PfTransportStats* stats) {
  const int32_t chk = check_args(t, a);
  if (chk != PF_OK) return chk;
  cudaStream_t s = (cudaStream_t)stream;
  const int32_t rc = transport_run(t, a, s, 0, 0);
  if (rc != PF_OK) return rc;
  bool conv = false;
  const int32_t rs = read_stats(t, s, a->rtol, stats, &conv);
  if (rs != PF_OK) return rs;
  return conv ? PF_OK : PF_CELL_FAILURES;
}

extern "C" int32_t pf_transport_enqueue(PfTransport* t, const PfTransportArgs* a, int32_t inner_iterations,
                                        int32_t refinements, void* stream) {
  const int32_t chk = check_args(t, a);
  if (chk != PF_OK) return chk;
  if (inner_iterations < 1 || inner_iterations > 10000 || refinements < 1 || refinements > 100) return PF_ERR_INVALID;
  return transport_run(t, a, (cudaStream_t)stream, inner_iterations, refinements);
}

extern "C" int32_t pf_transport_read_stats(PfTransport* t, double rtol, void* stream, PfTransportStats* stats) {
  if (!t || !(rtol > 0.0)) return PF_ERR_INVALID;
  bool conv = false;
  const int32_t rs = read_stats(t, (cudaStream_t)stream, rtol, stats, &conv);
  if (rs != PF_OK) return rs;
  return conv ? PF_OK : PF_CELL_FAILURES;
}
