// pfgpu_multi.cu -- one persistent launch over the cells of several networks.
//
// The operator-split step of a heterogeneous problem -- regions whose
// chemistry has different reaction networks (ncomp 3 ... 24), each with its
// own cells -- runs here as a single persistent kernel instead of one launch
// per network.  Every block walks the networks in the order given (the
// costliest first); for each it stages that network's tables into shared
// memory (TMA bulk copy, bounded mbarrier wait) and runs the group-per-cell
// step (group_body) on that network's work queue until the queue is empty,
// then moves on.  A network's queue therefore drains while other blocks are
// still busy on it or already on the next one: the SMs idle only at the very
// end of the launch, not once per network.  The per-network work (tables,
// scratch, work queue, counters, cell order) is exactly what the
// single-network launch uses, so every cell's result is bit for bit the
// single-network group kernel's with the same group size.
#include "pfgpu_group.cuh"

namespace pfgpu {
namespace multi {

// the (lanes per cell, rows per lane) variants the multi-network kernel
// carries: 4 lanes for ncomp 5-16, 8 lanes for ncomp 1-24
__host__ __device__ constexpr int variant_of(int G, int R) {
  return G == 4 ? (R >= 2 && R <= 4 ? R - 2 : -1) : (G == 8 ? (R >= 1 && R <= 3 ? 2 + R : -1) : -1);
}

struct Net {
  DevNet net;  // ent_staged set for the launch's block size
  PfCellState st;
  const double* scratch;
  unsigned long long* queue;     // the network's work-queue counter (zeroed)
  unsigned long long* counters;  // its reductions (zeroed)
  int variant;
  int threads;  // threads of the block that work on this network (whole warps)
};

struct Args {
  int nnets;
  double dt;
  Net nets[PF_MULTI_MAX_NETS];
};

template <int G, int R>
__device__ __forceinline__ void run(const Net& m, double dt, unsigned char* smem) {
  // warps beyond the network's workspace wait at the next barrier
  if ((int)threadIdx.x < m.threads)
    group::group_body<G, R, false>(m.net, m.net.grp, m.st, dt, m.scratch, m.queue, m.counters, PfAdjointArgs{},
                                   nullptr, smem, m.threads);
}

__global__ void __launch_bounds__(256, 1) rstep_multi_kernel(const __grid_constant__ Args args) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t tma_bar;
  for (int k = 0; k < args.nnets; ++k) {
    const Net& m = args.nets[k];
    // every warp is done with the previous network's tables and workspace
    __syncthreads();
    if (!group::stage_tables(m.net, smem, &tma_bar, (uint32_t)(k & 1), k == 0, m.counters)) return;
    switch (m.variant) {
      case 0: run<4, 2>(m, args.dt, smem); break;
      case 1: run<4, 3>(m, args.dt, smem); break;
      case 2: run<4, 4>(m, args.dt, smem); break;
      case 3: run<8, 1>(m, args.dt, smem); break;
      case 4: run<8, 2>(m, args.dt, smem); break;
      case 5: run<8, 3>(m, args.dt, smem); break;
      default: break;
    }
  }
}

}  // namespace multi

int multi_lanes_for(const DevNet& net, int preferred) {
  auto ok = [&](int G) {
    return group_supported(net, G) && multi::variant_of(G, (net.n + G - 1) / G) >= 0;
  };
  if ((preferred == 4 || preferred == 8) && ok(preferred)) return preferred;
  if (ok(4)) return 4;
  if (ok(8)) return 8;
  return 0;
}

int launch_rstep_multi(const MultiNetLaunch* nets, int nnets, double dt, int threads_per_block, int blocks_per_sm,
                       int num_sms, cudaStream_t stream) {
  if (nnets < 1 || nnets > PF_MULTI_MAX_NETS) return -1;
  multi::Args args{};
  args.nnets = nnets;
  args.dt = dt;
  size_t smem = 0;
  for (int k = 0; k < nnets; ++k) {
    const MultiNetLaunch& in = nets[k];
    const int G = in.lanes_per_cell, R = (in.net.n + G - 1) / G;
    const int v = multi::variant_of(G, R);
    if (v < 0 || !group_supported(in.net, G)) return -1;
    // as many whole warps of the block as the network's per-cell workspace
    // lets fit in shared memory
    int threads = threads_per_block;
    PfLaunchConfig cfg{threads, blocks_per_sm, 0, G};
    while (threads > 32 && group_smem_bytes(in.net, cfg, false) > 227u * 1024u) {
      threads -= 32;
      cfg.threads_per_block = threads;
    }
    if (group_smem_bytes(in.net, cfg, false) > 227u * 1024u) return -1;
    multi::Net& m = args.nets[k];
    m.net = in.net;
    m.net.ent_staged = group_entries_staged(in.net, cfg, false) ? 1 : 0;
    m.st = in.st;
    m.scratch = in.scratch;
    m.queue = in.queue;
    m.counters = in.counters;
    m.variant = v;
    m.threads = threads;
    const size_t b = group_smem_bytes(in.net, cfg, false);
    smem = b > smem ? b : smem;
  }
  // the per-network set-up pre-pass (logK(T), K' and ln guess per cell)
  for (int k = 0; k < nnets; ++k) {
    const int rc = launch_cell_setup(nets[k].net, nets[k].st, const_cast<double*>(nets[k].scratch), stream);
    if (rc) return rc;
  }
  cudaError_t e = cudaFuncSetAttribute(multi::rstep_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return (int)e;
  multi::rstep_multi_kernel<<<num_sms * blocks_per_sm, threads_per_block, smem, stream>>>(args);
  return (int)cudaGetLastError();
}

}  // namespace pfgpu
