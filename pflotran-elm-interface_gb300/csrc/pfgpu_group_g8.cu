// pfgpu_group_g8.cu -- the group-per-cell step kernel with 8 lanes per cell.
#include "pfgpu_group.cuh"

namespace pfgpu {
int launch_group_g8(const DevNet& net, const GroupTabs& gt, const PfCellState& st, double dt, int R, size_t smem,
                    int grid, int tpb, const double* scratch, unsigned long long* queue, unsigned long long* counters,
                    const PfAdjointArgs* adj, double* adj_store, cudaStream_t stream) {
  switch (R) {
    case 1:
      return group::launch_k<8, 1>(net, gt, st, dt, smem, grid, tpb, scratch, queue, counters, adj, adj_store,
                                    stream);
    case 2:
      return group::launch_k<8, 2>(net, gt, st, dt, smem, grid, tpb, scratch, queue, counters, adj, adj_store,
                                    stream);
    case 3:
      return group::launch_k<8, 3>(net, gt, st, dt, smem, grid, tpb, scratch, queue, counters, adj, adj_store,
                                    stream);
    default:
      return -1;
  }
}
}  // namespace pfgpu
