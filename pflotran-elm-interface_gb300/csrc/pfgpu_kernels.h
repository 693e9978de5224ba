// pfgpu_kernels.h -- launchers shared between the C-ABI translation unit and
// the kernel translation units.
#pragma once
#include "pfgpu_common.cuh"

namespace pfgpu {

// K1: one thread per cell, direct form (pfgpu_plain.cu)
int launch_rstep_plain(const DevNet& net, const PfCellState& st, double dt,
                       unsigned long long* counters, cudaStream_t stream);

// K2: persistent lane-refilling kernel (pfgpu_batched.cu).
// queue: device counter zeroed by the caller (cudaMemsetAsync) before launch.
// counters[0] += Newton iterations, counters[1] += failed cells,
// counters[2] = error flags (bit 0: table staging timed out).
// cfg.lanes_per_cell > 1 runs the group kernel; with adj it needs adj_store
// (group_adj_store_doubles), otherwise adj runs on one lane per cell.
int launch_rstep_batched(const DevNet& net, const PfCellState& st, double dt,
                         const PfLaunchConfig& cfg, int num_sms, double* scratch,
                         unsigned long long* queue, unsigned long long* counters,
                         cudaStream_t stream, const PfAdjointArgs* adj = nullptr,
                         double* adj_store = nullptr);
// K3: the same step with a group of lanes per cell (pfgpu_group.cu); used by
// launch_rstep_batched when cfg.lanes_per_cell > 1
bool group_supported(const DevNet& net, int lanes_per_cell);
size_t group_smem_bytes(const DevNet& net, const PfLaunchConfig& cfg, bool adj = false);
// doubles of the adjoint's substep store (iterate and dt of each substep)
size_t group_adj_store_doubles(const DevNet& net, int64_t ncells);
int launch_rstep_group(const DevNet& net, const GroupTabs& gt, const PfCellState& st, double dt,
                       const PfLaunchConfig& cfg, int num_sms, const double* scratch, unsigned long long* queue,
                       unsigned long long* counters, cudaStream_t stream, const PfAdjointArgs* adj = nullptr,
                       double* adj_store = nullptr);
// whether a group launch of this configuration stages the per-entry tables
bool group_entries_staged(const DevNet& net, const PfLaunchConfig& cfg, bool adj);
// the batched kernels' per-cell set-up pre-pass (pfgpu_batched.cu)
int launch_cell_setup(const DevNet& net, const PfCellState& st, double* scratch, cudaStream_t stream);
// one persistent launch over several networks' cells (pfgpu_multi.cu): per
// network its tables, state, set-up scratch, work-queue counter and
// reductions (both zeroed by the caller), and the group size
struct MultiNetLaunch {
  DevNet net;
  PfCellState st;
  double* scratch;
  unsigned long long* queue;
  unsigned long long* counters;
  int lanes_per_cell;
};
// the group size the multi-network kernel runs a network with (the preferred
// one when it carries it), 0 when it carries none for this network
int multi_lanes_for(const DevNet& net, int preferred);
int launch_rstep_multi(const MultiNetLaunch* nets, int nnets, double dt, int threads_per_block, int blocks_per_sm,
                       int num_sms, cudaStream_t stream);
// host: the group kernel's lookup tables from the host copies of the packed
// network blocks
int group_build_tables(const DevNet& net, const int32_t* h_ints, const double* h_dbls, void** d_buf,
                       GroupTabs* out);
// doubles of per-cell scratch the batched kernel's setup pre-pass writes
size_t batched_scratch_doubles(const DevNet& net, int64_t ncells);
// shared memory bytes a batched launch of this config needs
size_t batched_smem_bytes(const DevNet& net, const PfLaunchConfig& cfg);
bool batched_supported(const DevNet& net);
// one lane per cell: ncomp has an instantiation of the persistent kernel
bool lane_supported(const DevNet& net);

// auxvar kernels (pfgpu_aux.cu)
int launch_update_auxvars(const DevNet& net, const PfCellState& st, int update_act,
                          cudaStream_t stream);
int launch_update_activity_coefs(const DevNet& net, const PfCellState& st, cudaStream_t stream);

// global-implicit assembly (pfgpu_girt.cu).  Per-network lookup tables, all
// device pointers into one allocation, CSR over Jacobian entries
// f = row*n + col:
//   e_sec_*  the secondaries contributing to dtotal(row, col): secondary
//            index and nu_row*nu_col, ascending secondary
//   e_mn_*   the kinetic-mineral derivative terms: CSR slot of the column
//            species in the mineral's reaction, mineral index, nu_row
struct GirtTabs {
  // one device buffer [int32 part (ibytes, 16-byte padded) | double part]:
  //   per complex i, the species pairs (p <= q) of its reaction: CSR s_pair
  //   (ptr at o_spp, packed symmetric index at o_spk, nu_p nu_q at d_spc);
  //   per flat entry row*n+col, the kinetic minerals whose reaction holds
  //   both species: CSR m_ent (ptr at o_mep, mineral at o_mem, nu_row nu_col
  //   at d_mec)
  const void* buf;
  int32_t ibytes, dbytes;
  int32_t o_spp, o_spk, o_mep, o_mem;  // offsets in int32 words
  int32_t d_spc, d_mec;                // offsets in doubles
};
// host: build the tables from the host copies of the packed network blocks
// and upload them (*d_buf: the one device allocation)
int girt_build_tables(const DevNet& net, const int32_t* h_ints, const double* h_dbls, void** d_buf,
                      GirtTabs* out);
size_t girt_smem_bytes(const DevNet& net, const GirtTabs& gt, bool with_lna, bool e_in_smem, int* threads_per_block,
                       int* staged);
// RTUpdateAuxVars then the column kernel; a PfStatus
// e_scratch: nsym x ncells doubles of global memory for the packed sum of
// d total/d m (NULL: in shared memory)
int launch_girt_assemble(const DevNet& net, const GirtTabs& gt, const PfCellState& st, const PfGirtArgs& a,
                         int num_sms, cudaStream_t stream, double* e_scratch);

}  // namespace pfgpu
