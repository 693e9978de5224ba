// pfgpu_group.cu -- the operator-split step with a group of G lanes per cell.
//
// Same step as rstep_batched_kernel (RStep/RReact, reaction.F90:3564-4055),
// for larger networks.  One lane per cell keeps every per-cell array in that
// lane's registers or local memory; from ncomp ~16 up that is several KB per
// lane (the Jacobian alone is 4.6 KB at ncomp 24), which spills past L1 and
// leaves a few warps per SM.  Here G lanes (2, 4 or 8) share one cell:
//
//   * the cell's Jacobian, power table, secondary molalities and kinetic-
//     mineral terms live in a per-cell shared-memory workspace;
//   * lane r of the group owns the species / Jacobian rows i = r, r+G, ...
//     (R = ceil(n/G) of them) and holds their Newton state in registers;
//     secondary complexes and minerals are split round-robin over the lanes;
//   * a row owner assembles its Jacobian rows from per-species lists of the
//     secondaries and minerals that contain the species (no two lanes write
//     one entry);
//   * the LU is right-looking Gaussian elimination with the reference's
//     implicit pivoting (pivot = argmax VV_i |a_ik| over the remaining rows,
//     utility.F90:645-666), the right-hand side eliminated alongside, rows
//     not swapped but tracked; the pivot search is a shuffle reduction over
//     the group, each lane updates its own rows, back substitution runs by
//     columns so that every lane stays busy;
//   * every decision (convergence, cuts, substeps) uses group reductions
//     whose result is bitwise identical in all lanes of the group, so the
//     group follows one control path.
// The work queue hands out cells to groups exactly as the one-lane kernel
// hands them to lanes.  Log formulation only (the launch falls back to the
// one-lane kernel otherwise).
//
// ADJ = true adds the implicit adjoint of the step (pf_adjoint), as in the
// one-lane kernel: the converged iterate and dt of every substep go to a
// global store [PF_ADJ_MAX_SUBSTEPS][n + 1][ncells]; when the group finishes
// the forward step it walks the substeps backwards, rebuilding the exact
// Jacobian at each stored iterate (true mineral derivative), solving
// J u = B Tbar (B the minerals' part of J), lambda = (Tbar - u)/(psv/dt),
// and accumulating theta_bar += (dT/dtheta)^T u - (dR/dtheta)^T lambda.
// Gradients of the network parameters collect per lane over its own
// complexes and minerals and are reduced over the warp at the end.
#include <algorithm>
#include <vector>

#include "pfgpu_group.cuh"

namespace pfgpu {
// rows per lane the instantiations cover (pfgpu_group_g*.cu)
static bool group_rows_ok(int G, int R) {
  return (G == 2 && R >= 2 && R <= 6) || (G == 4 && R >= 2 && R <= 4) || (G == 8 && R >= 1 && R <= 3);
}

#define PF_GROUP_DECL(GG)                                                                                      \
  int launch_group_g##GG(const DevNet& net, const GroupTabs& gt, const PfCellState& st, double dt, int R,      \
                         size_t smem, int grid, int tpb, const double* scratch, unsigned long long* queue,     \
                         unsigned long long* counters, const PfAdjointArgs* adj, double* adj_store,            \
                         cudaStream_t stream);
PF_GROUP_DECL(2)
PF_GROUP_DECL(4)
PF_GROUP_DECL(8)
#undef PF_GROUP_DECL

bool group_supported(const DevNet& net, int lanes_per_cell) {
  if (lanes_per_cell != 2 && lanes_per_cell != 4 && lanes_per_cell != 8) return false;
  if (!net.o.use_log_formulation) return false;
  if (net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER &&
      net.o.act_coef_update_algorithm == PF_ACT_COEF_ALGO_NEWTON)
    return false;
  if (net.ns > PF_MAX_NSEC || net.nm > PF_MAX_NMNRL) return false;
  // rate prefactors with activity coefficients moving each Newton iteration:
  // the plain kernel (the prefactor's complexes' activities would follow them)
  if ((net.flags & NETF_PREFACTOR) && net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER) return false;
  if (net.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER && net.o.use_activity_h2o)
    return false;  // water activity moving each Newton iteration: the plain kernel
  const int R = (net.n + lanes_per_cell - 1) / lanes_per_cell;
  return group_rows_ok(lanes_per_cell, R);
}

// the per-entry assembly tables are staged in shared memory when they fit
// beside the block's cells, else read through L1
bool group_entries_staged(const DevNet& net, const PfLaunchConfig& cfg, bool adj) {
  const int G = cfg.lanes_per_cell > 0 ? cfg.lanes_per_cell : 1;
  const size_t cells = (size_t)cfg.threads_per_block / (size_t)G;
  const size_t ws = cells * ((size_t)group::ws_doubles(net, adj, G) * 8 + (size_t)net.n * 8);
  return (size_t)net.int_words_grp * 4 + (size_t)net.dbl_words_grp * 8 + ws <= 227u * 1024u;
}

size_t group_smem_bytes(const DevNet& net, const PfLaunchConfig& cfg, bool adj) {
  const int G = cfg.lanes_per_cell > 0 ? cfg.lanes_per_cell : 1;
  const size_t cells = (size_t)cfg.threads_per_block / (size_t)G;
  const size_t ws = cells * ((size_t)group::ws_doubles(net, adj, G) * 8 + (size_t)net.n * 8);
  const bool full = group_entries_staged(net, cfg, adj);
  const size_t tables = full ? (size_t)net.int_words_grp * 4 + (size_t)net.dbl_words_grp * 8
                             : (size_t)net.int_words_core * 4 + (size_t)net.dbl_words_core * 8;
  return tables + ws;
}

size_t group_adj_store_doubles(const DevNet& net, int64_t ncells) {
  return (size_t)PF_ADJ_MAX_SUBSTEPS * (size_t)(net.n + 1) * (size_t)ncells;
}

int launch_rstep_group(const DevNet& net, const GroupTabs& gt, const PfCellState& st, double dt,
                       const PfLaunchConfig& cfg, int num_sms, const double* scratch, unsigned long long* queue,
                       unsigned long long* counters, cudaStream_t stream, const PfAdjointArgs* adj,
                       double* adj_store) {
  const int G = cfg.lanes_per_cell;
  const int R = (net.n + G - 1) / G;
  const size_t smem = group_smem_bytes(net, cfg, adj != nullptr);
  const int tpb = cfg.threads_per_block;
  const int grid = num_sms * cfg.blocks_per_sm;
  DevNet nl = net;
  nl.ent_staged = group_entries_staged(net, cfg, adj != nullptr) ? 1 : 0;
  if (G == 2) return launch_group_g2(nl, gt, st, dt, R, smem, grid, tpb, scratch, queue, counters, adj, adj_store, stream);
  if (G == 4) return launch_group_g4(nl, gt, st, dt, R, smem, grid, tpb, scratch, queue, counters, adj, adj_store, stream);
  if (G == 8) return launch_group_g8(nl, gt, st, dt, R, smem, grid, tpb, scratch, queue, counters, adj, adj_store, stream);
  return -1;
}

int group_build_tables(const DevNet& net, const int32_t* I, const double* D, void** d_buf, GroupTabs* out) {
  const int n = net.n;
  std::vector<std::vector<int32_t>> ss(n), sp(n), mm(n), mp(n);
  for (int s = 0; s < net.ns; ++s)
    for (int p = I[net.o_sec_ptr + s]; p < I[net.o_sec_ptr + s + 1]; ++p) {
      ss[I[net.o_sec_idx + p]].push_back(s);
      sp[I[net.o_sec_idx + p]].push_back(p);
    }
  for (int m = 0; m < net.nm; ++m)
    for (int p = I[net.o_mnrl_ptr + m]; p < I[net.o_mnrl_ptr + m + 1]; ++p) {
      mm[I[net.o_mnrl_idx + p]].push_back(m);
      mp[I[net.o_mnrl_idx + p]].push_back(p);
    }
  std::vector<int32_t> ints;
  auto csr = [&](const std::vector<std::vector<int32_t>>& a, const std::vector<std::vector<int32_t>>& b, int* o_ptr,
                 int* o_a, int* o_b) {
    *o_ptr = (int)ints.size();
    int cnt = 0;
    for (auto& rw : a) { ints.push_back(cnt); cnt += (int)rw.size(); }
    ints.push_back(cnt);
    *o_a = (int)ints.size();
    for (auto& rw : a) ints.insert(ints.end(), rw.begin(), rw.end());
    *o_b = (int)ints.size();
    for (auto& rw : b) ints.insert(ints.end(), rw.begin(), rw.end());
  };
  int o1, o2, o3, o4, o5, o6;
  csr(ss, sp, &o1, &o2, &o3);
  csr(mm, mp, &o4, &o5, &o6);
  const int o7 = (int)ints.size();
  {
    std::vector<int> perm(net.ns);
    for (int k = 0; k < net.ns; ++k) perm[k] = k;
    auto len = [&](int k) { return I[net.o_sec_ptr + k + 1] - I[net.o_sec_ptr + k]; };
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return len(a) > len(b); });
    ints.insert(ints.end(), perm.begin(), perm.end());
    if (net.ns == 0) ints.push_back(0);
  }
  // the stoichiometric coefficients along the same lists, after the ints
  std::vector<double> nus;
  for (auto& rw : sp)
    for (int p : rw) nus.push_back(D[net.o_sec_nu + p]);
  const size_t o_mnu = nus.size();
  for (auto& rw : mp)
    for (int p : rw) nus.push_back(D[net.o_mnrl_nu + p]);
  while (ints.size() % 4) ints.push_back(0);
  const size_t ibytes = ints.size() * 4;
  void* buf = nullptr;
  if (cudaMalloc(&buf, ibytes + nus.size() * 8 + 8) != cudaSuccess) return PF_ERR_CUDA;
  if (cudaMemcpy(buf, ints.data(), ibytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      (!nus.empty() &&
       cudaMemcpy((char*)buf + ibytes, nus.data(), nus.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)) {
    cudaFree(buf);
    return PF_ERR_CUDA;
  }
  const int32_t* d = (const int32_t*)buf;
  out->sp_nu = reinterpret_cast<const double*>((const char*)buf + ibytes);
  out->mp_nu = out->sp_nu + o_mnu;
  out->sp_ptr = d + o1;
  out->sp_s = d + o2;
  out->sp_p = d + o3;
  out->mp_ptr = d + o4;
  out->mp_m = d + o5;
  out->mp_p = d + o6;
  out->s_perm = d + o7;
  *d_buf = buf;
  return PF_OK;
}

}  // namespace pfgpu
