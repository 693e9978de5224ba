// pfgpu_api.cu -- the C ABI (include/pfgpu.h): network upload, argument
// checking, kernel dispatch, the status reduction and the host-buffer path.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "pfgpu_common.cuh"
#include "pfgpu_kernels.h"

using namespace pfgpu;

extern "C" int32_t pf_equilibrate_constraint_impl(const DevNet* net, const PfCellState* st,
                                                  const int32_t* ctype, const PfConstraintReaction* creact,
                                                  const double* cconc, int use_prev, int32_t* iterations,
                                                  int max_iterations, void* stream);

struct PfNetwork {
  DevNet dev{};
  void* d_tables = nullptr;
  unsigned long long* d_counters = nullptr;  // [0] queue [1] its [2] fails [3] err [4] max its [5] max substeps
  unsigned long long* h_counters = nullptr;  // pinned mirror
  int32_t* d_ctype = nullptr;                // constraint types [PF_MAX_NCOMP], then reactions
  PfConstraintReaction* d_creact = nullptr;  // [PF_MAX_NCOMP], inside the d_ctype allocation
  double* d_scratch = nullptr;               // batched kernel per-cell scratch
  size_t scratch_cap = 0;                    // doubles
  std::vector<double> dbls_base;             // host copy of the double block at create
  std::vector<int32_t> ints_base;            // host copy of the int block
  void* d_girt = nullptr;                    // global-implicit lookup tables (built on first use)
  void* d_group = nullptr;                   // group-kernel inverse lists (dev.grp points into it)
  PfLaunchConfig launch_lane{};              // last one-lane-per-cell configuration (adjoint)
  GirtTabs girt{};
  size_t ib = 0;                             // byte offset of the double block
  PfLaunchConfig launch{};
  int device = 0;
  int num_sms = 0;
  // host-path arena (grow-only)
  void* d_arena = nullptr;
  size_t arena_bytes = 0;
  // host-path pipeline: copy-in, compute and copy-out streams, per-chunk
  // events, counters and the chunk-local work-queue orders (pinned)
  cudaStream_t s_in = nullptr, s_comp = nullptr, s_out = nullptr;
  cudaEvent_t ev_in[16] = {}, ev_comp[16] = {}, ev_start = nullptr;
  unsigned long long* d_ccounters = nullptr;  // [16][8]
  unsigned long long* h_ccounters = nullptr;
  int64_t* h_order = nullptr;
  size_t h_order_cap = 0;
};

namespace {

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? PF_OK : PF_ERR_CUDA; }

size_t pad16(size_t bytes) { return (bytes + 15) & ~size_t(15); }

int validate_desc(const PfNetworkDesc* d) {
  if (!d) return PF_ERR_INVALID;
  if (d->ncomp < 1 || d->nsec < 0 || d->nmnrl < 0) return PF_ERR_INVALID;
  if (d->ncomp > PF_MAX_NCOMP || d->nsec > PF_MAX_NSEC || d->nmnrl > PF_MAX_NMNRL) return PF_ERR_TOO_LARGE;
  if (!d->pri_Z || !d->pri_a0) return PF_ERR_INVALID;
  if (d->nsec > 0 && (!d->sec_nspec || !d->sec_spec || !d->sec_stoich || !d->sec_logK || !d->sec_Z ||
                      !d->sec_a0 || d->sec_stride < 1))
    return PF_ERR_INVALID;
  for (int i = 0; i < d->nsec; ++i) {
    if (d->sec_nspec[i] < 0 || d->sec_nspec[i] > d->sec_stride || d->sec_nspec[i] > PF_MAX_SPEC_PER_RXN)
      return PF_ERR_INVALID;
    for (int s = 0; s < d->sec_nspec[i]; ++s) {
      int k = d->sec_spec[i * d->sec_stride + s];
      if (k < 0 || k >= d->ncomp) return PF_ERR_INVALID;
    }
  }
  if (d->nmnrl > 0 && (!d->mnrl_nspec || !d->mnrl_spec || !d->mnrl_stoich || !d->mnrl_logK ||
                       !d->mnrl_rate_constant || !d->mnrl_activation_energy || !d->mnrl_molar_vol ||
                       !d->mnrl_affinity_threshold || !d->mnrl_rate_limiter || !d->mnrl_irreversible ||
                       d->mnrl_stride < 1))
    return PF_ERR_INVALID;
  for (int m = 0; m < d->nmnrl; ++m) {
    if (d->mnrl_nspec[m] < 0 || d->mnrl_nspec[m] > d->mnrl_stride || d->mnrl_nspec[m] > PF_MAX_SPEC_PER_RXN)
      return PF_ERR_INVALID;
    for (int s = 0; s < d->mnrl_nspec[m]; ++s) {
      int k = d->mnrl_spec[m * d->mnrl_stride + s];
      if (k < 0 || k >= d->ncomp) return PF_ERR_INVALID;
    }
  }
  if (d->opts.maximum_reaction_iterations < 1 || d->opts.maximum_reaction_cuts < 0) return PF_ERR_INVALID;
  if (const PfSorptionDesc* sd = d->sorption) {
    if (sd->nkd < 0 || sd->nionx < 0) return PF_ERR_INVALID;
    if (sd->nkd > PF_MAX_NKD || sd->nionx > PF_MAX_NIONX) return PF_ERR_TOO_LARGE;
    if (sd->kd_units != PF_KD_UNIT_KG_M3_BULK && sd->kd_units != PF_KD_UNIT_MLW_GSOIL) return PF_ERR_INVALID;
    if (sd->nkd > 0 && (!sd->kd_spec || !sd->kd_type || !sd->kd_coeff)) return PF_ERR_INVALID;
    for (int r = 0; r < sd->nkd; ++r) {
      if (sd->kd_spec[r] < 0 || sd->kd_spec[r] >= d->ncomp) return PF_ERR_INVALID;
      if (sd->kd_type[r] < PF_SORPTION_LINEAR || sd->kd_type[r] > PF_SORPTION_FREUNDLICH) return PF_ERR_INVALID;
      if (sd->kd_type[r] == PF_SORPTION_LANGMUIR && !sd->kd_langmuir_b) return PF_ERR_INVALID;
      if (sd->kd_type[r] == PF_SORPTION_FREUNDLICH && !sd->kd_freundlich_n) return PF_ERR_INVALID;
      if (sd->kd_mineral && (sd->kd_mineral[r] < -1 || sd->kd_mineral[r] >= d->nmnrl)) return PF_ERR_INVALID;
    }
    if (sd->nionx > 0 && (!sd->ionx_ncation || !sd->ionx_cation || !sd->ionx_k || !sd->ionx_cec ||
                          sd->ionx_stride < 1))
      return PF_ERR_INVALID;
    for (int r = 0; r < sd->nionx; ++r) {
      if (sd->ionx_ncation[r] < 1 || sd->ionx_ncation[r] > sd->ionx_stride ||
          sd->ionx_ncation[r] > PF_MAX_IONX_CATIONS)
        return PF_ERR_INVALID;
      for (int j = 0; j < sd->ionx_ncation[r]; ++j) {
        const int k = sd->ionx_cation[r * sd->ionx_stride + j];
        if (k < 0 || k >= d->ncomp || d->pri_Z[k] == 0.0) return PF_ERR_INVALID;  // cations carry charge
      }
      if (sd->ionx_mineral && (sd->ionx_mineral[r] < -1 || sd->ionx_mineral[r] >= d->nmnrl)) return PF_ERR_INVALID;
    }
    if (sd->nsrfcplx_rxn < 0 || sd->nsrfcplx < 0) return PF_ERR_INVALID;
    if (sd->nsrfcplx_rxn > PF_MAX_NSRFCPLX_RXN || sd->nsrfcplx > PF_MAX_NSRFCPLX) return PF_ERR_TOO_LARGE;
    if (sd->nsrfcplx_rxn > 0) {
      if (!sd->srfcplx_rxn_ptr || !sd->srfcplx_surf_type || !sd->srfcplx_site_density || !sd->srfcplx_nspec ||
          !sd->srfcplx_spec || !sd->srfcplx_stoich || !sd->srfcplx_free_site_stoich || !sd->srfcplx_logK ||
          sd->srfcplx_stride < 1)
        return PF_ERR_INVALID;
      if (sd->srfcplx_rxn_ptr[0] != 0 || sd->srfcplx_rxn_ptr[sd->nsrfcplx_rxn] != sd->nsrfcplx) return PF_ERR_INVALID;
      for (int r = 0; r < sd->nsrfcplx_rxn; ++r) {
        if (sd->srfcplx_rxn_ptr[r + 1] <= sd->srfcplx_rxn_ptr[r]) return PF_ERR_INVALID;  // a site has complexes
        const int t = sd->srfcplx_surf_type[r];
        if (t != PF_SURF_NULL && t != PF_SURF_MINERAL && t != PF_SURF_ROCK) return PF_ERR_INVALID;
        if (t == PF_SURF_MINERAL &&
            (!sd->srfcplx_mineral || sd->srfcplx_mineral[r] < 0 || sd->srfcplx_mineral[r] >= d->nmnrl))
          return PF_ERR_INVALID;
      }
      for (int k = 0; k < sd->nsrfcplx; ++k) {
        const int ns = sd->srfcplx_nspec[k];
        if (ns < 0 || ns > sd->srfcplx_stride || ns > PF_MAX_SPEC_PER_RXN) return PF_ERR_INVALID;
        for (int p = 0; p < ns; ++p) {
          const int j = sd->srfcplx_spec[k * sd->srfcplx_stride + p];
          if (j < 0 || j >= d->ncomp) return PF_ERR_INVALID;
        }
        if (!(sd->srfcplx_free_site_stoich[k] > 0.0)) return PF_ERR_INVALID;
      }
    }
  }
  if (const PfPrefactorDesc* pf = d->prefactors) {
    if (!pf->num_prefactors || !pf->rate || !pf->activation_energy || !pf->nspec || !pf->spec || !pf->alpha ||
        !pf->beta || !pf->atten_coef)
      return PF_ERR_INVALID;
    for (int m = 0; m < d->nmnrl; ++m) {
      const int np = pf->num_prefactors[m];
      if (np < 0 || np > PF_MAX_PREFACTORS) return PF_ERR_INVALID;
      // the derivative of a secondary prefactor species leaves the complex's
      // species count in place of the mineral's (reaction_mineral.F90:1046);
      // a later primary species of the same mineral then walks that many of
      // the mineral's species (:1033-1038), which must exist
      int cnt = d->mnrl_nspec[m];
      for (int p = 0; p < np; ++p) {
        const int ns = pf->nspec[m * PF_MAX_PREFACTORS + p];
        if (ns < 0 || ns > PF_MAX_PREFACTOR_SPECIES) return PF_ERR_INVALID;
        for (int k = 0; k < ns; ++k) {
          const int id = pf->spec[(m * PF_MAX_PREFACTORS + p) * PF_MAX_PREFACTOR_SPECIES + k];
          if (id >= d->ncomp || -id - 1 >= d->nsec) return PF_ERR_INVALID;
          if (id < 0) cnt = d->sec_nspec[-id - 1];
          else if (cnt > d->mnrl_nspec[m]) return PF_ERR_UNSUPPORTED;
        }
      }
    }
  }
  if (d->opts.act_coef_update_frequency < 0 || d->opts.act_coef_update_frequency > 2) return PF_ERR_INVALID;
  return PF_OK;
}

int validate_state(const PfNetwork* net, const PfCellState* s) {
  if (!net || !s) return PF_ERR_INVALID;
  if (s->ncells < 0) return PF_ERR_INVALID;
  if (s->ncells == 0) return PF_OK;
  if (!s->total || !s->pri_molal || !s->pri_act_coef || !s->porosity || !s->saturation || !s->den_kg ||
      !s->volume)
    return PF_ERR_INVALID;
  if (net->dev.ns > 0 && (!s->sec_act_coef || !s->sec_molal)) return PF_ERR_INVALID;
  if (net->dev.nm > 0 && (!s->mnrl_volfrac || !s->mnrl_area || !s->mnrl_rate)) return PF_ERR_INVALID;
  if (!net->dev.o.isothermal && !s->temperature) return PF_ERR_INVALID;
  if (has_sorption(net->dev) && !s->total_sorb) return PF_ERR_INVALID;
  if (net->dev.nsrx > 0 && !s->srfcplx_free_site) return PF_ERR_INVALID;
  if (net->dev.nionx > 0 && !s->ionx_ref_sorbed) return PF_ERR_INVALID;
  if (net->dev.o.use_activity_h2o && !s->ln_act_h2o) return PF_ERR_INVALID;
  return PF_OK;
}

PfLaunchConfig default_launch(const DevNet& dev) {
  PfLaunchConfig c{};
  c.threads_per_block = 128;
  c.blocks_per_sm = 1;
  if (!lane_supported(dev)) {
    // no one-lane instantiation for this ncomp: a group of lanes per cell
    for (int g : {4, 8, 2}) {
      if (!group_supported(dev, g)) continue;
      c.lanes_per_cell = g;
      while (c.threads_per_block > 32 && batched_smem_bytes(dev, c) > 227u * 1024u) c.threads_per_block -= 32;
      if (batched_smem_bytes(dev, c) <= 227u * 1024u) return c;
      c.threads_per_block = 128;
    }
    c.lanes_per_cell = 0;
  }
  c.jac_in_shared = dev.n <= 12 ? 1 : 0;
  // shrink until one block fits the 227 KB opt-in shared memory
  while (c.threads_per_block > 32 && batched_smem_bytes(dev, c) > 227u * 1024u) c.threads_per_block -= 32;
  if (batched_smem_bytes(dev, c) > 227u * 1024u) c.jac_in_shared = 0;
  return c;
}

}  // namespace

extern "C" {

const char* pf_version(void) { return "pfgpu 0.1 (sm_103a, FP64)"; }

int32_t pf_network_create(const PfNetworkDesc* d, PfNetwork** out) {
  if (!out) return PF_ERR_INVALID;
  *out = nullptr;
  int rc = validate_desc(d);
  if (rc) return rc;
  const int n = d->ncomp, ns = d->nsec, nm = d->nmnrl;
  // CSR rows
  std::vector<int32_t> ints;
  std::vector<double> dbls;
  DevNet dev{};
  dev.n = n;
  dev.ns = ns;
  dev.nm = nm;
  dev.o_sec_ptr = (int)ints.size();
  int nnz = 0;
  for (int i = 0; i < ns; ++i) { ints.push_back(nnz); nnz += d->sec_nspec[i]; }
  ints.push_back(nnz);
  dev.nnz_s = nnz;
  dev.o_sec_idx = (int)ints.size();
  for (int i = 0; i < ns; ++i)
    for (int s = 0; s < d->sec_nspec[i]; ++s) ints.push_back(d->sec_spec[i * d->sec_stride + s]);
  dev.o_mnrl_ptr = (int)ints.size();
  nnz = 0;
  for (int m = 0; m < nm; ++m) { ints.push_back(nnz); nnz += d->mnrl_nspec[m]; }
  ints.push_back(nnz);
  dev.nnz_m = nnz;
  dev.o_mnrl_idx = (int)ints.size();
  for (int m = 0; m < nm; ++m)
    for (int s = 0; s < d->mnrl_nspec[m]; ++s) ints.push_back(d->mnrl_spec[m * d->mnrl_stride + s]);
  dev.o_irrev = (int)ints.size();
  for (int m = 0; m < nm; ++m) ints.push_back(d->mnrl_irreversible[m]);
  // product-form tables
  int neg_mask = 0;
  auto code_of = [&](double nu, int k) -> int {
    if (nu == 1.0) return k;
    if (nu == 2.0) return n + k;
    if (nu == -1.0) { neg_mask |= 1 << k; return 2 * n + k; }
    if (nu == -2.0) { neg_mask |= 1 << k; return 3 * n + k; }
    return -1;
  };
  dev.o_sec_pidx = (int)ints.size();
  for (int i = 0; i < ns; ++i)
    for (int s2 = 0; s2 < d->sec_nspec[i]; ++s2)
      ints.push_back(code_of(d->sec_stoich[i * d->sec_stride + s2], d->sec_spec[i * d->sec_stride + s2]));
  // the pair tables of the one-lane kernel go to the end of the blocks
  // (lane_ints / pair coefficients, offsets fixed up there), so that the
  // group kernel stages only the prefix it reads
  std::vector<int32_t> spair_idx, mpair_idx, lane_ints;
  std::vector<double> spair_coef, mpair_coef;
  dev.o_spair_ptr = (int)lane_ints.size();
  for (int i = 0; i < ns; ++i) {
    lane_ints.push_back((int32_t)spair_idx.size());
    const int b = i * d->sec_stride, cnt = d->sec_nspec[i];
    for (int p = 0; p < cnt; ++p)
      for (int q = p; q < cnt; ++q) {
        const int kp = d->sec_spec[b + p], kq = d->sec_spec[b + q];
        const int lo = kp < kq ? kp : kq, hi = kp < kq ? kq : kp;
        spair_idx.push_back(lo * n + hi);
        spair_coef.push_back(d->sec_stoich[b + p] * d->sec_stoich[b + q]);
      }
  }
  lane_ints.push_back((int32_t)spair_idx.size());
  dev.o_spair_idx = (int)lane_ints.size();
  lane_ints.insert(lane_ints.end(), spair_idx.begin(), spair_idx.end());
  dev.o_mnrl_pidx = (int)ints.size();
  for (int m = 0; m < nm; ++m)
    for (int s2 = 0; s2 < d->mnrl_nspec[m]; ++s2)
      ints.push_back(code_of(d->mnrl_stoich[m * d->mnrl_stride + s2], d->mnrl_spec[m * d->mnrl_stride + s2]));
  dev.o_mpair_ptr = (int)lane_ints.size();
  for (int m = 0; m < nm; ++m) {
    lane_ints.push_back((int32_t)mpair_idx.size());
    const int b = m * d->mnrl_stride, cnt = d->mnrl_nspec[m];
    for (int p = 0; p < cnt; ++p)
      for (int q = 0; q < cnt; ++q) {
        mpair_idx.push_back(d->mnrl_spec[b + p] * n + d->mnrl_spec[b + q]);
        mpair_coef.push_back(d->mnrl_stoich[b + p] * d->mnrl_stoich[b + q]);
      }
  }
  lane_ints.push_back((int32_t)mpair_idx.size());
  dev.o_mpair_idx = (int)lane_ints.size();
  lane_ints.insert(lane_ints.end(), mpair_idx.begin(), mpair_idx.end());
  dev.neg_mask = neg_mask;
  // per-entry Jacobian assembly (group kernel, LDL^T): every lower-triangle
  // entry (i >= j, row-major, e = i(i+1)/2 + j) with the complexes and the
  // minerals that contain both species and the coefficient nu_i nu_j
  std::vector<int32_t> ent_sc, ent_mm, ent_ints;
  std::vector<double> ent_cf, ent_mcf;
  {
    std::vector<std::vector<std::pair<int, double>>> es(n * (n + 1) / 2), em(n * (n + 1) / 2);
    for (int sx = 0; sx < ns; ++sx)
      for (int a = 0; a < d->sec_nspec[sx]; ++a)
        for (int b = 0; b < d->sec_nspec[sx]; ++b) {
          const int i = d->sec_spec[sx * d->sec_stride + a], j = d->sec_spec[sx * d->sec_stride + b];
          if (j > i) continue;
          es[i * (i + 1) / 2 + j].push_back(
              {sx, d->sec_stoich[sx * d->sec_stride + a] * d->sec_stoich[sx * d->sec_stride + b]});
        }
    for (int m = 0; m < nm; ++m)
      for (int a = 0; a < d->mnrl_nspec[m]; ++a)
        for (int b = 0; b < d->mnrl_nspec[m]; ++b) {
          const int i = d->mnrl_spec[m * d->mnrl_stride + a], j = d->mnrl_spec[m * d->mnrl_stride + b];
          if (j > i) continue;
          em[i * (i + 1) / 2 + j].push_back(
              {m, d->mnrl_stoich[m * d->mnrl_stride + a] * d->mnrl_stoich[m * d->mnrl_stride + b]});
        }
    // the group kernel deals the entries round-robin to the lanes of a
    // group: listed longest first, the lanes of one round sum lists of about
    // the same length (a diagonal entry collects every complex of its
    // species, an off-diagonal one a few), so fewer lanes wait in each round;
    // every entry is summed the same way in any order
    const int ne = n * (n + 1) / 2;
    std::vector<int> eord(ne), eflat(ne);
    for (int i = 0, e = 0; i < n; ++i)
      for (int j = 0; j <= i; ++j, ++e) {
        eord[e] = e;
        eflat[e] = i * n + j;
      }
    std::stable_sort(eord.begin(), eord.end(), [&](int a, int b) {
      return es[a].size() + em[a].size() > es[b].size() + em[b].size();
    });
    // into ent_ints (offsets relative to it, fixed up where it is appended)
    dev.o_ent_ij = (int)ent_ints.size();
    for (int e : eord) ent_ints.push_back(eflat[e]);
    dev.o_ent_ptr = (int)ent_ints.size();
    for (int e : eord) {
      ent_ints.push_back((int32_t)ent_sc.size());
      for (auto& pr : es[e]) { ent_sc.push_back(pr.first); ent_cf.push_back(pr.second); }
    }
    ent_ints.push_back((int32_t)ent_sc.size());
    dev.o_ent_sc = (int)ent_ints.size();
    ent_ints.insert(ent_ints.end(), ent_sc.begin(), ent_sc.end());
    dev.o_ent_mptr = (int)ent_ints.size();
    for (int e : eord) {
      ent_ints.push_back((int32_t)ent_mm.size());
      for (auto& pr : em[e]) { ent_mm.push_back(pr.first); ent_mcf.push_back(pr.second); }
    }
    ent_ints.push_back((int32_t)ent_mm.size());
    dev.o_ent_mm = (int)ent_ints.size();
    ent_ints.insert(ent_ints.end(), ent_mm.begin(), ent_mm.end());
  }
  // sorption: K_D rows; ion-exchange reactions as CSR over their cations
  const PfSorptionDesc* sd = d->sorption;
  const int nkd = sd ? sd->nkd : 0, nix = sd ? sd->nionx : 0;
  dev.nkd = nkd;
  dev.nionx = nix;
  dev.kd_units = sd ? sd->kd_units : 0;
  dev.soil_density = sd ? sd->soil_particle_density : 0.0;
  dev.o_kd_spec = (int)ints.size();
  for (int r = 0; r < nkd; ++r) ints.push_back(sd->kd_spec[r]);
  dev.o_kd_type = (int)ints.size();
  for (int r = 0; r < nkd; ++r) ints.push_back(sd->kd_type[r]);
  dev.o_kd_min = (int)ints.size();
  for (int r = 0; r < nkd; ++r) ints.push_back(sd->kd_mineral ? sd->kd_mineral[r] : -1);
  dev.o_ix_ptr = (int)ints.size();
  {
    int cnt = 0;
    for (int r = 0; r < nix; ++r) { ints.push_back(cnt); cnt += sd->ionx_ncation[r]; }
    ints.push_back(cnt);
  }
  dev.o_ix_cat = (int)ints.size();
  for (int r = 0; r < nix; ++r)
    for (int j = 0; j < sd->ionx_ncation[r]; ++j) ints.push_back(sd->ionx_cation[r * sd->ionx_stride + j]);
  dev.o_ix_min = (int)ints.size();
  for (int r = 0; r < nix; ++r) ints.push_back(sd->ionx_mineral ? sd->ionx_mineral[r] : -1);
  dev.o_ix_zflag = (int)ints.size();
  for (int r = 0; r < nix; ++r) {  // eqionx_rxn_Z_flag, reaction_database.F90:2905-2919
    bool zf = false;
    for (int i = 0; i < sd->ionx_ncation[r] && !zf; ++i)
      for (int j = 0; j < sd->ionx_ncation[r]; ++j)
        if (std::fabs(d->pri_Z[sd->ionx_cation[r * sd->ionx_stride + i]] -
                      d->pri_Z[sd->ionx_cation[r * sd->ionx_stride + j]]) > 0.1) {
          zf = true;
          break;
        }
    ints.push_back(zf ? 1 : 0);
  }
  // surface complexation: reactions' complex ranges, types, minerals,
  // stoichiometry flags; the complexes' species CSR
  const int nsx = sd ? sd->nsrfcplx_rxn : 0, nsc = nsx ? sd->nsrfcplx : 0;
  dev.nsrx = nsx;
  dev.nsrc = nsc;
  dev.o_sx_ptr = (int)ints.size();
  for (int r = 0; r <= nsx && nsx; ++r) ints.push_back(sd->srfcplx_rxn_ptr[r]);
  dev.o_sx_type = (int)ints.size();
  for (int r = 0; r < nsx; ++r) ints.push_back(sd->srfcplx_surf_type[r]);
  dev.o_sx_min = (int)ints.size();
  for (int r = 0; r < nsx; ++r) ints.push_back(sd->srfcplx_mineral ? sd->srfcplx_mineral[r] : -1);
  dev.o_sx_flag = (int)ints.size();
  for (int r = 0; r < nsx; ++r) {  // srfcplxrxn_stoich_flag (reaction_database.F90:2801-2803)
    int f = 0;
    for (int k = sd->srfcplx_rxn_ptr[r]; k < sd->srfcplx_rxn_ptr[r + 1]; ++k)
      f = f || sd->srfcplx_free_site_stoich[k] > 1.0;
    ints.push_back(f);
  }
  dev.o_sx_cptr = (int)ints.size();
  {
    int cnt = 0;
    for (int k = 0; k < nsc; ++k) { ints.push_back(cnt); cnt += sd->srfcplx_nspec[k]; }
    if (nsc) ints.push_back(cnt);
  }
  dev.o_sx_spec = (int)ints.size();
  for (int k = 0; k < nsc; ++k)
    for (int p = 0; p < sd->srfcplx_nspec[k]; ++p) ints.push_back(sd->srfcplx_spec[k * sd->srfcplx_stride + p]);
  // staged prefixes of the group kernel: [core] without, [grp] with the
  // per-entry tables (staged when they fit beside a block's cells)
  while (ints.size() % 4) ints.push_back(0);
  dev.int_words_core = (int)ints.size();
  {
    const int base = (int)ints.size();
    dev.o_ent_ij += base;
    dev.o_ent_ptr += base;
    dev.o_ent_sc += base;
    dev.o_ent_mptr += base;
    dev.o_ent_mm += base;
    ints.insert(ints.end(), ent_ints.begin(), ent_ints.end());
  }
  while (ints.size() % 4) ints.push_back(0);  // 16-byte boundary: the group kernel's staged prefix ends here
  dev.int_words_grp = (int)ints.size();
  {
    const int base = (int)ints.size();
    dev.o_spair_ptr += base;
    dev.o_spair_idx += base;
    dev.o_mpair_ptr += base;
    dev.o_mpair_idx += base;
    ints.insert(ints.end(), lane_ints.begin(), lane_ints.end());
  }
  // rate prefactors (read from global memory by the kernels that carry them)
  const PfPrefactorDesc* pfd = d->prefactors;
  bool any_pref = false;
  for (int m = 0; pfd && m < nm; ++m) any_pref = any_pref || pfd->num_prefactors[m] > 0;
  const int MP = PF_MAX_PREFACTORS, MPS = PF_MAX_PREFACTORS * PF_MAX_PREFACTOR_SPECIES;
  dev.o_pf_cnt = (int)ints.size();
  for (int m = 0; m < nm; ++m) ints.push_back(any_pref ? pfd->num_prefactors[m] : 0);
  dev.o_pf_nsp = (int)ints.size();
  for (int k = 0; k < nm * MP; ++k) ints.push_back(any_pref ? pfd->nspec[k] : 0);
  dev.o_pf_id = (int)ints.size();
  for (int k = 0; k < nm * MPS; ++k) ints.push_back(any_pref ? pfd->spec[k] : 0);
  while (ints.size() % 4) ints.push_back(0);
  auto put = [&](const double* src, int count, double dflt) {
    int off = (int)dbls.size();
    for (int k = 0; k < count; ++k) dbls.push_back(src ? src[k] : dflt);
    return off;
  };
  dev.o_sec_nu = (int)dbls.size();
  for (int i = 0; i < ns; ++i)
    for (int s = 0; s < d->sec_nspec[i]; ++s) dbls.push_back(d->sec_stoich[i * d->sec_stride + s]);
  dev.o_sec_logK = put(d->sec_logK, ns, 0.0);
  dev.o_sec_logKcoef = put(d->sec_logKcoef, 5 * ns, 0.0);
  dev.o_pri_Z = put(d->pri_Z, n, 0.0);
  dev.o_pri_a0 = put(d->pri_a0, n, 0.0);
  dev.o_sec_Z = put(d->sec_Z, ns, 0.0);
  dev.o_sec_a0 = put(d->sec_a0, ns, 0.0);
  dev.o_mnrl_nu = (int)dbls.size();
  for (int m = 0; m < nm; ++m)
    for (int s = 0; s < d->mnrl_nspec[m]; ++s) dbls.push_back(d->mnrl_stoich[m * d->mnrl_stride + s]);
  dev.o_mnrl_logK = put(d->mnrl_logK, nm, 0.0);
  dev.o_mnrl_logKcoef = put(d->mnrl_logKcoef, 5 * nm, 0.0);
  dev.o_rate = put(d->mnrl_rate_constant, nm, 0.0);
  dev.o_ea = put(d->mnrl_activation_energy, nm, 0.0);
  dev.o_molar_vol = put(d->mnrl_molar_vol, nm, 0.0);
  dev.o_thresh = put(d->mnrl_affinity_threshold, nm, 0.0);
  dev.o_limiter = put(d->mnrl_rate_limiter, nm, 0.0);
  dev.o_msf = put(d->mnrl_min_scale_factor, nm, 1.0);
  dev.o_temkin = put(d->mnrl_Temkin_const, nm, 1.0);
  dev.o_power = put(d->mnrl_affinity_power, nm, 1.0);
  dev.o_kd_coeff = put(nkd ? sd->kd_coeff : nullptr, nkd, 0.0);
  dev.o_kd_b = put(nkd ? sd->kd_langmuir_b : nullptr, nkd, 0.0);
  dev.o_kd_n = put(nkd ? sd->kd_freundlich_n : nullptr, nkd, 1.0);
  dev.o_ix_k = (int)dbls.size();
  for (int r = 0; r < nix; ++r)
    for (int j = 0; j < sd->ionx_ncation[r]; ++j) dbls.push_back(sd->ionx_k[r * sd->ionx_stride + j]);
  dev.o_ix_cec = put(nix ? sd->ionx_cec : nullptr, nix, 0.0);
  dev.o_sx_dens = put(nsx ? sd->srfcplx_site_density : nullptr, nsx, 0.0);
  dev.o_sx_nu = (int)dbls.size();
  for (int k = 0; k < nsc; ++k)
    for (int p = 0; p < sd->srfcplx_nspec[k]; ++p) dbls.push_back(sd->srfcplx_stoich[k * sd->srfcplx_stride + p]);
  dev.o_sx_nuf = put(nsc ? sd->srfcplx_free_site_stoich : nullptr, nsc, 1.0);
  dev.o_sx_logK = put(nsc ? sd->srfcplx_logK : nullptr, nsc, 0.0);
  dev.o_sx_logKcoef = put(nsc ? sd->srfcplx_logKcoef : nullptr, 5 * nsc, 0.0);
  dev.o_sx_h2o = put(nsc ? sd->srfcplx_h2o_stoich : nullptr, nsc, 0.0);
  while (dbls.size() % 2) dbls.push_back(0.0);
  dev.dbl_words_core = (int)dbls.size();
  dev.o_ent_cf = put(ent_cf.data(), (int)ent_cf.size(), 0.0);
  dev.o_ent_mcf = put(ent_mcf.data(), (int)ent_mcf.size(), 0.0);
  while (dbls.size() % 2) dbls.push_back(0.0);  // 16-byte boundary: end of the group kernel's prefix
  dev.dbl_words_grp = (int)dbls.size();
  dev.o_spair_coef = put(spair_coef.data(), (int)spair_coef.size(), 0.0);
  dev.o_mpair_coef = put(mpair_coef.data(), (int)mpair_coef.size(), 0.0);
  dev.o_pf_rate = put(any_pref ? pfd->rate : nullptr, nm * MP, 0.0);
  dev.o_pf_ea = put(any_pref ? pfd->activation_energy : nullptr, nm * MP, 0.0);
  dev.o_pf_alpha = put(any_pref ? pfd->alpha : nullptr, nm * MPS, 0.0);
  dev.o_pf_beta = put(any_pref ? pfd->beta : nullptr, nm * MPS, 0.0);
  dev.o_pf_atten = put(any_pref ? pfd->atten_coef : nullptr, nm * MPS, 0.0);
  dev.o_sec_h2o = put(d->sec_h2o_stoich, ns, 0.0);
  dev.o_mnrl_h2o = put(d->mnrl_h2o_stoich, nm, 0.0);
  bool any_h2o = false;
  for (int i = 0; d->sec_h2o_stoich && i < ns; ++i) any_h2o = any_h2o || d->sec_h2o_stoich[i] != 0.0;
  for (int m = 0; d->mnrl_h2o_stoich && m < nm; ++m) any_h2o = any_h2o || d->mnrl_h2o_stoich[m] != 0.0;
  for (int k = 0; nsc && sd->srfcplx_h2o_stoich && k < nsc; ++k) any_h2o = any_h2o || sd->srfcplx_h2o_stoich[k] != 0.0;
  while (dbls.size() % 2) dbls.push_back(0.0);
  dev.flags = (d->sec_logKcoef ? NETF_SEC_LOGKCOEF : 0) | (d->mnrl_logKcoef ? NETF_MNRL_LOGKCOEF : 0) |
              (d->mnrl_min_scale_factor ? NETF_MSF : 0) | (d->mnrl_Temkin_const ? NETF_TEMKIN : 0) |
              (d->mnrl_affinity_power ? NETF_POWER : 0) | (any_pref ? NETF_PREFACTOR : 0) |
              (any_h2o ? NETF_H2O : 0) | ((nsc && sd->srfcplx_logKcoef) ? NETF_SX_LOGKCOEF : 0);
  dev.int_words = (int)ints.size();
  dev.dbl_words = (int)dbls.size();
  dev.A = d->debyeA;
  dev.B = d->debyeB;
  dev.Bdot = d->debyeBdot;
  dev.o = d->opts;
  if (!dev.o.isothermal && ((ns > 0 && !d->sec_logKcoef) || (nm > 0 && !d->mnrl_logKcoef)))
    return PF_ERR_INVALID;

  PfNetwork* net = new (std::nothrow) PfNetwork();
  if (!net) return PF_ERR_INVALID;
  const size_t ib = pad16(ints.size() * 4), db = pad16(dbls.size() * 8);
  cudaError_t e = cudaGetDevice(&net->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&net->num_sms, cudaDevAttrMultiProcessorCount, net->device);
  if (e == cudaSuccess) e = cudaMalloc(&net->d_tables, ib + db);
  if (e == cudaSuccess) e = cudaMemcpy(net->d_tables, ints.data(), ints.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy((char*)net->d_tables + ib, dbls.data(), dbls.size() * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&net->d_counters, 8 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost(&net->h_counters, 8 * sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = cudaMalloc(&net->d_ctype, pad16(PF_MAX_NCOMP * sizeof(int32_t)) + PF_MAX_NCOMP * sizeof(PfConstraintReaction));
  if (e == cudaSuccess)
    net->d_creact = reinterpret_cast<PfConstraintReaction*>(reinterpret_cast<char*>(net->d_ctype) +
                                                            pad16(PF_MAX_NCOMP * sizeof(int32_t)));
  if (e != cudaSuccess) {
    pf_network_destroy(net);
    return PF_ERR_CUDA;
  }
  dev.ints = (const int32_t*)net->d_tables;
  dev.dbls = (const double*)((char*)net->d_tables + ib);
  net->dbls_base = dbls;
  net->ints_base = ints;
  net->ib = ib;
  if (group_build_tables(dev, ints.data(), dbls.data(), &net->d_group, &dev.grp) != PF_OK) {
    pf_network_destroy(net);
    return PF_ERR_CUDA;
  }
  net->dev = dev;
  net->launch = default_launch(dev);
  net->launch_lane = net->launch;
  *out = net;
  return PF_OK;
}

// Internal accessors for pfgpu_noalloc.cu (not part of the public header).
int32_t pf_internal_network_view(PfNetwork* net, DevNet* dev, PfLaunchConfig* cfg, int* num_sms,
                                 unsigned long long** counters) {
  if (!net) return PF_ERR_INVALID;
  *dev = net->dev;
  *cfg = net->launch;
  *num_sms = net->num_sms;
  *counters = net->d_counters;
  return PF_OK;
}

int32_t pf_internal_check_rstep(PfNetwork* net, const PfCellState* state, double dt);
int32_t pf_internal_read_step_stats(PfNetwork* net, int64_t ncells, void* stream, PfStepStats* stats);

int32_t pf_network_destroy(PfNetwork* net) {
  if (!net) return PF_ERR_INVALID;
  if (net->d_tables) cudaFree(net->d_tables);
  if (net->d_counters) cudaFree(net->d_counters);
  if (net->h_counters) cudaFreeHost(net->h_counters);
  if (net->d_arena) cudaFree(net->d_arena);
  for (int c = 0; c < 16; ++c) {
    if (net->ev_in[c]) cudaEventDestroy(net->ev_in[c]);
    if (net->ev_comp[c]) cudaEventDestroy(net->ev_comp[c]);
  }
  if (net->ev_start) cudaEventDestroy(net->ev_start);
  if (net->s_in) cudaStreamDestroy(net->s_in);
  if (net->s_comp) cudaStreamDestroy(net->s_comp);
  if (net->s_out) cudaStreamDestroy(net->s_out);
  if (net->d_ccounters) cudaFree(net->d_ccounters);
  if (net->h_ccounters) cudaFreeHost(net->h_ccounters);
  if (net->h_order) cudaFreeHost(net->h_order);
  if (net->d_ctype) cudaFree(net->d_ctype);
  if (net->d_scratch) cudaFree(net->d_scratch);
  if (net->d_girt) cudaFree(net->d_girt);
  if (net->d_group) cudaFree(net->d_group);
  delete net;
  return PF_OK;
}

int32_t pf_network_set_options(PfNetwork* net, const PfOptions* opts) {
  if (!net || !opts) return PF_ERR_INVALID;
  if (opts->maximum_reaction_iterations < 1 || opts->maximum_reaction_cuts < 0) return PF_ERR_INVALID;
  if (opts->act_coef_update_frequency < 0 || opts->act_coef_update_frequency > 2) return PF_ERR_INVALID;
  if (!opts->isothermal && ((net->dev.ns > 0 && !(net->dev.flags & NETF_SEC_LOGKCOEF)) ||
                            (net->dev.nm > 0 && !(net->dev.flags & NETF_MNRL_LOGKCOEF))))
    return PF_ERR_INVALID;
  net->dev.o = *opts;
  // the launch configuration was chosen for the old options: a group of
  // lanes per cell that the new ones rule out (e.g. the linear formulation)
  // goes back to one lane per cell, or to the default for the new options
  const PfLaunchConfig& c = net->launch;
  const bool ok = c.lanes_per_cell > 1 ? group_supported(net->dev, c.lanes_per_cell) : lane_supported(net->dev);
  if (!ok) {
    const bool lane_cfg = net->launch_lane.lanes_per_cell <= 1 && lane_supported(net->dev) &&
                          batched_smem_bytes(net->dev, net->launch_lane) <= 227u * 1024u;
    net->launch = lane_cfg ? net->launch_lane : default_launch(net->dev);
  }
  return PF_OK;
}

static int ensure_scratch_doubles(PfNetwork* net, size_t need);
static int ensure_scratch(PfNetwork* net, int64_t ncells) {
  return ensure_scratch_doubles(net, batched_scratch_doubles(net->dev, ncells));
}
static int ensure_scratch_doubles(PfNetwork* net, size_t need) {
  if (need <= net->scratch_cap) return PF_OK;
  if (net->d_scratch) cudaFree(net->d_scratch);
  net->d_scratch = nullptr;
  net->scratch_cap = 0;
  if (cudaMalloc(&net->d_scratch, need * sizeof(double)) != cudaSuccess) return PF_ERR_CUDA;
  net->scratch_cap = need;
  return PF_OK;
}

int32_t pf_network_reserve(PfNetwork* net, int64_t ncells) {
  if (!net || ncells < 0) return PF_ERR_INVALID;
  return ensure_scratch(net, ncells);
}

int32_t pf_network_set_launch(PfNetwork* net, const PfLaunchConfig* cfg) {
  if (!net || !cfg) return PF_ERR_INVALID;
  if (cfg->threads_per_block < 32 || cfg->threads_per_block > 256 || cfg->threads_per_block % 32 ||
      cfg->blocks_per_sm < 1 || cfg->blocks_per_sm > 16)
    return PF_ERR_INVALID;
  const int G = cfg->lanes_per_cell;
  if (G != 0 && G != 1 && G != 2 && G != 4 && G != 8) return PF_ERR_INVALID;
  if (G > 1 && !group_supported(net->dev, G)) return PF_ERR_UNSUPPORTED;
  if (G <= 1 && !lane_supported(net->dev)) return PF_ERR_UNSUPPORTED;
  if (batched_smem_bytes(net->dev, *cfg) > 227u * 1024u) return PF_ERR_TOO_LARGE;
  net->launch = *cfg;
  if (G <= 1) net->launch_lane = *cfg;
  return PF_OK;
}

int32_t pf_network_get_launch(const PfNetwork* net, PfLaunchConfig* cfg) {
  if (!net || !cfg) return PF_ERR_INVALID;
  *cfg = net->launch;
  return PF_OK;
}

static int check_rstep(PfNetwork* net, const PfCellState* state, double dt, int32_t kernel) {
  int rc = validate_state(net, state);
  if (rc) return rc;
  if (!(dt > 0.0) && !state->dt_cell) return PF_ERR_INVALID;
  if (kernel != PF_KERNEL_PLAIN && kernel != PF_KERNEL_BATCHED) return PF_ERR_INVALID;
  // activity coefficients by the NEWTON algorithm at every Newton iteration:
  // the plain kernel (batched_supported refuses the combination)
  if (kernel == PF_KERNEL_BATCHED && !batched_supported(net->dev)) return PF_ERR_UNSUPPORTED;
  return PF_OK;
}

int32_t pf_internal_check_rstep(PfNetwork* net, const PfCellState* state, double dt) {
  return check_rstep(net, state, dt, PF_KERNEL_BATCHED);
}

// zero counters[0..8) and launch the step on stream s ([0] is the work queue;
// scratch: the batched kernel's per-cell set-up values for these cells)
static int enqueue_rstep(PfNetwork* net, const PfCellState* state, double dt, int32_t kernel,
                         unsigned long long* counters, double* scratch, cudaStream_t s) {
  if (cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess) return PF_ERR_CUDA;
  int lr;
  if (kernel == PF_KERNEL_PLAIN)
    lr = launch_rstep_plain(net->dev, *state, dt, counters + 1, s);
  else
    lr = launch_rstep_batched(net->dev, *state, dt, net->launch, net->num_sms, scratch, counters, counters + 1,
                              s);
  return lr != 0 ? PF_ERR_CUDA : PF_OK;
}

// Synchronises s, copies the counters of the last step into the pinned mirror
// and fills stats: PF_ERR_TIMEOUT when a launch-level wait ran out,
// PF_CELL_FAILURES when cells failed, else PF_OK.
static int read_step_stats(PfNetwork* net, int64_t ncells, cudaStream_t s, PfStepStats* stats) {
  cudaError_t e = cudaMemcpyAsync(net->h_counters, net->d_counters, 8 * sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return PF_ERR_CUDA;
  const unsigned long long* h = net->h_counters;
  stats->cells = ncells;
  stats->newton_iterations = (int64_t)h[1];
  stats->failed_cells = (int64_t)h[2];
  stats->max_newton_iterations = (int32_t)h[4];
  stats->max_substeps = (int32_t)h[5];
  if (h[3]) return PF_ERR_TIMEOUT;
  return stats->failed_cells ? PF_CELL_FAILURES : PF_OK;
}

int32_t pf_rstep(PfNetwork* net, const PfCellState* state, double dt, int32_t kernel, void* stream,
                 PfStepStats* stats) {
  int rc = check_rstep(net, state, dt, kernel);
  if (rc) return rc;
  if (state->ncells == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return PF_OK;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (kernel == PF_KERNEL_BATCHED) {
    rc = ensure_scratch(net, state->ncells);
    if (rc) return rc;
  }
  rc = enqueue_rstep(net, state, dt, kernel, net->d_counters, net->d_scratch, s);
  if (rc) return rc;
  if (!stats) return PF_OK;
  return read_step_stats(net, state->ncells, s, stats);
}

int32_t pf_internal_read_step_stats(PfNetwork* net, int64_t ncells, void* stream, PfStepStats* stats) {
  return read_step_stats(net, ncells, (cudaStream_t)stream, stats);
}

int32_t pf_rstep_multi(PfNetwork* const* nets, const PfCellState* states, int32_t nnets, double dt, void* stream,
                       PfStepStats* stats) {
  if (!nets || !states || nnets < 1 || nnets > PF_MULTI_MAX_NETS) return PF_ERR_INVALID;
  MultiNetLaunch L[PF_MULTI_MAX_NETS];
  int nl = 0, device = -1, sms = 0;
  for (int k = 0; k < nnets; ++k) {
    PfNetwork* net = nets[k];
    if (!net) return PF_ERR_INVALID;
    int rc = check_rstep(net, &states[k], dt, PF_KERNEL_BATCHED);
    if (rc) return rc;
    if (device < 0) {
      device = net->device;
      sms = net->num_sms;
    } else if (net->device != device) {
      return PF_ERR_INVALID;
    }
    const int G = multi_lanes_for(net->dev, net->launch.lanes_per_cell);
    if (!G) return PF_ERR_UNSUPPORTED;
    if (states[k].ncells == 0) continue;
    rc = ensure_scratch(net, states[k].ncells);
    if (rc) return rc;
    L[nl].net = net->dev;
    L[nl].st = states[k];
    L[nl].scratch = net->d_scratch;
    L[nl].queue = net->d_counters;
    L[nl].counters = net->d_counters + 1;
    L[nl].lanes_per_cell = G;
    ++nl;
  }
  cudaStream_t s = (cudaStream_t)stream;
  for (int k = 0; k < nnets; ++k)
    if (cudaMemsetAsync(nets[k]->d_counters, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess)
      return PF_ERR_CUDA;
  if (nl > 0) {
    // one block of 256 threads per SM (the group kernels' registers allow
    // one); a network whose workspace does not fit 256 threads' cells runs
    // on fewer of the block's warps
    if (launch_rstep_multi(L, nl, dt, 256, 1, sms, s) != 0) return PF_ERR_CUDA;
  }
  if (!stats) return PF_OK;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < nnets && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(nets[k]->h_counters, nets[k]->d_counters, 8 * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return PF_ERR_CUDA;
  bool timeout = false, failures = false;
  for (int k = 0; k < nnets; ++k) {
    const unsigned long long* h = nets[k]->h_counters;
    stats[k].cells = states[k].ncells;
    stats[k].newton_iterations = (int64_t)h[1];
    stats[k].failed_cells = (int64_t)h[2];
    stats[k].max_newton_iterations = (int32_t)h[4];
    stats[k].max_substeps = (int32_t)h[5];
    timeout = timeout || h[3];
    failures = failures || h[2];
  }
  if (timeout) return PF_ERR_TIMEOUT;
  return failures ? PF_CELL_FAILURES : PF_OK;
}

int32_t pf_update_auxvars(PfNetwork* net, const PfCellState* state, int32_t update_activity_coefs,
                          void* stream) {
  int rc = validate_state(net, state);
  if (rc) return rc;
  if (update_activity_coefs && (net->dev.ns > 0) && !state->sec_act_coef) return PF_ERR_INVALID;
  return launch_update_auxvars(net->dev, *state, update_activity_coefs, (cudaStream_t)stream) ? PF_ERR_CUDA
                                                                                              : PF_OK;
}

int32_t pf_update_activity_coefs(PfNetwork* net, const PfCellState* state, void* stream) {
  int rc = validate_state(net, state);
  if (rc) return rc;
  return launch_update_activity_coefs(net->dev, *state, (cudaStream_t)stream) ? PF_ERR_CUDA : PF_OK;
}

int32_t pf_network_shift_parameters(PfNetwork* net, const double* dlogK_sec, const double* dlogK_mnrl,
                                    const double* dlnk) {
  if (!net) return PF_ERR_INVALID;
  const DevNet& d = net->dev;
  std::vector<double> v = net->dbls_base;
  const bool csec = d.flags & NETF_SEC_LOGKCOEF, cmin = d.flags & NETF_MNRL_LOGKCOEF;
  for (int i = 0; dlogK_sec && i < d.ns; ++i) {
    v[d.o_sec_logK + i] += dlogK_sec[i];
    if (csec) v[d.o_sec_logKcoef + 5 * i + 1] += dlogK_sec[i];
  }
  for (int m = 0; dlogK_mnrl && m < d.nm; ++m) {
    v[d.o_mnrl_logK + m] += dlogK_mnrl[m];
    if (cmin) v[d.o_mnrl_logKcoef + 5 * m + 1] += dlogK_mnrl[m];
  }
  for (int m = 0; dlnk && m < d.nm; ++m) v[d.o_rate + m] = v[d.o_rate + m] * std::exp(dlnk[m]);
  if (cudaMemcpy((char*)net->d_tables + net->ib, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return PF_ERR_CUDA;
  return PF_OK;
}

int32_t pf_adjoint(PfNetwork* net, const PfCellState* state, double dt, const PfAdjointArgs* a, void* stream) {
  int rc = validate_state(net, state);
  if (rc) return rc;
  if (!a || !(dt > 0.0 || state->dt_cell)) return PF_ERR_INVALID;
  const DevNet& d = net->dev;
  if (!batched_supported(d)) return PF_ERR_UNSUPPORTED;
  if (d.o.act_coef_update_frequency == PF_ACT_COEF_NEWTON_ITER) return PF_ERR_UNSUPPORTED;
  if (has_sorption(d)) return PF_ERR_UNSUPPORTED;  // no adjoint of the sorption terms
  if (d.flags & NETF_PREFACTOR) return PF_ERR_UNSUPPORTED;  // nor of the rate prefactors
  if (!a->dL_dtotal0 || (d.nm > 0 && (!a->dL_dlnarea || !a->dL_dlogK_mnrl || !a->dL_dlnk)) ||
      (d.ns > 0 && !a->dL_dlogK_sec) || (!a->weight && !a->dL_dtotal) || (a->weight && !a->target))
    return PF_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (state->ncells == 0) return PF_OK;
  // the group kernel carries the adjoint with a substep store after the
  // setup scratch; otherwise one lane per cell with the last such config
  const bool grp = net->launch.lanes_per_cell > 1 &&
                   group_smem_bytes(d, net->launch, true) <= 227u * 1024u;
  if (!grp && !lane_supported(d)) return PF_ERR_UNSUPPORTED;
  const size_t base = batched_scratch_doubles(d, state->ncells);
  rc = ensure_scratch_doubles(net, base + (grp ? group_adj_store_doubles(d, state->ncells) : 0));
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  if (d.ns) e = cudaMemsetAsync(a->dL_dlogK_sec, 0, d.ns * sizeof(double), s);
  if (e == cudaSuccess && d.nm) e = cudaMemsetAsync(a->dL_dlogK_mnrl, 0, d.nm * sizeof(double), s);
  if (e == cudaSuccess && d.nm) e = cudaMemsetAsync(a->dL_dlnk, 0, d.nm * sizeof(double), s);
  if (e == cudaSuccess && a->loss) e = cudaMemsetAsync(a->loss, 0, sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->d_counters, 0, 8 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return PF_ERR_CUDA;
  if (launch_rstep_batched(d, *state, dt, grp ? net->launch : net->launch_lane, net->num_sms, net->d_scratch,
                           net->d_counters, net->d_counters + 1, s, a, grp ? net->d_scratch + base : nullptr) != 0)
    return PF_ERR_CUDA;
  return PF_OK;
}

int32_t pf_girt_assemble(PfNetwork* net, const PfCellState* state, const PfGirtArgs* a, void* stream) {
  int rc = validate_state(net, state);
  if (rc) return rc;
  if (!a || a->nx < 1 || a->ny < 1 || a->nz < 1 || !(a->dt > 0.0) || !a->total_k || !a->rowptr ||
      !a->colidx || !a->residual || !a->values || !(a->dx > 0) || !(a->dy > 0) || !(a->dz > 0))
    return PF_ERR_INVALID;
  if ((int64_t)a->nx * a->ny * a->nz != state->ncells) return PF_ERR_INVALID;
  if (has_sorption(net->dev) && !a->total_sorb_k) return PF_ERR_INVALID;
  if ((a->nx > 1 && !a->qx) || (a->ny > 1 && !a->qy) || (a->nz > 1 && !a->qz)) return PF_ERR_INVALID;
  if (!state->sec_molal && net->dev.ns) return PF_ERR_INVALID;
  // the per-cell K cache: not with the water activity on (ln a_H2O follows
  // the molalities, so K a_H2O^nu changes from one Newton iteration to the next)
  if (a->k_cache && water_on(net->dev)) return PF_ERR_UNSUPPORTED;
  if (!net->d_girt) {
    rc = girt_build_tables(net->dev, net->ints_base.data(), net->dbls_base.data(), &net->d_girt, &net->girt);
    if (rc) return rc;
  }
  // the packed sum of d total/d m in global memory ([entry][cell], the
  // network's grow-only scratch): the shared-memory scratch per cell would
  // cap the resident warps
  const size_t nsym = (size_t)net->dev.n * (net->dev.n + 1) / 2;
  rc = ensure_scratch_doubles(net, nsym * (size_t)state->ncells);
  if (rc) return rc;
  if (girt_smem_bytes(net->dev, net->girt, (net->dev.flags & NETF_PREFACTOR) || a->numerical_derivatives, false,
                      nullptr, nullptr) > 227u * 1024u)
    return PF_ERR_TOO_LARGE;
  return launch_girt_assemble(net->dev, net->girt, *state, *a, net->num_sms, (cudaStream_t)stream,
                              net->d_scratch);
}

int32_t pf_equilibrate_constraint_ex(PfNetwork* net, const PfCellState* state, const int32_t* ctype,
                                     const PfConstraintReaction* creact, const double* cconc, int32_t use_prev,
                                     int32_t* iterations, void* stream) {
  int rc = validate_state(net, state);
  if (rc) return rc;
  if (!ctype || !cconc || (net->dev.ns > 0 && !state->sec_act_coef)) return PF_ERR_INVALID;
  const int n = net->dev.n;
  int ncb = 0;
  bool reactions = false;
  for (int j = 0; j < n; ++j) {
    if (ctype[j] < PF_CONSTRAINT_TOTAL || ctype[j] > PF_CONSTRAINT_GAS) return PF_ERR_INVALID;
    ncb += ctype[j] == PF_CONSTRAINT_CHARGE_BAL;
    if (ctype[j] == PF_CONSTRAINT_MINERAL || ctype[j] == PF_CONSTRAINT_GAS) {
      if (!creact) return PF_ERR_INVALID;
      const PfConstraintReaction& R = creact[j];
      if (R.nspec < 1 || R.nspec > n) return PF_ERR_INVALID;
      for (int p = 0; p < R.nspec; ++p)
        if (R.spec[p] < 0 || R.spec[p] >= n) return PF_ERR_INVALID;
      reactions = true;
    }
  }
  if (ncb > 1) return PF_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(net->d_ctype, ctype, n * sizeof(int32_t), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return PF_ERR_CUDA;
  if (reactions &&
      cudaMemcpyAsync(net->d_creact, creact, n * sizeof(PfConstraintReaction), cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    return PF_ERR_CUDA;
  return pf_equilibrate_constraint_impl(&net->dev, state, net->d_ctype, net->d_creact, cconc, use_prev,
                                        iterations, 10000, stream);
}

int32_t pf_equilibrate_constraint(PfNetwork* net, const PfCellState* state, const int32_t* ctype,
                                  const double* cconc, int32_t use_prev, int32_t* iterations, void* stream) {
  if (net && ctype)
    for (int j = 0; j < net->dev.n; ++j)
      if (ctype[j] == PF_CONSTRAINT_MINERAL || ctype[j] == PF_CONSTRAINT_GAS) return PF_ERR_INVALID;
  return pf_equilibrate_constraint_ex(net, state, ctype, nullptr, cconc, use_prev, iterations, stream);
}

// The host-buffer step's chunk plan: cells [0, N) in chunks starting on
// whole 64-cell groups (aligned slices); up to 2^18 cells one chunk, else
// three: N/10 cells, the rest, N/10 cells.  Nothing hides the first chunk's
// copy in or the last one's copy out, and each launch costs about half a
// millisecond of ramp-up and tail (the persistent kernel's last cells); at
// the bench's chemistry a chunk's copies take about an eighth of its
// compute, so the first chunk's compute covers the middle one's copy in and
// the last one's covers its copy out.  Measured at 10^6 cells,
// device-resident: one launch 43.4 ms, these three 44.7 ms, four equal
// chunks 45.4 ms, six (N/32 at either end) 47.9 ms.  Writes the K + 1
// boundaries (cstart[0] = 0, cstart[K] = N) and returns K.
static int host_chunk_plan(int64_t N, int64_t cstart[4]) {
  const int64_t target = 262144;
  auto r64 = [](int64_t x) { return (x + 63) / 64 * 64; };
  int K = 1;
  cstart[0] = 0;
  if (N > target) {
    const int64_t edge = r64((N + 9) / 10);
    cstart[K++] = edge;
    cstart[K++] = (N - edge) / 64 * 64;  // the last chunk takes the ragged end
  }
  cstart[K] = N;
  return K;
}

// The chunk plan for tests of the host logic (no device work).
int32_t pf_internal_host_chunk_plan(int64_t ncells, int64_t* starts) {
  if (ncells < 0 || !starts) return -1;
  return host_chunk_plan(ncells, starts);
}

// Host-buffer step, pipelined over chunks of cells: chunk c's inputs go in on
// one stream while earlier chunks compute on a second and finished chunks'
// results come back on a third.  Each chunk has its own counters and set-up
// scratch.  (Chunks computing side by side on several streams were slower:
// the persistent kernels then compete for the SMs.)  On the
// device each chunk is its own compact SoA block (every field's rows for the
// chunk gathered from the host's strided rows by one 2-D copy); a chunk's
// work-queue order is the caller's order restricted to the chunk, renumbered
// locally.
int32_t pf_rstep_host(PfNetwork* net, const PfCellState* h, double dt, int32_t kernel, PfStepStats* stats) {
  int rc = check_rstep(net, h, dt, kernel);
  if (rc) return rc;
  const int64_t N = h->ncells;
  if (N == 0) return pf_rstep(net, h, dt, kernel, nullptr, stats);
  const int n = net->dev.n, ns = net->dev.ns, nm = net->dev.nm, nx = net->dev.nionx;
  struct Field {
    void* host;
    int rows;
    int esize;
    bool in, out;
  };
  const int d8 = sizeof(double), i4 = sizeof(int32_t);
  Field f[] = {
      {h->total, n, d8, true, true},           {h->pri_molal, n, d8, true, true},
      {h->pri_act_coef, n, d8, true, true},    {h->sec_act_coef, ns, d8, true, true},
      {h->sec_molal, ns, d8, true, true},      {h->mnrl_volfrac, nm, d8, true, true},
      {h->mnrl_area, nm, d8, true, false},     {h->mnrl_rate, nm, d8, false, true},
      {(void*)h->porosity, 1, d8, true, false}, {(void*)h->saturation, 1, d8, true, false},
      {(void*)h->den_kg, 1, d8, true, false},  {(void*)h->volume, 1, d8, true, false},
      {(void*)h->temperature, 1, d8, true, false}, {(void*)h->dt_cell, 1, d8, true, false},
      {h->status, 1, i4, false, true},         {h->newton_its, 1, i4, false, true},
      {h->num_substeps, 1, i4, false, true},
      {(void*)h->cell_order, 1, (int)sizeof(int64_t), false, false},  // remapped per chunk below
      {h->total_sorb, n, d8, true, true},      {h->ionx_ref_sorbed, nx, d8, true, true},
      {h->ln_act_h2o, 1, d8, true, true},
      {h->srfcplx_free_site, net->dev.nsrx, d8, true, true}, {h->srfcplx_conc, net->dev.nsrc, d8, false, true},
  };
  const int nf = sizeof(f) / sizeof(f[0]);
  int64_t cstart[4];
  const int K = host_chunk_plan(N, cstart);
  auto cells_of = [&](int c) { return cstart[c + 1] - cstart[c]; };
  auto chunk_bytes = [&](int64_t nc) {
    size_t b = 0;
    for (int k = 0; k < nf; ++k)
      if (f[k].host) b += pad16((size_t)f[k].rows * nc * f[k].esize);
    return b;
  };
  size_t arena_off[4];
  arena_off[0] = 0;
  for (int c = 0; c < K; ++c) arena_off[c + 1] = arena_off[c] + chunk_bytes(cells_of(c));
  const size_t need = arena_off[K];
  if (need > net->arena_bytes) {
    if (net->d_arena) cudaFree(net->d_arena);
    net->d_arena = nullptr;
    net->arena_bytes = 0;
    if (cudaMalloc(&net->d_arena, need) != cudaSuccess) return PF_ERR_CUDA;
    net->arena_bytes = need;
  }
  cudaError_t e = cudaSuccess;
  if (!net->s_in) {
    for (cudaStream_t* st : {&net->s_in, &net->s_comp, &net->s_out})
      if (e == cudaSuccess) e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
    for (int c = 0; c < 16 && e == cudaSuccess; ++c) {
      e = cudaEventCreateWithFlags(&net->ev_in[c], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&net->ev_comp[c], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&net->ev_start, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&net->d_ccounters, 16 * 8 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&net->h_ccounters, 16 * 8 * sizeof(unsigned long long));
    if (e != cudaSuccess) return PF_ERR_CUDA;
  }
  if (kernel == PF_KERNEL_BATCHED) {
    rc = ensure_scratch(net, N);
    if (rc) return rc;
  }
  // the step's device buffers may still be in use by work on the legacy stream
  e = cudaEventRecord(net->ev_start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(net->s_in, net->ev_start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(net->s_comp, net->ev_start, 0);
  if (e != cudaSuccess) return PF_ERR_CUDA;
  // chunk c's block of field k (nullptr for a field the caller did not pass)
  auto dev_field = [&](int c, int k) -> char* {
    if (!f[k].host) return nullptr;
    size_t off = arena_off[c];
    for (int q = 0; q < k; ++q)
      if (f[q].host) off += pad16((size_t)f[q].rows * cells_of(c) * f[q].esize);
    return (char*)net->d_arena + off;
  };
  // an error after copies were enqueued: let them finish before returning,
  // they read and write the caller's buffers
  auto fail = [&](int code) {
    cudaStreamSynchronize(net->s_in);
    cudaStreamSynchronize(net->s_comp);
    cudaStreamSynchronize(net->s_out);
    return code;
  };
  // 2-D copy of field k for chunk c: rows of nc elements, host pitch N, device pitch nc
  auto copy = [&](int c, int k, bool to_dev, cudaStream_t st) {
    const int64_t nc = cells_of(c);
    const size_t es = f[k].esize, w = (size_t)nc * es;
    char* hp = (char*)f[k].host + (size_t)cstart[c] * es;
    char* dp = dev_field(c, k);
    return to_dev ? cudaMemcpy2DAsync(dp, w, hp, (size_t)N * es, w, f[k].rows, cudaMemcpyHostToDevice, st)
                  : cudaMemcpy2DAsync(hp, (size_t)N * es, dp, w, w, f[k].rows, cudaMemcpyDeviceToHost, st);
  };
  const int kord = 17;  // the order's slot in f[]
  auto copy_in = [&](int c) {
    for (int k = 0; k < nf && e == cudaSuccess; ++k)
      if (f[k].host && f[k].in && f[k].rows > 0) e = copy(c, k, true, net->s_in);
  };
  // the chunk's local order to the device, on the input stream (a copy on
  // another stream can still queue behind the inputs on the same copy engine)
  auto copy_order = [&](int c) {
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dev_field(c, kord), net->h_order + cstart[c], (size_t)cells_of(c) * sizeof(int64_t),
                          cudaMemcpyHostToDevice, net->s_in);
  };
  // chunk-local orders.  Chunk 0 (cells [0, n0)) gets its order in a first
  // pass while its inputs are in flight, and the copy of that order follows
  // them, ahead of the other chunks' inputs: chunk 0's compute waits for it.
  // Its local order is the order's entries below n0 in sequence, written
  // branch-free (a slot past the end takes the writes once chunk 0 is
  // complete).  The other chunks' orders, and the check that the order is a
  // permutation (a bitmap of the cells seen), come after chunk 0's compute is
  // enqueued, while it runs, and before any result is copied back, so that a
  // refused order leaves the caller's buffers untouched.
  const int64_t n0 = cells_of(0);
  copy_in(0);
  if (e != cudaSuccess) return fail(PF_ERR_CUDA);
  // h_order: the chunk-local orders, the slot past them, then the bitmap
  const size_t order_words = (size_t)N + 1 + (size_t)(N + 63) / 64;
  if (h->cell_order) {
    if (net->h_order_cap < order_words) {
      if (net->h_order) cudaFreeHost(net->h_order);
      net->h_order = nullptr;
      net->h_order_cap = 0;
      if (cudaMallocHost(&net->h_order, order_words * sizeof(int64_t)) != cudaSuccess) return fail(PF_ERR_CUDA);
      net->h_order_cap = order_words;
    }
    int64_t* ho = net->h_order;
    int64_t p = 0;
    for (int64_t i = 0; i < N; ++i) {
      const int64_t o = h->cell_order[i];
      if (o < 0 || o >= N) return fail(PF_ERR_INVALID);
      ho[p < n0 ? p : N] = o;
      p += o < n0;
    }
    if (p != n0) return fail(PF_ERR_INVALID);  // not a permutation
    copy_order(0);
  }
  if (e == cudaSuccess) e = cudaEventRecord(net->ev_in[0], net->s_in);
  for (int c = 1; c < K && e == cudaSuccess; ++c) {
    copy_in(c);
    // with an order, chunk c's inputs are complete once its order is copied
    if (e == cudaSuccess && !h->cell_order) e = cudaEventRecord(net->ev_in[c], net->s_in);
  }
  if (e != cudaSuccess) return fail(PF_ERR_CUDA);
  // the rest of the chunks' orders (entries in range: checked above) and
  // the permutation check
  auto remap_rest = [&]() {
    uint64_t* seen = (uint64_t*)(net->h_order + N + 1);
    std::memset(seen, 0, (size_t)(N + 63) / 64 * sizeof(uint64_t));
    int64_t pos[4];
    for (int c = 1; c < K; ++c) pos[c] = cstart[c];
    for (int64_t i = 0; i < N; ++i) {
      const int64_t o = h->cell_order[i];
      const uint64_t bit = 1ull << (o & 63);
      if (seen[o >> 6] & bit) return false;  // a cell twice
      seen[o >> 6] |= bit;
      if (o < n0) continue;  // chunk 0's, placed in the first pass
      int c = 1;
      while (o >= cstart[c + 1]) ++c;  // o < N = cstart[K]
      if (pos[c] >= cstart[c + 1]) return false;
      net->h_order[pos[c]++] = o - cstart[c];
    }
    return true;
  };
  for (int c = 0; c < K && e == cudaSuccess; ++c) {
    const int64_t nc = cells_of(c);
    PfCellState d = *h;
    d.ncells = nc;
    double** dfl[] = {&d.total, &d.pri_molal, &d.pri_act_coef, &d.sec_act_coef, &d.sec_molal, &d.mnrl_volfrac,
                      &d.mnrl_area, &d.mnrl_rate};
    for (int k = 0; k < 8; ++k) *dfl[k] = (double*)dev_field(c, k);
    const double** cfl[] = {&d.porosity, &d.saturation, &d.den_kg, &d.volume, &d.temperature, &d.dt_cell};
    for (int k = 0; k < 6; ++k) *cfl[k] = (const double*)dev_field(c, 8 + k);
    d.status = (int32_t*)dev_field(c, 14);
    d.newton_its = (int32_t*)dev_field(c, 15);
    d.num_substeps = (int32_t*)dev_field(c, 16);
    d.cell_order = (const int64_t*)dev_field(c, kord);
    d.total_sorb = (double*)dev_field(c, 18);
    d.ionx_ref_sorbed = (double*)dev_field(c, 19);
    d.ln_act_h2o = (double*)dev_field(c, 20);
    d.srfcplx_free_site = (double*)dev_field(c, 21);
    d.srfcplx_conc = (double*)dev_field(c, 22);
    cudaStream_t sc = net->s_comp;
    e = cudaStreamWaitEvent(sc, net->ev_in[c], 0);
    if (e != cudaSuccess) break;
    rc = enqueue_rstep(net, &d, dt, kernel, net->d_ccounters + 8 * c,
                       net->d_scratch ? net->d_scratch + batched_scratch_doubles(net->dev, cstart[c]) : nullptr,
                       sc);
    if (rc) return fail(rc);
    if (c == 0 && h->cell_order) {
      if (!remap_rest()) return fail(PF_ERR_INVALID);
      for (int q = 1; q < K && e == cudaSuccess; ++q) {
        copy_order(q);
        if (e == cudaSuccess) e = cudaEventRecord(net->ev_in[q], net->s_in);
      }
      if (e != cudaSuccess) break;
    }
    e = cudaEventRecord(net->ev_comp[c], sc);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(net->s_out, net->ev_comp[c], 0);
    for (int k = 0; k < nf && e == cudaSuccess; ++k)
      if (f[k].host && f[k].out && f[k].rows > 0) e = copy(c, k, false, net->s_out);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(net->h_ccounters, net->d_ccounters, (size_t)K * 8 * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, net->s_out);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->s_out);
  if (e != cudaSuccess) return fail(PF_ERR_CUDA);
  PfStepStats st{};
  st.cells = N;
  bool timeout = false;
  for (int c = 0; c < K; ++c) {
    const unsigned long long* q = net->h_ccounters + 8 * c;
    st.newton_iterations += (int64_t)q[1];
    st.failed_cells += (int64_t)q[2];
    timeout = timeout || q[3];
    st.max_newton_iterations = std::max(st.max_newton_iterations, (int32_t)q[4]);
    st.max_substeps = std::max(st.max_substeps, (int32_t)q[5]);
  }
  if (stats) *stats = st;
  if (timeout) return PF_ERR_TIMEOUT;
  return st.failed_cells ? PF_CELL_FAILURES : PF_OK;
}

}  // extern "C"
