/*
 * pfgpu.h -- C ABI of the GB300 (sm_103a) per-cell geochemistry engine.
 *
 * The engine replaces PFLOTRAN's per-cell reaction loops:
 *   - the operator-split cell loop that calls RStep/RReact once per cell
 *     (src/pflotran/pmc_subsurface_osrt.F90:346-378,
 *      src/pflotran/reaction.F90:3564-4055), and
 *   - the per-cell accumulation/reaction blocks and 7-point flux blocks that
 *     RTResidual/RTJacobian assemble in global-implicit mode
 *     (src/pflotran/reactive_transport.F90:1964-3349).
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, int32 status codes.  No library
 *     ever aborts or prints; every entry point returns a PfStatus.
 *   - Species/component ids are 0-based (Fortran ids minus one).
 *   - Per-cell arrays are structure-of-arrays, component-major:
 *       value(k, cell) = array[k * ncells + cell]
 *     so that a warp reading component k of 32 consecutive cells issues one
 *     coalesced 256-byte transaction.  The Fortran shim packs the AoS
 *     rt_auxvar/global_auxvar/material_auxvar types into this layout.
 *   - Device entry points take device pointers and a cudaStream_t passed as
 *     void*; host entry points (suffix _host) take host pointers and do the
 *     copies themselves.
 *   - All arithmetic is IEEE FP64.
 */
#ifndef PFGPU_H_
#define PFGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum PfStatus {
  PF_OK = 0,
  PF_CELL_FAILURES = 1,      /* call succeeded; some cells report status != 0 */
  PF_ERR_INVALID = -1,       /* bad argument (null pointer, size, id range)   */
  PF_ERR_UNSUPPORTED = -2,   /* network feature this engine does not handle  */
  PF_ERR_CUDA = -3,          /* a CUDA runtime call failed                    */
  PF_ERR_TOO_LARGE = -4,     /* ncomp/nsec/nmnrl above the compiled maxima     */
  PF_ERR_TIMEOUT = -5        /* a bounded device wait ran out                  */
} PfStatus;

/* per-cell status codes written to PfCellState.status */
enum {
  PF_CELL_OK = 0,
  PF_CELL_TOO_MANY_CUTS = 1, /* RStep: num_cuts > maximum_reaction_cuts      */
  PF_CELL_NAN = 2,           /* non-finite residual or activity coefficient  */
  PF_CELL_NOT_RUN = -1       /* pf_rstep_noalloc: the launch ended before it
                                reached the cell (a launch-level wait ran out) */
};

/* reaction%act_coef_update_frequency, src/pflotran/reaction_aux.F90:392 */
enum { PF_ACT_COEF_OFF = 0, PF_ACT_COEF_TIMESTEP = 1, PF_ACT_COEF_NEWTON_ITER = 2 };
/* reaction%act_coef_update_algorithm, src/pflotran/reaction_aux.F90:393 */
enum { PF_ACT_COEF_ALGO_LAG = 0, PF_ACT_COEF_ALGO_NEWTON = 1 };

/* Kernel forms for pf_rstep. */
enum {
  PF_KERNEL_PLAIN = 0,   /* one thread per cell, direct form, no queue       */
  PF_KERNEL_BATCHED = 1  /* persistent, lane-refilling work queue, ncomp-
                            specialised, tables staged in shared memory      */
};

/* Compiled maxima (per network). */
#define PF_MAX_NCOMP 24
#define PF_MAX_NSEC 96
#define PF_MAX_NMNRL 16
#define PF_MAX_SPEC_PER_RXN 24
#define PF_MAX_NKD 8            /* isotherm (K_D) reactions            */
#define PF_MAX_NIONX 4          /* ion-exchange reactions              */
#define PF_MAX_IONX_CATIONS 8   /* cations per ion-exchange reaction   */
#define PF_MAX_NSRFCPLX_RXN 4   /* surface complexation reactions (sites) */
#define PF_MAX_NSRFCPLX 16      /* surface complexes over all reactions  */

/* isotherm types (reaction_isotherm_aux.F90 SORPTION_*) */
enum { PF_SORPTION_LINEAR = 1, PF_SORPTION_LANGMUIR = 2, PF_SORPTION_FREUNDLICH = 3 };
/* K_D units (isotherm%ikd_units) */
enum { PF_KD_UNIT_KG_M3_BULK = 0, PF_KD_UNIT_MLW_GSOIL = 1 };
/* surface types of a surface complexation reaction (srfcplxrxn_surf_type):
 * the site density is mol/m^3 bulk (NULL), per unit volume fraction of a
 * kinetic mineral (MINERAL), or per kg of solid, times the soil particle
 * density and (1 - porosity) (ROCK) */
enum { PF_SURF_NULL = 0, PF_SURF_MINERAL = 1, PF_SURF_ROCK = 2 };

/*
 * Equilibrium sorption (RTotalSorb, reaction.F90:4783-4832): equilibrium
 * surface complexation (RTotalSorbEqSurfCplx1,
 * reaction_surf_complex.F90:641-900), equilibrium ion exchange
 * (RTotalSorbEqIonx, reaction.F90:4906-5140) and K_D isotherms
 * (RTotalSorbKD, reaction_isotherm.F90:273-359), in that order, added to
 * the accumulation as total_sorb * volume (RAccumulationSorb[Derivative],
 * reaction.F90:5144-5210).  Dynamic K_D and multirate sorption are not
 * built.  Supported by pf_update_auxvars, pf_equilibrate_constraint[_ex]
 * and pf_rstep (the plain kernel and the one-lane batched kernel; a launch
 * configuration with several lanes per cell is refused) and
 * pf_girt_assemble (sorbed accumulation S*V/dt and its derivative
 * dS/dm*V/dt on the diagonal block, reactive_transport.F90:2412, 3183);
 * pf_adjoint returns PF_ERR_UNSUPPORTED for a network with sorption.
 * Surface complex k of reaction r (k from srfcplx_rxn_ptr[r] to
 * srfcplx_rxn_ptr[r+1]-1): S_k = exp(-logK_k ln10 + nu_fk ln S_x
 * + sum_j nu_jk ln a_j (+ h2o_k ln a_H2O)), S_x the reaction's free-site
 * concentration from its site balance (a Newton iteration when some nu_fk
 * > 1, else closed form), warm-started from PfCellState.srfcplx_free_site.
 */
typedef struct PfSorptionDesc {
  int32_t nkd;                    /* isotherm reactions, <= PF_MAX_NKD             */
  int32_t kd_units;               /* PF_KD_UNIT_*                                   */
  const int32_t* kd_spec;         /* [nkd] primary index (isotherm%eqkdspecid - 1)  */
  const int32_t* kd_type;         /* [nkd] PF_SORPTION_*                            */
  const double* kd_coeff;         /* [nkd] eqisothermcoeff                          */
  const double* kd_langmuir_b;    /* [nkd] or NULL                                  */
  const double* kd_freundlich_n;  /* [nkd] or NULL                                  */
  const int32_t* kd_mineral;      /* [nkd] kinetic mineral scaling K_D by its volume
                                     fraction (eqkdmineral - 1), -1 none; or NULL */
  double soil_particle_density;   /* kg/m^3, used with PF_KD_UNIT_MLW_GSOIL        */
  int32_t nionx;                  /* ion-exchange reactions, <= PF_MAX_NIONX        */
  int32_t ionx_stride;            /* row stride of ionx_cation / ionx_k             */
  const int32_t* ionx_ncation;    /* [nionx] eqionx_rxn_cationid(0,:)               */
  const int32_t* ionx_cation;     /* [nionx*stride] primary index; the first is the
                                     reference cation                              */
  const double* ionx_k;           /* [nionx*stride] selectivity eqionx_rxn_k         */
  const double* ionx_cec;         /* [nionx] eqionx_rxn_CEC, mol/m^3 bulk            */
  const int32_t* ionx_mineral;    /* [nionx] kinetic mineral whose volume fraction
                                     scales the CEC (eqionx_rxn_to_surf - 1), -1
                                     none; or NULL                                 */
  /* equilibrium surface complexation (surface_complexation_type,
   * reaction_surface_complexation_aux.F90) */
  int32_t nsrfcplx_rxn;           /* reactions (sites), <= PF_MAX_NSRFCPLX_RXN      */
  int32_t nsrfcplx;               /* complexes of all reactions, <= PF_MAX_NSRFCPLX */
  const int32_t* srfcplx_rxn_ptr; /* [nsrfcplx_rxn + 1] (srfcplxrxn_to_complex)     */
  const int32_t* srfcplx_surf_type;   /* [nsrfcplx_rxn] PF_SURF_*                   */
  const int32_t* srfcplx_mineral;     /* [nsrfcplx_rxn] kinetic mineral of a MINERAL
                                         surface (srfcplxrxn_to_surf - 1), or NULL */
  const double* srfcplx_site_density; /* [nsrfcplx_rxn] srfcplxrxn_site_density     */
  int32_t srfcplx_stride;             /* row stride of srfcplx_spec / _stoich       */
  const int32_t* srfcplx_nspec;       /* [nsrfcplx] srfcplxspecid(0,:)              */
  const int32_t* srfcplx_spec;        /* [nsrfcplx*stride] primary index            */
  const double* srfcplx_stoich;       /* [nsrfcplx*stride]                          */
  const double* srfcplx_free_site_stoich; /* [nsrfcplx]                             */
  const double* srfcplx_logK;         /* [nsrfcplx] at the reference temperature    */
  const double* srfcplx_logKcoef;     /* [nsrfcplx*5] or NULL (isothermal)          */
  const double* srfcplx_h2o_stoich;   /* [nsrfcplx] srfcplxh2ostoich, or NULL       */
} PfSorptionDesc;

/*
 * Kinetic-mineral rate prefactors (the PREFACTOR blocks of a mineral's
 * kinetics; kinmnrl_num_prefactors, kinmnrl_pref_*, kinmnrl_prefactor_id of
 * mineral_type, reaction_mineral_aux.F90:118-125, filled at
 * reaction_database.F90:2280-2335).  A mineral with num_prefactors > 0 uses
 *   sum_p rate_p * Arrhenius_p * prod_s exp(alpha_s ln a_s - ln(1 + K_s a_s^beta_s))
 * in place of its rate constant times its Arrhenius factor
 * (RKineticMineral, reaction_mineral.F90:820-858), with the derivative of
 * :976-1070.  Species: primary j as j (0-based), secondary complex i as
 * -(i+1) (the reference's negative ids).  Arrays are dense:
 * [nmnrl][PF_MAX_PREFACTORS] and [nmnrl][PF_MAX_PREFACTORS]
 * [PF_MAX_PREFACTOR_SPECIES].  Supported by the plain step kernel
 * (PF_KERNEL_PLAIN) and the global-implicit assembly; PF_KERNEL_BATCHED,
 * pf_set_launch_config and pf_adjoint return PF_ERR_UNSUPPORTED for such a
 * network.  pf_network_create returns PF_ERR_UNSUPPORTED when a primary
 * prefactor species follows a secondary one whose complex has more species
 * than the mineral (the reference's derivative would index past the
 * mineral's species there, reaction_mineral.F90:1033-1046).
 */
#define PF_MAX_PREFACTORS 4
#define PF_MAX_PREFACTOR_SPECIES 4
typedef struct PfPrefactorDesc {
  const int32_t* num_prefactors;     /* [nmnrl] 0..PF_MAX_PREFACTORS             */
  const double* rate;                /* kinmnrl_pref_rate, mol/m^2/s              */
  const double* activation_energy;   /* kinmnrl_pref_activation_energy, J/mol (0 =
                                        none)                                    */
  const int32_t* nspec;              /* kinmnrl_prefactor_id(0,:,:)               */
  const int32_t* spec;               /* species ids as above                      */
  const double* alpha;               /* kinmnrl_pref_alpha                        */
  const double* beta;                /* kinmnrl_pref_beta                         */
  const double* atten_coef;          /* kinmnrl_pref_atten_coef (0 allowed: no
                                        denominator)                             */
} PfPrefactorDesc;

/*
 * Solver options: the CHEMISTRY-block fields of reaction_rt_type with the
 * defaults of ReactionCreate (src/pflotran/reaction_aux.F90:371-556).
 */
typedef struct PfOptions {
  int32_t use_log_formulation;          /* reaction_base.F90:33 (deck: LOG_FORMULATION) */
  int32_t act_coef_update_frequency;    /* PF_ACT_COEF_*                       */
  int32_t act_coef_update_algorithm;    /* PF_ACT_COEF_ALGO_*                  */
  int32_t maximum_reaction_cuts;        /* 10                                  */
  int32_t maximum_reaction_iterations;  /* 20                                  */
  int32_t use_total_as_guess;           /* 0                                   */
  int32_t isothermal;                   /* 1: logK fixed; 0: logK(T) per cell  */
  int32_t fork_literal_rsolve;          /* 1: RSolve skips back-substitution as
                                           reaction.F90:5501-5504 does when
                                           solve_error is passed (update = 0).
                                           Documentation aid; default 0.      */
  double max_dlnC_rreact;               /* 5                                   */
  double max_relative_change_tolerance; /* 1e-6                                */
  double max_residual_tolerance;        /* 1e-12                               */
  double max_rel_residual_tolerance;    /* 1e-8                                */
  int32_t use_activity_h2o;             /* reaction%use_activity_h2o (deck:
                                           ACTIVITY_H2O): RActivityCoefficients
                                           sets ln a_H2O = ln(1 - 0.017 (sum of
                                           molalities)) (reaction.F90:4537-4547,
                                           4604-4611), added with each reaction's
                                           water coefficient to its ln Q/K.  0   */
} PfOptions;

/*
 * Flattened reaction network (reaction_rt_type, reaction_aux.F90:123-311,
 * and mineral_type, reaction_mineral_aux.F90:82-138).
 *
 * Secondary (aqueous complex) i:
 *   sec_nspec[i]                     = eqcplxspecid(0,i)
 *   sec_spec[i*sec_stride + s]       = eqcplxspecid(s+1,i) - 1
 *   sec_stoich[i*sec_stride + s]     = eqcplxstoich(s+1,i)
 * Kinetic mineral m: same scheme with mnrl_* and mnrl_stride
 *   (kinmnrlspecid / kinmnrlstoich).
 * logK coefficient fits: 5 per reaction (ReactionInterpolateLogK,
 * reaction_aux.F90:1285-1312); may be NULL when isothermal.
 * Optional TST arrays (min_scale_factor, Temkin_const, affinity_power) are
 * NULL when the reference leaves them unassociated
 * (reaction_database.F90:2039-2092); the rate formulas differ by branch.
 */
typedef struct PfNetworkDesc {
  int32_t ncomp;   /* naqcomp (no immobile species)          */
  int32_t nsec;    /* neqcplx                                 */
  int32_t nmnrl;   /* mineral%nkinmnrl                        */
  int32_t sec_stride;
  int32_t mnrl_stride;
  int32_t h_ion_id;                   /* 0-based id of H+, -1 if none (pH output) */
  const int32_t* sec_nspec;           /* [nsec]                */
  const int32_t* sec_spec;            /* [nsec*sec_stride]     */
  const double* sec_stoich;           /* [nsec*sec_stride]     */
  const double* sec_logK;             /* [nsec] at the reference temperature */
  const double* sec_logKcoef;         /* [nsec*5] or NULL      */
  const double* pri_Z;                /* [ncomp] primary_spec_Z  */
  const double* pri_a0;               /* [ncomp] primary_spec_a0 */
  const double* sec_Z;                /* [nsec]  eqcplx_Z        */
  const double* sec_a0;               /* [nsec]  eqcplx_a0       */
  const int32_t* mnrl_nspec;          /* [nmnrl]               */
  const int32_t* mnrl_spec;           /* [nmnrl*mnrl_stride]   */
  const double* mnrl_stoich;          /* [nmnrl*mnrl_stride]   */
  const double* mnrl_logK;            /* [nmnrl]               */
  const double* mnrl_logKcoef;        /* [nmnrl*5] or NULL     */
  const double* mnrl_rate_constant;   /* [nmnrl] mol/m^2/s     */
  const double* mnrl_activation_energy; /* [nmnrl] J/mol (0 = none) */
  const double* mnrl_molar_vol;       /* [nmnrl] m^3/mol       */
  const double* mnrl_affinity_threshold; /* [nmnrl]            */
  const double* mnrl_rate_limiter;    /* [nmnrl]               */
  const int32_t* mnrl_irreversible;   /* [nmnrl]               */
  const double* mnrl_min_scale_factor; /* [nmnrl] or NULL      */
  const double* mnrl_Temkin_const;    /* [nmnrl] or NULL       */
  const double* mnrl_affinity_power;  /* [nmnrl] or NULL       */
  double debyeA, debyeB, debyeBdot;   /* reaction_database.F90:931-1022 */
  PfOptions opts;
  const PfSorptionDesc* sorption;     /* NULL: no sorption                        */
  const PfPrefactorDesc* prefactors;  /* NULL: no mineral has rate prefactors     */
  const double* sec_h2o_stoich;       /* [nsec] eqcplxh2ostoich (0: no water in the
                                         reaction, eqcplxh2oid = 0), or NULL      */
  const double* mnrl_h2o_stoich;      /* [nmnrl] kinmnrlh2ostoich, or NULL         */
} PfNetworkDesc;

/*
 * Per-cell state, structure-of-arrays (value(k,cell) = a[k*ncells+cell]).
 * Mirrors rt_auxvar (reactive_transport_aux.F90:21-74), global_auxvar
 * (global_aux.F90:11-35) and material_auxvar (material_aux.F90:53-77).
 */
typedef struct PfCellState {
  int64_t ncells;
  double* total;          /* [ncomp]  total(:,1), mol/L; in: transported total */
  double* pri_molal;      /* [ncomp]  in: guess (free ion); out: solution     */
  double* pri_act_coef;   /* [ncomp]                                           */
  double* sec_act_coef;   /* [nsec]                                            */
  double* sec_molal;      /* [nsec]                                            */
  double* mnrl_volfrac;   /* [nmnrl]                                           */
  double* mnrl_area;      /* [nmnrl]  m^2/m^3 bulk                             */
  double* mnrl_rate;      /* [nmnrl]  out: mol/m^3/s                           */
  const double* porosity; /* [1]                                               */
  const double* saturation;
  const double* den_kg;   /* kg/m^3                                            */
  const double* volume;   /* m^3                                               */
  const double* temperature; /* C (used when !isothermal)                      */
  const double* dt_cell;  /* [1] per-cell operator-split dt, or NULL = uniform  */
  int32_t* status;        /* [1] out: PF_CELL_*                                */
  int32_t* newton_its;    /* [1] out: Newton iterations summed over substeps   */
  int32_t* num_substeps;  /* [1] out                                           */
  const int64_t* cell_order; /* optional permutation of 0..ncells-1: the order in
                              which the batched kernel's work queue hands out
                              cells (e.g. descending previous iteration count);
                              NULL = natural order.  Results do not depend on it. */
  /* networks with sorption only (NULL otherwise): */
  double* total_sorb;      /* [ncomp] total_sorb_eq, mol/m^3 bulk; in: the
                              sorbed total of the fixed accumulation; out: at
                              the solution                                     */
  double* ionx_ref_sorbed; /* [nionx] eqionx_ref_cation_sorbed_conc: the ion-
                              exchange Newton's warm start, carried between
                              calls as the reference carries it                */
  double* ln_act_h2o;      /* [1] rt_auxvar%ln_act_h2o (in; out where activity
                              coefficients are updated); NULL reads as 0.
                              Required when use_activity_h2o                   */
  /* networks with surface complexation only (NULL otherwise): */
  double* srfcplx_free_site; /* [nsrfcplx_rxn] srfcplxrxn_free_site_conc, mol/m^3
                                bulk: the site balance's warm start, updated in
                                place as the reference updates rt_auxvar         */
  double* srfcplx_conc;      /* [nsrfcplx] eqsrfcplx_conc (out, mol/m^3 bulk) of
                                the last evaluation, or NULL                    */
} PfCellState;

typedef struct PfStepStats {
  int64_t cells;
  int64_t failed_cells;
  int64_t newton_iterations;   /* sum over cells */
  int32_t max_newton_iterations;
  int32_t max_substeps;
} PfStepStats;

typedef struct PfNetwork PfNetwork;   /* opaque: device-resident tables */

/* ---------------------------------------------------------------- network */
/* Validates and uploads the network tables to the current CUDA device.
 * Replaces the setup-time flattening in BasisInit
 * (reaction_database.F90:812-2367) as seen by the cell loop. */
int32_t pf_network_create(const PfNetworkDesc* desc, PfNetwork** out);
int32_t pf_network_destroy(PfNetwork* net);
/* Copy of the descriptor's options; lets a caller change tolerances without
 * re-uploading tables (e.g. the tight mode of the parity tests). */
int32_t pf_network_set_options(PfNetwork* net, const PfOptions* opts);
/* Pre-allocates the per-cell scratch of the batched kernel for up to ncells
 * cells (pf_rstep grows it on demand otherwise; call this before capturing
 * pf_rstep into a CUDA graph, since allocation cannot be captured). */
int32_t pf_network_reserve(PfNetwork* net, int64_t ncells);

/* ------------------------------------------------------------ operator split */
/*
 * pf_rstep -- one operator-split reaction step for every cell.
 * Replaces the loop body at src/pflotran/pmc_subsurface_osrt.F90:349-378,
 * i.e. for each cell: guess = pri_molal; RStep(guess, rt_auxvar, ...)
 * (src/pflotran/reaction.F90:3564-3738, RReact :3742-4055).
 * dt: option%tran_dt [s] (ignored for cells when state->dt_cell != NULL).
 * kernel: PF_KERNEL_PLAIN or PF_KERNEL_BATCHED.
 * stats: optional (NULL); when given the call synchronises the stream and
 * reduces the per-cell counters (the MPI_Allreduce of rstep_error at
 * pmc_subsurface_osrt.F90:381 becomes this device reduction).
 * Returns PF_OK, PF_CELL_FAILURES (stats->failed_cells > 0) or PF_ERR_*.
 */
int32_t pf_rstep(PfNetwork* net, const PfCellState* state, double dt,
                 int32_t kernel, void* stream, PfStepStats* stats);

/*
 * pf_update_auxvars -- RTUpdateAuxVars for cells
 * (src/pflotran/reactive_transport.F90:3525-3660): optionally
 * RActivityCoefficients (reaction.F90:4368-4614), then RTotal
 * (reaction.F90:4618-4759) from pri_molal; writes total and sec_molal.
 */
int32_t pf_update_auxvars(PfNetwork* net, const PfCellState* state,
                          int32_t update_activity_coefs, void* stream);

/*
 * pf_update_activity_coefs -- RTUpdateActivityCoefficients for cells
 * (src/pflotran/reactive_transport.F90:3441-3521): activity coefficients
 * only, totals untouched (the TIMESTEP update of pm_osrt.F90:145-151).
 */
int32_t pf_update_activity_coefs(PfNetwork* net, const PfCellState* state,
                                 void* stream);

/*
 * pf_rstep_host -- the same step through host buffers: copies the state to
 * the device, runs pf_rstep (kernel form as given), copies results back.
 * Host arrays use the same SoA layout.  This is the entry point a Fortran
 * caller binds through iso_c_binding (contiguous temporaries via c_loc).
 * Large states go in chunks whose copies in and out overlap the compute;
 * host_state->cell_order (host memory) is restricted to each chunk, and an
 * order that is not a permutation of 0..ncells-1 returns PF_ERR_INVALID
 * with the caller's arrays untouched.
 */
int32_t pf_rstep_host(PfNetwork* net, const PfCellState* host_state,
                      double dt, int32_t kernel, PfStepStats* stats);

/*
 * pf_rstep_noalloc -- pf_rstep with the batched kernel, for callers that must
 * not allocate device memory during the step.  No counterpart in the
 * reference (PFLOTRAN's Fortran loop has no device memory to allocate).
 * Callers that cannot let a library call cudaMalloc -- a host model whose GPU
 * memory belongs to another framework's pool, or a coupled run with a fixed
 * device footprint -- use this instead of pf_rstep: the per-cell scratch
 * lives in a fixed 32 MiB device array inside the library (held on every
 * device that loads it until exit), and the call allocates nothing.  Limit:
 * (ncomp + nsec + nmnrl) * ncells <= 4,194,304; larger states return
 * PF_ERR_TOO_LARGE (split them across calls).  Each call outside a stream
 * capture resolves the array's device address (after a cudaDeviceReset it
 * may move); a call inside a capture uses the last one, so make one call on
 * the device before capturing.  All calls share the one array, so calls that overlap on
 * the GPU (other streams, other threads) race; serialise them.  The launch
 * configuration and option checks are pf_rstep's.  Before the launch every
 * status entry is set to PF_CELL_NOT_RUN; the kernel overwrites it for each
 * cell it finishes.  stats: optional, as for pf_rstep (the call then
 * synchronises the stream and returns PF_ERR_TIMEOUT or PF_CELL_FAILURES as
 * pf_rstep does; the counters are read through the network's own pinned
 * buffer, nothing is allocated).
 */
int32_t pf_rstep_noalloc(PfNetwork* net, const PfCellState* state, double dt, void* stream,
                         PfStepStats* stats);

/*
 * pf_rstep_multi -- one operator-split step for the cells of several
 * networks (a heterogeneous domain: regions whose chemistry has different
 * reaction networks, ncomp up to 24) in one persistent launch.  No
 * counterpart in the reference, whose cell loop calls RStep cell by cell
 * whatever the cell's chemistry (pmc_subsurface_osrt.F90:346-378); each cell's
 * step is exactly pf_rstep's with the batched kernel and a group of lanes per
 * cell.  nets[k] and states[k] (device arrays, each state's cell_order
 * honoured) for k < nnets <= PF_MULTI_MAX_NETS, every network on the current
 * device; the launch works through the networks in array order (list the
 * costliest first), every block staging a network's tables and pulling its
 * cells until its queue is empty, then moving to the next, so the SMs idle
 * only at the end of the launch.  Each network runs with 4 or 8 lanes per
 * cell: its own launch configuration's group size when that is one of
 * those, else the first of 4, 8 it supports.  A network the group kernel does
 * not support (sorption, rate prefactors, the linear formulation, activity by
 * the NEWTON algorithm or water activity at every Newton iteration) makes the
 * call return PF_ERR_UNSUPPORTED.  stats: NULL, or an array of nnets
 * (the call then synchronises the stream; PF_CELL_FAILURES when any network
 * had failed cells, PF_ERR_TIMEOUT when a table-staging wait ran out).
 * Per-network scratch grows as pf_rstep's does (pf_network_reserve first,
 * before capturing the call into a CUDA graph).
 */
#define PF_MULTI_MAX_NETS 16
int32_t pf_rstep_multi(PfNetwork* const* nets, const PfCellState* states, int32_t nnets, double dt, void* stream,
                       PfStepStats* stats);

/* ----------------------------------------------------------------- adjoint */
/* Largest number of RStep substeps (dt cuts) whose converged states the
 * adjoint keeps per cell; cells with more report adj_status 2. */
#define PF_ADJ_MAX_SUBSTEPS 16

/*
 * Arguments of pf_adjoint (device pointers, component-major like the state).
 * The loss is L = sum_cells sum_k weight*(total_final - target)^2 when weight
 * and target are given; otherwise dL/dtotal_final is taken from dL_dtotal
 * (the backward pass of an autograd wrapper).  Gradients are with respect to
 * an additive shift of every logK (secondary and mineral, applied at every
 * temperature), ln of every rate constant, ln of every cell's mineral area,
 * and every cell's initial (transported) total.
 */
typedef struct PfAdjointArgs {
  const double* weight;      /* [ncomp][ncells] or NULL                      */
  const double* target;      /* [ncomp][ncells] (with weight)                 */
  const double* dL_dtotal;   /* [ncomp][ncells] used when weight == NULL     */
  double* dL_dtotal0;        /* [ncomp][ncells] out                           */
  double* dL_dlnarea;        /* [nmnrl][ncells] out                           */
  double* dL_dlogK_sec;      /* [nsec]  out, summed over cells                */
  double* dL_dlogK_mnrl;     /* [nmnrl] out, summed over cells                */
  double* dL_dlnk;           /* [nmnrl] out, summed over cells                */
  double* loss;              /* [1] out (weight given) or NULL                */
  int32_t* adj_status;       /* [ncells] out: 0 ok, 1 forward failed (no
                                gradient), 2 more than PF_ADJ_MAX_SUBSTEPS
                                substeps, 3 singular adjoint system          */
} PfAdjointArgs;

/*
 * pf_adjoint -- the operator-split step (as pf_rstep, batched kernel; the
 * state is advanced exactly as pf_rstep would) followed, per cell, by the
 * implicit-function-theorem adjoint of the step.  No counterpart in the
 * reference (PFLOTRAN has no derivatives of RStep with respect to its
 * parameters).  For each substep, from the last backwards, it solves
 * J^T lambda = (dT/dln m)^T Tbar at that substep's converged free-ion
 * molalities m, with the exact Jacobian of the residual
 * (psv/dt)(T(m) - T_prev) + R(m) of RReact (reaction.F90:3899-3916), and
 * accumulates the parameter gradients; Newton iterates are recomputed, not
 * stored (only the substep end states are kept).  Output arrays are zeroed by
 * the call.  Requires the log formulation or the linear one (both solve the
 * same equations) and activity coefficients OFF or TIMESTEP.
 */
int32_t pf_adjoint(PfNetwork* net, const PfCellState* state, double dt,
                   const PfAdjointArgs* args, void* stream);

/* Shifts the network's parameters from their values at pf_network_create:
 * logK of every secondary and kinetic mineral += dlogK (at every temperature:
 * for temperature fits the constant coefficient moves), rate constants
 * *= exp(dlnk).  Host arrays; NULL leaves that group at its base value.
 * Used to evaluate losses away from the base point (finite differences,
 * optimisation steps). */
int32_t pf_network_shift_parameters(PfNetwork* net, const double* dlogK_sec,
                                    const double* dlogK_mnrl, const double* dlnk);

/* ---------------------------------------------------- global implicit (GIRT) */
/*
 * Residual and Jacobian of the global-implicit reactive-transport system on a
 * structured grid nx*ny*nz (cell index i + nx*(j + ny*k)), 7-point stencil,
 * zero-flux outer boundary: replaces RTResidual (reactive_transport.F90:1964)
 * and RTJacobian (:2788) for that grid -- per internal connection TFluxCoef/
 * TFlux/TFluxDerivative (transport.F90:378-565) with the harmonic mean of
 * TDispersion (:52-232), per cell RTAccumulation[Derivative] and
 * RReaction[Derivative], ADD_VALUES in the reference's connection order,
 * then the log-formulation column scaling (MatDiagonalScaleLocal, :2879).
 * The state holds the current Newton iterate (pri_molal) and the activity
 * coefficients; total and sec_molal are updated (RTUpdateAuxVars), and with
 * sorption total_sorb and the ion-exchange warm start.
 */
typedef struct PfGirtArgs {
  int32_t nx, ny, nz;
  double dx, dy, dz;                 /* m (cell sizes; faces dy*dz, dx*dz, dx*dy) */
  const double* qx;                  /* [nz][ny][nx-1] Darcy flux across x faces, m/s,
                                        positive from cell i to cell i+1 */
  const double* qy;                  /* [nz][ny-1][nx] */
  const double* qz;                  /* [nz-1][ny][nx] */
  double diffusion_coefficient;      /* m^2/s, all components */
  double tortuosity;
  double dispersivity;               /* longitudinal, m */
  const double* total_k;             /* [ncomp][ncells] totals at the start of the
                                        time step (fixed accumulation) */
  double dt;                         /* s */
  const int32_t* rowptr;             /* BAIJ pattern from pf_girt_pattern (device) */
  const int32_t* colidx;
  double* residual;                  /* [ncells*ncomp] out, PETSc block-interleaved */
  double* values;                    /* [nnzb*ncomp*ncomp] out, SeqBAIJ blocks,
                                        each column-major */
  const double* total_sorb_k;        /* [ncomp][ncells] sorbed totals at the start of
                                        the step, mol/m^3 bulk (the sorbed part of the
                                        fixed accumulation, RAccumulationSorb at
                                        reactive_transport.F90:1026); required when the
                                        network has sorption, else ignored (NULL) */
  int32_t numerical_derivatives;     /* option%transport%numerical_derivatives: the
                                        reaction part of the diagonal blocks by
                                        forward differences (RReactionDerivative,
                                        reaction.F90:4176-4230; perturbation 1e-5 m_j)
                                        instead of analytically.  pf_rstep has no such
                                        mode: the reference stops there for OSRT
                                        (reaction.F90:3918-3920) */
  double* k_cache;                   /* optional (NULL: none), [nsec + nmnrl][ncells]:
                                        each cell's K_i / gamma_i of every complex, then
                                        K_m of every kinetic mineral, at the cell's
                                        temperature (ReactionInterpolateLogK,
                                        reaction_aux.F90:1285-1312).  The Newton
                                        iterations of one time step assemble at the
                                        same temperatures and activity coefficients
                                        (activity updated per time step), so the first
                                        computes these and the others read them.
                                        Not with the water activity on
                                        (PF_ERR_UNSUPPORTED) */
  int32_t k_cache_valid;             /* 0: compute the K and store them in k_cache;
                                        1: read them from k_cache (what a call with 0
                                        stored, temperatures, logK and the complexes'
                                        activity coefficients unchanged since) */
} PfGirtArgs;

/* Host: block-row pattern of the 7-point structured-grid matrix (block
 * columns ascending).  rowptr[ncells+1], colidx[nnzb]; either may be NULL to
 * query the size.  Returns nnzb (>= 0) or a PfStatus (< 0). */
int32_t pf_girt_pattern(int32_t nx, int32_t ny, int32_t nz, int32_t* rowptr, int32_t* colidx);

int32_t pf_girt_assemble(PfNetwork* net, const PfCellState* state, const PfGirtArgs* args,
                         void* stream);

/* ------------------------------------------------- operator-split transport */
/*
 * The transport half of an operator-split step on a structured grid
 * nx*ny*nz (cell index i + nx*(j + ny*k)): replaces the transport solve of
 * PMCSubsurfaceOSRTStepDT (src/pflotran/pmc_subsurface_osrt.F90:259-330) --
 * the fixed accumulation psv*T_k, the matrix of RTCalculateTransportMatrix
 * (reactive_transport.F90:1469-1703) with TFluxCoef (transport.F90:495-565)
 * and the harmonic-mean dispersion of TDispersion, the right-hand side
 * psv*T_k/dt of RTCalculateRHS_t1 (:1239-1465), and one linear solve per
 * component (all components share the matrix).  Boundary conditions on the
 * six outer faces and sources/sinks follow the boundary and source loops
 * of both routines (TDispersionBC transport.F90:236-374, TFluxCoefBC
 * :569-609, TSrcSinkCoef :613-673); a face without a condition is closed
 * (zero flux).  Solved on the device, all components at once, by
 * mixed-precision iterative refinement (FP64 residual and update, FP32
 * Jacobi-preconditioned BiCGStab corrections) from T_k to
 * ||b - A x|| <= rtol ||b|| in FP64.  No counterpart in the reference for
 * the solver choice (PETSc KSP there).
 */
/* the outer faces, in this order; a face's cells are indexed j + ny*k on
 * the x faces, i + nx*k on the y faces, i + nx*j on the z faces */
enum { PF_FACE_XM = 0, PF_FACE_XP = 1, PF_FACE_YM = 2, PF_FACE_YP = 3, PF_FACE_ZM = 4, PF_FACE_ZP = 5 };
/* transport boundary condition types (tran_condition%itype as TDispersionBC
 * and TFluxCoefBC treat them); the boundary connection's distance is half
 * the cell's width, its area the face's */
enum {
  PF_BC_ZERO_FLUX = 0,              /* no boundary connection (closed face)       */
  PF_BC_DIRICHLET = 1,              /* DIRICHLET_BC: advection in from, and
                                       dispersion against, the boundary totals    */
  PF_BC_DIRICHLET_ZERO_GRADIENT = 2, /* DIRICHLET_ZERO_GRADIENT_BC: as Dirichlet
                                       where the flux enters, advection only where
                                       it leaves                                  */
  PF_BC_ZERO_GRADIENT = 3           /* ZERO_GRADIENT_BC (also NEUMANN_BC and
                                       CONCENTRATION_SS): advection only          */
};
/* source/sink types (tran_src_sink_type of TSrcSinkCoef) */
enum {
  PF_SRC_VOLUMETRIC = 0,  /* q m^3/s: injection carries src_total in, extraction
                             removes the cell's water                              */
  PF_SRC_EQUILIBRIUM = 1, /* EQUILIBRIUM_SS: relaxation at 1e-3 L/s toward src_total */
  PF_SRC_MASS_RATE = 2    /* MASS_RATE_SS: src_total is a rate, mol/s               */
};
typedef struct PfTransportArgs {
  int32_t nx, ny, nz, ncomp;
  double dx, dy, dz;                 /* m */
  const double* qx;                  /* [nz][ny][nx-1] Darcy flux, m/s, + from i to i+1 */
  const double* qy;                  /* [nz][ny-1][nx] */
  const double* qz;                  /* [nz-1][ny][nx] */
  double diffusion_coefficient;      /* m^2/s */
  double tortuosity;
  double dispersivity;               /* m */
  const double* porosity;            /* [ncells] */
  const double* saturation;          /* [ncells] */
  const double* volume;              /* [ncells] m^3 */
  double dt;                         /* s (option%tran_dt) */
  double* total;                     /* [ncomp][ncells] mol/L: in T_k, out T_k+1 */
  double rtol;                       /* relative residual tolerance */
  int32_t max_iterations;
  /* boundary conditions, per face (all PF_BC_ZERO_FLUX: a closed box) */
  int32_t bc_type[6];                /* PF_BC_*                                      */
  const double* bc_q[6];             /* [face cells] Darcy flux through the face, m/s,
                                        positive into the domain; NULL = no flow      */
  const double* bc_total[6];         /* [ncomp][face cells] totals of the boundary
                                        water, mol/L (rt_auxvars_bc%total)           */
  double bc_saturation[6];           /* saturation at the boundary
                                        (global_auxvars_bc%sat)                      */
  /* sources and sinks (source_sink_list), applied in array order */
  int32_t nsrc;
  const int32_t* src_cell;           /* [nsrc] cell index                            */
  const int32_t* src_type;           /* [nsrc] PF_SRC_*                              */
  const double* src_q;               /* [nsrc] m^3/s, positive: injection            */
  const double* src_total;           /* [ncomp][nsrc] mol/L (mol/s: PF_SRC_MASS_RATE) */
} PfTransportArgs;

typedef struct PfTransportStats {
  int32_t iterations;                /* inner (FP32) BiCGStab iterations, all components in step */
  int32_t converged;                 /* 1 when every component met rtol */
  double max_rel_residual;           /* max over components of the FP64 ||b - A x|| / ||b|| */
  int32_t refinements;               /* FP64 refinement cycles (residual, inner solve, update) */
  int32_t max_cycle_iterations;      /* most inner iterations any component took in one cycle */
} PfTransportStats;

typedef struct PfTransport PfTransport;  /* opaque: device work space of one grid */

int32_t pf_transport_create(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp, PfTransport** out);
int32_t pf_transport_destroy(PfTransport* t);
/* PF_OK, PF_CELL_FAILURES (not converged within max_iterations; totals hold
 * the last iterate) or PF_ERR_*. */
int32_t pf_transport_step(PfTransport* t, const PfTransportArgs* args, void* stream,
                          PfTransportStats* stats);
/* The same solve with a fixed schedule: `refinements` cycles of
 * `inner_iterations` inner iterations, enqueued on `stream` with no host
 * synchronisation (capturable in a CUDA graph; converged components make
 * the remaining work no-ops).  args->max_iterations is not used.  Returns
 * PF_OK once enqueued; pf_transport_read_stats then reports whether the
 * schedule met args->rtol (pf_transport_step's stats give a schedule:
 * refinements + 1 cycles of max_cycle_iterations + 2). */
int32_t pf_transport_enqueue(PfTransport* t, const PfTransportArgs* args, int32_t inner_iterations,
                             int32_t refinements, void* stream);
/* Synchronises `stream` and fills stats from the last solve's device
 * counters: PF_OK if every component met rtol, else PF_CELL_FAILURES. */
int32_t pf_transport_read_stats(PfTransport* t, double rtol, void* stream, PfTransportStats* stats);

/* ----------------------------------------------------------- constraints */
/* Constraint types (transport_constraint_rt.F90:22-34 subset). */
enum {
  PF_CONSTRAINT_TOTAL = 1,
  PF_CONSTRAINT_FREE = 2,
  PF_CONSTRAINT_PH = 3,
  PF_CONSTRAINT_CHARGE_BAL = 4,
  PF_CONSTRAINT_LOG = 5,
  PF_CONSTRAINT_MINERAL = 6,  /* equilibrium with a mineral: ln(Q/K) = 0 (reaction.F90:1755-1779) */
  PF_CONSTRAINT_GAS = 7       /* a gas partial pressure: ln(Q/K) = ln p (reaction.F90:1781-1811) */
};

/* The reaction of a MINERAL or GAS constraint row: the mineral's or gas's
 * reaction in the primary species (water dropped, its activity is one), as
 * the reference holds it in mineral%mnrlspecid/mnrlstoich/mnrl_logK and
 * gas%paseqspecid/paseqstoich/paseqlogK.  Any mineral or gas of the
 * database, kinetic or not. */
typedef struct PfConstraintReaction {
  int32_t nspec;                  /* species in the reaction, 1..ncomp */
  int32_t temperature_dependent;  /* 1: logK from logKcoef at the cell temperature */
  int32_t spec[PF_MAX_NCOMP];     /* primary indices, 0-based */
  double stoich[PF_MAX_NCOMP];
  double logK;                    /* used when temperature_dependent = 0 */
  double logKcoef[5];             /* c1 ln T + c2 + c3 T + c4/T + c5/T^2, T in K */
} PfConstraintReaction;

/*
 * pf_equilibrate_constraint -- ReactionEquilibrateConstraint
 * (src/pflotran/reaction.F90:1328-2115) for every cell, restricted to the
 * aqueous constraint types above (no mineral/gas/sorption constraints).
 * ctype: host array [ncomp], one type per primary component.
 * cconc: device array [ncomp][ncells]: total (mol/L), free (mol/L),
 *        log10 free, pH, or the charge-balance species' initial guess.
 * On return pri_molal, pri_act_coef, sec_act_coef, sec_molal and total hold
 * the equilibrated state; iterations[cell] (device, optional) holds the
 * Newton count or -1 when the cell did not converge within 10000 iterations
 * or produced a non-positive molality (the reference stops the run there).
 */
int32_t pf_equilibrate_constraint(PfNetwork* net, const PfCellState* state,
                                  const int32_t* ctype, const double* cconc,
                                  int32_t use_prev_soln_as_guess,
                                  int32_t* iterations, void* stream);
/* The same with MINERAL and GAS rows.  creact: host array [ncomp]; entry j
 * is read only when ctype[j] is MINERAL or GAS (may be NULL when no row is).
 * cconc for a MINERAL row: the free-ion guess (mol/L); for a GAS row: the
 * partial pressure (bar), or its log10 when <= 0. */
int32_t pf_equilibrate_constraint_ex(PfNetwork* net, const PfCellState* state,
                                     const int32_t* ctype, const PfConstraintReaction* creact,
                                     const double* cconc, int32_t use_prev_soln_as_guess,
                                     int32_t* iterations, void* stream);

/* ------------------------------------------------------------ capabilities */
/* Kernel launch configuration for the batched form; chosen by the
 * autotuner (pfgpu.autotune) and settable per network.
 * lanes_per_cell 0 or 1: one lane per cell (ncomp-specialised kernel);
 * 2, 4 or 8: a group of lanes shares each cell, the Jacobian in shared memory
 * (larger networks; log formulation only; pf_adjoint always uses one lane
 * per cell with the last such configuration set, or the default). */
typedef struct PfLaunchConfig {
  int32_t threads_per_block;  /* multiple of 32                        */
  int32_t blocks_per_sm;      /* persistent grid = SMs * blocks_per_sm */
  int32_t jac_in_shared;      /* 1: Jacobian in shared memory, 0: local (one lane per cell) */
  int32_t lanes_per_cell;     /* 0/1, 2, 4 or 8                        */
} PfLaunchConfig;
int32_t pf_network_set_launch(PfNetwork* net, const PfLaunchConfig* cfg);
int32_t pf_network_get_launch(const PfNetwork* net, PfLaunchConfig* cfg);

/* Library version / build info string (static storage). */
const char* pf_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PFGPU_H_ */
