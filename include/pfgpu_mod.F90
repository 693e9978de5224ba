! pfgpu_mod.F90 -- Fortran 2003 binding of the C ABI in pfgpu.h, for PFLOTRAN.
!
! The derived types mirror the header's structs member for member
! (bind(C): same order, same interoperable kinds); the interfaces declare
! every entry point.  tests/test_fortran_binding.py parses this file and
! checks each type's member names, order, kinds and byte offsets against
! the C structs as compiled from pfgpu.h, so the two cannot drift apart.
!
! Replaces, in the reference (fmyuan/pflotran-elm-interface):
!   - the operator-split cell loop of PMCSubsurfaceOSRTStepDT
!     (src/pflotran/pmc_subsurface_osrt.F90:346-378), one RStep per cell
!     (src/pflotran/reaction.F90:3564-3567), by one pf_rstep_host call over
!     all cells (pfgpu_osrt_react below shows the gather and the scatter);
!   - RTResidual/RTJacobian's per-cell and flux blocks on a structured grid
!     (src/pflotran/reactive_transport.F90:1964, 2788) by pf_girt_assemble;
!   - the OSRT transport solve (pmc_subsurface_osrt.F90:259-330) by
!     pf_transport_step.
! Ids are 0-based on the C side (Fortran ids minus one); per-cell arrays are
! component-major, value(k, cell) = a(cell + ncells*k), which is exactly a
! Fortran array dimensioned (ncells, ncomp).

module pfgpu_mod
  use, intrinsic :: iso_c_binding
  implicit none
  private

  ! ------------------------------------------------------------- status codes
  integer(c_int32_t), parameter, public :: PF_OK = 0, PF_CELL_FAILURES = 1, &
      PF_ERR_INVALID = -1, PF_ERR_UNSUPPORTED = -2, PF_ERR_CUDA = -3, &
      PF_ERR_TOO_LARGE = -4, PF_ERR_TIMEOUT = -5
  integer(c_int32_t), parameter, public :: PF_CELL_OK = 0, PF_CELL_TOO_MANY_CUTS = 1, &
      PF_CELL_NAN = 2, PF_CELL_NOT_RUN = -1
  integer(c_int32_t), parameter, public :: PF_ACT_COEF_OFF = 0, PF_ACT_COEF_TIMESTEP = 1, &
      PF_ACT_COEF_NEWTON_ITER = 2, PF_ACT_COEF_ALGO_LAG = 0, PF_ACT_COEF_ALGO_NEWTON = 1
  integer(c_int32_t), parameter, public :: PF_KERNEL_PLAIN = 0, PF_KERNEL_BATCHED = 1
  integer(c_int32_t), parameter, public :: PF_MAX_NCOMP = 24, PF_MAX_NSEC = 96, &
      PF_MAX_NMNRL = 16, PF_MAX_SPEC_PER_RXN = 24, PF_MAX_NKD = 8, PF_MAX_NIONX = 4, &
      PF_MAX_IONX_CATIONS = 8, PF_MAX_PREFACTORS = 4, PF_MAX_PREFACTOR_SPECIES = 4, &
      PF_ADJ_MAX_SUBSTEPS = 16, PF_MULTI_MAX_NETS = 16
  integer(c_int32_t), parameter, public :: PF_SORPTION_LINEAR = 1, PF_SORPTION_LANGMUIR = 2, &
      PF_SORPTION_FREUNDLICH = 3, PF_KD_UNIT_KG_M3_BULK = 0, PF_KD_UNIT_MLW_GSOIL = 1, &
      PF_SURF_NULL = 0, PF_SURF_MINERAL = 1, PF_SURF_ROCK = 2, PF_MAX_NSRFCPLX_RXN = 4, PF_MAX_NSRFCPLX = 16
  integer(c_int32_t), parameter, public :: PF_BC_ZERO_FLUX = 0, PF_BC_DIRICHLET = 1, &
      PF_BC_DIRICHLET_ZERO_GRADIENT = 2, PF_BC_ZERO_GRADIENT = 3, PF_SRC_VOLUMETRIC = 0, &
      PF_SRC_EQUILIBRIUM = 1, PF_SRC_MASS_RATE = 2
  integer(c_int32_t), parameter, public :: PF_CONSTRAINT_TOTAL = 1, PF_CONSTRAINT_FREE = 2, &
      PF_CONSTRAINT_PH = 3, PF_CONSTRAINT_CHARGE_BAL = 4, PF_CONSTRAINT_LOG = 5, &
      PF_CONSTRAINT_MINERAL = 6, PF_CONSTRAINT_GAS = 7

  ! ---------------------------------------------------------------- the types
  ! equilibrium sorption (RTotalSorb: K_D isotherms, ion exchange)
  type, bind(C), public :: pf_sorption_desc_t
    integer(c_int32_t) :: nkd, kd_units
    type(c_ptr) :: kd_spec, kd_type, kd_coeff, kd_langmuir_b, kd_freundlich_n, kd_mineral
    real(c_double) :: soil_particle_density
    integer(c_int32_t) :: nionx, ionx_stride
    type(c_ptr) :: ionx_ncation, ionx_cation, ionx_k, ionx_cec, ionx_mineral
    integer(c_int32_t) :: nsrfcplx_rxn, nsrfcplx
    type(c_ptr) :: srfcplx_rxn_ptr, srfcplx_surf_type, srfcplx_mineral, srfcplx_site_density
    integer(c_int32_t) :: srfcplx_stride
    type(c_ptr) :: srfcplx_nspec, srfcplx_spec, srfcplx_stoich, srfcplx_free_site_stoich, srfcplx_logK, &
                   srfcplx_logKcoef, srfcplx_h2o_stoich
  end type

  ! kinetic-mineral rate prefactors (kinmnrl_pref_*)
  type, bind(C), public :: pf_prefactor_desc_t
    type(c_ptr) :: num_prefactors, rate, activation_energy, nspec, spec, alpha, beta, atten_coef
  end type

  ! the CHEMISTRY block's solver options (reaction_aux.F90:371-556 defaults)
  type, bind(C), public :: pf_options_t
    integer(c_int32_t) :: use_log_formulation, act_coef_update_frequency, &
                          act_coef_update_algorithm, maximum_reaction_cuts, &
                          maximum_reaction_iterations, use_total_as_guess, &
                          isothermal, fork_literal_rsolve
    real(c_double) :: max_dlnC_rreact, max_relative_change_tolerance, &
                      max_residual_tolerance, max_rel_residual_tolerance
    integer(c_int32_t) :: use_activity_h2o
  end type

  ! the flattened network (reaction_rt_type, mineral_type)
  type, bind(C), public :: pf_network_desc_t
    integer(c_int32_t) :: ncomp, nsec, nmnrl, sec_stride, mnrl_stride, h_ion_id
    type(c_ptr) :: sec_nspec, sec_spec, sec_stoich, sec_logK, sec_logKcoef, &
                   pri_Z, pri_a0, sec_Z, sec_a0, &
                   mnrl_nspec, mnrl_spec, mnrl_stoich, mnrl_logK, mnrl_logKcoef, &
                   mnrl_rate_constant, mnrl_activation_energy, mnrl_molar_vol, &
                   mnrl_affinity_threshold, mnrl_rate_limiter, mnrl_irreversible, &
                   mnrl_min_scale_factor, mnrl_Temkin_const, mnrl_affinity_power
    real(c_double) :: debyeA, debyeB, debyeBdot
    type(pf_options_t) :: opts
    type(c_ptr) :: sorption                ! pf_sorption_desc_t or c_null_ptr
    type(c_ptr) :: prefactors              ! pf_prefactor_desc_t or c_null_ptr
    type(c_ptr) :: sec_h2o_stoich, mnrl_h2o_stoich
  end type

  ! per-cell state, structure of arrays (rt_auxvar, global_auxvar, material_auxvar)
  type, bind(C), public :: pf_cell_state_t
    integer(c_int64_t) :: ncells
    type(c_ptr) :: total, pri_molal, pri_act_coef, sec_act_coef, sec_molal, &
                   mnrl_volfrac, mnrl_area, mnrl_rate, porosity, saturation, &
                   den_kg, volume, temperature, dt_cell, status, newton_its, &
                   num_substeps, cell_order, total_sorb, ionx_ref_sorbed, ln_act_h2o, &
                   srfcplx_free_site, srfcplx_conc
  end type

  type, bind(C), public :: pf_step_stats_t
    integer(c_int64_t) :: cells, failed_cells, newton_iterations
    integer(c_int32_t) :: max_newton_iterations, max_substeps
  end type

  type, bind(C), public :: pf_adjoint_args_t
    type(c_ptr) :: weight, target, dL_dtotal, dL_dtotal0, dL_dlnarea, dL_dlogK_sec, &
                   dL_dlogK_mnrl, dL_dlnk, loss, adj_status
  end type

  type, bind(C), public :: pf_girt_args_t
    integer(c_int32_t) :: nx, ny, nz
    real(c_double) :: dx, dy, dz
    type(c_ptr) :: qx, qy, qz
    real(c_double) :: diffusion_coefficient, tortuosity, dispersivity
    type(c_ptr) :: total_k
    real(c_double) :: dt
    type(c_ptr) :: rowptr, colidx, residual, values, total_sorb_k
    integer(c_int32_t) :: numerical_derivatives
    type(c_ptr) :: k_cache                      ! optional per-cell K cache, (ncells, nsec + nmnrl)
    integer(c_int32_t) :: k_cache_valid         ! 0: fill it, 1: read it
  end type

  type, bind(C), public :: pf_transport_args_t
    integer(c_int32_t) :: nx, ny, nz, ncomp
    real(c_double) :: dx, dy, dz
    type(c_ptr) :: qx, qy, qz
    real(c_double) :: diffusion_coefficient, tortuosity, dispersivity
    type(c_ptr) :: porosity, saturation, volume
    real(c_double) :: dt
    type(c_ptr) :: total
    real(c_double) :: rtol
    integer(c_int32_t) :: max_iterations
    integer(c_int32_t) :: bc_type(6)            ! PF_BC_* per face x-, x+, y-, y+, z-, z+
    type(c_ptr) :: bc_q(6)                      ! face Darcy fluxes, m/s, + into the domain
    type(c_ptr) :: bc_total(6)                  ! boundary totals, (face cells, ncomp)
    real(c_double) :: bc_saturation(6)
    integer(c_int32_t) :: nsrc
    type(c_ptr) :: src_cell, src_type, src_q, src_total
  end type

  type, bind(C), public :: pf_transport_stats_t
    integer(c_int32_t) :: iterations, converged
    real(c_double) :: max_rel_residual
    integer(c_int32_t) :: refinements, max_cycle_iterations
  end type

  type, bind(C), public :: pf_constraint_reaction_t
    integer(c_int32_t) :: nspec, temperature_dependent
    integer(c_int32_t) :: spec(PF_MAX_NCOMP)
    real(c_double) :: stoich(PF_MAX_NCOMP)
    real(c_double) :: logK
    real(c_double) :: logKcoef(5)
  end type

  type, bind(C), public :: pf_launch_config_t
    integer(c_int32_t) :: threads_per_block, blocks_per_sm, jac_in_shared, lanes_per_cell
  end type

  ! ---------------------------------------------------------- entry points
  public :: pf_network_create, pf_network_destroy, pf_network_set_options, pf_network_reserve, &
            pf_rstep, pf_update_auxvars, pf_update_activity_coefs, pf_rstep_host, pf_rstep_noalloc, pf_rstep_multi, &
            pf_adjoint, pf_network_shift_parameters, pf_girt_pattern, pf_girt_assemble, &
            pf_transport_create, pf_transport_destroy, pf_transport_step, pf_transport_enqueue, &
            pf_transport_read_stats, pf_equilibrate_constraint, pf_equilibrate_constraint_ex, &
            pf_network_set_launch, pf_network_get_launch, pf_version
  public :: pfgpu_osrt_react

  interface
    integer(c_int32_t) function pf_network_create(desc, net) bind(C, name="pf_network_create")
      import :: c_int32_t, c_ptr, pf_network_desc_t
      type(pf_network_desc_t), intent(in) :: desc
      type(c_ptr), intent(out) :: net
    end function
    integer(c_int32_t) function pf_network_destroy(net) bind(C, name="pf_network_destroy")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: net
    end function
    integer(c_int32_t) function pf_network_set_options(net, opts) bind(C, name="pf_network_set_options")
      import :: c_int32_t, c_ptr, pf_options_t
      type(c_ptr), value :: net
      type(pf_options_t), intent(in) :: opts
    end function
    integer(c_int32_t) function pf_network_reserve(net, ncells) bind(C, name="pf_network_reserve")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: net
      integer(c_int64_t), value :: ncells
    end function
    ! device state, a cudaStream_t (c_null_ptr: the default stream); stats optional (c_null_ptr)
    integer(c_int32_t) function pf_rstep(net, state, dt, kernel, stream, stats) bind(C, name="pf_rstep")
      import :: c_int32_t, c_ptr, c_double, pf_cell_state_t
      type(c_ptr), value :: net, stream, stats
      type(pf_cell_state_t), intent(in) :: state
      real(c_double), value :: dt
      integer(c_int32_t), value :: kernel
    end function
    integer(c_int32_t) function pf_update_auxvars(net, state, update_activity_coefs, stream) &
        bind(C, name="pf_update_auxvars")
      import :: c_int32_t, c_ptr, pf_cell_state_t
      type(c_ptr), value :: net, stream
      type(pf_cell_state_t), intent(in) :: state
      integer(c_int32_t), value :: update_activity_coefs
    end function
    integer(c_int32_t) function pf_update_activity_coefs(net, state, stream) &
        bind(C, name="pf_update_activity_coefs")
      import :: c_int32_t, c_ptr, pf_cell_state_t
      type(c_ptr), value :: net, stream
      type(pf_cell_state_t), intent(in) :: state
    end function
    ! host state: the copies happen inside the call
    integer(c_int32_t) function pf_rstep_host(net, state, dt, kernel, stats) bind(C, name="pf_rstep_host")
      import :: c_int32_t, c_ptr, c_double, pf_cell_state_t, pf_step_stats_t
      type(c_ptr), value :: net
      type(pf_cell_state_t), intent(in) :: state
      real(c_double), value :: dt
      integer(c_int32_t), value :: kernel
      type(pf_step_stats_t), intent(out) :: stats
    end function
    integer(c_int32_t) function pf_rstep_noalloc(net, state, dt, stream, stats) bind(C, name="pf_rstep_noalloc")
      import :: c_int32_t, c_ptr, c_double, pf_cell_state_t
      type(c_ptr), value :: net, stream, stats
      type(pf_cell_state_t), intent(in) :: state
      real(c_double), value :: dt
    end function
    ! one persistent launch over several networks' cells; stats: c_null_ptr or c_loc of pf_step_stats_t(nnets)
    integer(c_int32_t) function pf_rstep_multi(nets, states, nnets, dt, stream, stats) bind(C, name="pf_rstep_multi")
      import :: c_int32_t, c_ptr, c_double, pf_cell_state_t
      type(c_ptr), intent(in) :: nets(*)
      type(pf_cell_state_t), intent(in) :: states(*)
      integer(c_int32_t), value :: nnets
      real(c_double), value :: dt
      type(c_ptr), value :: stream, stats
    end function
    integer(c_int32_t) function pf_adjoint(net, state, dt, args, stream) bind(C, name="pf_adjoint")
      import :: c_int32_t, c_ptr, c_double, pf_cell_state_t, pf_adjoint_args_t
      type(c_ptr), value :: net, stream
      type(pf_cell_state_t), intent(in) :: state
      real(c_double), value :: dt
      type(pf_adjoint_args_t), intent(in) :: args
    end function
    integer(c_int32_t) function pf_network_shift_parameters(net, dlogK_sec, dlogK_mnrl, dlnk) &
        bind(C, name="pf_network_shift_parameters")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: net, dlogK_sec, dlogK_mnrl, dlnk
    end function
    integer(c_int32_t) function pf_girt_pattern(nx, ny, nz, rowptr, colidx) bind(C, name="pf_girt_pattern")
      import :: c_int32_t, c_ptr
      integer(c_int32_t), value :: nx, ny, nz
      type(c_ptr), value :: rowptr, colidx
    end function
    integer(c_int32_t) function pf_girt_assemble(net, state, args, stream) bind(C, name="pf_girt_assemble")
      import :: c_int32_t, c_ptr, pf_cell_state_t, pf_girt_args_t
      type(c_ptr), value :: net, stream
      type(pf_cell_state_t), intent(in) :: state
      type(pf_girt_args_t), intent(in) :: args
    end function
    integer(c_int32_t) function pf_transport_create(nx, ny, nz, ncomp, tr) bind(C, name="pf_transport_create")
      import :: c_int32_t, c_ptr
      integer(c_int32_t), value :: nx, ny, nz, ncomp
      type(c_ptr), intent(out) :: tr
    end function
    integer(c_int32_t) function pf_transport_destroy(tr) bind(C, name="pf_transport_destroy")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: tr
    end function
    integer(c_int32_t) function pf_transport_step(tr, args, stream, stats) bind(C, name="pf_transport_step")
      import :: c_int32_t, c_ptr, pf_transport_args_t, pf_transport_stats_t
      type(c_ptr), value :: tr, stream
      type(pf_transport_args_t), intent(in) :: args
      type(pf_transport_stats_t), intent(out) :: stats
    end function
    integer(c_int32_t) function pf_transport_enqueue(tr, args, inner_iterations, refinements, stream) &
        bind(C, name="pf_transport_enqueue")
      import :: c_int32_t, c_ptr, pf_transport_args_t
      type(c_ptr), value :: tr, stream
      type(pf_transport_args_t), intent(in) :: args
      integer(c_int32_t), value :: inner_iterations, refinements
    end function
    integer(c_int32_t) function pf_transport_read_stats(tr, rtol, stream, stats) &
        bind(C, name="pf_transport_read_stats")
      import :: c_int32_t, c_ptr, c_double, pf_transport_stats_t
      type(c_ptr), value :: tr, stream
      real(c_double), value :: rtol
      type(pf_transport_stats_t), intent(out) :: stats
    end function
    integer(c_int32_t) function pf_equilibrate_constraint(net, state, ctype, cconc, use_prev, iterations, stream) &
        bind(C, name="pf_equilibrate_constraint")
      import :: c_int32_t, c_ptr, pf_cell_state_t
      type(c_ptr), value :: net, cconc, iterations, stream
      type(pf_cell_state_t), intent(in) :: state
      integer(c_int32_t), intent(in) :: ctype(*)
      integer(c_int32_t), value :: use_prev
    end function
    integer(c_int32_t) function pf_equilibrate_constraint_ex(net, state, ctype, creact, cconc, use_prev, &
                                                            iterations, stream) &
        bind(C, name="pf_equilibrate_constraint_ex")
      import :: c_int32_t, c_ptr, pf_cell_state_t, pf_constraint_reaction_t
      type(c_ptr), value :: net, cconc, iterations, stream
      type(pf_cell_state_t), intent(in) :: state
      integer(c_int32_t), intent(in) :: ctype(*)
      type(pf_constraint_reaction_t), intent(in) :: creact(*)
      integer(c_int32_t), value :: use_prev
    end function
    integer(c_int32_t) function pf_network_set_launch(net, cfg) bind(C, name="pf_network_set_launch")
      import :: c_int32_t, c_ptr, pf_launch_config_t
      type(c_ptr), value :: net
      type(pf_launch_config_t), intent(in) :: cfg
    end function
    integer(c_int32_t) function pf_network_get_launch(net, cfg) bind(C, name="pf_network_get_launch")
      import :: c_int32_t, c_ptr, pf_launch_config_t
      type(c_ptr), value :: net
      type(pf_launch_config_t), intent(out) :: cfg
    end function
    type(c_ptr) function pf_version() bind(C, name="pf_version")
      import :: c_ptr
    end function
  end interface

contains

  ! The operator-split reaction step for every cell, in place of the loop at
  ! pmc_subsurface_osrt.F90:346-378.  The caller gathers its auxvars into
  ! these arrays (one row per local cell, column per component: the C side's
  ! component-major layout) and scatters them back afterwards, as the
  ! reference's loop reads rt_auxvars(ghosted_id), global_auxvars and
  ! material_auxvars and writes pri_molal back into tran_xx (:372-373).
  ! rstep_error follows the reference's convention (1 when any cell failed;
  ! the MPI_Allreduce of :381 stays with the caller).
  subroutine pfgpu_osrt_react(net, ncells, ncomp, nsec, nmnrl, total, pri_molal, pri_act_coef, &
                              sec_act_coef, sec_molal, mnrl_volfrac, mnrl_area, mnrl_rate, &
                              porosity, saturation, den_kg, volume, temperature, status, &
                              newton_its, num_substeps, dt, rstep_error, sum_newton_iterations, ierr)
    type(c_ptr), intent(in) :: net
    integer, intent(in) :: ncells, ncomp, nsec, nmnrl
    real(c_double), target, intent(inout) :: total(ncells, ncomp), pri_molal(ncells, ncomp), &
        pri_act_coef(ncells, ncomp), sec_act_coef(ncells, max(nsec, 1)), &
        sec_molal(ncells, max(nsec, 1)), mnrl_volfrac(ncells, max(nmnrl, 1)), &
        mnrl_rate(ncells, max(nmnrl, 1))
    real(c_double), target, intent(in) :: mnrl_area(ncells, max(nmnrl, 1)), porosity(ncells), &
        saturation(ncells), den_kg(ncells), volume(ncells), temperature(ncells)
    integer(c_int32_t), target, intent(out) :: status(ncells), newton_its(ncells), num_substeps(ncells)
    real(c_double), intent(in) :: dt
    integer, intent(out) :: rstep_error
    integer(c_int64_t), intent(inout) :: sum_newton_iterations
    integer(c_int32_t), intent(out) :: ierr
    type(pf_cell_state_t) :: state
    type(pf_step_stats_t) :: stats

    state%ncells = int(ncells, c_int64_t)
    state%total = c_loc(total)
    state%pri_molal = c_loc(pri_molal)          ! in: the guess; out: the solution
    state%pri_act_coef = c_loc(pri_act_coef)
    state%sec_act_coef = c_loc(sec_act_coef)
    state%sec_molal = c_loc(sec_molal)
    state%mnrl_volfrac = c_loc(mnrl_volfrac)
    state%mnrl_area = c_loc(mnrl_area)
    state%mnrl_rate = c_loc(mnrl_rate)
    state%porosity = c_loc(porosity)
    state%saturation = c_loc(saturation)
    state%den_kg = c_loc(den_kg)
    state%volume = c_loc(volume)
    state%temperature = c_loc(temperature)
    state%dt_cell = c_null_ptr                  ! option%tran_dt for every cell
    state%status = c_loc(status)
    state%newton_its = c_loc(newton_its)
    state%num_substeps = c_loc(num_substeps)
    state%cell_order = c_null_ptr
    state%total_sorb = c_null_ptr               ! networks without sorption
    state%ionx_ref_sorbed = c_null_ptr
    state%ln_act_h2o = c_null_ptr
    state%srfcplx_free_site = c_null_ptr        ! networks without surface complexation
    state%srfcplx_conc = c_null_ptr
    if (nsec == 0) then
      state%sec_act_coef = c_null_ptr
      state%sec_molal = c_null_ptr
    end if
    ierr = pf_rstep_host(net, state, dt, PF_KERNEL_BATCHED, stats)
    rstep_error = 0
    if (stats%failed_cells > 0) rstep_error = 1
    sum_newton_iterations = sum_newton_iterations + stats%newton_iterations
  end subroutine pfgpu_osrt_react

end module pfgpu_mod
