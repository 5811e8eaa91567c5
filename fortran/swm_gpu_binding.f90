! swm_gpu_binding.f90 -- ISO_C_BINDING interfaces of include/swm_gpu.h.
!
! Written by fortran/gen_binding.py from the header; do not edit by hand.
! Every pointer argument is type(c_ptr), value: pass c_loc(array) of the
! Fortran (Nx, Ny) array (column-major = the C [Ny][Nx] layout the ABI
! uses) or c_null_ptr; handles (contexts, ensembles, solvers) are
! type(c_ptr).  Every integer function returns SWM_GPU_OK or an error
! code; c_string(swm_gpu_last_error()) is the message.
! Not compiled here (this image has no Fortran compiler).
module swm_gpu_binding
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SWM_GPU_OK = 0
  integer(c_int), parameter :: SWM_GPU_EINVAL = 1
  integer(c_int), parameter :: SWM_GPU_ECUDA = 2
  integer(c_int), parameter :: SWM_GPU_ENOMEM = 3
  integer(c_int), parameter :: SWM_GPU_ENOT_CONVERGED = 4
  integer(c_int), parameter :: SWM_GPU_EDEVICE = 5
  integer(c_int), parameter :: SWM_MODE_NONE = 0
  integer(c_int), parameter :: SWM_MODE_NONLINEAR = 1
  integer(c_int), parameter :: SWM_MODE_LIN_REST = 2
  integer(c_int), parameter :: SWM_MODE_LIN_MEAN = 3
  integer(c_int), parameter :: SWM_MIX_LAPLACE = 0
  integer(c_int), parameter :: SWM_MIX_BIHARMONIC = 1
  integer(c_int), parameter :: SWM_PATH_PLAIN_FP64 = 0
  integer(c_int), parameter :: SWM_PATH_FUSED_FP64 = 1
  integer(c_int), parameter :: SWM_PATH_FUSED_FP32C = 2
  integer(c_int), parameter :: SWM_F_U = 0
  integer(c_int), parameter :: SWM_F_V = 1
  integer(c_int), parameter :: SWM_F_ETA = 2
  integer(c_int), parameter :: SWM_F_D = 3
  integer(c_int), parameter :: SWM_F_DH = 4
  integer(c_int), parameter :: SWM_F_DU = 5
  integer(c_int), parameter :: SWM_F_DV = 6
  integer(c_int), parameter :: SWM_F_EDENS = 7
  integer(c_int), parameter :: SWM_F_POT = 8
  integer(c_int), parameter :: SWM_F_ZETA = 9
  integer(c_int), parameter :: SWM_F_MU = 10
  integer(c_int), parameter :: SWM_F_MV = 11
  integer(c_int), parameter :: SWM_F_H = 12
  integer(c_int), parameter :: SWM_F_HU = 13
  integer(c_int), parameter :: SWM_F_HV = 14
  integer(c_int), parameter :: SWM_F_HETA = 15
  integer(c_int), parameter :: SWM_F_IMPL_U = 16
  integer(c_int), parameter :: SWM_F_IMPL_V = 17
  integer(c_int), parameter :: SWM_F_IMPL_ETA = 18
  integer(c_int), parameter :: SWM_F_GAMMA_LIN_U = 19
  integer(c_int), parameter :: SWM_F_GAMMA_LIN_V = 20
  integer(c_int), parameter :: SWM_F_GAMMA_LIN_ETA = 21
  integer(c_int), parameter :: SWM_F_GAMMA_SQ_U = 22
  integer(c_int), parameter :: SWM_F_GAMMA_SQ_V = 23
  integer(c_int), parameter :: SWM_F_FX = 24
  integer(c_int), parameter :: SWM_F_FY = 25
  integer(c_int), parameter :: SWM_F_FETA = 26
  integer(c_int), parameter :: SWM_F_U_BS = 27
  integer(c_int), parameter :: SWM_F_V_BS = 28
  integer(c_int), parameter :: SWM_F_ZETA_BS = 29
  integer(c_int), parameter :: SWM_F_LATMIX_U = 30
  integer(c_int), parameter :: SWM_F_LATMIX_V = 31
  integer(c_int), parameter :: SWM_F_GU = 32
  integer(c_int), parameter :: SWM_F_GV = 33
  integer(c_int), parameter :: SWM_F_GETA = 34
  integer(c_int), parameter :: SWM_F_PSI = 35
  integer(c_int), parameter :: SWM_F_NFIELDS = 36
  integer(c_int), parameter :: SWM_TERM_GAMMA_LIN_U = 0
  integer(c_int), parameter :: SWM_TERM_GAMMA_LIN_V = 1
  integer(c_int), parameter :: SWM_TERM_GAMMA_LIN_ETA = 2
  integer(c_int), parameter :: SWM_TERM_GAMMA_SQ_U = 3
  integer(c_int), parameter :: SWM_TERM_GAMMA_SQ_V = 4
  integer(c_int), parameter :: SWM_DAMP_UNIFORM = 0
  integer(c_int), parameter :: SWM_DAMP_SPONGE = 1
  integer(c_int), parameter :: SWM_DAMP_FILE = 2
  integer(c_int), parameter :: SWM_SPONGE_N = 1
  integer(c_int), parameter :: SWM_SPONGE_S = 2
  integer(c_int), parameter :: SWM_SPONGE_W = 4
  integer(c_int), parameter :: SWM_SPONGE_E = 8
  integer(c_int), parameter :: SWM_FRC_WIND = 0
  integer(c_int), parameter :: SWM_FRC_OSC = 1
  integer(c_int), parameter :: SWM_FRC_CUSTOM = 2
  integer(c_int), parameter :: SWM_FRC_HEAT = 3
  integer(c_int), parameter :: SWM_FRC_EMF = 4
  integer(c_int), parameter :: SWM_CMP_ZONAL = 0
  integer(c_int), parameter :: SWM_CMP_MERID = 1
  integer(c_int), parameter :: SWM_CMP_CONT = 2
  integer(c_int), parameter :: SWM_CMP_U2 = 3
  integer(c_int), parameter :: SWM_CMP_V2 = 4
  integer(c_int), parameter :: SWM_CMP_REY = 5
  integer(c_int), parameter :: TRC_F_CH = 0
  integer(c_int), parameter :: TRC_F_C = 1
  integer(c_int), parameter :: TRC_F_G = 2
  integer(c_int), parameter :: TRC_F_UHC = 3
  integer(c_int), parameter :: TRC_F_VHC = 4
  integer(c_int), parameter :: TRC_F_DIFF = 5
  integer(c_int), parameter :: TRC_F_IMPL = 6
  integer(c_int), parameter :: SWM_NOALLOC_MAX_NY = 8192

  type, bind(C) :: swm_gpu_config
    integer(c_int32_t) :: nx, ny
    integer(c_int32_t) :: mode
    integer(c_int32_t) :: lateral_mixing
    integer(c_int32_t) :: quadratic_friction
    integer(c_int32_t) :: barotropic
    integer(c_int32_t) :: mixing_kind
    integer(c_int32_t) :: coriolis_approx
    integer(c_int32_t) :: tracer_nan_guard
    integer(c_int32_t) :: damping_additive
    integer(c_int32_t) :: mask_psi_bs
    integer(c_int32_t) :: tracer_flux
    integer(c_int32_t) :: frozen_flow
    real(c_double) :: dt, G, Ah, A, OMEGA, RHO0
    real(c_double) :: lbc, theta0
    real(c_double) :: lon_s, lon_e, lat_s, lat_e
    real(c_double) :: H_overwrite
    real(c_double) :: ab_chi, minD
    real(c_double) :: tau_scale
    real(c_double) :: bih
    integer(c_int32_t) :: path
    integer(c_int32_t) :: reserved
  end type swm_gpu_config

  interface
    function swm_gpu_last_error() bind(C) result(res)
      import :: c_ptr
      type(c_ptr) :: res
    end function swm_gpu_last_error
    integer(c_int) function swm_gpu_create(cfg, out_) bind(C)
      import :: c_int, c_ptr, swm_gpu_config
      type(swm_gpu_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: out_
    end function swm_gpu_create
    integer(c_int) function swm_gpu_destroy(ctx) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function swm_gpu_destroy
    integer(c_int) function swm_gpu_synchronize(ctx) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function swm_gpu_synchronize
    function swm_gpu_stream(ctx) bind(C) result(res)
      import :: c_ptr
      type(c_ptr) :: res
      type(c_ptr), value :: ctx
    end function swm_gpu_stream
    integer(c_int64_t) function swm_gpu_launch_count(ctx) bind(C)
      import :: c_int64_t, c_ptr
      type(c_ptr), value :: ctx
    end function swm_gpu_launch_count
    integer(c_int) function swm_gpu_step_shape(ctx, rows, masked_cost, blocks) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: rows
      type(c_ptr), value :: masked_cost
      type(c_ptr), value :: blocks
    end function swm_gpu_step_shape
    integer(c_int) function swm_gpu_plan_step_tiles(mixing, nx, ny, mask_words, rows, masked_cost, &
        tiles, capacity) bind(C)
      import :: c_double, c_int, c_ptr
      integer(c_int), value :: mixing
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      type(c_ptr), value :: mask_words
      real(c_double), value :: rows
      real(c_double), value :: masked_cost
      type(c_ptr), value :: tiles
      integer(c_int), value :: capacity
    end function swm_gpu_plan_step_tiles
    integer(c_int) function swm_gpu_step_strip_columns(mixing) bind(C)
      import :: c_int
      integer(c_int), value :: mixing
    end function swm_gpu_step_strip_columns
    integer(c_int) function swm_gpu_domain(ctx, H, H_missing) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: H
      type(c_ptr), value :: H_missing
    end function swm_gpu_domain
    integer(c_int) function swm_gpu_timestep_init(ctx, psi_bs) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: psi_bs
    end function swm_gpu_timestep_init
    integer(c_int) function swm_gpu_add_damping(ctx, term, typ, value, sl_length, sl_cutoff, &
        sponge_flags, file_data) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: term
      integer(c_int), value :: typ
      real(c_double), value :: value
      real(c_double), value :: sl_length
      real(c_double), value :: sl_cutoff
      integer(c_int), value :: sponge_flags
      type(c_ptr), value :: file_data
    end function swm_gpu_add_damping
    integer(c_int) function swm_gpu_finish_damping(ctx) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function swm_gpu_finish_damping
    integer(c_int) function swm_gpu_add_stream(ctx, typ, component, omega, is_constant, d1, d2, &
        id) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: typ
      integer(c_int), value :: component
      real(c_double), value :: omega
      integer(c_int), value :: is_constant
      type(c_ptr), value :: d1
      type(c_ptr), value :: d2
      type(c_ptr), value :: id
    end function swm_gpu_add_stream
    integer(c_int) function swm_gpu_set_stream_data(ctx, id, d1, d2) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: id
      type(c_ptr), value :: d1
      type(c_ptr), value :: d2
    end function swm_gpu_set_stream_data
    integer(c_int) function swm_gpu_set_stream_rows(ctx, id, rows1, rows2) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: id
      type(c_ptr), value :: rows1
      type(c_ptr), value :: rows2
    end function swm_gpu_set_stream_rows
    integer(c_int) function swm_gpu_stream_records(ctx, id, part, nrec, records) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: id
      integer(c_int), value :: part
      integer(c_int), value :: nrec
      type(c_ptr), value :: records
    end function swm_gpu_stream_records
    integer(c_int) function swm_gpu_stream_interp(ctx, id, part, r0, r1, t, t0, t1) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: id
      integer(c_int), value :: part
      integer(c_int), value :: r0
      integer(c_int), value :: r1
      real(c_double), value :: t
      real(c_double), value :: t0
      real(c_double), value :: t1
    end function swm_gpu_stream_interp
    integer(c_int) function swm_gpu_forcing_init(ctx) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function swm_gpu_forcing_init
    integer(c_int) function swm_gpu_initial_conditions(ctx, eta, u, v) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: eta
      type(c_ptr), value :: u
      type(c_ptr), value :: v
    end function swm_gpu_initial_conditions
    integer(c_int) function swm_gpu_step(ctx, itt) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: itt
    end function swm_gpu_step
    integer(c_int) function swm_gpu_advance(ctx, itt) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: itt
    end function swm_gpu_advance
    integer(c_int) function swm_gpu_run(ctx, itt0, nsteps) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: itt0
      integer(c_int64_t), value :: nsteps
    end function swm_gpu_run
    integer(c_int) function swm_gpu_run_monitor(ctx, itt0, nsteps, stream_id, rows1, rows2, &
        out3) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: itt0
      integer(c_int64_t), value :: nsteps
      integer(c_int), value :: stream_id
      type(c_ptr), value :: rows1
      type(c_ptr), value :: rows2
      type(c_ptr), value :: out3
    end function swm_gpu_run_monitor
    integer(c_int) function swm_gpu_get_field(ctx, field, host_out) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      type(c_ptr), value :: host_out
    end function swm_gpu_get_field
    integer(c_int) function swm_gpu_set_field(ctx, field, host_in) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      type(c_ptr), value :: host_in
    end function swm_gpu_set_field
    integer(c_int) function swm_gpu_get_field_async(ctx, field, host_out, ticket) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      type(c_ptr), value :: host_out
      type(c_ptr), value :: ticket
    end function swm_gpu_get_field_async
    integer(c_int) function swm_gpu_wait(ctx, ticket) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: ticket
    end function swm_gpu_wait
    integer(c_int) function swm_gpu_ready(ctx, ticket) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: ticket
    end function swm_gpu_ready
    integer(c_int) function swm_gpu_host_register(host, bytes) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: host
      integer(c_int64_t), value :: bytes
    end function swm_gpu_host_register
    integer(c_int) function swm_gpu_host_unregister(host) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: host
    end function swm_gpu_host_unregister
    integer(c_int) function swm_gpu_get_metric(ctx, which, grid, host_out) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: which
      integer(c_int), value :: grid
      type(c_ptr), value :: host_out
    end function swm_gpu_get_metric
    integer(c_int) function swm_gpu_get_mask(ctx, grid, host_out) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: grid
      type(c_ptr), value :: host_out
    end function swm_gpu_get_mask
    integer(c_int) function swm_gpu_streamfunction(ctx, psi_out) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: psi_out
    end function swm_gpu_streamfunction
    integer(c_int) function swm_gpu_diag_accumulate(ctx, slot, field, square, weight) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: slot
      integer(c_int), value :: field
      integer(c_int), value :: square
      real(c_double), value :: weight
    end function swm_gpu_diag_accumulate
    integer(c_int) function swm_gpu_diag_mean(ctx, slot, host_out, count_out) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: slot
      type(c_ptr), value :: host_out
      type(c_ptr), value :: count_out
    end function swm_gpu_diag_mean
    integer(c_int) function swm_gpu_integrals(ctx, out3) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: out3
    end function swm_gpu_integrals
    integer(c_int) function swm_gpu_integrals_async(ctx, out3, ticket) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: out3
      type(c_ptr), value :: ticket
    end function swm_gpu_integrals_async
    integer(c_int) function swm_gpu_integrals_noalloc(ctx, out3) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: out3
    end function swm_gpu_integrals_noalloc
    integer(c_int) function swm_gpu_ensemble_create(members, n, out_) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), intent(out) :: members
      integer(c_int), value :: n
      type(c_ptr), intent(out) :: out_
    end function swm_gpu_ensemble_create
    integer(c_int) function swm_gpu_ensemble_destroy(ens) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
    end function swm_gpu_ensemble_destroy
    integer(c_int) function swm_gpu_ensemble_run(ens, itt0, nsteps) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ens
      integer(c_int64_t), value :: itt0
      integer(c_int64_t), value :: nsteps
    end function swm_gpu_ensemble_run
    integer(c_int) function swm_gpu_ensemble_integrals(ens, out_) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
      type(c_ptr), value :: out_
    end function swm_gpu_ensemble_integrals
    integer(c_int) function swm_gpu_ensemble_run_monitor(ens, itt0, nsteps, rows, out_) bind(C)
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ens
      integer(c_int64_t), value :: itt0
      integer(c_int64_t), value :: nsteps
      type(c_ptr), value :: rows
      type(c_ptr), value :: out_
    end function swm_gpu_ensemble_run_monitor
    integer(c_int) function swm_gpu_ensemble_synchronize(ens) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
    end function swm_gpu_ensemble_synchronize
    function swm_gpu_ensemble_stream(ens) bind(C) result(res)
      import :: c_ptr
      type(c_ptr) :: res
      type(c_ptr), value :: ens
    end function swm_gpu_ensemble_stream
    integer(c_int64_t) function swm_gpu_ensemble_launch_count(ens) bind(C)
      import :: c_int64_t, c_ptr
      type(c_ptr), value :: ens
    end function swm_gpu_ensemble_launch_count
    integer(c_int) function swm_gpu_ensemble_rows(ens) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
    end function swm_gpu_ensemble_rows
    integer(c_int) function trc_gpu_add(ctx, kappa_h, cons, gamma_c, C, C0, gamma_field, &
        cons_field, id) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), value :: kappa_h
      real(c_double), value :: cons
      real(c_double), value :: gamma_c
      type(c_ptr), value :: C
      type(c_ptr), value :: C0
      type(c_ptr), value :: gamma_field
      type(c_ptr), value :: cons_field
      type(c_ptr), value :: id
    end function trc_gpu_add
    integer(c_int) function trc_gpu_init(ctx) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function trc_gpu_init
    integer(c_int) function trc_gpu_get_field(ctx, tracer, field, host_out) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: tracer
      integer(c_int), value :: field
      type(c_ptr), value :: host_out
    end function trc_gpu_get_field
    integer(c_int) function elsolv_sor_gpu_init(ctx) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function elsolv_sor_gpu_init
    integer(c_int) function elsolv_sor_gpu_solve(ctx, B, chi, eps, first_guess, iterations, &
        anorm) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), value :: B
      type(c_ptr), value :: chi
      real(c_double), value :: eps
      integer(c_int), value :: first_guess
      type(c_ptr), value :: iterations
      type(c_ptr), value :: anorm
    end function elsolv_sor_gpu_solve
    integer(c_int) function swm_gpu_nondivergent(ctx, first_guess, eps, u_nd, v_nd, chi, &
        iterations) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: first_guess
      real(c_double), value :: eps
      type(c_ptr), value :: u_nd
      type(c_ptr), value :: v_nd
      type(c_ptr), value :: chi
      type(c_ptr), value :: iterations
    end function swm_gpu_nondivergent
    integer(c_int) function swm_gpu_check_division(n, seed, mismatches) bind(C)
      import :: c_int, c_int64_t, c_ptr
      integer(c_int64_t), value :: n
      integer(c_int64_t), value :: seed
      type(c_ptr), value :: mismatches
    end function swm_gpu_check_division
    integer(c_int) function swm_helm_create(nx, ny, dx, dy, lambda, H, ocean, out_) bind(C)
      import :: c_double, c_int, c_ptr
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      real(c_double), value :: dx
      real(c_double), value :: dy
      real(c_double), value :: lambda
      type(c_ptr), value :: H
      type(c_ptr), value :: ocean
      type(c_ptr), intent(out) :: out_
    end function swm_helm_create
    integer(c_int) function swm_helm_destroy(h) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function swm_helm_destroy
    function swm_helm_stream(h) bind(C) result(res)
      import :: c_ptr
      type(c_ptr) :: res
      type(c_ptr), value :: h
    end function swm_helm_stream
    integer(c_int64_t) function swm_helm_launch_count(h) bind(C)
      import :: c_int64_t, c_ptr
      type(c_ptr), value :: h
    end function swm_helm_launch_count
    integer(c_int) function swm_helm_apply(h, psi, out_) bind(C)
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: psi
      type(c_ptr), value :: out_
    end function swm_helm_apply
    integer(c_int) function swm_helm_solve_fp64(h, rhs, psi, omega, rtol, max_sweeps, sweeps, &
        relres) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: rhs
      type(c_ptr), value :: psi
      real(c_double), value :: omega
      real(c_double), value :: rtol
      integer(c_int), value :: max_sweeps
      type(c_ptr), value :: sweeps
      type(c_ptr), value :: relres
    end function swm_helm_solve_fp64
    integer(c_int) function swm_helm_solve_mixed(h, rhs, psi, omega, rtol, inner_tol, max_sweeps, &
        sweeps, outer, relres) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: rhs
      type(c_ptr), value :: psi
      real(c_double), value :: omega
      real(c_double), value :: rtol
      real(c_double), value :: inner_tol
      integer(c_int), value :: max_sweeps
      type(c_ptr), value :: sweeps
      type(c_ptr), value :: outer
      type(c_ptr), value :: relres
    end function swm_helm_solve_mixed
    integer(c_int) function swm_helm_autotune(h, rhs, omega_lo, omega_hi, ngrid, trial_sweeps, &
        omega, block_x, block_y) bind(C)
      import :: c_double, c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: rhs
      real(c_double), value :: omega_lo
      real(c_double), value :: omega_hi
      integer(c_int), value :: ngrid
      integer(c_int), value :: trial_sweeps
      type(c_ptr), value :: omega
      type(c_ptr), value :: block_x
      type(c_ptr), value :: block_y
    end function swm_helm_autotune
  end interface

contains

  ! the NUL-terminated C string p as a Fortran string
  function c_string(p) result(s)
    type(c_ptr), intent(in) :: p
    character(len=:), allocatable :: s
    character(kind=c_char), pointer :: a(:)
    integer :: n
    s = ""
    if (.not. c_associated(p)) return
    call c_f_pointer(p, a, [4096])
    n = 0
    do while (n < 4096)
      if (a(n + 1) == c_null_char) exit
      n = n + 1
    end do
    allocate(character(len=n) :: s)
    s = transfer(a(1:n), s)
  end function c_string

end module swm_gpu_binding
