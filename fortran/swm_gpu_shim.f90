! swm_gpu_shim.f90 -- the GPU bodies behind the reference's module entry points.
!
! The reference keeps its routine names and argument lists; under the CPP
! switch SWM_GPU their bodies call the subroutines below, which drive the C
! ABI of include/swm_gpu.h through swm_gpu_binding.  One context serves the
! model (the reference runs one basin per process).  Error codes become the
! reference's log_fatal; SOR non-convergence becomes its warning.
!
!   SWM_initSWM (swm_module.f90:37-48)          -> gpu_init, after the
!        configuration (model.h switches, &model_nl, &domain_nl) is filled
!        into a swm_gpu_config and the damping/forcing records are added
!   SWM_timestep_step (swm_nonlinear_timestep_module.f90:164-180)
!        and TRC_timestep (tracer_module.f90:109-123) -> gpu_timestep(itt)
!   model_advance (model.f90:238-259)           -> gpu_advance(itt), then
!        gpu_fetch for the registry arrays a diagnostics task writes now
!   init_ElSolv_SOR (ElSolv_SOR.f90:44-66)      -> gpu_sor_init
!   main_ElSolv_SOR (ElSolv_SOR.f90:150-222)    -> gpu_sor_solve
!   SWM_finishSWM (swm_module.f90:56-65)        -> gpu_finish
!
! Not compiled here (this image has no Fortran compiler); the same calls run
! from Python through ctypes in the tests (swm_gb300/model.py).
module swm_gpu_shim
  use iso_c_binding
  use swm_gpu_binding
  use logging, only : log_fatal, log_warn
  implicit none
  private
  type(c_ptr), save, public :: swm_gpu_ctx = c_null_ptr
  public :: gpu_check, gpu_init, gpu_timestep, gpu_advance, gpu_fetch, gpu_sor_init, gpu_sor_solve, gpu_finish

contains

  ! stop with the library's message unless rc is SWM_GPU_OK
  subroutine gpu_check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    if (rc /= SWM_GPU_OK) call log_fatal(what // ": " // c_string(swm_gpu_last_error()))
  end subroutine gpu_check

  ! create the context and set up the domain (H on the H grid, may be
  ! absent) and the time stepping; psi_bs only under LINEARISED_MEAN_STATE
  subroutine gpu_init(cfg, H, psi_bs)
    type(swm_gpu_config), intent(in) :: cfg
    real(c_double), dimension(:, :), intent(in), target, contiguous, optional :: H, psi_bs
    type(c_ptr) :: pH, ppsi
    pH = c_null_ptr
    ppsi = c_null_ptr
    if (present(H)) pH = c_loc(H)
    if (present(psi_bs)) ppsi = c_loc(psi_bs)
    call gpu_check(swm_gpu_create(cfg, swm_gpu_ctx), "swm_gpu_create")
    call gpu_check(swm_gpu_domain(swm_gpu_ctx, pH, c_null_ptr), "swm_gpu_domain")
    call gpu_check(swm_gpu_timestep_init(swm_gpu_ctx, ppsi), "swm_gpu_timestep_init")
  end subroutine gpu_init

  subroutine gpu_timestep(itt)
    integer, intent(in) :: itt
    call gpu_check(swm_gpu_step(swm_gpu_ctx, int(itt, c_int64_t)), "swm_gpu_step")
  end subroutine gpu_timestep

  subroutine gpu_advance(itt)
    integer, intent(in) :: itt
    call gpu_check(swm_gpu_advance(swm_gpu_ctx, int(itt, c_int64_t)), "swm_gpu_advance")
  end subroutine gpu_advance

  ! the current device copy of a registry field (SWM_F_*) into arr(Nx, Ny)
  subroutine gpu_fetch(field, arr)
    integer(c_int), intent(in) :: field
    real(c_double), dimension(:, :), intent(inout), target, contiguous :: arr
    call gpu_check(swm_gpu_get_field(swm_gpu_ctx, field, c_loc(arr)), "swm_gpu_get_field")
  end subroutine gpu_fetch

  subroutine gpu_sor_init()
    call gpu_check(elsolv_sor_gpu_init(swm_gpu_ctx), "elsolv_sor_gpu_init")
  end subroutine gpu_sor_init

  ! main_ElSolv_SOR(B, chi, epsilon, first_guess): chi holds the first guess
  ! on entry and the solution on return
  subroutine gpu_sor_solve(B, chi, epsilon, first_guess)
    real(c_double), dimension(:, :), intent(in), target, contiguous :: B
    real(c_double), dimension(:, :), intent(inout), target, contiguous :: chi
    real(c_double), intent(in) :: epsilon
    logical, intent(in) :: first_guess
    integer(c_int) :: rc
    integer(c_int), target :: iters
    real(c_double), target :: anorm
    integer(c_int) :: fg
    fg = 0
    if (first_guess) fg = 1
    rc = elsolv_sor_gpu_solve(swm_gpu_ctx, c_loc(B), c_loc(chi), epsilon, fg, c_loc(iters), c_loc(anorm))
    if (rc == SWM_GPU_ENOT_CONVERGED) then
      call log_warn("main_ElSolv_SOR: maximum number of iterations reached")
    else
      call gpu_check(rc, "elsolv_sor_gpu_solve")
    end if
  end subroutine gpu_sor_solve

  subroutine gpu_finish()
    integer(c_int) :: rc
    if (c_associated(swm_gpu_ctx)) rc = swm_gpu_destroy(swm_gpu_ctx)
    swm_gpu_ctx = c_null_ptr
  end subroutine gpu_finish

end module swm_gpu_shim
