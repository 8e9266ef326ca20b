! funwave_gpu.F90 -- ISO_C_BINDING interface of libfunwave_gpu for a Fortran
! host (the reference's own driver, src/main.F), one interface per entry
! point of funwave_gpu.h.
!
! FW_PARAMS mirrors the C struct fw_params field by field, in the same order
! and with the same types (C_INT for int, C_DOUBLE for double), so that
! fw_params_default and fw_create read and write exactly the caller's
! object.  tests/test_fortran_module.py checks the field list, every bound
! name and every argument count against funwave_gpu.h.
!
! Host arrays are the reference's MODULE GLOBAL arrays (Eta(Mloc,Nloc),
! P(Mloc1,Nloc), Q(Mloc,Nloc1), ...), Fortran-ordered with their ghost
! cells.  A build with -DDOUBLE_PRECISION passes them to fw_get_field /
! fw_set_field (REAL(8)); a single-precision build (REAL(SP) = REAL(4),
! mod_param.F:58-68) passes them to fw_get_field_f32 / fw_set_field_f32.
! Masks are default INTEGER in both.  Names are NUL-terminated:
! 'Eta'//C_NULL_CHAR.
MODULE FUNWAVE_GPU
  USE ISO_C_BINDING
  IMPLICIT NONE

  INTEGER(C_INT), PARAMETER :: FW_OK = 0
  INTEGER(C_INT), PARAMETER :: FW_ERR_CUDA = -1, FW_ERR_OOM = -2, FW_ERR_BAD_PARAM = -3
  INTEGER(C_INT), PARAMETER :: FW_ERR_BLOWUP = -4, FW_ERR_NAN = -5, FW_ERR_UNSUPPORTED = -6
  INTEGER(C_INT), PARAMETER :: FW_ERR_NOT_READY = -7, FW_ERR_NO_DEVICE = -8, FW_ERR_IO = -9
  INTEGER(C_INT), PARAMETER :: FW_ERR_TIMEOUT = -10
  INTEGER(C_INT), PARAMETER :: FW_PREC_FP64 = 0, FW_PREC_MIXED = 1
  INTEGER(C_INT), PARAMETER :: FW_WK_NONE = 0, FW_WK_REG = 1, FW_WK_JON_2D = 2
  INTEGER(C_INT), PARAMETER :: FW_SPREAD_WRAPPED_NORMAL = 0, FW_SPREAD_COS2S = 1
  INTEGER(C_INT), PARAMETER :: FW_TUNE_LEN = 14, FW_TUNE_FRESH = 1
  INTEGER(C_LONG_LONG), PARAMETER :: FW_DT_DEVICE_MAX_CELLS = 134217728_C_LONG_LONG

  ! the input.txt keys of the hot path (fw_params of funwave_gpu.h)
  TYPE, BIND(C) :: FW_PARAMS
    INTEGER(C_INT) :: Mglob, Nglob
    REAL(C_DOUBLE) :: DX, DY
    INTEGER(C_INT) :: periodic
    INTEGER(C_INT) :: dispersion
    REAL(C_DOUBLE) :: gamma1, gamma2, gamma3, beta_ref
    INTEGER(C_INT) :: viscosity_breaking
    INTEGER(C_INT) :: show_breaking
    REAL(C_DOUBLE) :: cbrk1, cbrk2
    REAL(C_DOUBLE) :: wavemaker_cbrk
    REAL(C_DOUBLE) :: nu_bkg
    REAL(C_DOUBLE) :: swe_eta_dep
    REAL(C_DOUBLE) :: cfl
    INTEGER(C_INT) :: fixed_dt
    REAL(C_DOUBLE) :: dt_fixed
    REAL(C_DOUBLE) :: froude_cap
    REAL(C_DOUBLE) :: min_depth
    REAL(C_DOUBLE) :: min_depth_frc
    INTEGER(C_INT) :: eta_limiter
    REAL(C_DOUBLE) :: trough_limit, crest_limit
    INTEGER(C_INT) :: direct_sponge
    REAL(C_DOUBLE) :: sponge_west, sponge_east, sponge_south, sponge_north
    REAL(C_DOUBLE) :: r_sponge, a_sponge
    INTEGER(C_INT) :: friction_sponge
    REAL(C_DOUBLE) :: cd_fixed
    INTEGER(C_INT) :: wavemaker
    REAL(C_DOUBLE) :: amp_wk, tperiod, dep_wk, xc_wk, yc_wk, theta_wk, delta_wk
    REAL(C_DOUBLE) :: time_ramp, ywidth_wk
    REAL(C_DOUBLE) :: freq_peak, freq_min, freq_max
    REAL(C_DOUBLE) :: gamma_tma, hmo, theta_peak, sigma_theta
    INTEGER(C_INT) :: nfreq, ntheta
    INTEGER(C_INT) :: spreading
    REAL(C_DOUBLE) :: spread_s
    INTEGER(C_INT) :: precision
    INTEGER(C_INT) :: device
    INTEGER(C_INT) :: track_hmax
    INTEGER(C_INT) :: track_hmin, track_umax, track_mfmax
    REAL(C_DOUBLE) :: steady_time
    REAL(C_DOUBLE) :: t_intv_mean
    INTEGER(C_INT) :: track_roller
    INTEGER(C_INT) :: track_radiation
  END TYPE FW_PARAMS

  INTERFACE
    ! --- context --------------------------------------------------------
    SUBROUTINE fw_params_default(p) BIND(C, NAME="fw_params_default")
      IMPORT :: FW_PARAMS
      TYPE(FW_PARAMS), INTENT(OUT) :: p
    END SUBROUTINE
    INTEGER(C_INT) FUNCTION fw_create(p, ctx) BIND(C, NAME="fw_create")
      IMPORT :: C_INT, C_PTR, FW_PARAMS
      TYPE(FW_PARAMS), INTENT(IN) :: p
      TYPE(C_PTR), INTENT(OUT) :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_destroy(ctx) BIND(C, NAME="fw_destroy")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    ! depth: Mglob x Nglob; eta, u, v, phases: C_LOC(...) or C_NULL_PTR
    INTEGER(C_INT) FUNCTION fw_init(ctx, depth, eta, u, v, phases) BIND(C, NAME="fw_init")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: depth(*)
      TYPE(C_PTR), VALUE :: eta, u, v, phases
    END FUNCTION

    ! --- fields and scalars ---------------------------------------------
    ! host: C_LOC of a REAL(8) array (INTEGER for MASK, MASK9, MASK_STRUC)
    INTEGER(C_INT) FUNCTION fw_get_field(ctx, name, host) BIND(C, NAME="fw_get_field")
      IMPORT :: C_INT, C_PTR, C_CHAR
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      TYPE(C_PTR), VALUE :: host
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_set_field(ctx, name, host) BIND(C, NAME="fw_set_field")
      IMPORT :: C_INT, C_PTR, C_CHAR
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      TYPE(C_PTR), VALUE :: host
    END FUNCTION
    ! REAL(4) host arrays of a single-precision build (not the masks)
    INTEGER(C_INT) FUNCTION fw_get_field_f32(ctx, name, host) BIND(C, NAME="fw_get_field_f32")
      IMPORT :: C_INT, C_PTR, C_CHAR, C_FLOAT
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      REAL(C_FLOAT), INTENT(OUT) :: host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_set_field_f32(ctx, name, host) BIND(C, NAME="fw_set_field_f32")
      IMPORT :: C_INT, C_PTR, C_CHAR, C_FLOAT
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      REAL(C_FLOAT), INTENT(IN) :: host(*)
    END FUNCTION
    ! names(k) = C_LOC of a NUL-terminated name, host(k) = C_LOC of its array
    INTEGER(C_INT) FUNCTION fw_set_fields_f32(ctx, n, names, host) BIND(C, NAME="fw_set_fields_f32")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: n
      TYPE(C_PTR), INTENT(IN) :: names(*), host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_get_fields_f32(ctx, n, names, host) BIND(C, NAME="fw_get_fields_f32")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: n
      TYPE(C_PTR), INTENT(IN) :: names(*), host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_set_fields(ctx, n, names, host) BIND(C, NAME="fw_set_fields")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: n
      TYPE(C_PTR), INTENT(IN) :: names(*), host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_get_fields(ctx, n, names, host) BIND(C, NAME="fw_get_fields")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: n
      TYPE(C_PTR), INTENT(IN) :: names(*), host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_get_points(ctx, name, n, I, J, out) BIND(C, NAME="fw_get_points")
      IMPORT :: C_INT, C_PTR, C_CHAR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      INTEGER(C_INT), VALUE :: n
      INTEGER(C_INT), INTENT(IN) :: I(*), J(*)
      REAL(C_DOUBLE), INTENT(OUT) :: out(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_get_scalar(ctx, name, val) BIND(C, NAME="fw_get_scalar")
      IMPORT :: C_INT, C_PTR, C_CHAR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      REAL(C_DOUBLE), INTENT(OUT) :: val
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_set_scalar(ctx, name, val) BIND(C, NAME="fw_set_scalar")
      IMPORT :: C_INT, C_PTR, C_CHAR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      REAL(C_DOUBLE), VALUE :: val
    END FUNCTION

    ! --- time stepping (main.F:284-535) --------------------------------
    INTEGER(C_INT) FUNCTION fw_begin_step(ctx) BIND(C, NAME="fw_begin_step")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_stage(ctx, istage) BIND(C, NAME="fw_stage")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: istage
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_end_step(ctx, status) BIND(C, NAME="fw_end_step")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), INTENT(OUT) :: status
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_step(ctx, nsteps, status) BIND(C, NAME="fw_step")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: nsteps
      INTEGER(C_INT), INTENT(OUT) :: status
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_step_async(ctx, nsteps) BIND(C, NAME="fw_step_async")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: nsteps
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_step_wait(ctx, status) BIND(C, NAME="fw_step_wait")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), INTENT(OUT) :: status
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_sync(ctx) BIND(C, NAME="fw_sync")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION

    ! --- ensembles of independent runs ----------------------------------
    INTEGER(C_INT) FUNCTION fw_ensemble_step(ctxs, n, nsteps, status) BIND(C, NAME="fw_ensemble_step")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), INTENT(IN) :: ctxs(*)
      INTEGER(C_INT), VALUE :: n, nsteps
      INTEGER(C_INT), INTENT(OUT) :: status(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_ensemble_create(ctxs, n, ens) BIND(C, NAME="fw_ensemble_create")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), INTENT(IN) :: ctxs(*)
      INTEGER(C_INT), VALUE :: n
      TYPE(C_PTR), INTENT(OUT) :: ens
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_ensemble_run(ens, nsteps, status) BIND(C, NAME="fw_ensemble_run")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ens
      INTEGER(C_INT), VALUE :: nsteps
      INTEGER(C_INT), INTENT(OUT) :: status(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_ensemble_destroy(ens) BIND(C, NAME="fw_ensemble_destroy")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ens
    END FUNCTION

    ! --- learned coarse-grid correction (device tensors as C_PTR) --------
    INTEGER(C_INT) FUNCTION fw_net_create(seed, net) BIND(C, NAME="fw_net_create")
      IMPORT :: C_INT, C_PTR, C_LONG_LONG
      INTEGER(C_LONG_LONG), VALUE :: seed
      TYPE(C_PTR), INTENT(OUT) :: net
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_destroy(net) BIND(C, NAME="fw_net_destroy")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: net
    END FUNCTION
    INTEGER(C_LONG_LONG) FUNCTION fw_net_num_params(net) BIND(C, NAME="fw_net_num_params")
      IMPORT :: C_LONG_LONG, C_PTR
      TYPE(C_PTR), VALUE :: net
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_get_params(net, host) BIND(C, NAME="fw_net_get_params")
      IMPORT :: C_INT, C_PTR, C_FLOAT
      TYPE(C_PTR), VALUE :: net
      REAL(C_FLOAT), INTENT(OUT) :: host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_set_params(net, host) BIND(C, NAME="fw_net_set_params")
      IMPORT :: C_INT, C_PTR, C_FLOAT
      TYPE(C_PTR), VALUE :: net
      REAL(C_FLOAT), INTENT(IN) :: host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_get_grads(net, host) BIND(C, NAME="fw_net_get_grads")
      IMPORT :: C_INT, C_PTR, C_FLOAT
      TYPE(C_PTR), VALUE :: net
      REAL(C_FLOAT), INTENT(OUT) :: host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_forward(net, x, B, H, W, y, stream) BIND(C, NAME="fw_net_forward")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: net, x
      INTEGER(C_INT), VALUE :: B, H, W
      TYPE(C_PTR), VALUE :: y, stream
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_loss_grad(net, x, target, wmask, B, H, W, loss, stream) &
        BIND(C, NAME="fw_net_loss_grad")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: net, x, target, wmask
      INTEGER(C_INT), VALUE :: B, H, W
      TYPE(C_PTR), VALUE :: loss, stream          ! loss: C_LOC of a REAL(8) or C_NULL_PTR
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_adam(net, lr, beta1, beta2, eps, stream) BIND(C, NAME="fw_net_adam")
      IMPORT :: C_INT, C_PTR, C_FLOAT
      TYPE(C_PTR), VALUE :: net
      REAL(C_FLOAT), VALUE :: lr, beta1, beta2, eps
      TYPE(C_PTR), VALUE :: stream
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_set_wait_limit(net, polls) BIND(C, NAME="fw_net_set_wait_limit")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: net
      INTEGER(C_INT), VALUE :: polls             ! unsigned in C
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_correct(ctx, net, max_corr, applied) BIND(C, NAME="fw_correct")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx, net
      REAL(C_DOUBLE), VALUE :: max_corr
      TYPE(C_PTR), VALUE :: applied               ! C_LOC of an INTEGER or C_NULL_PTR
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_last_check(net, out) BIND(C, NAME="fw_net_last_check")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: net
      REAL(C_DOUBLE), INTENT(OUT) :: out(5)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_net_set_shore_band(net, cells) BIND(C, NAME="fw_net_set_shore_band")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: net
      INTEGER(C_INT), VALUE :: cells
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_correct_run(ctx, net, nsteps, max_corr, status) BIND(C, NAME="fw_correct_run")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx, net
      INTEGER(C_INT), VALUE :: nsteps
      REAL(C_DOUBLE), VALUE :: max_corr
      INTEGER(C_INT), INTENT(OUT) :: status
    END FUNCTION

    ! --- one entry point per reference unit -----------------------------
    INTEGER(C_INT) FUNCTION fw_exchange(ctx) BIND(C, NAME="fw_exchange")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_estimate_dt(ctx) BIND(C, NAME="fw_estimate_dt")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_cal_dispersion(ctx) BIND(C, NAME="fw_cal_dispersion")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_fluxes(ctx) BIND(C, NAME="fw_fluxes")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_source_terms(ctx) BIND(C, NAME="fw_source_terms")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_estimate_huv(ctx, istage) BIND(C, NAME="fw_estimate_huv")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: istage
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_update_mask(ctx) BIND(C, NAME="fw_update_mask")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_wave_breaking(ctx) BIND(C, NAME="fw_wave_breaking")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_sponge_damping(ctx) BIND(C, NAME="fw_sponge_damping")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION

    ! --- checkpoint / restart -------------------------------------------
    INTEGER(C_INT) FUNCTION fw_checkpoint(ctx, path) BIND(C, NAME="fw_checkpoint")
      IMPORT :: C_INT, C_PTR, C_CHAR
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_restore(ctx, path) BIND(C, NAME="fw_restore")
      IMPORT :: C_INT, C_PTR, C_CHAR
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
    END FUNCTION

    ! --- asynchronous output ---------------------------------------------
    INTEGER(C_INT) FUNCTION fw_output_begin(ctx, n, names, host) BIND(C, NAME="fw_output_begin")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: n
      TYPE(C_PTR), INTENT(IN) :: names(*), host(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_output_wait(ctx) BIND(C, NAME="fw_output_wait")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_output_done(ctx) BIND(C, NAME="fw_output_done")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_host_alloc(bytes, ptr) BIND(C, NAME="fw_host_alloc")
      IMPORT :: C_INT, C_PTR, C_SIZE_T
      INTEGER(C_SIZE_T), VALUE :: bytes
      TYPE(C_PTR), INTENT(OUT) :: ptr
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_host_free(ptr) BIND(C, NAME="fw_host_free")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ptr
    END FUNCTION

    ! --- diagnostics and launch-shape tuning ----------------------------
    INTEGER(C_LONG_LONG) FUNCTION fw_launch_count(ctx) BIND(C, NAME="fw_launch_count")
      IMPORT :: C_LONG_LONG, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_time_kernel(ctx, name, nrep, ms) BIND(C, NAME="fw_time_kernel")
      IMPORT :: C_INT, C_PTR, C_CHAR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: name(*)
      INTEGER(C_INT), VALUE :: nrep
      REAL(C_DOUBLE), INTENT(OUT) :: ms
    END FUNCTION
    TYPE(C_PTR) FUNCTION fw_stream(ctx) BIND(C, NAME="fw_stream")
      IMPORT :: C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_autotune(ctx, flags) BIND(C, NAME="fw_autotune")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: flags
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_get_tuning(ctx, tuning) BIND(C, NAME="fw_get_tuning")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), INTENT(OUT) :: tuning(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION fw_set_tuning(ctx, tuning) BIND(C, NAME="fw_set_tuning")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), INTENT(IN) :: tuning(*)
    END FUNCTION

    ! --- the CFL step on caller-owned device arrays, allocating nothing ---
    ! U, V, H, DT, TIME: device addresses (e.g. from !$acc host_data
    ! use_device, or C_DEVLOC of CUDA Fortran device arrays); TIME may be
    ! C_NULL_PTR; stream: a cudaStream_t or C_NULL_PTR
    INTEGER(C_INT) FUNCTION fw_estimate_dt_device(Mloc, Nloc, DX, DY, U, V, H, MinDepthFrc, CFL, dt_fixed, &
        DT, TIME, stream) BIND(C, NAME="fw_estimate_dt_device")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      INTEGER(C_INT), VALUE :: Mloc, Nloc
      REAL(C_DOUBLE), VALUE :: DX, DY
      TYPE(C_PTR), VALUE :: U, V, H
      REAL(C_DOUBLE), VALUE :: MinDepthFrc, CFL, dt_fixed
      TYPE(C_PTR), VALUE :: DT, TIME, stream
    END FUNCTION

    ! text of a status code: a NUL-terminated C string (C_F_POINTER to read)
    TYPE(C_PTR) FUNCTION fw_strerror(status) BIND(C, NAME="fw_strerror")
      IMPORT :: C_INT, C_PTR
      INTEGER(C_INT), VALUE :: status
    END FUNCTION
  END INTERFACE
END MODULE FUNWAVE_GPU
