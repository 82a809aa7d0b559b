!> letkf_gpu_c -- iso_c_binding interface to the GB300 analysis library
!! (include/letkf_gpu.h, liblgpu.so).
!!
!! The reference binds C the same way (src/letkf_config.F90:23-60 over
!! src/letkf_config_c.cpp).  Every derived type below is BIND(C) and mirrors
!! the C struct of the same name field by field; tests/abi_c/test_abi.c prints
!! the C layout and tests/test_abi.py checks these declarations against it,
!! so the two cannot drift apart.  Index arguments (grid_s_idx, bkg_t_var,
!! groups, observation indices) are 0-based on the C side.
MODULE letkf_gpu_c
  USE, INTRINSIC :: iso_c_binding
  IMPLICIT NONE

  ! lgpu_status
  INTEGER(c_int), PARAMETER :: LGPU_OK = 0
  INTEGER(c_int), PARAMETER :: LGPU_ERR_ARG = 1
  INTEGER(c_int), PARAMETER :: LGPU_ERR_CUDA = 2
  INTEGER(c_int), PARAMETER :: LGPU_ERR_NOMEM = 3
  INTEGER(c_int), PARAMETER :: LGPU_ERR_UNSUPPORTED_LOCALIZER = 4
  INTEGER(c_int), PARAMETER :: LGPU_ERR_CONFIG = 5
  INTEGER(c_int), PARAMETER :: LGPU_ERR_ORDER = 6
  INTEGER(c_int), PARAMETER :: LGPU_ERR_CAPACITY = 7
  INTEGER(c_int), PARAMETER :: LGPU_ERR_NONFINITE = 8
  INTEGER(c_int), PARAMETER :: LGPU_ERR_EIG = 9
  INTEGER(c_int), PARAMETER :: LGPU_ERR_UNSUPPORTED = 10

  INTEGER(c_int), PARAMETER :: LGPU_MAX_INTERP = 16
  INTEGER(c_int), PARAMETER :: LGPU_MAX_IDS = 32
  INTEGER(c_int), PARAMETER :: LGPU_MAX_LEVELS = 128
  INTEGER(c_int), PARAMETER :: LGPU_MAX_K = 128
  INTEGER(c_int), PARAMETER :: LGPU_NOALLOC_MAX_LIST = 262144

  INTEGER(c_int), PARAMETER :: LGPU_VARIANT_AUTO = 0
  INTEGER(c_int), PARAMETER :: LGPU_VARIANT_PLAIN = 1
  INTEGER(c_int), PARAMETER :: LGPU_VARIANT_BATCHED_TC = 2
  INTEGER(c_int), PARAMETER :: LGPU_VARIANT_LEARNED = 3

  INTEGER(c_int), PARAMETER :: LGPU_PREC_FP32 = 0
  INTEGER(c_int), PARAMETER :: LGPU_PREC_FP32_RESOLVE = 1
  INTEGER(c_int), PARAMETER :: LGPU_PREC_FP64 = 2

  !> solver: section (src/letkf_solver.F90:86-101)
  TYPE, BIND(C) :: lgpu_solver_config
     REAL(c_float)  :: rtps
     REAL(c_float)  :: rtpp
     REAL(c_float)  :: mul
     INTEGER(c_int) :: save_diag
  END TYPE lgpu_solver_config

  !> one {lat, radius} entry of a linearinterp_lat table (src/letkf_loc.F90:251-294)
  TYPE, BIND(C) :: lgpu_interp_point
     REAL(c_float) :: lat
     REAL(c_float) :: radius
  END TYPE lgpu_interp_point

  !> localization: section of loc_novrt / loc_ocean / loc_vtgc
  TYPE, BIND(C) :: lgpu_loc_config
     TYPE(c_ptr)    :: cls            ! NUL-terminated class name
     INTEGER(c_int) :: n_hz
     TYPE(c_ptr)    :: hz             ! lgpu_interp_point(n_hz)
     INTEGER(c_int) :: n_hz_sat
     TYPE(c_ptr)    :: hz_sat         ! lgpu_interp_point(n_hz_sat)
     REAL(c_float)  :: tloc_prof
     REAL(c_float)  :: tloc_sat
     INTEGER(c_int) :: vtloc_surf
     REAL(c_float)  :: bkg_t_delta
     INTEGER(c_int) :: bkg_t_var      ! 0-based index into the statevars
     INTEGER(c_int) :: n_sat_obs
     TYPE(c_ptr)    :: sat_obs        ! INTEGER(c_int)(n_sat_obs)
     INTEGER(c_int) :: n_sat_plats
     TYPE(c_ptr)    :: sat_plats      ! INTEGER(c_int)(n_sat_plats)
     REAL(c_float)  :: vtloc
     INTEGER(c_int) :: nlev
     TYPE(c_ptr)    :: lev_depth      ! REAL(c_float)(nlev)
  END TYPE lgpu_loc_config

  !> letkf_statevar_spec (src/letkf_state.F90:83-98)
  TYPE, BIND(C) :: lgpu_statevar
     INTEGER(c_int) :: grid_s_idx     ! 0-based
     INTEGER(c_int) :: levels
     REAL(c_float)  :: ana_inc_max
     REAL(c_float)  :: ana_bounds(2)
  END TYPE lgpu_statevar

  !> letkf_observation (src/letkf_obs.F90:57-68) as structure of arrays
  TYPE, BIND(C) :: lgpu_obs
     TYPE(c_ptr) :: lat
     TYPE(c_ptr) :: lon
     TYPE(c_ptr) :: zdim
     TYPE(c_ptr) :: time
     TYPE(c_ptr) :: val
     TYPE(c_ptr) :: err
     TYPE(c_ptr) :: obsid
     TYPE(c_ptr) :: platid
  END TYPE lgpu_obs

  !> device and host-link times of the last lgpu_solver_run
  TYPE, BIND(C) :: lgpu_timings
     REAL(c_float)      :: total_ms
     REAL(c_float)      :: index_ms
     REAL(c_float)      :: prep_ms
     REAL(c_float)      :: gram_ms
     REAL(c_float)      :: eig_ms
     REAL(c_float)      :: update_ms
     INTEGER(c_int)     :: launches
     INTEGER(c_int)     :: units
     INTEGER(c_long_long) :: kept_pairs
     INTEGER(c_int)     :: variant
     REAL(c_float)      :: tiles_ms
     INTEGER(c_long_long) :: mma_chunks
     INTEGER(c_int)     :: mma_n
     INTEGER(c_int)     :: precision
     INTEGER(c_int)     :: fp64_units
     REAL(c_float)      :: fp64_ms
     REAL(c_float)      :: h2d_obs_ms
     REAL(c_float)      :: host_obs_ms
     REAL(c_float)      :: h2d_state_ms
     REAL(c_float)      :: d2h_state_ms
     REAL(c_float)      :: span_ms
     REAL(c_float)      :: host_run_ms
     INTEGER(c_long_long) :: h2d_state_bytes
     INTEGER(c_long_long) :: d2h_state_bytes
  END TYPE lgpu_timings

  !> learned form (no counterpart in the reference)
  TYPE, BIND(C) :: lgpu_learn_config
     INTEGER(c_int)     :: nx
     INTEGER(c_int)     :: ny
     INTEGER(c_int)     :: stride
     INTEGER(c_int)     :: hidden
     REAL(c_float)      :: judge_frac
     REAL(c_float)      :: gate_frac
     REAL(c_float)      :: sample_frac
     INTEGER(c_int)     :: train_cap
     INTEGER(c_long_long) :: seed
  END TYPE lgpu_learn_config

  TYPE, BIND(C) :: lgpu_learn_stats
     INTEGER(c_int)     :: coarse
     INTEGER(c_int)     :: judged
     INTEGER(c_int)     :: fallback
     INTEGER(c_int)     :: gated
     INTEGER(c_int)     :: inferred
     REAL(c_float)      :: judge_rms
     REAL(c_float)      :: judge_ref_rms
     REAL(c_float)      :: tau
     INTEGER(c_long_long) :: train_rows
     REAL(c_float)      :: exact_ms
     REAL(c_float)      :: feature_ms
     REAL(c_float)      :: network_ms
     REAL(c_float)      :: apply_ms
  END TYPE lgpu_learn_stats

  INTERFACE
     INTEGER(c_int) FUNCTION lgpu_create(device, h) BIND(C, name="lgpu_create")
       IMPORT :: c_int, c_ptr
       INTEGER(c_int), VALUE :: device
       TYPE(c_ptr), INTENT(out) :: h
     END FUNCTION lgpu_create

     SUBROUTINE lgpu_destroy(h) BIND(C, name="lgpu_destroy")
       IMPORT :: c_ptr
       TYPE(c_ptr), VALUE :: h
     END SUBROUTINE lgpu_destroy

     TYPE(c_ptr) FUNCTION lgpu_last_error(h) BIND(C, name="lgpu_last_error")
       IMPORT :: c_ptr
       TYPE(c_ptr), VALUE :: h
     END FUNCTION lgpu_last_error

     INTEGER(c_int) FUNCTION lgpu_solver_init(h, cfg) BIND(C, name="lgpu_solver_init")
       IMPORT :: c_int, c_ptr, lgpu_solver_config
       TYPE(c_ptr), VALUE :: h
       TYPE(lgpu_solver_config), INTENT(in) :: cfg
     END FUNCTION lgpu_solver_init

     INTEGER(c_int) FUNCTION lgpu_loc_init(h, cfg) BIND(C, name="lgpu_loc_init")
       IMPORT :: c_int, c_ptr, lgpu_loc_config
       TYPE(c_ptr), VALUE :: h
       TYPE(lgpu_loc_config), INTENT(in) :: cfg
     END FUNCTION lgpu_loc_init

     INTEGER(c_int) FUNCTION lgpu_loc_maxgroups(h) BIND(C, name="lgpu_loc_maxgroups")
       IMPORT :: c_int, c_ptr
       TYPE(c_ptr), VALUE :: h
     END FUNCTION lgpu_loc_maxgroups

     INTEGER(c_int) FUNCTION lgpu_set_variant(h, variant) BIND(C, name="lgpu_set_variant")
       IMPORT :: c_int, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: variant
     END FUNCTION lgpu_set_variant

     INTEGER(c_int) FUNCTION lgpu_set_precision(h, mode, gap_threshold) BIND(C, name="lgpu_set_precision")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: mode
       REAL(c_float), VALUE :: gap_threshold
     END FUNCTION lgpu_set_precision

     INTEGER(c_int) FUNCTION lgpu_set_grid(h, nij, lat, lon, mask) BIND(C, name="lgpu_set_grid")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: nij
       REAL(c_float), INTENT(in) :: lat(*), lon(*)
       INTEGER(c_int), INTENT(in) :: mask(*)
     END FUNCTION lgpu_set_grid

     INTEGER(c_int) FUNCTION lgpu_set_state(h, k, ns, state, mean, sprd, nvars, vars) &
          BIND(C, name="lgpu_set_state")
       IMPORT :: c_int, c_float, c_ptr, lgpu_statevar
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: k, ns, nvars
       REAL(c_float), INTENT(in) :: state(*), mean(*), sprd(*)
       TYPE(lgpu_statevar), INTENT(in) :: vars(*)
     END FUNCTION lgpu_set_state

     INTEGER(c_int) FUNCTION lgpu_bind_state(h, k, ns, state, mean, sprd, nvars, vars) &
          BIND(C, name="lgpu_bind_state")
       IMPORT :: c_int, c_float, c_ptr, lgpu_statevar
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: k, ns, nvars
       REAL(c_float) :: state(*), mean(*), sprd(*)   ! background in, analysis out (in place)
       TYPE(lgpu_statevar), INTENT(in) :: vars(*)
     END FUNCTION lgpu_bind_state

     INTEGER(c_int) FUNCTION lgpu_set_state_members(h, k, ns, members, nvars, vars) &
          BIND(C, name="lgpu_set_state_members")
       IMPORT :: c_int, c_float, c_ptr, lgpu_statevar
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: k, ns, nvars
       REAL(c_float), INTENT(in) :: members(*)
       TYPE(lgpu_statevar), INTENT(in) :: vars(*)
     END FUNCTION lgpu_set_state_members

     INTEGER(c_int) FUNCTION lgpu_set_obs(h, nobs, obs, hx, hx_mean) BIND(C, name="lgpu_set_obs")
       IMPORT :: c_int, c_float, c_ptr, lgpu_obs
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: nobs
       TYPE(lgpu_obs), INTENT(in) :: obs
       REAL(c_float), INTENT(in) :: hx(*), hx_mean(*)
     END FUNCTION lgpu_set_obs

     INTEGER(c_int) FUNCTION lgpu_set_obs_raw(h, nobs, obs, qc, hx_members, nobs_kept) &
          BIND(C, name="lgpu_set_obs_raw")
       IMPORT :: c_int, c_float, c_ptr, lgpu_obs
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: nobs
       TYPE(lgpu_obs), INTENT(in) :: obs
       INTEGER(c_int), INTENT(in) :: qc(*)
       REAL(c_float), INTENT(in) :: hx_members(*)
       INTEGER(c_int), INTENT(out) :: nobs_kept
     END FUNCTION lgpu_set_obs_raw

     INTEGER(c_int) FUNCTION lgpu_solver_run(h) BIND(C, name="lgpu_solver_run")
       IMPORT :: c_int, c_ptr
       TYPE(c_ptr), VALUE :: h
     END FUNCTION lgpu_solver_run

     INTEGER(c_int) FUNCTION lgpu_get_state(h, state, mean, sprd) BIND(C, name="lgpu_get_state")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       REAL(c_float), INTENT(out) :: state(*), mean(*), sprd(*)
     END FUNCTION lgpu_get_state

     INTEGER(c_int) FUNCTION lgpu_get_diag(h, maxhz, obscount, lg_obscount, lg_obsloc) &
          BIND(C, name="lgpu_get_diag")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       REAL(c_float), INTENT(out) :: maxhz(*), obscount(*), lg_obscount(*), lg_obsloc(*)
     END FUNCTION lgpu_get_diag

     INTEGER(c_int) FUNCTION lgpu_get_timings(h, t) BIND(C, name="lgpu_get_timings")
       IMPORT :: c_int, c_ptr, lgpu_timings
       TYPE(c_ptr), VALUE :: h
       TYPE(lgpu_timings), INTENT(out) :: t
     END FUNCTION lgpu_get_timings

     INTEGER(c_int) FUNCTION lgpu_solver_final(h) BIND(C, name="lgpu_solver_final")
       IMPORT :: c_int, c_ptr
       TYPE(c_ptr), VALUE :: h
     END FUNCTION lgpu_solver_final

     INTEGER(c_int) FUNCTION lgpu_get_obslist(h, ij, group, idx, rloc, cap, n, ncand) &
          BIND(C, name="lgpu_get_obslist")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: ij, group, cap
       INTEGER(c_int), INTENT(out) :: idx(*)
       REAL(c_float), INTENT(out) :: rloc(*)
       INTEGER(c_int), INTENT(out) :: n, ncand
     END FUNCTION lgpu_get_obslist

     INTEGER(c_int) FUNCTION lgpu_get_obslist_noalloc(h, ij, group, idx, rloc, cap, n, ncand) &
          BIND(C, name="lgpu_get_obslist_noalloc")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: ij, group, cap
       INTEGER(c_int), INTENT(out) :: idx(*)
       REAL(c_float), INTENT(out) :: rloc(*)
       INTEGER(c_int), INTENT(out) :: n, ncand
     END FUNCTION lgpu_get_obslist_noalloc

     INTEGER(c_int) FUNCTION lgpu_write_diag(h, path, nx, ny, lat_nom, lon_nom) BIND(C, name="lgpu_write_diag")
       IMPORT :: c_int, c_float, c_ptr, c_char
       TYPE(c_ptr), VALUE :: h
       CHARACTER(kind=c_char), INTENT(in) :: path(*)   ! NUL-terminated
       INTEGER(c_int), VALUE :: nx, ny
       REAL(c_float), INTENT(in) :: lat_nom(*), lon_nom(*)
     END FUNCTION lgpu_write_diag

     INTEGER(c_int) FUNCTION lgpu_get_loc_diag(h, surf_lvl) BIND(C, name="lgpu_get_loc_diag")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       REAL(c_float), INTENT(out) :: surf_lvl(*)
     END FUNCTION lgpu_get_loc_diag

     INTEGER(c_int) FUNCTION lgpu_write_loc_diag(h, path, nx, ny, lat_nom, lon_nom, nz, vert_nom) &
          BIND(C, name="lgpu_write_loc_diag")
       IMPORT :: c_int, c_float, c_ptr, c_char
       TYPE(c_ptr), VALUE :: h
       CHARACTER(kind=c_char), INTENT(in) :: path(*)   ! NUL-terminated
       INTEGER(c_int), VALUE :: nx, ny, nz
       REAL(c_float), INTENT(in) :: lat_nom(*), lon_nom(*), vert_nom(*)
     END FUNCTION lgpu_write_loc_diag

     INTEGER(c_int) FUNCTION lgpu_host_alloc(bytes, ptr) BIND(C, name="lgpu_host_alloc")
       IMPORT :: c_int, c_size_t, c_ptr
       INTEGER(c_size_t), VALUE :: bytes
       TYPE(c_ptr), INTENT(out) :: ptr
     END FUNCTION lgpu_host_alloc

     INTEGER(c_int) FUNCTION lgpu_host_free(ptr) BIND(C, name="lgpu_host_free")
       IMPORT :: c_int, c_ptr
       TYPE(c_ptr), VALUE :: ptr
     END FUNCTION lgpu_host_free

     INTEGER(c_int) FUNCTION lgpu_learn_init(h, cfg) BIND(C, name="lgpu_learn_init")
       IMPORT :: c_int, c_ptr, lgpu_learn_config
       TYPE(c_ptr), VALUE :: h
       TYPE(lgpu_learn_config), INTENT(in) :: cfg
     END FUNCTION lgpu_learn_init

     INTEGER(c_int) FUNCTION lgpu_learn_collect(h, rows) BIND(C, name="lgpu_learn_collect")
       IMPORT :: c_int, c_long_long, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_long_long), INTENT(out) :: rows
     END FUNCTION lgpu_learn_collect

     INTEGER(c_int) FUNCTION lgpu_learn_train(h, epochs, batch, lr, loss) BIND(C, name="lgpu_learn_train")
       IMPORT :: c_int, c_float, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: epochs, batch
       REAL(c_float), VALUE :: lr
       REAL(c_float), INTENT(out) :: loss
     END FUNCTION lgpu_learn_train

     INTEGER(c_int) FUNCTION lgpu_learn_stats_get(h, out) BIND(C, name="lgpu_learn_stats_get")
       IMPORT :: c_int, c_ptr, lgpu_learn_stats
       TYPE(c_ptr), VALUE :: h
       TYPE(lgpu_learn_stats), INTENT(out) :: out
     END FUNCTION lgpu_learn_stats_get

     INTEGER(c_int) FUNCTION lgpu_learn_set_network(h, use_network) BIND(C, name="lgpu_learn_set_network")
       IMPORT :: c_int, c_ptr
       TYPE(c_ptr), VALUE :: h
       INTEGER(c_int), VALUE :: use_network
     END FUNCTION lgpu_learn_set_network
  END INTERFACE

CONTAINS

  !> the library's last error message as a Fortran string
  FUNCTION lgpu_error_string(h) RESULT(msg)
    TYPE(c_ptr), INTENT(in) :: h
    CHARACTER(:), ALLOCATABLE :: msg
    CHARACTER(kind=c_char), POINTER :: p(:)
    INTEGER :: n
    TYPE(c_ptr) :: cp
    INTERFACE
       INTEGER(c_size_t) FUNCTION c_strlen(s) BIND(C, name="strlen")
         IMPORT :: c_ptr, c_size_t
         TYPE(c_ptr), VALUE :: s
       END FUNCTION c_strlen
    END INTERFACE
    cp = lgpu_last_error(h)
    IF (.NOT. C_ASSOCIATED(cp)) THEN
       msg = "unknown error"
       RETURN
    END IF
    n = INT(c_strlen(cp))
    CALL C_F_POINTER(cp, p, [n])
    ALLOCATE(CHARACTER(n) :: msg)
    msg = TRANSFER(p(1:n), msg)
  END FUNCTION lgpu_error_string

END MODULE letkf_gpu_c
