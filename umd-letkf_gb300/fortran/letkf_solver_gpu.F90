!> letkf_solver -- the GB300 replacement of the reference's solver module
!! (src/letkf_solver.F90).  It keeps the module name and the three public
!! procedures, so letkf_run (src/letkf.F90:152,158,167) calls it unchanged; a
!! build selects this file instead of src/letkf_solver.F90 (e.g. a CMake
!! option LETKF_ENABLE_GPU), links -llgpu -lcudart, and compiles
!! letkf_gpu_c.F90 before it.
!!
!! What it reads and writes are the reference's module globals:
!!   lat_ij, lon_ij, mask_ij, state_ij, state_mean_ij, state_sprd_ij,
!!   statevars, grid_ns, grid_nx, grid_ny, hzgrids, vtgrids (letkf_state);
!!   obs_def, obs_hx, obs_hx_mean (letkf_obs); localizer_class (letkf_loc);
!!   ens_size, ij_count (letkf_mpi).
!! The analysis is written back into state_ij / state_mean_ij /
!! state_sprd_ij in place, as src/letkf_solver.F90:288,299-379 do; the
!! library uploads the background and downloads the analysis while it
!! computes.
!!
!! The count of valid observations after the QC compaction of
!! letkf_obs_read (src/letkf_obs.F90:480-488) is a local there; the
!! integration adds one public variable to letkf_obs, set after that loop:
!!     INTEGER, PUBLIC, PROTECTED :: obs_nvalid = 0   ! and: obs_nvalid = nobs
!! Only obs_def(1:obs_nvalid) and obs_hx(:, 1:obs_nvalid) are passed.
!!
!! Localizer plugins reach the device as parameter descriptors: loc_novrt
!! and loc_ocean are mapped here from their public components; any other
!! class stops the run with letkf_mpi_abort (there is no CPU fallback).
!! Every nonzero status of the library goes to letkf_mpi_abort with the
!! library's message, the reference's error behaviour.
MODULE letkf_solver
  USE, INTRINSIC :: iso_c_binding
  USE letkf_config
  USE letkf_mpi
  USE letkf_loc
  USE letkf_loc_novrt_mod, ONLY: letkf_loc_novrt
  USE letkf_loc_ocean_mod, ONLY: letkf_loc_ocean
  USE letkf_state
  USE letkf_obs
  USE letkf_gpu_c
  IMPLICIT NONE
  PRIVATE

  PUBLIC :: letkf_solver_init
  PUBLIC :: letkf_solver_run
  PUBLIC :: letkf_solver_final

  TYPE(c_ptr) :: h = c_null_ptr
  LOGICAL :: save_diag = .TRUE.
  CHARACTER(:), ALLOCATABLE :: diag_file

CONTAINS

  !> src/letkf_solver.F90:73-142: the solver: section and its validation (the
  !! library checks rtps/rtpp/mul with the reference's messages)
  SUBROUTINE letkf_solver_init(config)
    TYPE(configuration), INTENT(in) :: config
    TYPE(configuration) :: infl_config
    TYPE(lgpu_solver_config) :: c
    REAL :: infl_mul, infl_rtps, infl_rtpp

    CALL config%get("save_diag", save_diag, .TRUE.)
    CALL config%get("diag_file", diag_file, "diag.solver.nc")
    IF (config%found("inflation")) THEN
       CALL config%get("inflation", infl_config)
    ELSE
       infl_config = config
    END IF
    CALL infl_config%get("mul", infl_mul, default=1.0)
    CALL infl_config%get("rtps", infl_rtps, default=0.0)
    CALL infl_config%get("rtpp", infl_rtpp, default=0.0)
    IF (pe_isroot) THEN
       PRINT *, "solver.inflation.rtps=", infl_rtps
       PRINT *, "solver.inflation.rtpp=", infl_rtpp
       PRINT *, "solver.inflation.mul= ", infl_mul
    END IF

    c%rtps = infl_rtps
    c%rtpp = infl_rtpp
    c%mul = infl_mul
    c%save_diag = MERGE(1, 0, save_diag)
    IF (lgpu_create(0_c_int, h) /= LGPU_OK) CALL letkf_mpi_abort("letkf_gpu: no usable GB300 device")
    CALL check(lgpu_solver_init(h, c))
    CALL localizer_to_device()
  END SUBROUTINE letkf_solver_init


  !> src/letkf_solver.F90:150-389: the column loop, on the device
  SUBROUTINE letkf_solver_run()
    INTEGER(c_int), ALLOCATABLE :: m(:)
    TYPE(lgpu_statevar), ALLOCATABLE :: v(:)
    REAL(c_float), ALLOCATABLE, TARGET :: olat(:), olon(:), oz(:), ot(:), oval(:), oerr(:)
    INTEGER(c_int), ALLOCATABLE, TARGET :: oid(:), opl(:)
    REAL(c_float), ALLOCATABLE :: lvl(:)
    TYPE(lgpu_obs) :: ob
    INTEGER :: i, n

    ALLOCATE(m(ij_count))
    m = MERGE(1, 0, mask_ij)
    CALL check(lgpu_set_grid(h, INT(ij_count, c_int), lat_ij, lon_ij, m))

    ALLOCATE(v(SIZE(statevars)))
    DO i = 1, SIZE(statevars)
       v(i)%grid_s_idx = statevars(i)%grid_s_idx - 1
       v(i)%levels = statevars(i)%levels
       v(i)%ana_inc_max = statevars(i)%ana_inc_max
       v(i)%ana_bounds = statevars(i)%ana_bounds
    END DO
    ! in place: the run reads the background from these arrays and leaves the
    ! analysis in them
    CALL check(lgpu_bind_state(h, INT(ens_size, c_int), INT(grid_ns, c_int), state_ij, state_mean_ij, &
         state_sprd_ij, INT(SIZE(v), c_int), v))

    n = obs_nvalid
    olat = obs_def(1:n)%lat
    olon = obs_def(1:n)%lon
    oz = obs_def(1:n)%zdim
    ot = obs_def(1:n)%time
    oval = obs_def(1:n)%val
    oerr = obs_def(1:n)%err
    oid = obs_def(1:n)%obsid
    opl = obs_def(1:n)%platid
    ob%lat = C_LOC(olat)
    ob%lon = C_LOC(olon)
    ob%zdim = C_LOC(oz)
    ob%time = C_LOC(ot)
    ob%val = C_LOC(oval)
    ob%err = C_LOC(oerr)
    ob%obsid = C_LOC(oid)
    ob%platid = C_LOC(opl)
    CALL check(lgpu_set_obs(h, INT(n, c_int), ob, obs_hx, obs_hx_mean))

    CALL check(lgpu_solver_run(h))

    ! loc_ocean's diagnostics as its groups() would have left them
    ! (src/subclass.letkf_localizer/letkf_loc_ocean.F90:353-358), so that its
    ! own final() writes diag.loc_ocean.nc unchanged
    SELECT TYPE (p => localizer_class)
    TYPE IS (letkf_loc_ocean)
       IF (p%save_diag .AND. p%vtloc_surf_src /= 0) THEN
          ALLOCATE(lvl(ij_count))
          CALL check(lgpu_get_loc_diag(h, lvl))
          DO i = 1, ij_count
             IF (mask_ij(i)) CYCLE
             p%diag_vtloc_surf_lvl(i) = lvl(i)
             p%diag_vtloc_surf_dpth(i) = vtgrids(1)%vert_nom(INT(lvl(i)))
          END DO
       END IF
    END SELECT
  END SUBROUTINE letkf_solver_run


  !> src/letkf_solver.F90:397-527: the diagnostics file, then the device freed
  SUBROUTINE letkf_solver_final()
    IF (save_diag .AND. pe_isroot) &
         CALL check(lgpu_write_diag(h, TRIM(diag_file)//c_null_char, INT(grid_nx, c_int), INT(grid_ny, c_int), &
         hzgrids(1)%lat_nom, hzgrids(1)%lon_nom))
    CALL check(lgpu_solver_final(h))
    CALL lgpu_destroy(h)
    h = c_null_ptr
  END SUBROUTINE letkf_solver_final


  !> the device descriptor of localizer_class: the parameters its init()
  !! read (src/subclass.letkf_localizer/letkf_loc_novrt.F90:38-50,
  !! letkf_loc_ocean.F90:30-59); the library copies them
  SUBROUTINE localizer_to_device()
    TYPE(lgpu_loc_config) :: lc
    TYPE(lgpu_interp_point), ALLOCATABLE, TARGET :: hz(:), hz_sat(:)
    INTEGER(c_int), ALLOCATABLE, TARGET :: sat_obs(:), sat_plats(:)
    CHARACTER(len=16, kind=c_char), TARGET :: cls
    INTEGER :: i

    lc%n_hz = 0
    lc%hz = c_null_ptr
    lc%n_hz_sat = 0
    lc%hz_sat = c_null_ptr
    lc%tloc_prof = -1.0
    lc%tloc_sat = -1.0
    lc%vtloc_surf = 0
    lc%bkg_t_delta = 0.0
    lc%bkg_t_var = -1
    lc%n_sat_obs = 0
    lc%sat_obs = c_null_ptr
    lc%n_sat_plats = 0
    lc%sat_plats = c_null_ptr
    lc%vtloc = 0.0
    lc%nlev = 0
    lc%lev_depth = c_null_ptr

    SELECT TYPE (p => localizer_class)
    TYPE IS (letkf_loc_novrt)
       cls = "loc_novrt"//c_null_char
       hz = interp_points(p%hzdist)
    TYPE IS (letkf_loc_ocean)
       cls = "loc_ocean"//c_null_char
       hz = interp_points(p%hzdist_prof)
       hz_sat = interp_points(p%hzdist_sat)
       lc%n_hz_sat = SIZE(hz_sat)
       lc%hz_sat = C_LOC(hz_sat)
       lc%tloc_prof = p%tloc_prof
       lc%tloc_sat = p%tloc_sat
       lc%vtloc_surf = p%vtloc_surf_src
       lc%bkg_t_delta = p%bkg_t_delta
       DO i = 1, SIZE(statevars)
          IF (statevars(i)%grid_s_idx == p%bkg_t_var_idx) lc%bkg_t_var = i - 1
       END DO
       IF (ALLOCATED(p%surf_obs)) THEN
          sat_obs = p%surf_obs
          lc%n_sat_obs = SIZE(sat_obs)
          IF (SIZE(sat_obs) > 0) lc%sat_obs = C_LOC(sat_obs)
       END IF
       IF (ALLOCATED(p%surf_plats)) THEN
          sat_plats = p%surf_plats
          lc%n_sat_plats = SIZE(sat_plats)
          IF (SIZE(sat_plats) > 0) lc%sat_plats = C_LOC(sat_plats)
       END IF
    CLASS DEFAULT
       CALL letkf_mpi_abort('letkf_gpu: localizer class "'//localizer_class%name()// &
            '" has no device descriptor')
    END SELECT
    lc%cls = C_LOC(cls)
    lc%n_hz = SIZE(hz)
    lc%hz = C_LOC(hz)
    CALL check(lgpu_loc_init(h, lc))
  END SUBROUTINE localizer_to_device


  !> a linearinterp_lat table (src/letkf_loc.F90:126-133) as {lat, radius}
  !! points; the table is already padded with 0 and 90 degrees, which the
  !! library's own padding leaves unchanged
  FUNCTION interp_points(t) RESULT(pts)
    TYPE(linearinterp_lat), INTENT(in) :: t
    TYPE(lgpu_interp_point), ALLOCATABLE :: pts(:)
    INTEGER :: i
    ALLOCATE(pts(t%npoints))
    DO i = 1, t%npoints
       pts(i)%lat = t%lat(i)
       pts(i)%radius = t%dist(i)
    END DO
  END FUNCTION interp_points


  SUBROUTINE check(rc)
    INTEGER(c_int), INTENT(in) :: rc
    IF (rc /= LGPU_OK) CALL letkf_mpi_abort("letkf_gpu: "//lgpu_error_string(h))
  END SUBROUTINE check

END MODULE letkf_solver
