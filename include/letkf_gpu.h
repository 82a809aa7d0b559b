/*
 * letkf_gpu.h -- C ABI of the GB300 (sm_103a) LETKF per-gridpoint analysis.
 *
 * This library replaces the analysis path of UMD-LETKF: the local
 * observation search, Gaspari-Cohn localisation, the LETKF core solve and
 * the ensemble update with its relaxation/inflation/bounds epilogue.  It is
 * called from the host exactly where the reference calls its solver module:
 *
 *   reference (Fortran module letkf_solver)        this ABI
 *   ------------------------------------------    ----------------------------
 *   letkf_solver_init(config)                      lgpu_solver_init
 *     src/letkf_solver.F90:73-142
 *   letkf_loc_init(config) + plugin %init          lgpu_loc_init
 *     src/letkf_loc.F90:164-210, plugin init
 *   module globals lat_ij/lon_ij/mask_ij           lgpu_set_grid
 *     src/letkf_state.F90:166-173
 *   module globals state_ij/state_mean_ij/         lgpu_set_state
 *     state_sprd_ij, statevars
 *     src/letkf_state.F90:176-208, :83-98
 *   module globals obs_def/obs_hx/obs_hx_mean      lgpu_set_obs
 *     src/letkf_obs.F90:57-68, :164-171
 *   letkf_solver_run()                             lgpu_solver_run
 *     src/letkf_solver.F90:150-389
 *   in-place update of the state module arrays     lgpu_get_state
 *     src/letkf_solver.F90:288,299-379
 *   diagnostics written by letkf_solver_final      lgpu_get_diag
 *     src/letkf_solver.F90:131-140,212,220,265-268
 *   letkf_solver_final()                           lgpu_solver_final
 *     src/letkf_solver.F90:397-527
 *
 * Conventions
 *   - Plain C types and host pointers only; the library owns every device
 *     buffer behind the opaque handle.  Host arrays are borrowed for the
 *     duration of a call.
 *   - Layouts are the reference's Fortran column-major arrays read as C:
 *       state[ij][slab][member]   (state_ij(k, ns, ij))
 *       mean[ij][slab], sprd[ij][slab]
 *       hx[obs][member]           (obs_hx(k, nobs))
 *       lg_obscount[group][ij]    (diag_lg_obscount(ij, maxgroups))
 *     Indices (slabs, groups, observation indices) are 0-based.
 *   - Every call returns an lgpu_status; on failure lgpu_last_error() holds a
 *     message.  The reference aborts the MPI job in these cases
 *     (letkf_mpi_abort, src/letkf_mpi.F90:159-169); the caller decides.
 *   - One host thread per handle; calls on a handle are not re-entrant.
 *   - There is no CPU fallback: without a usable sm_103a device every call
 *     that needs it fails with LGPU_ERR_CUDA.
 */
#ifndef LETKF_GPU_H
#define LETKF_GPU_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lgpu_handle lgpu_handle;

typedef enum lgpu_status {
  LGPU_OK = 0,
  LGPU_ERR_ARG = 1,                   /* bad argument (NULL, size, range) */
  LGPU_ERR_CUDA = 2,                  /* CUDA runtime error / no device */
  LGPU_ERR_NOMEM = 3,                 /* device allocation failed */
  LGPU_ERR_UNSUPPORTED_LOCALIZER = 4, /* localization.class not registered */
  LGPU_ERR_CONFIG = 5,                /* invalid solver / localizer settings */
  LGPU_ERR_ORDER = 6,                 /* call made before its inputs were set */
  LGPU_ERR_CAPACITY = 7,              /* a static limit was exceeded */
  LGPU_ERR_NONFINITE = 8,             /* non-finite analysis produced */
  LGPU_ERR_EIG = 9,                   /* eigensolver did not converge */
  LGPU_ERR_UNSUPPORTED = 10           /* size outside what this build supports */
} lgpu_status;

#define LGPU_MAX_INTERP 16   /* linearinterp_lat points per table */
#define LGPU_MAX_IDS 32      /* sat_obs / sat_plats list entries */
#define LGPU_MAX_LEVELS 128  /* loc_vtgc level groups */
#define LGPU_MAX_K 128       /* ensemble size supported by this build */

/* Solver settings: the keys letkf_solver_init reads (src/letkf_solver.F90:86-101).
 * Validation matches :113-125 (0<=rtps<=1, 0<=rtpp<=1, not both, mul>=1). */
typedef struct lgpu_solver_config {
  float rtps;      /* solver.inflation.rtps, default 0 */
  float rtpp;      /* solver.inflation.rtpp, default 0 */
  float mul;       /* solver.inflation.mul, default 1 */
  int save_diag;   /* solver.save_diag, default 1 */
} lgpu_solver_config;

/* One {lat, radius} entry of a linearinterp_lat table (src/letkf_loc.F90:251-294). */
typedef struct lgpu_interp_point { float lat; float radius; } lgpu_interp_point;

/* Localizer selection and parameters (localization: section).
 *   cls = "loc_novrt"  (src/subclass.letkf_localizer/letkf_loc_novrt.F90)
 *         uses hz (localization.hzloc.value)
 *   cls = "loc_ocean"  (src/subclass.letkf_localizer/letkf_loc_ocean.F90)
 *         uses hz (hzloc_prof), hz_sat (hzloc_sat), tloc_prof, tloc_sat,
 *         sat_obs, sat_plats, vtloc_surf (0 none, 1 bkg_t), bkg_t_delta,
 *         bkg_t_var (index into the statevars given to lgpu_set_state)
 *   cls = "loc_vtgc"   horizontal GC times vertical GC with one group per
 *         level (a plugin added by this project for depth localisation)
 *         uses hz, vtloc (metres), nlev + lev_depth (vertical grid)
 * The class name is matched case-insensitively, as letkf_loc_init does. */
typedef struct lgpu_loc_config {
  const char *cls;
  int n_hz; const lgpu_interp_point *hz;
  int n_hz_sat; const lgpu_interp_point *hz_sat;
  float tloc_prof, tloc_sat;          /* <= 0 disables (default -1) */
  int vtloc_surf;
  float bkg_t_delta;
  int bkg_t_var;
  int n_sat_obs; const int *sat_obs;
  int n_sat_plats; const int *sat_plats;
  float vtloc;
  int nlev; const float *lev_depth;
} lgpu_loc_config;

/* letkf_statevar_spec (src/letkf_state.F90:83-98), 0-based grid_s_idx. */
typedef struct lgpu_statevar {
  int grid_s_idx;
  int levels;
  float ana_inc_max;      /* default 9.99e36 */
  float ana_bounds[2];    /* default {-9.99e36, 9.99e36} */
} lgpu_statevar;

/* letkf_observation (src/letkf_obs.F90:57-68) as structure-of-arrays, after
 * the reference's QC compaction (only qc == 0 observations). */
typedef struct lgpu_obs {
  const float *lat, *lon, *zdim, *time, *val, *err;
  const int *obsid, *platid;
} lgpu_obs;

/* Device time of the last lgpu_solver_run, from CUDA events on the
 * library's stream. */
typedef struct lgpu_timings {
  float total_ms;    /* whole run */
  float index_ms;    /* observation preparation + spatial index */
  float prep_ms;     /* per-column localisation parameters */
  float gram_ms;     /* search + localisation + Gram/RHS */
  float eig_ms;      /* eigensolve + transform */
  float update_ms;   /* X_b * T + relaxation/inflation/bounds epilogue */
  int launches;      /* kernels launched by the run */
  int units;         /* (column, group) solve units */
  long long kept_pairs;   /* sum over units of kept local observations (only when counted) */
  int variant;       /* variant that ran (LGPU_VARIANT_PLAIN / _BATCHED_TC / _LEARNED) */
  float tiles_ms;    /* BATCHED_TC: part of gram_ms spent building the tile candidate streams */
  long long mma_chunks;  /* BATCHED_TC: (tile, group, pass, 16-observation chunk) steps that ran MMAs */
  int mma_n;         /* BATCHED_TC: features per pass (MMA N); executed TF32 flops =
                        mma_chunks * 3 products * 2 * 128 * mma_n * 16 */
  int precision;     /* eigensolve precision mode of the run (LGPU_PREC_*) */
  int fp64_units;    /* units whose eigensolve ran in FP64 (re-solved, or all under LGPU_PREC_FP64) */
  float fp64_ms;     /* part of eig_ms spent in the FP64 eigensolve */
  /* host link and host time (the end-to-end view of a run) */
  float h2d_obs_ms;      /* the last lgpu_set_obs: observation upload (CUDA events around its copies) */
  float host_obs_ms;     /* the last lgpu_set_obs: host wall time of the call */
  float h2d_state_ms;    /* bound state: background upload (mean and spread, then the members), on the copy stream (0 otherwise) */
  float d2h_state_ms;    /* bound state: analysis download, summed over the column chunks (0 otherwise) */
  float span_ms;         /* run start to the end of the last analysis download (total_ms without a bound state) */
  float host_run_ms;     /* host wall time of lgpu_solver_run */
  long long h2d_state_bytes;  /* bound state: bytes uploaded by the run */
  long long d2h_state_bytes;  /* bound state: bytes downloaded by the run */
} lgpu_timings;

/* Gram variants.  PLAIN: one CTA per (column, group), FP32 on the CUDA
 * cores.  BATCHED_TC: tiles of 128 neighbouring columns share their
 * observations; the Gram of a tile is one GEMM on the tensor cores (tcgen05,
 * TF32 with a three-term hi/lo split, FP32 accumulation).  AUTO (default)
 * runs both forms, timed, on the first analysis after lgpu_set_grid,
 * lgpu_loc_init or a change of ensemble size, and keeps the faster one
 * (PLAIN below k = 8); the first analysis therefore takes longer.  Both
 * forms give bit-identical observation lists and keep decisions. */
#define LGPU_VARIANT_AUTO 0
#define LGPU_VARIANT_PLAIN 1
#define LGPU_VARIANT_BATCHED_TC 2
/* LEARNED (after lgpu_learn_init and lgpu_learn_train; loc_novrt only): exact
 * solves (PLAIN Gram) on the columns of a coarse lattice, a random judge
 * sample and the columns the confidence gate sends back; every other column
 * gets the bilinear interpolation of the coarse (W, w-bar) corrected by the
 * learned network.  The update and its epilogue are those of the exact
 * forms.  No counterpart in the reference, which solves every column
 * (src/letkf_solver.F90:203-384). */
#define LGPU_VARIANT_LEARNED 3

int lgpu_create(int device, lgpu_handle **out);
void lgpu_destroy(lgpu_handle *h);
const char *lgpu_last_error(const lgpu_handle *h);

int lgpu_solver_init(lgpu_handle *h, const lgpu_solver_config *cfg);
int lgpu_loc_init(lgpu_handle *h, const lgpu_loc_config *cfg);
int lgpu_loc_maxgroups(const lgpu_handle *h);
int lgpu_set_variant(lgpu_handle *h, int variant);   /* no reference counterpart: selects the Gram kernel */

/* Precision of the eigensolve and transform (src/letkf_core.F90:100-141,
 * FP32 ssyev in the reference); no reference counterpart.  The Gram stays
 * FP32 in every mode.
 * FP32 (default): FP32 throughout, the reference's precision.
 * FP32_RESOLVE: FP32, and a unit is solved again in FP64 when its FP32
 *   solve failed (no convergence, a non-positive or non-finite eigenvalue)
 *   or when two of its relevant eigenvalues lie within gap_threshold *
 *   lambda_max of each other.  Relevant eigenvalues are those above the
 *   (k-1) floor of Yb^T R^-1 Yb + (k-1) I by more than the FP32 rounding
 *   level (4 k eps lambda_max): the floor is exactly degenerate whenever the
 *   unit has fewer observations than members and does not make T
 *   ill-conditioned.  gap_threshold <= 0 takes 1e-6.
 * FP64: every unit's eigensolve and transform in FP64 (results stored FP32).
 * Under LGPU_VARIANT_LEARNED the mode applies to the exact solves. */
#define LGPU_PREC_FP32 0
#define LGPU_PREC_FP32_RESOLVE 1
#define LGPU_PREC_FP64 2
int lgpu_set_precision(lgpu_handle *h, int mode, float gap_threshold);

int lgpu_set_grid(lgpu_handle *h, int nij, const float *lat, const float *lon, const int *mask);
int lgpu_set_state(lgpu_handle *h, int k, int ns, const float *state, const float *mean,
                   const float *sprd, int nvars, const lgpu_statevar *vars);
int lgpu_set_obs(lgpu_handle *h, int nobs, const lgpu_obs *obs, const float *hx, const float *hx_mean);

/* letkf_obs_read's post-processing on the device (src/letkf_obs.F90:459-488),
 * the step before the analysis: hx_members holds the full observation-
 * operator values of every member [nobs][k]; the library forms
 * hx_mean = SUM(hx,1)/k and the perturbations, drops observations with
 * qc > 0 keeping the order of the rest, and then holds what lgpu_set_obs
 * would.  qc may be NULL (every observation kept).  *nobs_kept receives
 * the count after compaction. */
int lgpu_set_obs_raw(lgpu_handle *h, int nobs, const lgpu_obs *obs, const int *qc, const float *hx_members,
                     int *nobs_kept);

/* letkf_state_init's background statistics on the device
 * (src/letkf_state.F90:326-334): members holds the full ensemble
 * [ij][slab][member]; the library forms mean = SUM(x,1)/k, the
 * perturbations and sprd = SQRT(DOT(x',x')/(k-1)) and then holds what
 * lgpu_set_state would. */
int lgpu_set_state_members(lgpu_handle *h, int k, int ns, const float *members, int nvars,
                           const lgpu_statevar *vars);

/* Verification of the two calls above: copy back the prepared background
 * (perturbations, mean, spread) and the prepared observation arrays
 * (kept observations only: hx perturbations [n][k], hx_mean, and the
 * compacted lat/lon/val/err). */
int lgpu_get_background(lgpu_handle *h, float *state, float *mean, float *sprd);
int lgpu_get_obs_prepared(lgpu_handle *h, float *hx, float *hx_mean, float *lat, float *lon, float *val, float *err);

int lgpu_solver_run(lgpu_handle *h);

int lgpu_get_state(lgpu_handle *h, float *state, float *mean, float *sprd);

/* letkf_solver_run's in-place state (src/letkf_solver.F90:283-330 overwrites
 * state_ij, state_mean_ij, state_sprd_ij with the analysis): binds the
 * caller's arrays (layout and arguments as lgpu_set_state).  Each following
 * lgpu_solver_run reads the background from them and writes the analysis
 * back into them before it returns.  The background mean and spread are
 * uploaded first; the members follow on a copy stream once the Gram has run,
 * concurrently with the eigensolve (host<->device copies in flight slow the
 * tile-stream and Gram kernels, not the eigensolve or update); the
 * eigensolve and update run in column chunks whose update waits for its
 * members and whose analysis is downloaded while the next chunks are
 * computed.  Page-locked arrays (lgpu_host_alloc) give full link speed.  The arrays must stay allocated and untouched by the caller while
 * lgpu_solver_run executes; lgpu_set_state or another lgpu_bind_state
 * releases them. */
int lgpu_bind_state(lgpu_handle *h, int k, int ns, float *state, float *mean, float *sprd, int nvars,
                    const lgpu_statevar *vars);
int lgpu_get_diag(lgpu_handle *h, float *maxhz, float *obscount, float *lg_obscount, float *lg_obsloc);
int lgpu_get_timings(const lgpu_handle *h, lgpu_timings *t);
int lgpu_solver_final(lgpu_handle *h);

/* Verification: the local observation list of (ij, group) in canonical order
 * (ascending observation index) with its localisation weights; *n receives
 * the full count (entries beyond cap are not written), *ncand the number of
 * search candidates (diag_obscount).  Needs a prior lgpu_solver_run. */
int lgpu_get_obslist(lgpu_handle *h, int ij, int group, int *idx, float *rloc, int cap,
                     int *n, int *ncand);

/* lgpu_get_obslist for callers that cannot allocate device memory.
 * No counterpart in the reference (the reference builds its lists in Fortran
 * automatic arrays on the host stack).  It is meant for hosts that drive the
 * analysis from inside their own memory manager -- a model that takes its
 * device memory as one pool at start-up and hands it out itself, or a
 * cycling driver whose memory footprint is fixed once it starts -- where the
 * lazily grown list buffer of lgpu_get_obslist is not allowed.  Same
 * arguments, results and canonical order as lgpu_get_obslist.  It calls no
 * cudaMalloc/cudaFree: its scratch is one fixed __device__ array of
 * 4 * LGPU_NOALLOC_MAX_LIST + 64 ints (about 4 MB) that every device loading
 * the library holds until the process exits.  Handles whose observation
 * table is larger than LGPU_NOALLOC_MAX_LIST are rejected with
 * LGPU_ERR_CAPACITY.  All calls share that array, which keeps the last
 * call's contents (each call clears its counters and flags first): calls
 * that overlap on the GPU race and must be serialised by the caller.  The
 * first call on a device looks up the array's address. */
#define LGPU_NOALLOC_MAX_LIST 262144
int lgpu_get_obslist_noalloc(lgpu_handle *h, int ij, int group, int *idx, float *rloc, int cap,
                             int *n, int *ncand);


/* ---- Learned form: interpolation of (W, w-bar) with a learned correction.
 * No counterpart in the reference (it solves every column exactly).
 *
 * The grid must be a regular lattice, column ij = i + nx * j (i longitude,
 * j latitude), with nx a multiple of `stride`.  Columns with i % stride == 0
 * and j % stride == 0 are the coarse lattice.  The network maps, per column,
 * the bilinear interpolation of the four coarse neighbours' (W, w-bar)
 * (k*k + k values) and 16 observation-geometry features (local count, sums
 * of localisation weights, nearest-observation distance, innovation
 * moments, position in the coarse cell, neighbour spread) to a correction
 * of (W, w-bar): layers din -> hidden -> hidden -> dout, GELU, BF16 weights
 * and activations with FP32 accumulation; inference on the tensor cores
 * (tcgen05 kind::f16), training on the CUDA cores (Adam). */
typedef struct lgpu_learn_config {
  int nx, ny;            /* lattice */
  int stride;            /* coarse lattice stride (>= 2) */
  int hidden;            /* hidden width, a multiple of 16 (512) */
  float judge_frac;      /* fraction of the other columns solved exactly every analysis to judge the network (0.02) */
  float gate_frac;       /* fraction of calibration columns whose network output is large enough to send them to the exact solve (0.05) */
  float sample_frac;     /* fraction of the other columns of a collected analysis added to the training rows */
  int train_cap;         /* training rows kept */
  unsigned long long seed;
} lgpu_learn_config;

typedef struct lgpu_learn_stats {
  int coarse;            /* exact: coarse lattice columns */
  int judged;            /* exact: judge sample */
  int fallback;          /* exact: columns without four coarse neighbours */
  int gated;             /* exact: sent back by the gate */
  int inferred;          /* columns whose transform came from the network */
  float judge_rms;       /* RMS over judged, ungated columns of ||T_net - T_exact||_F / k */
  float judge_ref_rms;   /* RMS of ||T_exact - I||_F / k over the same columns */
  float tau;             /* gate threshold (RMS of the standardised network output) */
  long long train_rows;  /* training rows stored */
  float exact_ms, feature_ms, network_ms, apply_ms;   /* device time of the learned stages */
} lgpu_learn_stats;

int lgpu_learn_init(lgpu_handle *h, const lgpu_learn_config *cfg);
/* Runs an exact analysis (the AUTO / PLAIN / BATCHED_TC form in force; the
 * analysis result is the exact one) and adds training rows: network inputs
 * and residual targets (exact - interpolated) of a sample of the
 * non-lattice columns.  *rows receives the number of rows stored. */
int lgpu_learn_collect(lgpu_handle *h, long long *rows);
/* Standardises the stored rows (first call), runs `epochs` passes of Adam
 * with mini-batches of `batch` rows, then calibrates the gate threshold.
 * Once two or more analyses were collected, the rows of the last one are
 * held out of training and calibrate the gate.  *loss receives the mean
 * training loss of the last epoch (standardised units). */
int lgpu_learn_train(lgpu_handle *h, int epochs, int batch, float lr, float *loss);
int lgpu_learn_stats_get(lgpu_handle *h, lgpu_learn_stats *out);
/* use_network = 0: the LEARNED variant applies the bare interpolation (no
 * correction, the gate only for columns without four coarse neighbours): the
 * method without the network, for comparison. */
int lgpu_learn_set_network(lgpu_handle *h, int use_network);
/* Network parameters (FP32 masters; W1, b1, W2, b2, W3, b3 row-major
 * [out][in]); n must equal the count lgpu_learn_param_count returns. */
long long lgpu_learn_param_count(lgpu_handle *h);
int lgpu_learn_get_params(lgpu_handle *h, float *params, long long n);
int lgpu_learn_set_params(lgpu_handle *h, const float *params, long long n);

/* Verification of the network kernels (standalone, allocates): for rows x
 * [rows][din] (rounded to BF16 inside) and targets t [rows][dout], with the
 * parameters given (rounded to BF16 inside), returns the mean squared error
 * *loss, its gradient (FP32, the parameter layout) from the training
 * kernels, the output of the CUDA-core forward y_simt and of the tensor-core
 * forward y_tc ([rows][dout] each; any may be null). */
int lgpu_mlp_debug(int device, int din, int hidden, int dout, int rows, const float *params, const float *x,
                   const float *t, float *loss, float *grad, float *y_simt, float *y_tc);

/* ---- Diagnostics files (save_diag) ----------------------------------------
 * letkf_solver_final's diag.solver.nc (src/letkf_solver.F90:397-527) from
 * the last run: dimensions time (1), lat (ny), lon (nx), loc_group; lat and
 * lon from lat_nom / lon_nom; col_maxhz, col_obscount [time][lat][lon] and
 * lg_obscount, lg_obsloc [time][loc_group][lat][lon] with the reference's
 * attributes.  The grid must be nx * ny columns, column ij = i + nx * j.
 * Masked columns hold 0, as the reference's initialised arrays do. */
int lgpu_write_diag(lgpu_handle *h, const char *path, int nx, int ny, const float *lat_nom, const float *lon_nom);
/* loc_ocean with vtloc_surf (src/subclass.letkf_localizer/letkf_loc_ocean.F90
 * :353-358): the level count of each column's surface localisation group
 * (calc_mldlvl_bkgt, :408-427) in the last run; 0 on masked columns. */
int lgpu_get_loc_diag(lgpu_handle *h, float *surf_lvl);
/* loc_ocean_final's diag.loc_ocean.nc (letkf_loc_ocean.F90:249-322):
 * vtloc_surf_lvl and vtloc_surf_depth = vert_nom(vtloc_surf_lvl) per column
 * (vert_nom: the nz nominal level depths, vtgrids(1)%vert_nom). */
int lgpu_write_loc_diag(lgpu_handle *h, const char *path, int nx, int ny, const float *lat_nom,
                        const float *lon_nom, int nz, const float *vert_nom);

/* ---- File formats (host code, no device needed) ---------------------------
 * NetCDF classic files, read and written by the library's own implementation
 * of the published format: versions CDF-1 (classic), CDF-2 (64-bit offset)
 * and CDF-5 (64-bit data) are read, any numeric type converted; files are
 * written as CDF-1 (CDF-2 above 2 GiB), big-endian, data laid out as the
 * netCDF library lays it out.  NetCDF-4 (HDF5) files are refused with
 * LGPU_ERR_UNSUPPORTED.  These calls take no handle: their error message is
 * lgpu_io_last_error() (per thread).  Array arguments are in file order
 * (slowest dimension first: a Fortran (nx, ny, nz) variable is [nz][ny][nx]). */
const char *lgpu_io_last_error(void);
/* parse_ens_filename (src/letkf_state_helper.F90:445-510): "#ENSn#" becomes
 * the member number zero-padded to n digits (ensmem >= 0), "mean" (-1
 * background, -2 analysis) or "sprd" (-3, -4); "#TYPE#" becomes "ana" (members,
 * -2, -4) or "bkg" (-1, -3). */
int lgpu_ens_filename(const char *pattern, int ensmem, char *out, int cap);
int lgpu_nc_dim_len(const char *path, const char *dim, long long *len);
int lgpu_nc_var_info(const char *path, const char *var, int *ndims, long long *dims, int maxdims);
int lgpu_nc_read_float(const char *path, const char *var, float *out, long long n);
int lgpu_nc_read_int(const char *path, const char *var, int *out, long long n);
/* obsio_nc_read_obs (src/subclass.letkf_obsio/letkf_obsio_nc.F90:150-237):
 * dimension "obs"; variables obid, plat, lat, lon, depth, hr, val, err, qc.
 * With lat == NULL only *nobs is set (to size the arrays). */
int lgpu_read_obs_nc(const char *path, int cap, int *nobs, float *lat, float *lon, float *zdim, float *time,
                     float *val, float *err, int *obsid, int *platid, int *qc);
/* obsio_nc_read_hx (letkf_obsio_nc.F90:244-306): one member's H(x) ("hx"),
 * or "val" + "inc" when read_inc is set; the "obs" dimension must equal nobs. */
int lgpu_read_hx_nc(const char *path, int nobs, int read_inc, float *hx);
/* stateio_nc_read_state (src/subclass.letkf_stateio/letkf_stateio_nc.F90:
 * 196-245): variable `var` holding nx * ny * nz values ([nz][ny][nx]). */
int lgpu_read_state_nc(const char *path, const char *var, int nx, int ny, int nz, float *out);
/* stateio_nc_write_state (letkf_stateio_nc.F90:252-370) as a classic file
 * (the reference writes NetCDF-4 with deflate): dimensions time (record),
 * lon, lat and each vertical grid; coordinate variables lon, lat and the
 * vertical grids with the reference's attributes; state variable v as
 * [time][vt][lat][lon] on vertical grid var_vt[v], one record. */
int lgpu_write_state_nc(const char *path, int nx, int ny, const float *lon_nom, const float *lat_nom, int nvt,
                        const char *const *vt_names, const int *vt_len, const float *const *vt_nom, int nvar,
                        const char *const *names, const int *var_vt, const float *const *vals);
/* The two diagnostics files from host arrays (layouts as lgpu_write_diag /
 * lgpu_write_loc_diag). */
int lgpu_write_diag_nc(const char *path, int nx, int ny, int groups, const float *lat_nom, const float *lon_nom,
                       const float *maxhz, const float *obscount, const float *lg_obscount, const float *lg_obsloc);
int lgpu_write_loc_diag_nc(const char *path, int nx, int ny, const float *lat_nom, const float *lon_nom,
                           const float *surf_lvl, const float *surf_depth);

/* Page-locked host memory for callers that stream state in and out every
 * analysis (host<->device copies run at full link speed from it): an
 * anonymous mapping registered with CUDA (cudaMallocHost where that fails),
 * zero-filled.  Release it with lgpu_host_free. */
int lgpu_host_alloc(size_t bytes, void **ptr);
int lgpu_host_free(void *ptr);

/* Benchmark hygiene: overwrite `bytes` of device scratch memory (owned by the
 * handle) on the library's stream so the next run starts with a cold L2. */
int lgpu_flush_l2(lgpu_handle *h, size_t bytes);

/* Verification: evaluate the library's distance metric and Gaspari-Cohn
 * weights on the device.  dist[i] = distance (m) between points
 * (lat1[i], lon1[i]) and (lat2[i], lon2[i]).  gc must hold 2n floats:
 * gc[i] = the fast single-precision weight used in the search loop and
 * gc[n + i] = letkf_loc_gc(z[i], L[i]) evaluated exactly as the reference
 * does (REAL(8), rounded to REAL). */
int lgpu_debug_metric(lgpu_handle *h, int n, const float *lat1, const float *lon1,
                      const float *lat2, const float *lon2, float *dist);
int lgpu_debug_gc(lgpu_handle *h, int n, const float *z, const float *L, float *gc);
/* Verification of the batched Gram's fast weight path: for point pairs
 * (lat1, lon1)-(lat2, lon2) and horizontal scales L, out receives 5n floats:
 * the exact distance, the fast distance, letkf_loc_gc of the exact distance
 * (REAL(8), rounded to REAL), the fast weight of the fast distance, and the
 * fast distance with the short asin series (valid for half-chords <= 0.25). */
int lgpu_debug_weight(lgpu_handle *h, int n, const float *lat1, const float *lon1, const float *lat2,
                      const float *lon2, const float *L, float *out);

/* Verification of the eigensolve stage alone (src/letkf_core.F90:100-141
 * with infl = 1): gram holds nunits packed blocks (upper triangle of
 * Yb^T R^-1 rho Yb row-major, then the right-hand side b; k(k+3)/2 floats);
 * trans receives T = W + wbar 1^T, [unit][i][j] row-major.  The precision
 * mode of lgpu_set_precision applies; lgpu_get_timings then reports the
 * FP64-solved unit count in fp64_units (the other fields are not set). */
int lgpu_debug_transform(lgpu_handle *h, int nunits, int k, const float *gram, float *trans);

#ifdef __cplusplus
}
#endif
#endif
