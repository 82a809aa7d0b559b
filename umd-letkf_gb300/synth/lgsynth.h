/*
 * lgsynth.h -- seeded synthetic LETKF workloads (grid, background ensemble,
 * observations) for the GB300 analysis path, its tests and its benchmark.
 *
 * The reference (UMD-LETKF) reads its ensemble and observations from NetCDF
 * files; the regression data it uses is downloaded at configure time and is
 * not available.  These generators stand in for those files.  They produce
 * the module-global arrays the reference's solver consumes after its own
 * pre-processing has run:
 *   - state_ij(k,ns,ij) background perturbations, state_mean_ij, state_sprd_ij
 *     computed exactly as src/letkf_state.F90:326-334 does (float, k-1 spread);
 *   - obs_def (lat, lon, zdim, time, val, err, obsid, platid, qc), obs_hx as
 *     perturbations and obs_hx_mean, computed as src/letkf_obs.F90:459-466.
 *
 * Layouts are C, 0-based, and match the reference's Fortran column-major
 * arrays byte for byte: state[ij][slab][member], mean[ij][slab],
 * hx[obs][member].  Column ij runs longitude fastest, then latitude.
 *
 * PRNG: xoshiro256** (Blackman & Vigna, 2018) seeded through splitmix64,
 * one independent stream per (purpose, member) so the output does not depend
 * on the number of threads.  Normals: Box-Muller.
 */
#ifndef LGSYNTH_H
#define LGSYNTH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGS_MAXVARS 8

typedef struct lgs_var {
  char  name[16];
  int   grid_s_idx;     /* 0-based first slab of this variable */
  int   levels;         /* number of vertical levels (1 = 2-D) */
  float ana_inc_max;    /* default 9.99e36 (src/letkf_state.F90:95) */
  float ana_bounds[2];  /* default +-9.99e36 (src/letkf_state.F90:97) */
} lgs_var;

/* Options of the generic generator.  Zero / negative fields take the
 * defaults of the named workload. */
typedef struct lgs_options {
  int      workload;       /* LGS_W_* */
  uint64_t seed;
  int      nx, ny, nz;     /* grid (cell centred lon/lat, nz depth levels) */
  int      k;              /* ensemble size */
  int      n_profiles;     /* C2: number of T/S profiles */
  int      n_swaths;       /* C2: number of satellite swaths */
  int      swath_len;      /* C2: accepted obs per swath */
  int      n_obs;          /* C1/C3/C4: number of point obs */
  int      n_clusters;     /* C3/C4: number of Gaussian clusters */
  float    cluster_sigma_m;/* C3/C4: cluster standard deviation (m) */
  int      nthreads;       /* 0 = all available */
} lgs_options;

enum {
  LGS_W_C1 = 1,        /* 90x45x10, one 3-D temperature, k=20, 5,000 point obs */
  LGS_W_C2 = 2,        /* 720x360x40 ocean, T/S/SSH, k=40, profiles + swaths */
  LGS_W_C3 = 3,        /* 720x360x40 ocean, clustered obs, k=32 or 64 */
  LGS_W_C4 = 4,        /* 1440x720x50, T/S, k=100, clustered obs */
  LGS_W_SIMPLE3D = 5,  /* test/simple3d-style: 3 variables, two synthetic obs */
  LGS_W_OCEAN = 6      /* test/ocean vtloc-style: T/S/u/v, five synthetic obs */
};

typedef struct lgs_problem {
  int nx, ny, nz, ncol, k, ns, nvars, nobs;
  lgs_var vars[LGS_MAXVARS];
  float *lev_depth;      /* [nz] nominal level depth (m), vtgrids(1)%vert_nom */
  float *lat, *lon;      /* [ncol] degrees */
  int   *mask;           /* [ncol] nonzero = masked (land), mask_ij */
  float *state;          /* [ncol][ns][k] background perturbations */
  float *mean, *sprd;    /* [ncol][ns] */
  float *truth;          /* [ncol][ns] synthetic truth (diagnostics only) */
  /* observations (obs_def), already QC-compacted */
  float *olat, *olon, *oz, *otime, *oval, *oerr;
  int   *oobsid, *oplatid, *oqc;
  float *hx;             /* [nobs][k] perturbations */
  float *hx_mean;        /* [nobs] */
} lgs_problem;

/* Fill opt with the defaults of a workload (full published sizes). */
void lgs_default_options(int workload, lgs_options *opt);

/* Generate a problem.  Returns 0 on success, nonzero on a bad option or an
 * allocation failure.  Free with lgs_free. */
int lgs_generate(const lgs_options *opt, lgs_problem *out);
void lgs_free(lgs_problem *p);

/* Cycling experiments: one forecast step of members and truth (zonal
 * advection u m/s over dt s, diffusion kappa m^2/s) with the background
 * statistics recomputed; new clustered observations of the current state
 * (allocated here, freed by lgs_free_obs).  p may hold caller arrays. */
int lgs_forecast(lgs_problem *p, double u, double kappa, double dt, int nthreads);
int lgs_observe(const lgs_options *opt, lgs_problem *p, uint64_t centre_seed);
void lgs_free_obs(lgs_problem *p);

#ifdef __cplusplus
}
#endif
#endif
