/*
 * letkf_oracle.h -- CPU oracle for the LETKF per-gridpoint analysis path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (UMD-LETKF letkf_solver_run / letkf_core_solve / the localizer
 * plugins) used as the checker for the GPU library and as the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the GPU product never links or calls it.
 *
 * Parity status: the solver loop, core equations, Gaspari-Cohn function,
 * latitude interpolation and localizer plugins follow the reference source
 * line by line (citations in letkf_oracle.c) and are pinned by the
 * known-answer tests in tests/ plus a LAPACK (ssyev/dsyev) cross-check of the
 * eigensolver.  The observation-search metric is NOT pinned: the reference
 * delegates it to the geoKdTree submodule, which is absent, so the oracle and
 * the GPU library share a documented metric (great-circle distance on a
 * 6371 km sphere, evaluated by a fixed sequence of IEEE operations) and are
 * compared bit-exactly against each other.
 */
#ifndef LETKF_ORACLE_H
#define LETKF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAXINTERP 16
#define OR_MAXIDS 32
#define OR_MAXLEV 128
#define OR_MAXVARS 8

enum { OR_LOC_NOVRT = 0, OR_LOC_OCEAN = 1, OR_LOC_VTGC = 2 };

typedef struct or_interp {       /* linearinterp_lat (src/letkf_loc.F90:126-137) */
  int npoints;
  float lat[OR_MAXINTERP + 2];
  float dist[OR_MAXINTERP + 2];
} or_interp;

typedef struct or_loc {
  int cls;
  or_interp hz;                  /* novrt / vtgc: hzloc;  ocean: hzloc_prof */
  or_interp hz_sat;              /* ocean: hzloc_sat */
  float tloc_prof, tloc_sat;     /* ocean temporal localisation (<=0 off) */
  int vtloc_surf;                /* ocean: 0 none, 1 bkg_t */
  float bkg_t_delta;
  int bkg_t_idx, bkg_t_len;      /* 0-based first slab / levels of the T var */
  int n_sat_obs, sat_obs[OR_MAXIDS];
  int n_sat_plats, sat_plats[OR_MAXIDS];
  float vloc;                    /* vtgc vertical GC length scale (m) */
  int nlev;                      /* vtgc: number of level groups */
  float lev_depth[OR_MAXLEV];
  int maxgroups;
} or_loc;

typedef struct or_var { int grid_s_idx, levels; float ana_inc_max, ana_bounds[2]; } or_var;

typedef struct or_problem {
  int ncol, k, ns, nvars, nobs;
  or_var vars[OR_MAXVARS];
  const float *lat, *lon; const int *mask;
  const float *state, *mean, *sprd;          /* background: [ncol][ns][k], [ncol][ns] */
  const float *olat, *olon, *oz, *otime, *oval, *oerr;
  const int *oobsid, *oplatid;
  const float *hx, *hx_mean;                 /* [nobs][k], [nobs] */
  float rtps, rtpp, mul;
} or_problem;

typedef struct or_result {     /* outputs for the listed columns, compact */
  float *state, *mean, *sprd;  /* [ncl][ns][k], [ncl][ns], [ncl][ns] */
  float *maxhz, *obscount;     /* [ncl] */
  float *lg_obscount, *lg_obsloc;  /* [ncl][maxgroups] */
} or_result;

/* Build the oracle's search index and localizer tables.  Returns an opaque
 * context or NULL. */
void *or_create(const or_problem *p, const or_loc *loc);
void or_destroy(void *ctx);

/* Run the analysis for the listed columns (all columns when cols == NULL).
 * precision: 32 = float mirror of the reference arithmetic, 64 = double,
 * OR_PREC_LAPACK = the reference's own call sequence through the BLAS /
 * LAPACK routines registered with or_set_lapack (sgemm, ssyev: FP32).
 * Returns 0 on success. */
#define OR_PREC_LAPACK 1
int or_run(void *ctx, int precision, const int *cols, int ncl, or_result *res, int nthreads);

/* Local observation list of (column, group) in canonical order (ascending
 * observation index): returns the kept count n, writes min(n, cap) indices
 * and localisation weights; *ncand receives the search-candidate count. */
int or_obslist(void *ctx, int col, int group, int *idx, float *rloc, int cap, int *ncand);

/* Building blocks, exported for known-answer tests. */
float or_gc(float z, float L);                       /* letkf_loc_gc */
float or_interp_get(const or_interp *t, float lat);  /* linearinterp_lat_get_dist */
void or_interp_build(or_interp *t, int n, const float *lat, const float *radius);
void or_unitvec(float lat, float lon, float out[3]);
float or_dist(const float a[3], const float b[3]);
int or_eigh(int k, const double *A, double *lam, double *V);   /* Jacobi, ascending */
int or_core_solve(int precision, int k, int n, const float *hdxb, const float *rdiag,
                  const float *rloc, const float *dep, float infl, float *trans);

/* Fortran-convention BLAS sgemm and LAPACK ssyev (every argument by address)
 * for OR_PREC_LAPACK, e.g. an optimised library's entry points.  Returns 0
 * when both are non-NULL. */
typedef void (*or_sgemm_fn)(char *transa, char *transb, int *m, int *n, int *k, float *alpha, float *a, int *lda,
                            float *b, int *ldb, float *beta, float *c, int *ldc);
typedef void (*or_ssyev_fn)(char *jobz, char *uplo, int *n, float *a, int *lda, float *w, float *work, int *lwork,
                            int *info);
int or_set_lapack(or_sgemm_fn sgemm, or_ssyev_fn ssyev);

#ifdef __cplusplus
}
#endif
#endif
