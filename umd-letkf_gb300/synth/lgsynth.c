/*
 * lgsynth.c -- seeded synthetic LETKF workloads.  See lgsynth.h.
 *
 * Everything here is input preparation: the background statistics and the
 * observation-space mean/perturbation split are computed on the host with the
 * reference's own float semantics so that the analysis path sees exactly the
 * arrays the reference's letkf_solver_run would see:
 *   src/letkf_state.F90:326-334   mean = SUM(x,1)/k, x' = x - mean,
 *                                 sprd = SQRT(DOT(x',x')/(k-1))
 *   src/letkf_obs.F90:459-466     hx_mean = SUM(hx,1)/k, hx' = hx - hx_mean
 *   src/subclass.letkf_obsio/letkf_obsio_test.F90:146-220
 *                                 synthetic obs: nearest grid point, nearest
 *                                 level, val = (O-F) + mean(hx)
 */
#include "lgsynth.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.14159265358979323846
#define D2R (PI_D / 180.0)
#define EARTH_R 6371000.0

/* ---------------------------------------------------------------- PRNG -- */
typedef struct { uint64_t s[4]; int have; double spare; } rng_t;

static uint64_t splitmix64(uint64_t *x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static void rng_init(rng_t *r, uint64_t seed, uint64_t purpose, uint64_t stream) {
  uint64_t x = seed ^ (purpose * 0xD1B54A32D192ED03ULL) ^ (stream * 0x8CB92BA72F3D8DD7ULL);
  for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
  r->have = 0;
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t rng_next(rng_t *r) {
  uint64_t *s = r->s;
  uint64_t res = rotl(s[1] * 5, 7) * 9;
  uint64_t t = s[1] << 17;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
  s[2] ^= t; s[3] = rotl(s[3], 45);
  return res;
}
static inline double rng_unif(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static double rng_normal(rng_t *r) {
  if (r->have) { r->have = 0; return r->spare; }
  double u1 = 1.0 - rng_unif(r);     /* (0,1] */
  double u2 = rng_unif(r);
  double rad = sqrt(-2.0 * log(u1));
  r->spare = rad * sin(2.0 * PI_D * u2);
  r->have = 1;
  return rad * cos(2.0 * PI_D * u2);
}

/* ------------------------------------------------------------ helpers -- */
static int nthreads_of(const lgs_options *o) {
#ifdef _OPENMP
  return o->nthreads > 0 ? o->nthreads : omp_get_max_threads();
#else
  (void)o; return 1;
#endif
}

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

void lgs_free(lgs_problem *p) {
  if (!p) return;
  free(p->lev_depth); free(p->lat); free(p->lon); free(p->mask);
  free(p->state); free(p->mean); free(p->sprd); free(p->truth);
  free(p->olat); free(p->olon); free(p->oz); free(p->otime); free(p->oval);
  free(p->oerr); free(p->oobsid); free(p->oplatid); free(p->oqc);
  free(p->hx); free(p->hx_mean);
  memset(p, 0, sizeof(*p));
}

void lgs_default_options(int w, lgs_options *o) {
  memset(o, 0, sizeof(*o));
  o->workload = w;
  switch (w) {
  case LGS_W_C1: o->seed = 1001; o->nx = 90; o->ny = 45; o->nz = 10; o->k = 20; o->n_obs = 5000; break;
  case LGS_W_C2: o->seed = 1002; o->nx = 720; o->ny = 360; o->nz = 40; o->k = 40;
    o->n_profiles = 3000; o->n_swaths = 50; o->swath_len = 4000; break;
  case LGS_W_C3: o->seed = 1003; o->nx = 720; o->ny = 360; o->nz = 40; o->k = 32;
    o->n_obs = 500000; o->n_clusters = 12; o->cluster_sigma_m = 300e3f; break;
  case LGS_W_C4: o->seed = 1004; o->nx = 1440; o->ny = 720; o->nz = 50; o->k = 100;
    o->n_obs = 1000000; o->n_clusters = 12; o->cluster_sigma_m = 300e3f; break;
  case LGS_W_SIMPLE3D: o->seed = 1011; o->nx = 180; o->ny = 90; o->nz = 5; o->k = 50; break;
  case LGS_W_OCEAN: o->seed = 1012; o->nx = 180; o->ny = 90; o->nz = 20; o->k = 10; break;
  default: break;
  }
}

/* Analytic land mask (nonzero = land) used by the ocean workloads: two
 * low-order harmonics of longitude/latitude plus an Antarctic cap.  About a
 * quarter to a third of the sphere is land. */
static int land_at(double lat_deg, double lon_deg) {
  double p = lat_deg * D2R, l = lon_deg * D2R;
  if (lat_deg < -70.0) return 1;
  double f = 0.55 * sin(2.0 * l + 0.4) * cos(1.7 * p) + 0.45 * sin(3.0 * l - 1.0) * cos(2.3 * p + 0.5);
  return f > 0.42;
}

static void lonlat_to_xyz(double lat, double lon, double v[3]) {
  double p = lat * D2R, l = lon * D2R;
  v[0] = cos(p) * cos(l); v[1] = cos(p) * sin(l); v[2] = sin(p);
}
static void xyz_to_lonlat(const double v[3], double *lat, double *lon) {
  double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  *lat = asin(v[2] / n) / D2R;
  double lo = atan2(v[1], v[0]) / D2R;
  if (lo < 0) lo += 360.0;
  if (lo >= 360.0) lo -= 360.0;
  *lon = lo;
}

static int nearest_col(const lgs_problem *p, double lat, double lon) {
  double dlon = 360.0 / p->nx, dlat = 180.0 / p->ny;
  double lo = fmod(lon, 360.0); if (lo < 0) lo += 360.0;
  int i = (int)floor(lo / dlon); if (i >= p->nx) i = p->nx - 1; if (i < 0) i = 0;
  int j = (int)floor((lat + 90.0) / dlat); if (j >= p->ny) j = p->ny - 1; if (j < 0) j = 0;
  return i + p->nx * j;
}

/* nearest level, ties to the deeper one (letkf_obsio_test.F90:188-200) */
static int nearest_level(const lgs_problem *p, double z) {
  int best = 0; double bd = fabs(p->lev_depth[0] - z);
  for (int l = 1; l < p->nz; l++) {
    double d = fabs(p->lev_depth[l] - z);
    if (d <= bd) { bd = d; best = l; }
  }
  return best;
}

/* -------------------------------------------------------------- fields -- */
/* background mean field of variable v at column c, level l */
static double mean_field(int w, const lgs_problem *p, int v, int c, int l) {
  double lat = p->lat[c], lon = p->lon[c], z = p->lev_depth[l];
  double ph = lat * D2R, la = lon * D2R;
  switch (w) {
  case LGS_W_C1:
    return 10.0 + 15.0 * cos(ph) * exp(-z / 1000.0);
  case LGS_W_SIMPLE3D:
    if (v == 0) return 1.0 * cos(ph) * exp(-z / 500.0);
    if (v == 1) return 1.0 * sin(2.0 * la) * cos(ph);
    return 0.5 * cos(3.0 * ph) * exp(-z / 500.0);
  case LGS_W_OCEAN: {
    /* a mixed layer whose depth varies with latitude/longitude */
    double mld = 40.0 + 60.0 * (1.0 + sin(2.0 * la)) * cos(ph);
    double t0 = 4.0 + 22.0 * cos(ph) * cos(ph);
    if (v == 0) return z <= mld ? t0 : t0 - 12.0 * (1.0 - exp(-(z - mld) / 400.0)) * cos(ph);
    if (v == 1) return 34.5 + 0.8 * cos(ph) * exp(-z / 800.0);
    if (v == 2) return 0.3 * sin(la) * cos(ph) * exp(-z / 300.0);
    return 0.2 * cos(2.0 * la) * cos(ph) * exp(-z / 300.0);
  }
  default: /* C2, C3, C4: T, S, SSH */
    if (v == 0) return 2.0 + 26.0 * cos(ph) * cos(ph) * exp(-z / 700.0) + 1.5 * sin(2.0 * la) * exp(-z / 1500.0);
    if (v == 1) return 34.2 + 1.2 * cos(ph) * exp(-z / 1000.0) + 0.2 * sin(la);
    return 0.8 * cos(ph) * sin(2.0 * la + 0.3);
  }
}

static double var_sigma(int w, int v) {
  switch (w) {
  case LGS_W_C1: case LGS_W_SIMPLE3D: return 1.0;
  case LGS_W_OCEAN: return v == 0 ? 0.5 : (v == 1 ? 0.1 : 0.05);
  default: return v == 0 ? 1.0 : (v == 1 ? 0.2 : 0.05);
  }
}

/* one smoothed N(0, sigma) horizontal field: 3-point box filter in longitude
 * (periodic) then latitude (edge replicated), rescaled by 3 so the filtered
 * field keeps unit variance away from the edges */
static void smooth_field(rng_t *r, int nx, int ny, double sigma, float *out, double *t1, double *t2) {
  for (int c = 0; c < nx * ny; c++) t1[c] = rng_normal(r);
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      int im = (i + nx - 1) % nx, ip = (i + 1) % nx;
      t2[i + nx * j] = (t1[im + nx * j] + t1[i + nx * j] + t1[ip + nx * j]) / 3.0;
    }
  for (int j = 0; j < ny; j++) {
    int jm = j > 0 ? j - 1 : 0, jp = j < ny - 1 ? j + 1 : ny - 1;
    for (int i = 0; i < nx; i++)
      out[i + nx * j] = (float)(3.0 * sigma * (t2[i + nx * jm] + t2[i + nx * j] + t2[i + nx * jp]) / 3.0);
  }
}

/* ------------------------------------------------------------ problem -- */
static int setup_grid(int w, const lgs_options *o, lgs_problem *p) {
  p->nx = o->nx; p->ny = o->ny; p->nz = o->nz; p->k = o->k;
  p->ncol = p->nx * p->ny;
  if (p->nx <= 0 || p->ny <= 0 || p->nz <= 0 || p->k < 2) return 1;
  p->lev_depth = xcalloc(p->nz, sizeof(float));
  for (int l = 0; l < p->nz; l++) {
    double z;
    if (w == LGS_W_C1) z = 5.0 + 100.0 * l;
    else if (w == LGS_W_SIMPLE3D) { static const double d[] = {1, 10, 50, 100, 200, 400, 800, 1600}; z = l < 8 ? d[l] : 1600.0 + 400.0 * (l - 7); }
    else if (w == LGS_W_OCEAN) z = 5.0 + 1995.0 * pow((double)l / (p->nz - 1), 2.0);
    else z = 5.0 + 4995.0 * pow((double)l / (p->nz > 1 ? p->nz - 1 : 1), 2.0);
    p->lev_depth[l] = (float)z;
  }
  /* variables */
  const char *names[LGS_MAXVARS]; int lev[LGS_MAXVARS]; int nv = 0;
  switch (w) {
  case LGS_W_C1: names[0] = "T"; lev[0] = p->nz; nv = 1; break;
  case LGS_W_SIMPLE3D: names[0] = "state1"; names[1] = "state2"; names[2] = "state3";
    lev[0] = lev[1] = lev[2] = p->nz; nv = 3; break;
  case LGS_W_OCEAN: names[0] = "ocn_t"; names[1] = "ocn_s"; names[2] = "ocn_u"; names[3] = "ocn_v";
    lev[0] = lev[1] = lev[2] = lev[3] = p->nz; nv = 4; break;
  case LGS_W_C4: names[0] = "T"; names[1] = "S"; lev[0] = lev[1] = p->nz; nv = 2; break;
  default: names[0] = "T"; names[1] = "S"; names[2] = "SSH"; lev[0] = lev[1] = p->nz; lev[2] = 1; nv = 3; break;
  }
  p->nvars = nv; p->ns = 0;
  for (int v = 0; v < nv; v++) {
    memset(&p->vars[v], 0, sizeof(lgs_var));
    strncpy(p->vars[v].name, names[v], 15);
    p->vars[v].grid_s_idx = p->ns; p->vars[v].levels = lev[v];
    p->vars[v].ana_inc_max = 9.99e36f;
    p->vars[v].ana_bounds[0] = -9.99e36f; p->vars[v].ana_bounds[1] = 9.99e36f;
    p->ns += lev[v];
  }
  p->lat = xcalloc(p->ncol, sizeof(float)); p->lon = xcalloc(p->ncol, sizeof(float));
  p->mask = xcalloc(p->ncol, sizeof(int));
  if (!p->lat || !p->lon || !p->mask || !p->lev_depth) return 2;
  double dlon = 360.0 / p->nx, dlat = 180.0 / p->ny;
  int ocean = (w == LGS_W_C2 || w == LGS_W_C3 || w == LGS_W_C4 || w == LGS_W_OCEAN);
  for (int j = 0; j < p->ny; j++)
    for (int i = 0; i < p->nx; i++) {
      int c = i + p->nx * j;
      p->lon[c] = (float)((i + 0.5) * dlon);
      p->lat[c] = (float)(-90.0 + (j + 0.5) * dlat);
      p->mask[c] = ocean ? land_at(p->lat[c], p->lon[c]) : 0;
    }
  return 0;
}

/* members (full values) and truth, then the reference's background
 * mean/perturbation/spread split */
static int make_ensemble(int w, const lgs_options *o, lgs_problem *p) {
  size_t ncol = p->ncol, ns = p->ns, k = p->k;
  p->state = malloc(ncol * ns * k * sizeof(float));
  p->mean = malloc(ncol * ns * sizeof(float));
  p->sprd = malloc(ncol * ns * sizeof(float));
  p->truth = malloc(ncol * ns * sizeof(float));
  float *mf = malloc(ncol * ns * sizeof(float));  /* analytic mean field */
  if (!p->state || !p->mean || !p->sprd || !p->truth || !mf) { free(mf); return 2; }
  for (int v = 0; v < p->nvars; v++)
    for (int l = 0; l < p->vars[v].levels; l++) {
      int s = p->vars[v].grid_s_idx + l;
      for (size_t c = 0; c < ncol; c++) mf[c * ns + s] = (float)mean_field(w, p, v, (int)c, l);
    }
  int nth = nthreads_of(o);
  int nstreams = (int)k + 1;   /* members 0..k-1, truth = k */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
  for (int m = 0; m < nstreams; m++) {
    rng_t r; rng_init(&r, o->seed, 1, (uint64_t)m);
    float *f = malloc(ncol * sizeof(float));
    double *t1 = malloc(ncol * sizeof(double)), *t2 = malloc(ncol * sizeof(double));
    for (int v = 0; v < p->nvars; v++)
      for (int l = 0; l < p->vars[v].levels; l++) {
        int s = p->vars[v].grid_s_idx + l;
        smooth_field(&r, p->nx, p->ny, var_sigma(w, v), f, t1, t2);
        if (m < (int)k) {
          for (size_t c = 0; c < ncol; c++) p->state[(c * ns + s) * k + m] = mf[c * ns + s] + f[c];
        } else {
          for (size_t c = 0; c < ncol; c++) p->truth[c * ns + s] = mf[c * ns + s] + f[c];
        }
      }
    free(f); free(t1); free(t2);
  }
  free(mf);
  /* src/letkf_state.F90:326-334, float arithmetic in member order */
#pragma omp parallel for schedule(static) num_threads(nth)
  for (size_t cs = 0; cs < ncol * ns; cs++) {
    float *x = p->state + cs * k;
    float sum = 0.0f;
    for (size_t m = 0; m < k; m++) sum += x[m];
    float mean = sum / (float)k;
    float dot = 0.0f;
    for (size_t m = 0; m < k; m++) { x[m] = x[m] - mean; dot += x[m] * x[m]; }
    p->mean[cs] = mean;
    p->sprd[cs] = sqrtf(dot / (float)(k - 1));
  }
  return 0;
}

static int alloc_obs(lgs_problem *p, int n) {
  p->nobs = n;
  p->olat = xcalloc(n, 4); p->olon = xcalloc(n, 4); p->oz = xcalloc(n, 4); p->otime = xcalloc(n, 4);
  p->oval = xcalloc(n, 4); p->oerr = xcalloc(n, 4); p->oobsid = xcalloc(n, 4); p->oplatid = xcalloc(n, 4);
  p->oqc = xcalloc(n, 4); p->hx = xcalloc((size_t)n * p->k, 4); p->hx_mean = xcalloc(n, 4);
  return (p->olat && p->olon && p->oz && p->otime && p->oval && p->oerr && p->oobsid && p->oplatid &&
          p->oqc && p->hx && p->hx_mean) ? 0 : 2;
}

/* full member value of slab s at column c (perturbation + mean) */
static inline float member_val(const lgs_problem *p, int c, int s, int m) {
  return p->state[((size_t)c * p->ns + s) * p->k + m] + p->mean[(size_t)c * p->ns + s];
}

/* src/letkf_obs.F90:459-466 */
static void obs_split_hx(lgs_problem *p) {
  int k = p->k;
  for (int o = 0; o < p->nobs; o++) {
    float *h = p->hx + (size_t)o * k;
    float sum = 0.0f;
    for (int m = 0; m < k; m++) sum += h[m];
    float mean = sum / (float)k;
    for (int m = 0; m < k; m++) h[m] = h[m] - mean;
    p->hx_mean[o] = mean;
  }
}

/* nearest-column, exact-level observation operator, hx from full members */
static void obs_nearest(lgs_problem *p, int o, int slab, rng_t *r) {
  int c = nearest_col(p, p->olat[o], p->olon[o]);
  for (int m = 0; m < p->k; m++) p->hx[(size_t)o * p->k + m] = member_val(p, c, slab, m);
  p->oval[o] = (float)(p->truth[(size_t)c * p->ns + slab] + p->oerr[o] * rng_normal(r));
}

/* trilinear observation operator (bilinear between cell centres, linear in
 * depth) applied to each member and to the truth */
static void obs_trilinear(lgs_problem *p, int o, int var, rng_t *r) {
  double dlon = 360.0 / p->nx, dlat = 180.0 / p->ny;
  double x = p->olon[o] / dlon - 0.5, y = (p->olat[o] + 90.0) / dlat - 0.5;
  int i0 = (int)floor(x); double fx = x - i0;
  int j0 = (int)floor(y); double fy = y - j0;
  int i1 = i0 + 1, j1 = j0 + 1;
  i0 = ((i0 % p->nx) + p->nx) % p->nx; i1 = ((i1 % p->nx) + p->nx) % p->nx;
  if (j0 < 0) { j0 = 0; fy = 0.0; }
  if (j1 > p->ny - 1) { j1 = p->ny - 1; }
  if (j0 > p->ny - 1) j0 = p->ny - 1;
  int l0 = 0; double fz = 0.0; double z = p->oz[o];
  if (z <= p->lev_depth[0]) { l0 = 0; fz = 0.0; }
  else if (z >= p->lev_depth[p->nz - 1]) { l0 = p->nz - 1; fz = 0.0; }
  else {
    while (l0 < p->nz - 2 && p->lev_depth[l0 + 1] < z) l0++;
    fz = (z - p->lev_depth[l0]) / (p->lev_depth[l0 + 1] - p->lev_depth[l0]);
  }
  int l1 = l0 + 1 < p->nz ? l0 + 1 : l0;
  int s0 = p->vars[var].grid_s_idx + l0, s1 = p->vars[var].grid_s_idx + l1;
  int cs[4] = {i0 + p->nx * j0, i1 + p->nx * j0, i0 + p->nx * j1, i1 + p->nx * j1};
  double wh[4] = {(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy};
  for (int m = 0; m <= p->k; m++) {
    double v = 0.0;
    for (int q = 0; q < 4; q++) {
      double a, b;
      if (m < p->k) { a = member_val(p, cs[q], s0, m); b = member_val(p, cs[q], s1, m); }
      else { a = p->truth[(size_t)cs[q] * p->ns + s0]; b = p->truth[(size_t)cs[q] * p->ns + s1]; }
      v += wh[q] * ((1 - fz) * a + fz * b);
    }
    if (m < p->k) p->hx[(size_t)o * p->k + m] = (float)v;
    else p->oval[o] = (float)(v + p->oerr[o] * rng_normal(r));
  }
}

static void random_ocean_point(const lgs_problem *p, rng_t *r, double *lat, double *lon) {
  for (int tries = 0; tries < 100000; tries++) {
    double la = asin(2.0 * rng_unif(r) - 1.0) / D2R, lo = 360.0 * rng_unif(r);
    if (!p->mask[nearest_col(p, la, lo)]) { *lat = la; *lon = lo; return; }
  }
  *lat = 0.0; *lon = 180.0;
}

static int make_obs_c1(const lgs_options *o, lgs_problem *p) {
  if (alloc_obs(p, o->n_obs)) return 2;
  rng_t r; rng_init(&r, o->seed, 3, 0);
  for (int i = 0; i < p->nobs; i++) {
    p->olat[i] = (float)(asin(2.0 * rng_unif(&r) - 1.0) / D2R);
    p->olon[i] = (float)(360.0 * rng_unif(&r));
    p->oz[i] = (float)(5.0 + 900.0 * rng_unif(&r));
    p->otime[i] = 0.0f; p->oerr[i] = 0.5f; p->oobsid[i] = 1; p->oplatid[i] = 1;
  }
  rng_t re; rng_init(&re, o->seed, 4, 0);
  for (int i = 0; i < p->nobs; i++) obs_trilinear(p, i, 0, &re);
  obs_split_hx(p);
  return 0;
}

/* C2: T/S profiles at random ocean points + SSH/SST along great-circle swaths */
static int make_obs_c2(const lgs_options *o, lgs_problem *p) {
  int nprof = o->n_profiles, nl = p->vars[0].levels;
  int n = nprof * nl * 2 + o->n_swaths * o->swath_len;
  if (alloc_obs(p, n)) return 2;
  rng_t r; rng_init(&r, o->seed, 3, 0);
  rng_t re; rng_init(&re, o->seed, 4, 0);
  int i = 0;
  for (int q = 0; q < nprof; q++) {
    double la, lo; random_ocean_point(p, &r, &la, &lo);
    float t = (float)(6.0 * rng_unif(&r) - 3.0);
    for (int l = 0; l < nl; l++)
      for (int v = 0; v < 2; v++) {
        p->olat[i] = (float)la; p->olon[i] = (float)lo; p->oz[i] = p->lev_depth[l]; p->otime[i] = t;
        p->oerr[i] = v == 0 ? 0.5f : 0.05f; p->oobsid[i] = v + 1; p->oplatid[i] = 1;
        obs_nearest(p, i, p->vars[v].grid_s_idx + l, &re);
        i++;
      }
  }
  for (int sw = 0; sw < o->n_swaths; sw++) {
    double nvec[3]; double la0 = asin(2.0 * rng_unif(&r) - 1.0) / D2R, lo0 = 360.0 * rng_unif(&r);
    lonlat_to_xyz(la0, lo0, nvec);
    /* orthonormal a, b perpendicular to nvec */
    double a[3] = {-nvec[1], nvec[0], 0.0};
    double an = sqrt(a[0] * a[0] + a[1] * a[1]);
    if (an < 1e-6) { a[0] = 1; a[1] = 0; a[2] = 0; an = 1; }
    a[0] /= an; a[1] /= an;
    double b[3] = {nvec[1] * a[2] - nvec[2] * a[1], nvec[2] * a[0] - nvec[0] * a[2], nvec[0] * a[1] - nvec[1] * a[0]};
    double s = 2.0 * PI_D * rng_unif(&r), ds = 2.0 * PI_D / (o->swath_len * 1.6);
    int acc = 0;
    for (long step = 0; acc < o->swath_len && step < 100L * o->swath_len; step++, s += ds) {
      double jit = (rng_unif(&r) - 0.5) * (100e3 / EARTH_R);
      double v[3];
      for (int d = 0; d < 3; d++) v[d] = cos(s) * a[d] + sin(s) * b[d] + jit * nvec[d];
      double la, lo; xyz_to_lonlat(v, &la, &lo);
      if (p->mask[nearest_col(p, la, lo)]) continue;
      int ssh = (acc % 2) == 0;
      p->olat[i] = (float)la; p->olon[i] = (float)lo; p->oz[i] = 0.0f;
      p->otime[i] = (float)(6.0 * rng_unif(&r) - 3.0);
      p->oerr[i] = ssh ? 0.02f : 0.3f; p->oobsid[i] = ssh ? 3 : 4; p->oplatid[i] = 2;
      obs_nearest(p, i, ssh ? p->vars[2].grid_s_idx : p->vars[0].grid_s_idx, &re);
      i++; acc++;
    }
  }
  p->nobs = i;
  obs_split_hx(p);
  return 0;
}

/* C3/C4: clustered point obs (Gaussian clusters of given sigma + 10% uniform),
 * T/S at a random level, or SSH when the state has it */
static int make_obs_clustered_c(const lgs_options *o, lgs_problem *p, uint64_t centre_seed) {
  if (alloc_obs(p, o->n_obs)) return 2;
  rng_t r; rng_init(&r, centre_seed, 3, 0);
  rng_t re; rng_init(&re, o->seed, 4, 0);
  int nc = o->n_clusters > 0 ? o->n_clusters : 1;
  double cen[64][3];
  for (int c = 0; c < nc && c < 64; c++) { double la, lo; random_ocean_point(p, &r, &la, &lo); lonlat_to_xyz(la, lo, cen[c]); }
  if (centre_seed != o->seed) rng_init(&r, o->seed, 3, 0);   /* positions drawn with the observation seed */
  int has_ssh = p->nvars >= 3;
  for (int i = 0; i < p->nobs; i++) {
    double la, lo;
    for (;;) {
      if (rng_unif(&r) < 0.1) { la = asin(2.0 * rng_unif(&r) - 1.0) / D2R; lo = 360.0 * rng_unif(&r); }
      else {
        const double *c = cen[(int)(rng_unif(&r) * nc) % nc];
        double e1[3] = {-c[1], c[0], 0.0}; double en = sqrt(e1[0] * e1[0] + e1[1] * e1[1]);
        if (en < 1e-9) { e1[0] = 1; e1[1] = 0; en = 1; }
        e1[0] /= en; e1[1] /= en;
        double e2[3] = {c[1] * e1[2] - c[2] * e1[1], c[2] * e1[0] - c[0] * e1[2], c[0] * e1[1] - c[1] * e1[0]};
        double gx = rng_normal(&r) * o->cluster_sigma_m / EARTH_R, gy = rng_normal(&r) * o->cluster_sigma_m / EARTH_R;
        double v[3]; for (int d = 0; d < 3; d++) v[d] = c[d] + gx * e1[d] + gy * e2[d];
        xyz_to_lonlat(v, &la, &lo);
      }
      if (!p->mask[nearest_col(p, la, lo)]) break;
    }
    double u = rng_unif(&r);
    int kind = (has_ssh && u < 0.1) ? 2 : (u < 0.55 ? 0 : 1);
    int lvl = kind == 2 ? 0 : (int)(rng_unif(&r) * p->nz) % p->nz;
    p->olat[i] = (float)la; p->olon[i] = (float)lo; p->oz[i] = kind == 2 ? 0.0f : p->lev_depth[lvl];
    p->otime[i] = (float)(6.0 * rng_unif(&r) - 3.0);
    p->oerr[i] = kind == 0 ? 0.5f : (kind == 1 ? 0.05f : 0.02f);
    p->oobsid[i] = kind + 1; p->oplatid[i] = kind == 2 ? 2 : 1;
    obs_nearest(p, i, p->vars[kind].grid_s_idx + lvl, &re);
  }
  obs_split_hx(p);
  return 0;
}

/* letkf_obsio_test semantics (src/subclass.letkf_obsio/letkf_obsio_test.F90:146-220):
 * hx = member value at the nearest grid point and nearest level,
 * val = (O-F) + SUM(hx)/k */
typedef struct { int obsid, platid, var; float lat, lon, z, time, inc, err; } synth_ob;

static int make_obs_listed(lgs_problem *p, const synth_ob *list, int n) {
  if (alloc_obs(p, n)) return 2;
  for (int i = 0; i < n; i++) {
    const synth_ob *s = &list[i];
    float lo = s->lon; if (lo < 0) lo += 360.0f;
    p->olat[i] = s->lat; p->olon[i] = s->lon; p->oz[i] = s->z; p->otime[i] = s->time;
    p->oerr[i] = s->err; p->oobsid[i] = s->obsid; p->oplatid[i] = s->platid;
    /* nearest grid point by great-circle distance */
    double vo[3]; lonlat_to_xyz(s->lat, lo, vo);
    int best = 0; double bd = 1e300;
    for (int c = 0; c < p->ncol; c++) {
      double vc[3]; lonlat_to_xyz(p->lat[c], p->lon[c], vc);
      double d = (vo[0] - vc[0]) * (vo[0] - vc[0]) + (vo[1] - vc[1]) * (vo[1] - vc[1]) + (vo[2] - vc[2]) * (vo[2] - vc[2]);
      if (d < bd) { bd = d; best = c; }
    }
    int lvl = nearest_level(p, s->z);
    int slab = p->vars[s->var].grid_s_idx + (p->vars[s->var].levels > 1 ? lvl : 0);
    float sum = 0.0f;
    for (int m = 0; m < p->k; m++) {
      float h = p->state[((size_t)best * p->ns + slab) * p->k + m] + p->mean[(size_t)best * p->ns + slab];
      p->hx[(size_t)i * p->k + m] = h; sum += h;
    }
    p->oval[i] = s->inc + sum / (float)p->k;
  }
  obs_split_hx(p);
  return 0;
}

static int make_obs_clustered(const lgs_options *o, lgs_problem *p) { return make_obs_clustered_c(o, p, o->seed); }

int lgs_generate(const lgs_options *opt, lgs_problem *out) {
  memset(out, 0, sizeof(*out));
  lgs_options o; lgs_default_options(opt->workload, &o);
  /* caller overrides */
  if (opt->seed) o.seed = opt->seed;
  if (opt->nx > 0) o.nx = opt->nx;
  if (opt->ny > 0) o.ny = opt->ny;
  if (opt->nz > 0) o.nz = opt->nz;
  if (opt->k > 0) o.k = opt->k;
  if (opt->n_profiles > 0) o.n_profiles = opt->n_profiles;
  if (opt->n_swaths > 0) o.n_swaths = opt->n_swaths;
  if (opt->swath_len > 0) o.swath_len = opt->swath_len;
  if (opt->n_obs > 0) o.n_obs = opt->n_obs;
  if (opt->n_clusters > 0) o.n_clusters = opt->n_clusters;
  if (opt->cluster_sigma_m > 0) o.cluster_sigma_m = opt->cluster_sigma_m;
  o.nthreads = opt->nthreads;
  int w = o.workload;
  if (w < LGS_W_C1 || w > LGS_W_OCEAN) return 1;
  int rc = setup_grid(w, &o, out);
  if (!rc) rc = make_ensemble(w, &o, out);
  if (!rc) {
    switch (w) {
    case LGS_W_C1: rc = make_obs_c1(&o, out); break;
    case LGS_W_C2: rc = make_obs_c2(&o, out); break;
    case LGS_W_C3: case LGS_W_C4: rc = make_obs_clustered(&o, out); break;
    case LGS_W_SIMPLE3D: {
      /* test/simple3d/default.yaml:16-19 */
      synth_ob l[2] = {{1, 1, 0, 40.5f, 220.5f, 1.0f, 0.0f, 1.0f, 1.0f},
                       {2, 1, 1, 1.5f, 220.5f, 1.0f, 10.0f, -1.0f, 1.0f}};
      rc = make_obs_listed(out, l, 2); break;
    }
    case LGS_W_OCEAN: {
      /* test/ocean/vtloc.yaml:93-99: obs type ocn_t (id 1) for all; platforms
       * ocn_sat = 1, ocn_prf = 2 (ids in order of first appearance) */
      synth_ob l[5] = {{1, 1, 0, 20.0f, -140.0f, 5.0f, 0.0f, -1.0f, 0.1f},
                       {1, 2, 0, 0.0f, -140.0f, 5.0f, 0.0f, -1.0f, 1.0f},
                       {1, 2, 0, 0.0f, -150.0f, 5.0f, 0.0f, -1.0f, 1.0f},
                       {1, 2, 0, 0.0f, -160.0f, 5.0f, 0.0f, -1.0f, 1.0f},
                       {1, 2, 1, 0.0f, -160.0f, 5.0f, 0.0f, 0.5f, 1.0f}};
      rc = make_obs_listed(out, l, 5); break;
    }
    }
  }
  if (rc) lgs_free(out);
  return rc;
}

/* ---- cycling experiments (the learned analysis form) ----
 * One forecast step on the regular lattice: every member (mean +
 * perturbation) and the truth are advected by a zonal wind u (m/s) over dt
 * seconds (semi-Lagrangian, linear interpolation, periodic in longitude) and
 * diffused with kappa (m^2/s, one explicit 5-point step, the coefficients
 * capped at 0.2 for stability near the poles); the background mean,
 * perturbations and spread are then recomputed (src/letkf_state.F90:326-334).
 * p holds caller arrays (grid, state, mean, sprd, truth). */
static void advect_field(const lgs_problem *p, double u, double kappa, double dt, float *f, float *g) {
  const int nx = p->nx, ny = p->ny;
  const double dl = 2.0 * PI_D / nx, dphi = PI_D / ny;
  for (int j = 0; j < ny; j++) {
    const double phi = (-90.0 + (j + 0.5) * 180.0 / ny) * D2R;
    const double cphi = fmax(cos(phi), 1e-3);
    const double sh = u * dt / (EARTH_R * cphi * dl);   /* cells moved eastwards */
    const double fl = floor(sh);
    const int is = (int)fl;
    const double a = sh - fl;
    for (int i = 0; i < nx; i++) {
      int i0 = ((i - is) % nx + nx) % nx, i1 = ((i - is - 1) % nx + nx) % nx;
      g[i + nx * j] = (float)((1.0 - a) * f[i0 + nx * j] + a * f[i1 + nx * j]);
    }
  }
  for (int j = 0; j < ny; j++) {
    const double phi = (-90.0 + (j + 0.5) * 180.0 / ny) * D2R;
    const double dx = EARTH_R * fmax(cos(phi), 1e-3) * dl, dy = EARTH_R * dphi;
    const double cx = fmin(0.2, kappa * dt / (dx * dx)), cy = fmin(0.2, kappa * dt / (dy * dy));
    const int jm = j > 0 ? j - 1 : j, jp = j < ny - 1 ? j + 1 : j;
    for (int i = 0; i < nx; i++) {
      const int im = (i + nx - 1) % nx, ip = (i + 1) % nx;
      const double c = g[i + nx * j];
      f[i + nx * j] = (float)(c + cx * (g[ip + nx * j] - 2.0 * c + g[im + nx * j]) +
                              cy * (g[i + nx * jp] - 2.0 * c + g[i + nx * jm]));
    }
  }
}

int lgs_forecast(lgs_problem *p, double u, double kappa, double dt, int nthreads) {
  const size_t ncol = (size_t)p->ncol, ns = (size_t)p->ns, k = (size_t)p->k;
  if (ncol != (size_t)p->nx * p->ny) return 1;
  const int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
  const long long ntask = (long long)ns * (long long)(k + 1);
  int bad = 0;
#pragma omp parallel num_threads(nth)
  {
    float *f = malloc(ncol * sizeof(float)), *g = malloc(ncol * sizeof(float));
    if (!f || !g) {
#pragma omp atomic write
      bad = 1;
    } else {
#pragma omp for schedule(dynamic, 1)
      for (long long t = 0; t < ntask; t++) {
        const size_t s = (size_t)(t / (long long)(k + 1)), m = (size_t)(t % (long long)(k + 1));
        if (m < k) {
          for (size_t c = 0; c < ncol; c++) f[c] = p->state[(c * ns + s) * k + m] + p->mean[c * ns + s];
        } else {
          for (size_t c = 0; c < ncol; c++) f[c] = p->truth[c * ns + s];
        }
        advect_field(p, u, kappa, dt, f, g);
        if (m < k) {
          for (size_t c = 0; c < ncol; c++) p->state[(c * ns + s) * k + m] = f[c];   /* full values for now */
        } else {
          for (size_t c = 0; c < ncol; c++) p->truth[c * ns + s] = f[c];
        }
      }
    }
    free(f);
    free(g);
  }
  if (bad) return 2;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (size_t cs = 0; cs < ncol * ns; cs++) {
    float *x = p->state + cs * k;
    float sum = 0.0f;
    for (size_t m = 0; m < k; m++) sum += x[m];
    float mean = sum / (float)k;
    float dot = 0.0f;
    for (size_t m = 0; m < k; m++) { x[m] = x[m] - mean; dot += x[m] * x[m]; }
    p->mean[cs] = mean;
    p->sprd[cs] = sqrtf(dot / (float)(k - 1));
  }
  return 0;
}

/* New clustered observations of p's current background and truth: the
 * C3/C4 network with its cluster centres drawn from centre_seed (a persistent
 * observing network), positions and errors from opt->seed; the observation
 * arrays are allocated here and freed by lgs_free_obs. */
int lgs_observe(const lgs_options *opt, lgs_problem *p, uint64_t centre_seed) {
  lgs_options o;
  lgs_default_options(LGS_W_C3, &o);
  o.seed = opt->seed;
  if (opt->n_obs > 0) o.n_obs = opt->n_obs;
  if (opt->n_clusters > 0) o.n_clusters = opt->n_clusters;
  if (opt->cluster_sigma_m > 0) o.cluster_sigma_m = opt->cluster_sigma_m;
  return make_obs_clustered_c(&o, p, centre_seed);
}

void lgs_free_obs(lgs_problem *p) {
  free(p->olat); free(p->olon); free(p->oz); free(p->otime); free(p->oval); free(p->oerr);
  free(p->oobsid); free(p->oplatid); free(p->oqc); free(p->hx); free(p->hx_mean);
  p->olat = p->olon = p->oz = p->otime = p->oval = p->oerr = p->hx = p->hx_mean = NULL;
  p->oobsid = p->oplatid = p->oqc = NULL;
  p->nobs = 0;
}
