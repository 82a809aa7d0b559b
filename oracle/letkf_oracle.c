/*
 * letkf_oracle.c -- CPU oracle for the LETKF per-gridpoint analysis path.
 *
 * TEST INFRASTRUCTURE ONLY (see letkf_oracle.h).  Citations are to the
 * reference source tree (UMD-LETKF), path:line.
 *
 * Two arithmetic modes:
 *   precision 32: mirrors the reference's REAL (float) arithmetic step by
 *                 step, including its redundant Pa*hdxb_rinv product
 *                 (src/letkf_core.F90:118) and float post-processing.
 *                 The eigensolver is a double-precision cyclic Jacobi whose
 *                 output is rounded to float (stand-in for LAPACK ssyev).
 *   precision 64: the same steps in double (the FP64 oracle).
 *   OR_PREC_LAPACK: the reference's own sequence of library calls
 *                 (sgemm / ssyev / sgemm / sgemm / sgemm, then one sgemm
 *                 per slab) through an optimised BLAS / LAPACK the caller
 *                 registers: the timed CPU baseline, with the arithmetic
 *                 the reference binary runs.
 * In both modes observation distances and localisation weights are the
 * float values the reference passes around (REAL), computed by the shared
 * documented metric below and by letkf_loc_gc in double, as the reference
 * does (src/letkf_loc.F90:348-378).
 *
 * Build with -ffp-contract=off: the metric must be evaluated with exactly the
 * listed IEEE operations so that observation lists match the GPU library bit
 * for bit.
 */
#include "letkf_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------ metric ---- */
/* sin/cos of an angle in degrees, double precision: exact reduction by
 * multiples of 90 degrees, then Taylor polynomials (coefficients 1/n!) on
 * |x| <= pi/4, Horner order fixed. */
static void sincos_deg(double a, double *s, double *c) {
  double q = floor(a / 90.0 + 0.5);
  double r = a - 90.0 * q;
  double x = r * 0.017453292519943295;
  double x2 = x * x;
  double p = 2.8114572543455206e-15;
  p = p * x2 + -7.647163731819816e-13;
  p = p * x2 + 1.6059043836821613e-10;
  p = p * x2 + -2.505210838544172e-08;
  p = p * x2 + 2.7557319223985893e-06;
  p = p * x2 + -0.0001984126984126984;
  p = p * x2 + 0.008333333333333333;
  p = p * x2 + -0.16666666666666666;
  double sn = x + x * (x2 * p);
  double u = 4.779477332387385e-14;
  u = u * x2 + -1.1470745597729725e-11;
  u = u * x2 + 2.08767569878681e-09;
  u = u * x2 + -2.755731922398589e-07;
  u = u * x2 + 2.48015873015873e-05;
  u = u * x2 + -0.001388888888888889;
  u = u * x2 + 0.041666666666666664;
  u = u * x2 + -0.5;
  double cs = 1.0 + x2 * u;
  long qi = ((long)q % 4 + 4) % 4;
  switch (qi) {
  case 0: *s = sn; *c = cs; break;
  case 1: *s = cs; *c = -sn; break;
  case 2: *s = -sn; *c = -cs; break;
  default: *s = -cs; *c = sn; break;
  }
}

void or_unitvec(float lat, float lon, float out[3]) {
  double sp, cp, sl, cl;
  sincos_deg((double)lat, &sp, &cp);
  sincos_deg((double)lon, &sl, &cl);
  out[0] = (float)(cp * cl);
  out[1] = (float)(cp * sl);
  out[2] = (float)sp;
}

/* asin(x) for 0 <= x <= 0.5: Taylor series (2n)!/(4^n (n!)^2 (2n+1)),
 * coefficients rounded to float, Horner in x^2 */
static float asin_poly(float x) {
  float x2 = x * x;
  float p = 0.008390335366129875f;
  p = p * x2 + 0.009761609137058258f;
  p = p * x2 + 0.01155180111527443f;
  p = p * x2 + 0.013964843936264515f;
  p = p * x2 + 0.017352763563394547f;
  p = p * x2 + 0.022372158244252205f;
  p = p * x2 + 0.0303819440305233f;
  p = p * x2 + 0.0446428582072258f;
  p = p * x2 + 0.07500000298023224f;
  p = p * x2 + 0.1666666716337204f;
  return x + x * (x2 * p);
}

/* great-circle distance (m) between two float unit vectors:
 * theta = 2 asin(|a-b|/2), R = 6371 km */
float or_dist(const float a[3], const float b[3]) {
  float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  float c2 = (dx * dx + dy * dy) + dz * dz;
  float h = 0.5f * sqrtf(c2);
  if (h > 1.0f) h = 1.0f;
  float ang;
  if (h <= 0.5f) ang = asin_poly(h);
  else ang = 1.5707963705062866f - 2.0f * asin_poly(sqrtf((1.0f - h) * 0.5f));
  return 12742000.0f * ang;
}

/* -------------------------------------------------- localisation ---- */
/* src/letkf_loc.F90:251-294: the 0-degree point takes the first radius, the
 * 90-degree point the last one */
void or_interp_build(or_interp *t, int n, const float *lat, const float *radius) {
  memset(t, 0, sizeof(*t));
  float last_lat = 0.0f, last_r = 0.0f;
  for (int i = 0; i < n && i < OR_MAXINTERP; i++) {
    if (lat[i] > 0.0f && t->npoints == 0) { t->lat[0] = 0.0f; t->dist[0] = radius[i]; t->npoints = 1; }
    t->lat[t->npoints] = lat[i]; t->dist[t->npoints] = radius[i]; t->npoints++;
    last_lat = lat[i]; last_r = radius[i];
  }
  if (last_lat < 90.0f) { t->lat[t->npoints] = 90.0f; t->dist[t->npoints] = last_r; t->npoints++; }
}

/* src/letkf_loc.F90:302-320 */
float or_interp_get(const or_interp *t, float lat) {
  float al = fabsf(lat);
  int i = 0;
  while (i < t->npoints - 1 && al > t->lat[i]) i++;
  if (i == 0) return t->dist[0];
  float d = (al - t->lat[i - 1]) / (t->lat[i] - t->lat[i - 1]);
  return d * t->dist[i] + (1.0f - d) * t->dist[i - 1];
}

/* letkf_loc_gc, src/letkf_loc.F90:348-378: REAL(8) evaluation with the
 * reference's truncated coefficients, rounded to REAL */
float or_gc(float z, float L) {
  double c = (double)L / sqrt(0.3);
  double abs_z = (double)fabsf(z);
  double zc = abs_z / c;
  double z2 = zc * zc, z3 = z2 * zc, z4 = z2 * z2, z5 = z4 * zc;
  double res;
  if (abs_z >= 2.0 * c) res = 0.0;
  else if (abs_z > c)
    res = 0.08333 * z5 - 0.5 * z4 + 0.625 * z3 + 1.66667 * z2 - 5.0 * zc + 4.0 - 0.66667 * c / abs_z;
  else
    res = -0.25 * z5 + 0.5 * z4 + 0.625 * z3 - 1.66667 * z2 + 1.0;
  return (float)res;
}

/* -------------------------------------------------------- context ---- */
#define NB 180
typedef struct {
  or_problem p;
  or_loc loc;
  float *ou;        /* [nobs][3] unit vectors */
  float *cu;        /* [ncol][3] */
  unsigned char *surf;  /* ocean: obs counts as surface/satellite */
  int *bstart;      /* [NB+1] band offsets into border */
  int *border;      /* obs ids sorted by band, then lon, then id */
  double *blon;     /* lon of border entries */
} ctx_t;

typedef struct { double lon; int id; } lonid;
static int cmp_lonid(const void *a, const void *b) {
  const lonid *x = a, *y = b;
  if (x->lon < y->lon) return -1;
  if (x->lon > y->lon) return 1;
  return x->id - y->id;
}

static double norm_lon(double lon) { double l = fmod(lon, 360.0); if (l < 0) l += 360.0; if (l >= 360.0) l -= 360.0; return l; }
static int band_of(double lat) { int b = (int)floor(lat + 90.0); return b < 0 ? 0 : (b >= NB ? NB - 1 : b); }

void *or_create(const or_problem *p, const or_loc *loc) {
  ctx_t *c = calloc(1, sizeof(ctx_t));
  if (!c) return NULL;
  c->p = *p; c->loc = *loc;
  int no = p->nobs;
  c->ou = malloc(sizeof(float) * 3 * (no ? no : 1));
  c->cu = malloc(sizeof(float) * 3 * (p->ncol ? p->ncol : 1));
  c->surf = calloc(no ? no : 1, 1);
  c->bstart = calloc(NB + 1, sizeof(int));
  c->border = malloc(sizeof(int) * (no ? no : 1));
  c->blon = malloc(sizeof(double) * (no ? no : 1));
  lonid *tmp = malloc(sizeof(lonid) * (no ? no : 1));
  int *cnt = calloc(NB, sizeof(int));
  if (!c->ou || !c->cu || !c->surf || !c->bstart || !c->border || !c->blon || !tmp || !cnt) {
    free(tmp); free(cnt); or_destroy(c); return NULL;
  }
  for (int i = 0; i < no; i++) or_unitvec(p->olat[i], p->olon[i], c->ou + 3 * i);
  for (int i = 0; i < p->ncol; i++) or_unitvec(p->lat[i], p->lon[i], c->cu + 3 * i);
  /* surface classification, src/subclass.letkf_localizer/letkf_loc_ocean.F90:467-479:
   * starts TRUE and is cleared by either non-empty list that misses the id */
  for (int i = 0; i < no; i++) {
    int s = 1;
    if (loc->n_sat_obs > 0) { int f = 0; for (int j = 0; j < loc->n_sat_obs; j++) if (p->oobsid[i] == loc->sat_obs[j]) { f = 1; break; } if (!f) s = 0; }
    if (loc->n_sat_plats > 0) { int f = 0; for (int j = 0; j < loc->n_sat_plats; j++) if (p->oplatid[i] == loc->sat_plats[j]) { f = 1; break; } if (!f) s = 0; }
    c->surf[i] = (unsigned char)s;
  }
  for (int i = 0; i < no; i++) cnt[band_of(p->olat[i])]++;
  c->bstart[0] = 0;
  for (int b = 0; b < NB; b++) c->bstart[b + 1] = c->bstart[b] + cnt[b];
  memset(cnt, 0, sizeof(int) * NB);
  for (int i = 0; i < no; i++) {
    int b = band_of(p->olat[i]);
    int pos = c->bstart[b] + cnt[b]++;
    tmp[pos].lon = norm_lon(p->olon[i]); tmp[pos].id = i;
  }
  for (int b = 0; b < NB; b++) qsort(tmp + c->bstart[b], c->bstart[b + 1] - c->bstart[b], sizeof(lonid), cmp_lonid);
  for (int i = 0; i < no; i++) { c->border[i] = tmp[i].id; c->blon[i] = tmp[i].lon; }
  free(tmp); free(cnt);
  return c;
}

void or_destroy(void *vc) {
  ctx_t *c = vc;
  if (!c) return;
  free(c->ou); free(c->cu); free(c->surf); free(c->bstart); free(c->border); free(c->blon);
  free(c);
}

static int lower_bound_lon(const double *a, int lo, int hi, double v) {
  while (lo < hi) { int m = (lo + hi) / 2; if (a[m] < v) lo = m + 1; else hi = m; }
  return lo;
}

typedef struct { int id; float d; } id_dist;
static int cmp_id(const void *a, const void *b) {
  int x = ((const id_dist *)a)->id, y = ((const id_dist *)b)->id;
  return (x > y) - (x < y);
}

/* all obs with dist <= rmax, ascending id; returns count (-1: out of
 * memory), fills ids & dist */
static int search(const ctx_t *c, int col, float rmax, int *ids, float *dist) {
  const float *cu = c->cu + 3 * col;
  double latc = c->p.lat[col], lonc = norm_lon(c->p.lon[col]);
  double alpha = (double)rmax / 6371000.0 * (1.0 + 1e-6) + 1e-9;
  double adeg = alpha * 57.29577951308232 + 0.01;
  int full = (latc + adeg >= 90.0) || (latc - adeg <= -90.0) || alpha >= 1.5;
  double dlon = 180.0;
  if (!full) {
    double s = sin(alpha) / cos(latc * 0.017453292519943295);
    dlon = s >= 1.0 ? 180.0 : asin(s) * 57.29577951308232 + 0.01;
  }
  int b0 = band_of(latc - adeg), b1 = band_of(latc + adeg);
  int n = 0;
  for (int b = b0; b <= b1; b++) {
    int lo = c->bstart[b], hi = c->bstart[b + 1];
    int seg[2][2]; int nseg = 0;
    if (full || dlon >= 179.99) { seg[0][0] = lo; seg[0][1] = hi; nseg = 1; }
    else {
      double w0 = lonc - dlon, w1 = lonc + dlon;
      if (w0 < 0.0) {
        seg[nseg][0] = lower_bound_lon(c->blon, lo, hi, w0 + 360.0); seg[nseg][1] = hi; nseg++;
        seg[nseg][0] = lo; seg[nseg][1] = lower_bound_lon(c->blon, lo, hi, w1 + 1e-9); nseg++;
      } else if (w1 >= 360.0) {
        seg[nseg][0] = lower_bound_lon(c->blon, lo, hi, w0); seg[nseg][1] = hi; nseg++;
        seg[nseg][0] = lo; seg[nseg][1] = lower_bound_lon(c->blon, lo, hi, w1 - 360.0 + 1e-9); nseg++;
      } else {
        seg[0][0] = lower_bound_lon(c->blon, lo, hi, w0); seg[0][1] = lower_bound_lon(c->blon, lo, hi, w1 + 1e-9); nseg = 1;
      }
    }
    for (int s = 0; s < nseg; s++)
      for (int q = seg[s][0]; q < seg[s][1]; q++) {
        int id = c->border[q];
        float d = or_dist(cu, c->ou + 3 * id);
        if (d <= rmax) { ids[n] = id; dist[n] = d; n++; }
      }
  }
  /* canonical order: ascending observation index (indices are unique) */
  int sorted = 1;
  for (int i = 1; i < n && sorted; i++) sorted = ids[i] > ids[i - 1];
  if (!sorted) {
    id_dist *t = malloc(sizeof(id_dist) * (size_t)n);
    if (!t) return -1;
    for (int i = 0; i < n; i++) { t[i].id = ids[i]; t[i].d = dist[i]; }
    qsort(t, (size_t)n, sizeof(id_dist), cmp_id);
    for (int i = 0; i < n; i++) { ids[i] = t[i].id; dist[i] = t[i].d; }
    free(t);
  }
  return n;
}

/* localizer%maxhz (loc_novrt :155-161, loc_ocean :435-443) */
static float loc_maxhz(const ctx_t *c, int col) {
  float lat = c->p.lat[col];
  if (c->loc.cls == OR_LOC_OCEAN) {
    float a = or_interp_get(&c->loc.hz, lat), b = or_interp_get(&c->loc.hz_sat, lat);
    return a > b ? a : b;
  }
  return or_interp_get(&c->loc.hz, lat);
}

/* localizer%groups: slab -> group index (0-based), group ids.
 * loc_novrt :133-147 (one group), loc_ocean :331-400 with calc_mldlvl_bkgt
 * :408-427 (surface / below-mixed-layer split), loc_vtgc (one group per
 * level) */
static int loc_groups(const ctx_t *c, int col, int *slab_group, int *gid) {
  const or_problem *p = &c->p;
  if (c->loc.cls == OR_LOC_OCEAN && c->loc.vtloc_surf == 1) {
    const float *m = p->mean + (size_t)col * p->ns;
    float t0 = m[c->loc.bkg_t_idx];
    int mld = c->loc.bkg_t_len;
    for (int i = 1; i <= c->loc.bkg_t_len - 1; i++) {
      float t1 = m[c->loc.bkg_t_idx + i];
      if (fabsf(t0 - t1) > c->loc.bkg_t_delta) { mld = i; break; }
    }
    for (int s = 0; s < p->ns; s++) slab_group[s] = -1;
    for (int v = 0; v < p->nvars; v++)
      for (int j = 0; j < p->vars[v].levels; j++)
        slab_group[p->vars[v].grid_s_idx + j] = (j + 1 <= mld) ? 0 : 1;
    gid[0] = 0; gid[1] = 1;
    return 2;
  }
  if (c->loc.cls == OR_LOC_VTGC) {
    for (int s = 0; s < p->ns; s++) slab_group[s] = -1;
    for (int v = 0; v < p->nvars; v++)
      for (int j = 0; j < p->vars[v].levels; j++) slab_group[p->vars[v].grid_s_idx + j] = j;
    for (int g = 0; g < c->loc.nlev; g++) gid[g] = g;
    return c->loc.nlev;
  }
  for (int s = 0; s < p->ns; s++) slab_group[s] = 0;
  gid[0] = 0;   /* loc_ocean without vtloc leaves the id unset; taken as the surface group */
  return 1;
}

/* localizer%localize (loc_novrt :170-183, loc_ocean :451-506, loc_vtgc) */
static float loc_localize(const ctx_t *c, int col, int gid, int ob, float dist) {
  const or_problem *p = &c->p;
  float lat = p->lat[col];
  switch (c->loc.cls) {
  case OR_LOC_OCEAN:
    if (c->surf[ob]) {
      if (gid == 1) return 0.0f;
      float r = or_gc(dist, or_interp_get(&c->loc.hz_sat, lat));
      if (c->loc.tloc_sat > 0.0f) r = r * or_gc(p->otime[ob], c->loc.tloc_sat);
      return r;
    } else {
      float r = or_gc(dist, or_interp_get(&c->loc.hz, lat));
      if (c->loc.tloc_prof > 0.0f) r = r * or_gc(p->otime[ob], c->loc.tloc_prof);
      return r;
    }
  case OR_LOC_VTGC: {
    float rh = or_gc(dist, or_interp_get(&c->loc.hz, lat));
    float rv = or_gc(fabsf(p->oz[ob] - c->loc.lev_depth[gid]), c->loc.vloc);
    return rh * rv;
  }
  default:
    return or_gc(dist, or_interp_get(&c->loc.hz, lat));
  }
}

/* ------------------------------------------------------ eigensolver ---- */
/* Cyclic-by-row Jacobi for a symmetric matrix (Golub & Van Loan, Matrix
 * Computations, 4th ed., Alg. 8.5.3), double precision.  A is k x k
 * column-major (only the upper triangle is read, as ssyev('V','U') does);
 * returns eigenvalues ascending and eigenvectors in the columns of V. */
int or_eigh(int k, const double *Ain, double *lam, double *V) {
  double *A = malloc(sizeof(double) * k * k);
  if (!A) return -1;
  for (int j = 0; j < k; j++)
    for (int i = 0; i < k; i++) A[i + k * j] = (i <= j) ? Ain[i + k * j] : Ain[j + k * i];
  for (int j = 0; j < k; j++) for (int i = 0; i < k; i++) V[i + k * j] = (i == j);
  int sweep;
  for (sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, dia = 0.0;
    for (int j = 0; j < k; j++) { dia += A[j + k * j] * A[j + k * j]; for (int i = 0; i < j; i++) off += A[i + k * j] * A[i + k * j]; }
    if (off <= 1e-32 * dia || off == 0.0) break;
    for (int pp = 0; pp < k - 1; pp++)
      for (int q = pp + 1; q < k; q++) {
        double apq = A[pp + k * q];
        if (apq == 0.0) continue;
        double app = A[pp + k * pp], aqq = A[q + k * q];
        double th = (aqq - app) / (2.0 * apq);
        double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < k; r++) {       /* columns pp, q */
          double a = A[r + k * pp], b = A[r + k * q];
          A[r + k * pp] = cs * a - sn * b; A[r + k * q] = sn * a + cs * b;
        }
        for (int r = 0; r < k; r++) {       /* rows pp, q */
          double a = A[pp + k * r], b = A[q + k * r];
          A[pp + k * r] = cs * a - sn * b; A[q + k * r] = sn * a + cs * b;
        }
        for (int r = 0; r < k; r++) {
          double a = V[r + k * pp], b = V[r + k * q];
          V[r + k * pp] = cs * a - sn * b; V[r + k * q] = sn * a + cs * b;
        }
      }
  }
  for (int i = 0; i < k; i++) lam[i] = A[i + k * i];
  /* sort ascending (selection sort, stable for ties) */
  for (int i = 0; i < k; i++) {
    int m = i;
    for (int j = i + 1; j < k; j++) if (lam[j] < lam[m]) m = j;
    if (m != i) {
      double t = lam[i]; lam[i] = lam[m]; lam[m] = t;
      for (int r = 0; r < k; r++) { double tv = V[r + k * i]; V[r + k * i] = V[r + k * m]; V[r + k * m] = tv; }
    }
  }
  free(A);
  return sweep < 100 ? 0 : 1;
}

/* ------------------------------------------------------ core solve ---- */
/* src/letkf_core.F90:69-146.  hdxb is [n][k] (= Fortran hdxb(k,n)), trans is
 * k x k column-major (= Fortran trans(k,k)). */
static int core32(int k, int n, const float *hdxb, const float *rdiag, const float *rloc,
                  const float *dep, float infl, float *trans, float *ws) {
  float *rinv = ws, *work1 = rinv + (size_t)n * k, *eivec = work1 + k * k, *pa = eivec + k * k;
  float *work2 = pa + k * k, *work3 = work2 + (size_t)k * n, *eival = work3 + k;
  double *A = (double *)(eival + k + (k & 1)), *lam = A + k * k, *V = lam + k;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < k; i++) rinv[(size_t)j * k + i] = hdxb[(size_t)j * k + i] / rdiag[j] * rloc[j];
  for (int l = 0; l < k; l++)
    for (int i = 0; i < k; i++) {
      float s = 0.0f;
      for (int j = 0; j < n; j++) s += rinv[(size_t)j * k + i] * hdxb[(size_t)j * k + l];
      work1[i + k * l] = s;
    }
  float r = (float)(k - 1) * 1.0f / infl;
  for (int i = 0; i < k; i++) work1[i + k * i] += r;
  for (int t = 0; t < k * k; t++) A[t] = work1[t];
  int rc = or_eigh(k, A, lam, V);
  for (int i = 0; i < k; i++) eival[i] = (float)lam[i];
  for (int t = 0; t < k * k; t++) eivec[t] = (float)V[t];
  for (int i = 0; i < k; i++) for (int r2 = 0; r2 < k; r2++) work1[r2 + k * i] = eivec[r2 + k * i] / eival[i];
  for (int l = 0; l < k; l++)
    for (int i = 0; i < k; i++) {
      float s = 0.0f;
      for (int m = 0; m < k; m++) s += work1[i + k * m] * eivec[l + k * m];
      pa[i + k * l] = s;
    }
  for (int j = 0; j < n; j++)
    for (int i = 0; i < k; i++) {
      float s = 0.0f;
      for (int m = 0; m < k; m++) s += pa[i + k * m] * rinv[(size_t)j * k + m];
      work2[i + (size_t)k * j] = s;
    }
  for (int i = 0; i < k; i++) work3[i] = 0.0f;
  for (int j = 0; j < n; j++) for (int i = 0; i < k; i++) work3[i] = work3[i] + work2[i + (size_t)k * j] * dep[j];
  for (int j = 0; j < k; j++) {
    float rr = sqrtf((float)(k - 1) / eival[j]);
    for (int i = 0; i < k; i++) work1[i + k * j] = eivec[i + k * j] * rr;
  }
  for (int l = 0; l < k; l++)
    for (int i = 0; i < k; i++) {
      float s = 0.0f;
      for (int m = 0; m < k; m++) s += work1[i + k * m] * eivec[l + k * m];
      trans[i + k * l] = s;
    }
  for (int j = 0; j < k; j++) for (int i = 0; i < k; i++) trans[i + k * j] = trans[i + k * j] + work3[i];
  return rc;
}

static int core64(int k, int n, const float *hdxb, const float *rdiag, const float *rloc,
                  const float *dep, double infl, double *trans, double *ws) {
  double *rinv = ws, *G = rinv + (size_t)n * k, *lam = G + k * k, *V = lam + k, *b = V + k * k, *wb = b + k, *tmp = wb + k;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < k; i++) rinv[(size_t)j * k + i] = (double)hdxb[(size_t)j * k + i] / (double)rdiag[j] * (double)rloc[j];
  for (int l = 0; l < k; l++)
    for (int i = 0; i < k; i++) {
      double s = 0.0;
      for (int j = 0; j < n; j++) s += rinv[(size_t)j * k + i] * (double)hdxb[(size_t)j * k + l];
      G[i + k * l] = s;
    }
  for (int i = 0; i < k; i++) G[i + k * i] += (double)(k - 1) / infl;
  int rc = or_eigh(k, G, lam, V);
  for (int i = 0; i < k; i++) {
    double s = 0.0;
    for (int j = 0; j < n; j++) s += rinv[(size_t)j * k + i] * (double)dep[j];
    b[i] = s;
  }
  /* wbar = V diag(1/lam) V^T b */
  for (int m = 0; m < k; m++) { double s = 0.0; for (int i = 0; i < k; i++) s += V[i + k * m] * b[i]; tmp[m] = s / lam[m]; }
  for (int i = 0; i < k; i++) { double s = 0.0; for (int m = 0; m < k; m++) s += V[i + k * m] * tmp[m]; wb[i] = s; }
  for (int l = 0; l < k; l++)
    for (int i = 0; i < k; i++) {
      double s = 0.0;
      for (int m = 0; m < k; m++) s += V[i + k * m] * sqrt((double)(k - 1) / lam[m]) * V[l + k * m];
      trans[i + k * l] = s + wb[i];
    }
  return rc;
}

/* src/letkf_core.F90:69-146 as the reference calls its libraries: every
 * product through sgemm with the reference's arguments, the eigensolve
 * through ssyev('V','U') with its workspace size (64+2)*nbv
 * (src/letkf_core.F90:60).  The Fortran arrays hdxb(k,n) and trans(k,k) are
 * the column-major [n][k] and [k][k] buffers here. */
static or_sgemm_fn g_sgemm;
static or_ssyev_fn g_ssyev;

int or_set_lapack(or_sgemm_fn sgemm, or_ssyev_fn ssyev) {
  g_sgemm = sgemm;
  g_ssyev = ssyev;
  return (sgemm && ssyev) ? 0 : -1;
}

static int core_lapack(int k, int n, const float *hdxb, const float *rdiag, const float *rloc,
                       const float *dep, float infl, float *trans, float *ws) {
  float *rinv = ws, *work1 = rinv + (size_t)n * k, *eivec = work1 + k * k, *pa = eivec + k * k;
  float *work2 = pa + k * k, *work3 = work2 + (size_t)k * n, *eival = work3 + k, *evwork = eival + k;
  int lwork = (64 + 2) * k, info = 0;
  char cn = 'n', ct = 't', cv = 'V', cu = 'U';
  float one = 1.0f, zero = 0.0f;
  for (int j = 0; j < n; j++)                                              /* :92-94 */
    for (int i = 0; i < k; i++) rinv[(size_t)j * k + i] = hdxb[(size_t)j * k + i] / rdiag[j] * rloc[j];
  g_sgemm(&cn, &ct, &k, &k, &n, &one, rinv, &k, (float *)hdxb, &k, &zero, work1, &k);   /* :97-98 */
  float r = (float)(k - 1) * 1.0f / infl;                                  /* :101-104 */
  for (int i = 0; i < k; i++) work1[i + k * i] = work1[i + k * i] + r;
  g_ssyev(&cv, &cu, &k, work1, &k, eival, evwork, &lwork, &info);          /* :107 */
  memcpy(eivec, work1, sizeof(float) * k * k);                             /* :108 */
  for (int i = 0; i < k; i++)                                              /* :111-113 */
    for (int r2 = 0; r2 < k; r2++) work1[r2 + k * i] = eivec[r2 + k * i] / eival[i];
  g_sgemm(&cn, &ct, &k, &k, &k, &one, work1, &k, eivec, &k, &zero, pa, &k);            /* :114-115 */
  g_sgemm(&cn, &cn, &k, &n, &k, &one, pa, &k, rinv, &k, &zero, work2, &k);              /* :118-119 */
  for (int i = 0; i < k; i++) work3[i] = 0.0f;                             /* :122-125 */
  for (int j = 0; j < n; j++) for (int i = 0; i < k; i++) work3[i] = work3[i] + work2[i + (size_t)k * j] * dep[j];
  for (int j = 0; j < k; j++) {                                            /* :128-131 */
    float rr = sqrtf((float)(k - 1) / eival[j]);
    for (int i = 0; i < k; i++) work1[i + k * j] = eivec[i + k * j] * rr;
  }
  g_sgemm(&cn, &ct, &k, &k, &k, &one, work1, &k, eivec, &k, &zero, trans, &k);         /* :132-133 */
  for (int j = 0; j < k; j++) for (int i = 0; i < k; i++) trans[i + k * j] = trans[i + k * j] + work3[i];  /* :139-141 */
  return info == 0 ? 0 : 1;
}

int or_core_solve(int precision, int k, int n, const float *hdxb, const float *rdiag,
                  const float *rloc, const float *dep, float infl, float *trans) {
  int rc;
  if (precision == OR_PREC_LAPACK) {
    if (!g_sgemm || !g_ssyev) return -2;
    float *ws = malloc(sizeof(float) * (2 * (size_t)n * k + 3 * k * k + 68 * (size_t)k + 8));
    if (!ws) return -1;
    rc = core_lapack(k, n, hdxb, rdiag, rloc, dep, infl, trans, ws);
    free(ws);
    return rc;
  }
  if (precision == 64) {
    double *ws = malloc(sizeof(double) * ((size_t)n * k + 3 * k * k + 4 * k + 8));
    double *tr = malloc(sizeof(double) * k * k);
    rc = core64(k, n, hdxb, rdiag, rloc, dep, infl, tr, ws);
    for (int t = 0; t < k * k; t++) trans[t] = (float)tr[t];
    free(ws); free(tr);
  } else {
    size_t fl = 2 * (size_t)n * k + 4 * k * k + 4 * k + 8;
    float *ws = malloc(sizeof(float) * fl + sizeof(double) * (2 * k * k + k + 8));
    rc = core32(k, n, hdxb, rdiag, rloc, dep, infl, trans, ws);
    free(ws);
  }
  return rc;
}

/* ------------------------------------------------------ solver loop ---- */
typedef struct {
  int cap_n;
  int *ids; float *dist, *dep, *rdiag, *hdxb, *rloc_all;
  int *kidx; float *krloc, *kdep, *krdiag, *khdxb;
  void *core_ws; size_t core_ws_sz;
  int *slab_group, *gid;
  float *bkg; double *xd, *bkgd; float *tr32; double *tr64;
} thr_ws;

static int ws_grow(thr_ws *w, int n, int k, int ns, int maxg) {
  if (!w->slab_group) {
    w->slab_group = malloc(sizeof(int) * ns); w->gid = malloc(sizeof(int) * (maxg + 2));
    w->bkg = malloc(sizeof(float) * ns * k); w->xd = malloc(sizeof(double) * ns * k);
    w->bkgd = malloc(sizeof(double) * ns * k);
    w->tr32 = malloc(sizeof(float) * k * k); w->tr64 = malloc(sizeof(double) * k * k);
  }
  if (n <= w->cap_n) return 0;
  int cap = n + 1024;
  free(w->ids); free(w->dist); free(w->dep); free(w->rdiag); free(w->hdxb); free(w->rloc_all);
  free(w->kidx); free(w->krloc); free(w->kdep); free(w->krdiag); free(w->khdxb); free(w->core_ws);
  w->ids = malloc(sizeof(int) * cap); w->dist = malloc(sizeof(float) * cap);
  w->dep = malloc(sizeof(float) * cap); w->rdiag = malloc(sizeof(float) * cap);
  w->hdxb = malloc(sizeof(float) * (size_t)cap * k); w->rloc_all = malloc(sizeof(float) * cap);
  w->kidx = malloc(sizeof(int) * cap); w->krloc = malloc(sizeof(float) * cap);
  w->kdep = malloc(sizeof(float) * cap); w->krdiag = malloc(sizeof(float) * cap);
  w->khdxb = malloc(sizeof(float) * (size_t)cap * k);
  w->core_ws_sz = sizeof(double) * ((size_t)cap * k + 3 * k * k + 4 * k + 8) + sizeof(float) * (2 * (size_t)cap * k + 4 * k * k + 4 * k + 8) + sizeof(double) * (2 * k * k + k + 8);
  w->core_ws = malloc(w->core_ws_sz);
  w->cap_n = cap;
  return (w->ids && w->dist && w->hdxb && w->khdxb && w->core_ws) ? 0 : -1;
}

static void ws_free(thr_ws *w) {
  free(w->ids); free(w->dist); free(w->dep); free(w->rdiag); free(w->hdxb); free(w->rloc_all);
  free(w->kidx); free(w->krloc); free(w->kdep); free(w->krdiag); free(w->khdxb); free(w->core_ws);
  free(w->slab_group); free(w->gid); free(w->bkg); free(w->xd); free(w->bkgd); free(w->tr32); free(w->tr64);
}

static const float STDEV2MAX = 3.65148377f;   /* SQRT(40.0/3.0) in REAL, src/letkf_solver.F90:47 */

/* one column of letkf_solver_run, src/letkf_solver.F90:203-384 */
static int solve_column(const ctx_t *c, int precision, int col, int slot, or_result *res, thr_ws *w) {
  const or_problem *p = &c->p;
  int k = p->k, ns = p->ns, maxg = c->loc.maxgroups;
  float *xs = res->state + (size_t)slot * ns * k;
  float *xm = res->mean + (size_t)slot * ns, *xsp = res->sprd + (size_t)slot * ns;
  memcpy(xs, p->state + (size_t)col * ns * k, sizeof(float) * ns * k);
  memcpy(xm, p->mean + (size_t)col * ns, sizeof(float) * ns);
  memcpy(xsp, p->sprd + (size_t)col * ns, sizeof(float) * ns);
  if (res->maxhz) res->maxhz[slot] = 0.0f;
  if (res->obscount) res->obscount[slot] = 0.0f;
  for (int g = 0; g < maxg; g++) {
    if (res->lg_obscount) res->lg_obscount[(size_t)slot * maxg + g] = 0.0f;
    if (res->lg_obsloc) res->lg_obsloc[(size_t)slot * maxg + g] = 0.0f;
  }
  if (p->mask[col]) return 0;                              /* :207 */
  float maxhz = loc_maxhz(c, col);                         /* :210 */
  float rmax = maxhz * STDEV2MAX;                          /* :211 */
  if (res->maxhz) res->maxhz[slot] = maxhz;
  if (ws_grow(w, p->nobs, k, ns, maxg)) return -1;
  int n = search(c, col, rmax, w->ids, w->dist);           /* :217 */
  if (n < 0) return -1;
  if (res->obscount) res->obscount[slot] = (float)n;
  for (int i = 0; i < n; i++) {                            /* :224-229 */
    int id = w->ids[i];
    memcpy(w->hdxb + (size_t)i * k, p->hx + (size_t)id * k, sizeof(float) * k);
    w->rdiag[i] = p->oerr[id];
    w->dep[i] = p->oval[id] - p->hx_mean[id];
  }
  int ng = loc_groups(c, col, w->slab_group, w->gid);      /* :232 */
  const float *bkg_x = p->state + (size_t)col * ns * k;    /* :235-237 */
  const float *bkg_m = p->mean + (size_t)col * ns, *bkg_s = p->sprd + (size_t)col * ns;
  int rc = 0;
  if (precision == 64) for (int t = 0; t < ns * k; t++) w->xd[t] = bkg_x[t];
  for (int g = 0; g < ng; g++) {                           /* :241 */
    int nl = 0; float loc_sum = 0.0f;
    for (int i = 0; i < n; i++) {
      float r = loc_localize(c, col, w->gid[g], w->ids[i], w->dist[i]);
      if (r > 1.0e-4f) {
        loc_sum = loc_sum + r;
        w->kidx[nl] = w->ids[i]; w->krloc[nl] = r; w->kdep[nl] = w->dep[i]; w->krdiag[nl] = w->rdiag[i];
        memcpy(w->khdxb + (size_t)nl * k, w->hdxb + (size_t)i * k, sizeof(float) * k);
        nl++;
      }
    }
    if (res->lg_obscount && g < maxg) res->lg_obscount[(size_t)slot * maxg + g] = (float)nl;
    if (res->lg_obsloc && g < maxg) res->lg_obsloc[(size_t)slot * maxg + g] = loc_sum;
    if (nl > 0) {
      if (precision == 64) {
        rc |= core64(k, nl, w->khdxb, w->krdiag, w->krloc, w->kdep, 1.0, w->tr64, (double *)w->core_ws);
        for (int s = 0; s < ns; s++) {
          if (w->slab_group[s] != g) continue;
          for (int j = 0; j < k; j++) {
            double acc = 0.0;
            for (int i = 0; i < k; i++) acc += (double)bkg_x[s * k + i] * w->tr64[i + k * j];
            w->xd[s * k + j] = acc;
          }
        }
      } else if (precision == OR_PREC_LAPACK) {
        rc |= core_lapack(k, nl, w->khdxb, w->krdiag, w->krloc, w->kdep, 1.0f, w->tr32, (float *)w->core_ws);
        int one_i = 1;
        char cn = 'n';
        float one = 1.0f, zero = 0.0f;
        for (int s = 0; s < ns; s++) {                     /* :285-289 */
          if (w->slab_group[s] != g) continue;
          g_sgemm(&cn, &cn, &one_i, &k, &k, &one, (float *)bkg_x + s * k, &one_i, w->tr32, &k, &zero, xs + s * k,
                  &one_i);
        }
      } else {
        rc |= core32(k, nl, w->khdxb, w->krdiag, w->krloc, w->kdep, 1.0f, w->tr32, (float *)w->core_ws);
        for (int s = 0; s < ns; s++) {                     /* :285-289 */
          if (w->slab_group[s] != g) continue;
          for (int j = 0; j < k; j++) {
            float acc = 0.0f;
            for (int i = 0; i < k; i++) acc += bkg_x[s * k + i] * w->tr32[i + k * j];
            xs[s * k + j] = acc;
          }
        }
      }
    }
  }
  if (precision == 64) {
    /* :299-379 in double */
    double *x = w->xd;
    double *ma = w->bkgd;   /* reuse: analysis mean per slab at ma[s] */
    for (int s = 0; s < ns; s++) {
      double sum = 0.0;
      for (int m = 0; m < k; m++) { x[s * k + m] += bkg_m[s]; sum += x[s * k + m]; }
      ma[s] = sum / k;
      for (int m = 0; m < k; m++) x[s * k + m] -= ma[s];
    }
    for (int v = 0; v < p->nvars; v++)
      for (int j = p->vars[v].grid_s_idx; j < p->vars[v].grid_s_idx + p->vars[v].levels; j++) {
        double r = ma[j] - bkg_m[j];
        r = fmax(r, -(double)p->vars[v].ana_inc_max); r = fmin(r, (double)p->vars[v].ana_inc_max);
        r = fmax(r, (double)p->vars[v].ana_bounds[0] - bkg_m[j]); r = fmin(r, (double)p->vars[v].ana_bounds[1] - bkg_m[j]);
        ma[j] = r + bkg_m[j];
      }
    if (p->rtps > 0.0f)
      for (int s = 0; s < ns; s++) {
        double d = 0.0; for (int m = 0; m < k; m++) d += x[s * k + m] * x[s * k + m];
        double sa = sqrt(d / (k - 1));
        if (sa <= 0.0) continue;
        double f = (double)p->rtps * ((double)bkg_s[s] - sa) / sa + 1.0;
        for (int m = 0; m < k; m++) x[s * k + m] *= f;
      }
    if (p->rtpp > 0.0f)
      for (int s = 0; s < ns; s++)
        for (int m = 0; m < k; m++) x[s * k + m] = (double)p->rtpp * bkg_x[s * k + m] + (1.0 - (double)p->rtpp) * x[s * k + m];
    if (p->mul != 1.0f) for (int t = 0; t < ns * k; t++) x[t] *= (double)p->mul;
    for (int v = 0; v < p->nvars; v++)
      for (int j = p->vars[v].grid_s_idx; j < p->vars[v].grid_s_idx + p->vars[v].levels; j++) {
        double sum = 0.0;
        for (int m = 0; m < k; m++) {
          double r = x[j * k + m];
          r = fmax(r, (double)p->vars[v].ana_bounds[0] - ma[j]); r = fmin(r, (double)p->vars[v].ana_bounds[1] - ma[j]);
          x[j * k + m] = r; sum += r;
        }
        double r = sum / k;
        for (int m = 0; m < k; m++) x[j * k + m] -= r;
        ma[j] += r;
      }
    for (int s = 0; s < ns; s++) {
      double d = 0.0; for (int m = 0; m < k; m++) d += x[s * k + m] * x[s * k + m];
      xsp[s] = (float)sqrt(d / (k - 1));
      xm[s] = (float)ma[s];
      for (int m = 0; m < k; m++) xs[s * k + m] = (float)(x[s * k + m] + ma[s]);
    }
    return rc;
  }
  /* :299-303 recenter */
  for (int s = 0; s < ns; s++) {
    float sum = 0.0f;
    for (int m = 0; m < k; m++) { xs[s * k + m] = xs[s * k + m] + bkg_m[s]; }
    for (int m = 0; m < k; m++) sum += xs[s * k + m];
    xm[s] = sum / (float)k;
    for (int m = 0; m < k; m++) xs[s * k + m] = xs[s * k + m] - xm[s];
  }
  /* :308-318 increment and bounds clip */
  for (int v = 0; v < p->nvars; v++)
    for (int j = p->vars[v].grid_s_idx; j < p->vars[v].grid_s_idx + p->vars[v].levels; j++) {
      float r = xm[j] - bkg_m[j];
      r = fmaxf(r, -p->vars[v].ana_inc_max); r = fminf(r, p->vars[v].ana_inc_max);
      r = fmaxf(r, p->vars[v].ana_bounds[0] - bkg_m[j]); r = fminf(r, p->vars[v].ana_bounds[1] - bkg_m[j]);
      xm[j] = r + bkg_m[j];
    }
  /* :322-335 RTPS */
  if (p->rtps > 0.0f)
    for (int s = 0; s < ns; s++) {
      float d = 0.0f; for (int m = 0; m < k; m++) d += xs[s * k + m] * xs[s * k + m];
      xsp[s] = sqrtf(d / (float)(k - 1));
      if (xsp[s] <= 0.0f) continue;
      float f = p->rtps * (bkg_s[s] - xsp[s]) / xsp[s] + 1.0f;
      for (int m = 0; m < k; m++) xs[s * k + m] = xs[s * k + m] * f;
    }
  /* :339-344 RTPP */
  if (p->rtpp > 0.0f)
    for (int s = 0; s < ns; s++)
      for (int m = 0; m < k; m++) xs[s * k + m] = p->rtpp * bkg_x[s * k + m] + (1.0f - p->rtpp) * xs[s * k + m];
  /* :347-349 multiplicative */
  if (p->mul != 1.0f) for (int t = 0; t < ns * k; t++) xs[t] = xs[t] * p->mul;
  /* :357-371 member bounds, re-mean */
  for (int v = 0; v < p->nvars; v++)
    for (int j = p->vars[v].grid_s_idx; j < p->vars[v].grid_s_idx + p->vars[v].levels; j++) {
      for (int m = 0; m < k; m++) {
        float r = xs[j * k + m];
        r = fmaxf(r, p->vars[v].ana_bounds[0] - xm[j]); r = fminf(r, p->vars[v].ana_bounds[1] - xm[j]);
        xs[j * k + m] = r;
      }
      float sum = 0.0f; for (int m = 0; m < k; m++) sum += xs[j * k + m];
      float r = sum / (float)k;
      for (int m = 0; m < k; m++) xs[j * k + m] = xs[j * k + m] - r;
      xm[j] = xm[j] + r;
    }
  /* :375-379 spread, add mean */
  for (int s = 0; s < ns; s++) {
    float d = 0.0f; for (int m = 0; m < k; m++) d += xs[s * k + m] * xs[s * k + m];
    xsp[s] = sqrtf(d / (float)(k - 1));
    for (int m = 0; m < k; m++) xs[s * k + m] = xs[s * k + m] + xm[s];
  }
  return rc;
}

int or_run(void *vc, int precision, const int *cols, int ncl, or_result *res, int nthreads) {
  ctx_t *c = vc;
  if (!c || !res || !res->state || !res->mean || !res->sprd) return -1;
  if (precision != 32 && precision != 64 && precision != OR_PREC_LAPACK) return -2;
  if (precision == OR_PREC_LAPACK && (!g_sgemm || !g_ssyev)) return -2;
  if (c->p.k < 2 || c->loc.maxgroups < 1) return -3;
  int n = cols ? ncl : c->p.ncol;
  int nth = 1;
#ifdef _OPENMP
  nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
#endif
  int err = 0;
#pragma omp parallel num_threads(nth) reduction(|:err)
  {
    thr_ws w; memset(&w, 0, sizeof(w));
#pragma omp for schedule(dynamic, 4)
    for (int i = 0; i < n; i++) {
      int col = cols ? cols[i] : i;
      if (col < 0 || col >= c->p.ncol) { err |= 4; continue; }
      if (solve_column(c, precision, col, i, res, &w) < 0) err |= 8;
    }
    ws_free(&w);
  }
  return err;
}

int or_obslist(void *vc, int col, int group, int *idx, float *rloc, int cap, int *ncand) {
  ctx_t *c = vc;
  if (!c || col < 0 || col >= c->p.ncol) return -1;
  const or_problem *p = &c->p;
  int *ids = malloc(sizeof(int) * (p->nobs ? p->nobs : 1));
  float *dist = malloc(sizeof(float) * (p->nobs ? p->nobs : 1));
  int *sg = malloc(sizeof(int) * p->ns), gid[OR_MAXLEV + 2];
  if (ncand) *ncand = 0;
  int nl = 0;
  if (!p->mask[col]) {
    float rmax = loc_maxhz(c, col) * STDEV2MAX;
    int n = search(c, col, rmax, ids, dist);
    if (n < 0) n = 0, nl = -1;
    if (ncand) *ncand = n;
    int ng = loc_groups(c, col, sg, gid);
    if (group >= 0 && group < ng)
      for (int i = 0; i < n; i++) {
        float r = loc_localize(c, col, gid[group], ids[i], dist[i]);
        if (r > 1.0e-4f) {
          if (nl < cap) { idx[nl] = ids[i]; if (rloc) rloc[nl] = r; }
          nl++;
        }
      }
  }
  free(ids); free(dist); free(sg);
  return nl;
}
