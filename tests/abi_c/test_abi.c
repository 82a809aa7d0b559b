/* test_abi.c -- the C ABI of include/letkf_gpu.h exercised from plain C.
 *
 *   test_abi layout   prints every struct of the header as
 *                     "struct field offset size" lines and "struct - 0 size";
 *                     needs no device (tests/test_abi.py compares it with the
 *                     ctypes mirror and the Fortran BIND(C) types)
 *   test_abi          runs a small analysis through the ABI on device 0
 *                     (a 48 x 24 grid, two variables, k = 8, 400
 *                     observations, loc_novrt) and checks what a Fortran
 *                     host would rely on: status codes and messages, the
 *                     in-place analysis of a bound state, recentred
 *                     perturbations, diagnostics and timings, the list query
 *
 * The _Static_asserts pin the layouts on LP64 hosts (x86_64 and aarch64):
 * a header change that moves a field breaks this build. */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "letkf_gpu.h"

_Static_assert(sizeof(void *) == 8, "LP64 host expected");
_Static_assert(sizeof(lgpu_solver_config) == 16, "lgpu_solver_config size");
_Static_assert(sizeof(lgpu_interp_point) == 8, "lgpu_interp_point size");
_Static_assert(sizeof(lgpu_loc_config) == 104, "lgpu_loc_config size");
_Static_assert(offsetof(lgpu_loc_config, hz) == 16, "lgpu_loc_config.hz");
_Static_assert(offsetof(lgpu_loc_config, tloc_prof) == 40, "lgpu_loc_config.tloc_prof");
_Static_assert(offsetof(lgpu_loc_config, sat_obs) == 64, "lgpu_loc_config.sat_obs");
_Static_assert(offsetof(lgpu_loc_config, sat_plats) == 80, "lgpu_loc_config.sat_plats");
_Static_assert(offsetof(lgpu_loc_config, lev_depth) == 96, "lgpu_loc_config.lev_depth");
_Static_assert(sizeof(lgpu_statevar) == 20, "lgpu_statevar size");
_Static_assert(offsetof(lgpu_statevar, ana_bounds) == 12, "lgpu_statevar.ana_bounds");
_Static_assert(sizeof(lgpu_obs) == 64, "lgpu_obs size");
_Static_assert(offsetof(lgpu_timings, kept_pairs) == 32, "lgpu_timings.kept_pairs");
_Static_assert(offsetof(lgpu_timings, mma_chunks) == 48, "lgpu_timings.mma_chunks");
_Static_assert(offsetof(lgpu_timings, h2d_obs_ms) == 72, "lgpu_timings.h2d_obs_ms");
_Static_assert(offsetof(lgpu_timings, h2d_state_bytes) == 96, "lgpu_timings.h2d_state_bytes");
_Static_assert(sizeof(lgpu_timings) == 112, "lgpu_timings size");
_Static_assert(sizeof(lgpu_learn_config) == 40, "lgpu_learn_config size");
_Static_assert(offsetof(lgpu_learn_config, seed) == 32, "lgpu_learn_config.seed");
_Static_assert(sizeof(lgpu_learn_stats) == 56, "lgpu_learn_stats size");
_Static_assert(offsetof(lgpu_learn_stats, train_rows) == 32, "lgpu_learn_stats.train_rows");

#define FIELD(T, m) printf("%s %s %zu %zu\n", #T, #m, offsetof(T, m), sizeof(((T *)0)->m))
#define SIZE(T) printf("%s - 0 %zu\n", #T, sizeof(T))

static void layout(void) {
  FIELD(lgpu_solver_config, rtps); FIELD(lgpu_solver_config, rtpp); FIELD(lgpu_solver_config, mul);
  FIELD(lgpu_solver_config, save_diag); SIZE(lgpu_solver_config);
  FIELD(lgpu_interp_point, lat); FIELD(lgpu_interp_point, radius); SIZE(lgpu_interp_point);
  FIELD(lgpu_loc_config, cls); FIELD(lgpu_loc_config, n_hz); FIELD(lgpu_loc_config, hz);
  FIELD(lgpu_loc_config, n_hz_sat); FIELD(lgpu_loc_config, hz_sat); FIELD(lgpu_loc_config, tloc_prof);
  FIELD(lgpu_loc_config, tloc_sat); FIELD(lgpu_loc_config, vtloc_surf); FIELD(lgpu_loc_config, bkg_t_delta);
  FIELD(lgpu_loc_config, bkg_t_var); FIELD(lgpu_loc_config, n_sat_obs); FIELD(lgpu_loc_config, sat_obs);
  FIELD(lgpu_loc_config, n_sat_plats); FIELD(lgpu_loc_config, sat_plats); FIELD(lgpu_loc_config, vtloc);
  FIELD(lgpu_loc_config, nlev); FIELD(lgpu_loc_config, lev_depth); SIZE(lgpu_loc_config);
  FIELD(lgpu_statevar, grid_s_idx); FIELD(lgpu_statevar, levels); FIELD(lgpu_statevar, ana_inc_max);
  FIELD(lgpu_statevar, ana_bounds); SIZE(lgpu_statevar);
  FIELD(lgpu_obs, lat); FIELD(lgpu_obs, lon); FIELD(lgpu_obs, zdim); FIELD(lgpu_obs, time); FIELD(lgpu_obs, val);
  FIELD(lgpu_obs, err); FIELD(lgpu_obs, obsid); FIELD(lgpu_obs, platid); SIZE(lgpu_obs);
  FIELD(lgpu_timings, total_ms); FIELD(lgpu_timings, index_ms); FIELD(lgpu_timings, prep_ms);
  FIELD(lgpu_timings, gram_ms); FIELD(lgpu_timings, eig_ms); FIELD(lgpu_timings, update_ms);
  FIELD(lgpu_timings, launches); FIELD(lgpu_timings, units); FIELD(lgpu_timings, kept_pairs);
  FIELD(lgpu_timings, variant); FIELD(lgpu_timings, tiles_ms); FIELD(lgpu_timings, mma_chunks);
  FIELD(lgpu_timings, mma_n); FIELD(lgpu_timings, precision); FIELD(lgpu_timings, fp64_units);
  FIELD(lgpu_timings, fp64_ms); FIELD(lgpu_timings, h2d_obs_ms); FIELD(lgpu_timings, host_obs_ms);
  FIELD(lgpu_timings, h2d_state_ms); FIELD(lgpu_timings, d2h_state_ms); FIELD(lgpu_timings, span_ms);
  FIELD(lgpu_timings, host_run_ms); FIELD(lgpu_timings, h2d_state_bytes); FIELD(lgpu_timings, d2h_state_bytes);
  SIZE(lgpu_timings);
  FIELD(lgpu_learn_config, nx); FIELD(lgpu_learn_config, ny); FIELD(lgpu_learn_config, stride);
  FIELD(lgpu_learn_config, hidden); FIELD(lgpu_learn_config, judge_frac); FIELD(lgpu_learn_config, gate_frac);
  FIELD(lgpu_learn_config, sample_frac); FIELD(lgpu_learn_config, train_cap); FIELD(lgpu_learn_config, seed);
  SIZE(lgpu_learn_config);
  FIELD(lgpu_learn_stats, coarse); FIELD(lgpu_learn_stats, judged); FIELD(lgpu_learn_stats, fallback);
  FIELD(lgpu_learn_stats, gated); FIELD(lgpu_learn_stats, inferred); FIELD(lgpu_learn_stats, judge_rms);
  FIELD(lgpu_learn_stats, judge_ref_rms); FIELD(lgpu_learn_stats, tau); FIELD(lgpu_learn_stats, train_rows);
  FIELD(lgpu_learn_stats, exact_ms); FIELD(lgpu_learn_stats, feature_ms); FIELD(lgpu_learn_stats, network_ms);
  FIELD(lgpu_learn_stats, apply_ms); SIZE(lgpu_learn_stats);
}

static int failures = 0;
#define CHECK(cond, ...)                                   \
  do {                                                     \
    if (!(cond)) {                                         \
      fprintf(stderr, "FAIL line %d: ", __LINE__);         \
      fprintf(stderr, __VA_ARGS__);                        \
      fprintf(stderr, "\n");                               \
      failures++;                                          \
    }                                                      \
  } while (0)
#define CALL(h, expr)                                                                    \
  do {                                                                                   \
    int rc_ = (expr);                                                                    \
    if (rc_ != LGPU_OK) {                                                                \
      fprintf(stderr, "FAIL %s -> %d: %s\n", #expr, rc_, lgpu_last_error(h));            \
      return 1;                                                                          \
    }                                                                                    \
  } while (0)

/* xorshift + Box-Muller: a self-contained seeded generator */
static unsigned long long rs = 88172645463325252ULL;
static double unif(void) {
  rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17;
  return ((rs >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static double gauss(void) { return sqrt(-2.0 * log(unif())) * cos(6.283185307179586 * unif()); }

static int run(void) {
  enum { NX = 48, NY = 24, NCOL = NX * NY, K = 8, NZ = 3, NS = NZ + 1, NOBS = 400 };
  lgpu_handle *h = NULL;
  int rc = lgpu_create(0, &h);
  if (rc != LGPU_OK) { fprintf(stderr, "FAIL lgpu_create -> %d (no device?)\n", rc); return 1; }
  /* order and argument errors, as the reference aborts on them */
  CHECK(lgpu_solver_run(h) == LGPU_ERR_ORDER, "run before init");
  CHECK(strstr(lgpu_last_error(h), "solver_init") != NULL, "message: %s", lgpu_last_error(h));
  lgpu_solver_config bad = {1.5f, 0.0f, 1.0f, 1};
  CHECK(lgpu_solver_init(h, &bad) == LGPU_ERR_CONFIG, "rtps 1.5 accepted");
  lgpu_solver_config sc = {0.6f, 0.0f, 1.0f, 1};
  CALL(h, lgpu_solver_init(h, &sc));
  lgpu_interp_point hz[2] = {{0.0f, 600.0e3f}, {90.0f, 300.0e3f}};
  lgpu_loc_config lc;
  memset(&lc, 0, sizeof lc);
  lc.cls = "LOC_GAUSSIAN";
  lc.n_hz = 2;
  lc.hz = hz;
  lc.tloc_prof = lc.tloc_sat = -1.0f;
  CHECK(lgpu_loc_init(h, &lc) == LGPU_ERR_UNSUPPORTED_LOCALIZER, "unknown class accepted");
  lc.cls = "LOC_NOVRT";   /* matched case-insensitively */
  CALL(h, lgpu_loc_init(h, &lc));
  CHECK(lgpu_loc_maxgroups(h) == 1, "maxgroups %d", lgpu_loc_maxgroups(h));
  /* grid: cell centres, a land strip masked */
  static float lat[NCOL], lon[NCOL];
  static int mask[NCOL];
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NX; i++) {
      lat[i + NX * j] = -90.0f + (j + 0.5f) * 180.0f / NY;
      lon[i + NX * j] = (i + 0.5f) * 360.0f / NX;
      mask[i + NX * j] = (i >= 20 && i < 24) ? 1 : 0;
    }
  CALL(h, lgpu_set_grid(h, NCOL, lat, lon, mask));
  /* background: T on 3 levels + one 2-D variable; k members, zero-mean perturbations */
  static float state[NCOL * NS * K], mean[NCOL * NS], sprd[NCOL * NS], bkg[NCOL * NS * K], mean_b[NCOL * NS];
  for (int c = 0; c < NCOL; c++)
    for (int s = 0; s < NS; s++) {
      float *x = &state[((size_t)c * NS + s) * K];
      double m = 0.0, v = 0.0;
      for (int e = 0; e < K; e++) { x[e] = (float)gauss(); m += x[e]; }
      m /= K;
      for (int e = 0; e < K; e++) { x[e] = (float)(x[e] - m); v += (double)x[e] * x[e]; }
      mean[c * NS + s] = 10.0f + 5.0f * cosf(lat[c] * 0.0174533f) - s;
      sprd[c * NS + s] = (float)sqrt(v / (K - 1));
    }
  memcpy(bkg, state, sizeof state);
  memcpy(mean_b, mean, sizeof mean);
  lgpu_statevar vars[2] = {{0, NZ, 9.99e36f, {-9.99e36f, 9.99e36f}}, {NZ, 1, 9.99e36f, {-9.99e36f, 9.99e36f}}};
  CALL(h, lgpu_bind_state(h, K, NS, state, mean, sprd, 2, vars));
  /* observations of the first level of T at random points */
  static float olat[NOBS], olon[NOBS], oz[NOBS], ot[NOBS], oval[NOBS], oerr[NOBS], hx[NOBS * K], hxm[NOBS];
  static int oid[NOBS], opl[NOBS];
  for (int i = 0; i < NOBS; i++) {
    olat[i] = (float)(asin(2.0 * unif() - 1.0) * 57.29577951308232);
    olon[i] = (float)(360.0 * unif());
    oz[i] = 0.0f; ot[i] = 0.0f; oerr[i] = 0.5f; oid[i] = 1; opl[i] = 1;
    double m = 0.0;
    for (int e = 0; e < K; e++) { hx[i * K + e] = (float)gauss(); m += hx[i * K + e]; }
    m /= K;
    for (int e = 0; e < K; e++) hx[i * K + e] = (float)(hx[i * K + e] - m);
    hxm[i] = 10.0f;
    oval[i] = (float)(10.0 + 0.5 * gauss());
  }
  lgpu_obs ob = {olat, olon, oz, ot, oval, oerr, oid, opl};
  oerr[3] = 0.0f;
  CHECK(lgpu_set_obs(h, NOBS, &ob, hx, hxm) == LGPU_ERR_ARG, "zero error accepted");
  oerr[3] = 0.5f;
  CALL(h, lgpu_set_obs(h, NOBS, &ob, hx, hxm));
  CALL(h, lgpu_solver_run(h));
  /* the bound arrays now hold the analysis: full members and mean on active
   * columns; masked columns keep the background perturbation, mean and
   * spread, as the reference's solver loop skips them (src/letkf_solver.F90:207) */
  int changed = 0, masked_same = 1;
  double worst = 0.0;
  for (int c = 0; c < NCOL; c++)
    for (int s = 0; s < NS; s++) {
      const float *x = &state[((size_t)c * NS + s) * K];
      if (mask[c]) {
        for (int e = 0; e < K; e++)
          if (x[e] != bkg[((size_t)c * NS + s) * K + e]) masked_same = 0;
        if (mean[c * NS + s] != mean_b[c * NS + s]) masked_same = 0;
        continue;
      }
      double sum = 0.0, amp = 1e-6;
      for (int e = 0; e < K; e++) {
        CHECK(isfinite(x[e]), "non-finite analysis");
        sum += x[e] - mean[c * NS + s];
        amp = fmax(amp, fabs(x[e]));
      }
      worst = fmax(worst, fabs(sum) / amp);
      if (mean[c * NS + s] != mean_b[c * NS + s]) changed++;
    }
  CHECK(worst < 1e-4, "perturbations not recentred: %g", worst);
  CHECK(masked_same, "masked columns changed");
  CHECK(changed > 100, "analysis left the mean unchanged (%d slabs)", changed);
  /* diagnostics and timings */
  static float maxhz[NCOL], obsc[NCOL], lgc[NCOL], lgl[NCOL];
  CALL(h, lgpu_get_diag(h, maxhz, obsc, lgc, lgl));
  double kept = 0.0;
  for (int c = 0; c < NCOL; c++) {
    kept += lgc[c];
    if (mask[c]) CHECK(maxhz[c] == 0.0f && obsc[c] == 0.0f, "masked column diagnostics");
    else CHECK(maxhz[c] >= 300.0e3f && maxhz[c] <= 600.0e3f, "maxhz %g", maxhz[c]);
  }
  CHECK(kept > NOBS, "kept pairs %g", kept);
  lgpu_timings t;
  CALL(h, lgpu_get_timings(h, &t));
  CHECK(t.total_ms > 0.0f && t.launches > 0 && t.units == NCOL - 4 * NY, "timings %g %d %d", t.total_ms,
        t.launches, t.units);
  CHECK(t.h2d_state_bytes == (long long)4 * (NCOL * NS * K + 2 * NCOL * NS), "bound-state bytes %lld",
        t.h2d_state_bytes);
  /* the local list of the column nearest observation 0 */
  int best = 0;
  float bd = 1e30f;
  for (int c = 0; c < NCOL; c++) {
    float dla = lat[c] - olat[0], dlo = fabsf(lon[c] - olon[0]);
    if (dlo > 180.0f) dlo = 360.0f - dlo;
    if (!mask[c] && dla * dla + dlo * dlo < bd) { bd = dla * dla + dlo * dlo; best = c; }
  }
  static int idx[NOBS];
  static float rl[NOBS];
  int n = 0, ncand = 0;
  CALL(h, lgpu_get_obslist(h, best, 0, idx, rl, NOBS, &n, &ncand));
  CHECK(n > 0 && n <= ncand && n == (int)lgc[best], "list of %d, %d candidates, %g kept", n, ncand, lgc[best]);
  for (int i = 1; i < n; i++) CHECK(idx[i] > idx[i - 1], "list not in ascending order");
  for (int i = 0; i < n; i++) CHECK(rl[i] > 1.0e-4f && rl[i] <= 1.0f, "weight %g", rl[i]);
  int found = 0;
  for (int i = 0; i < n; i++) found |= idx[i] == 0;
  CHECK(found, "observation 0 missing from the list of its nearest column");
  CHECK(lgpu_get_obslist(h, NCOL, 0, idx, rl, NOBS, &n, &ncand) == LGPU_ERR_ARG, "bad column accepted");
  CALL(h, lgpu_solver_final(h));
  lgpu_destroy(h);
  if (failures) { fprintf(stderr, "%d checks failed\n", failures); return 1; }
  printf("abi ok: %d columns, %d kernel launches, %.3f ms, %d observations in the list of column %d\n", NCOL,
         t.launches, t.total_ms, n, best);
  return 0;
}

int main(int argc, char **argv) {
  if (argc > 1 && strcmp(argv[1], "layout") == 0) {
    layout();
    return 0;
  }
  return run();
}
