// lgpu_api.cu -- the C ABI (include/letkf_gpu.h): handle, validation that
// mirrors the reference's solver/localizer initialisation, uploads, the run
// orchestration on one CUDA stream, timings and verification helpers.
#include <algorithm>
#include <array>
#include <cctype>
#include <chrono>
#include <cstdint>
#include <mutex>
#include <unordered_map>
#include <utility>
#include <sys/mman.h>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <cmath>

#include "lgpu_internal.cuh"

using namespace lgpu;

namespace lgpu {
size_t gram_smem_bytes(int k);
cudaError_t noalloc_scratch(int device, int **out);
int noalloc_max_list();
cudaError_t launch_obslist_noalloc(cudaStream_t st, int gid, const ColPar *cp_col, const DevLoc &loc, ObsSorted obs,
                                   const IndexGeom *geom, int nobs, int *scratch);
cudaError_t launch_hx_stats(cudaStream_t st, int nobs, int k, float *hx, float *hx_mean, const int *qc, int *flag,
                            int *pos, int *total);
cudaError_t launch_compact(cudaStream_t st, int nobs, int k, const int *flag, const int *pos, const float *const *src_f,
                           float *const *dst_f, int nf, const int *const *src_i, int *const *dst_i, int ni,
                           const float *hx, float *hx_out, const float *hxm, float *hxm_out);
cudaError_t launch_state_stats(cudaStream_t st, long long ncs, int k, float *x, float *mean, float *sprd);
cudaError_t launch_eig_debug(cudaStream_t st, int nunits, int k, const float *G, const int *nkept, float *T,
                             int *status, int prec, float gap_thresh, int *nfp64);
}

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e == cudaSuccess) cap = bytes ? bytes : 16;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T> T *as() const { return static_cast<T *>(p); }
};

enum {
  B_LAT, B_LON, B_MASK, B_COL2ACT, B_ACTIVE,
  B_BKG, B_MEANB, B_SPRDB, B_ANA, B_MEANA, B_SPRDA, B_SLABVAR, B_SLABLEV, B_VARINC, B_VARLB, B_VARUB,
  B_OLAT, B_OLON, B_OZ, B_OTIME, B_OVAL, B_OERR, B_OOBSID, B_OPLATID, B_HX, B_HXM, B_SATOBS, B_SATPLATS,
  B_GEOM, B_CELL, B_COUNT, B_FILL, B_POSTMP, B_ORDER, B_ATMP, B_BTMP, B_SA, B_SB, B_SHX, B_SIDX, B_CSTART,
  B_CP, B_G, B_T, B_NKEPT, B_DMAXHZ, B_DOBSC, B_DLGC, B_DLGL, B_STATUS, B_LEVDEPTH,
  B_LIST_IDX, B_LIST_R, B_LIST_CNT, B_FLUSH, B_TILECOLS, B_TILEPAR, B_TILEN, B_TILEOFF, B_TILEREC, B_EIGSCR, B_WCACHE,
  B_RAW0, B_RAW1, B_RAW2, B_RAW3, B_RAW4, B_RAW5, B_RAW6, B_RAW7, B_RAWQC, B_RAWHX, B_RAWHXM, B_FLAG, B_POS,
  B_PTRS, B_TOTAL, B_GPART, B_GCNT, B_FLAGLIST, B_TCWORK, B_TCSEG,
  B_COUNT_ALL
};

}  // namespace

constexpr int kOutChunks = 8;   // column chunks of eigensolve / update / analysis download of a bound state

// Column range [c0, c1) of chunk c of n over ncol columns.  With n =
// kOutChunks (and at least 1,000 columns, so that none is empty) the chunks
// shrink towards the end (per mille of the columns below), so that the
// download of the last chunk, which nothing overlaps, is short; the earlier
// downloads overlap the following chunks' work.  Otherwise equal chunks,
// empty ones only at the end.
static void chunk_bounds(int ncol, int n, int c, int *c0, int *c1) {
  static const int kShare[kOutChunks + 1] = {0, 150, 300, 450, 590, 720, 840, 940, 1000};
  if (n == kOutChunks && ncol >= 1000) {
    *c0 = (int)((long long)ncol * kShare[c] / 1000);
    *c1 = (int)((long long)ncol * kShare[c + 1] / 1000);
  } else {
    const int per = (ncol + n - 1) / n;
    *c0 = std::min(ncol, c * per);
    *c1 = std::min(ncol, (c + 1) * per);
  }
}
constexpr int kSegChunks = 256;   // batched Gram: chunks of 16 observations per CTA at most
constexpr int kDrainChunks = 64;  // batched Gram: chunks per tensor-core accumulation (drained to a partial block)

struct LearnState;   // learned form (below)

struct lgpu_handle {
  int device = 0;
  cudaStream_t st = nullptr;
  cudaStream_t cst = nullptr;      // host<->device copies of a bound state
  cudaEvent_t ev[8] = {};
  cudaEvent_t ev_in[2] = {};       // bound state: mean/spread uploaded; members' upload started
  cudaEvent_t ev_tune[3] = {};     // AUTO: timing of the two Gram forms
  cudaEvent_t ev_cull[3] = {};     // batched Gram: timing of its two producer forms
  // per column chunk: eigensolve start, update start, update end, FP64 eigensolve start
  cudaEvent_t ev_chunk[kOutChunks][4] = {};
  cudaEvent_t ev_obs[2] = {};        // lgpu_set_obs: observation upload
  cudaEvent_t ev_up[2] = {};         // bound state: background upload (copy stream)
  cudaEvent_t ev_down[kOutChunks][2] = {};   // bound state: analysis download per chunk (download stream)
  cudaEvent_t ev_upc[kOutChunks] = {};       // bound state: background of column chunk c uploaded
  cudaEvent_t ev_gram_done = nullptr;        // bound state: the Gram has run (the members' upload starts)
  cudaStream_t dst = nullptr;                // bound state: analysis downloads (uploads run on cst)
  float obs_h2d_ms = 0.0f, obs_host_ms = 0.0f;
  float *bound_state = nullptr, *bound_mean = nullptr, *bound_sprd = nullptr;   // caller arrays (in place)
  std::string err;
  bool solver_ok = false, loc_ok = false, grid_ok = false, state_ok = false, obs_ok = false, ran = false;
  lgpu_solver_config scfg{0.0f, 0.0f, 1.0f, 1};
  DevLoc loc{};
  std::vector<int> sat_obs, sat_plats;
  std::vector<float> lev_depth;
  int bkg_t_var = -1;
  int ncol = 0, nact = 0;
  std::vector<int> h_col2act;
  int k = 0, ns = 0, kp = 0;
  std::vector<lgpu_statevar> vars;
  int nobs = 0;
  IndexGeom geom{};
  int ncell = 0;
  int nunits = 0;
  int variant = LGPU_VARIANT_AUTO;
  int ntiles = 0;
  bool used_tc = false;
  int mma_n = 0;
  int auto_choice = 0;   // AUTO: the Gram variant measured faster (0 = not yet measured)
  int gram_nseg = 1;     // most accumulation segments of a tile in the last batched Gram
  std::vector<int> h_tile_off;       // tile stream offsets of the last batched Gram (read back)
  // page-locked landing areas of the run's small device-to-host reads: a
  // pageable destination would queue them behind a bound state's upload
  int *pin_off = nullptr;            // tile stream offsets
  size_t pin_off_n = 0;
  int *pin_scr = nullptr;            // [0..3] status words, [4] FP64 re-solve count
  std::vector<TcWork> h_tc_work;     // its accumulation segments
  std::vector<TcSegTile> h_tc_seg;   // its tiles with more than one segment
  int tc_cull = -1;      // batched Gram producers: 1 with the warp-level cull, 0 without, -1 not yet measured
  float tc_tune_ms = 0.0f;   // time of the producer form the tuning run discarded (left out of AUTO's comparison)
  bool preloaded = false;    // the Gram kernels are loaded (before the first timed trial)
  int prec = LGPU_PREC_FP32;   // eigensolve precision mode
  float gap_thresh = 1e-6f;    // FP32_RESOLVE: relative eigenvalue gap that sends a unit to FP64
  DevBuf buf[B_COUNT_ALL];
  lgpu_timings tim{};
  LearnState *learn = nullptr;      // learned form, after lgpu_learn_init
  float *learn_wbar = nullptr;      // mean weights of every unit while training rows are collected
};

static void learn_free(lgpu_handle *h);

namespace {

int fail(lgpu_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(lgpu_handle *h, cudaError_t e, const char *what) {
  // a failed runtime call also leaves the thread's last-error state set;
  // clear it so that the next call's launch checks do not report it again
  // (a sticky context error stays and is reported by every later call)
  (void)cudaGetLastError();
  return fail(h, e == cudaErrorMemoryAllocation ? LGPU_ERR_NOMEM : LGPU_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_fail(h, _e, what); \
  } while (0)

std::string upper(const char *s) {
  std::string r(s ? s : "");
  for (auto &c : r) c = (char)std::toupper((unsigned char)c);
  return r;
}

// linearinterp_lat_init (src/letkf_loc.F90:251-294): pad with a 0-degree
// point carrying the first radius and a 90-degree point carrying the last.
int build_interp(lgpu_handle *h, Interp &t, int n, const lgpu_interp_point *pts, const char *name) {
  std::memset(&t, 0, sizeof(t));
  if (n <= 0 || !pts) return fail(h, LGPU_ERR_CONFIG, std::string("localizer needs a non-empty ") + name + " table");
  if (n > LGPU_MAX_INTERP) return fail(h, LGPU_ERR_CAPACITY, std::string(name) + " has more than 16 points");
  float last_lat = 0.0f, last_r = 0.0f;
  for (int i = 0; i < n; i++) {
    if (!(pts[i].radius > 0.0f)) return fail(h, LGPU_ERR_CONFIG, std::string(name) + " radius must be > 0");
    if (pts[i].lat > 0.0f && t.n == 0) { t.lat[0] = 0.0f; t.dist[0] = pts[i].radius; t.n = 1; }
    t.lat[t.n] = pts[i].lat;
    t.dist[t.n] = pts[i].radius;
    t.n++;
    last_lat = pts[i].lat;
    last_r = pts[i].radius;
  }
  if (last_lat < 90.0f) { t.lat[t.n] = 90.0f; t.dist[t.n] = last_r; t.n++; }
  return LGPU_OK;
}

// Tiles of (up to) 128 active columns that are close on the sphere: k-d
// bisection of the columns' unit vectors, splitting the widest coordinate at
// a multiple of 128 so that leaves hold exactly 128 columns where possible.
void kd_split(std::vector<std::array<float, 3>> &u, std::vector<int> &id, size_t lo, size_t hi,
              std::vector<int> &out) {
  const size_t n = hi - lo;
  if (n <= 128) {
    for (size_t i = lo; i < hi; i++) out.push_back(id[i]);
    for (size_t i = n; i < 128; i++) out.push_back(-1);
    return;
  }
  float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
  for (size_t i = lo; i < hi; i++)
    for (int d = 0; d < 3; d++) { mn[d] = std::min(mn[d], u[i][d]); mx[d] = std::max(mx[d], u[i][d]); }
  int ax = 0;
  for (int d = 1; d < 3; d++) if (mx[d] - mn[d] > mx[ax] - mn[ax]) ax = d;
  size_t half = (size_t)std::max<long long>(1, std::llround((double)n / 256.0)) * 128;
  if (half >= n) half = 128;
  std::vector<size_t> perm(n);
  for (size_t i = 0; i < n; i++) perm[i] = lo + i;
  std::nth_element(perm.begin(), perm.begin() + half, perm.end(), [&](size_t a, size_t b) {
    return u[a][ax] < u[b][ax] || (u[a][ax] == u[b][ax] && id[a] < id[b]);
  });
  std::vector<std::array<float, 3>> u2(n);
  std::vector<int> id2(n);
  for (size_t i = 0; i < n; i++) { u2[i] = u[perm[i]]; id2[i] = id[perm[i]]; }
  for (size_t i = 0; i < n; i++) { u[lo + i] = u2[i]; id[lo + i] = id2[i]; }
  kd_split(u, id, lo, lo + half, out);
  kd_split(u, id, lo + half, hi, out);
}

std::vector<int> build_tiles(const std::vector<int> &act, const float *lat, const float *lon) {
  const size_t n = act.size();
  std::vector<std::array<float, 3>> u(n);
  std::vector<int> id(act);
  for (size_t i = 0; i < n; i++) {
    const double p = lat[act[i]] * 0.017453292519943295, l = lon[act[i]] * 0.017453292519943295;
    u[i] = {(float)(std::cos(p) * std::cos(l)), (float)(std::cos(p) * std::sin(l)), (float)std::sin(p)};
  }
  std::vector<int> tiles;
  tiles.reserve((n / 128 + 2) * 128);
  if (n > 0) kd_split(u, id, 0, n, tiles);
  return tiles;
}

void build_geom(IndexGeom &g, int &ncell) {
  int off = 0;
  for (int b = 0; b < kNB; b++) {
    const double lat0 = -90.0 + b, lat1 = lat0 + 1.0;
    const double pole = std::max(std::fabs(lat0), std::fabs(lat1));
    int n = (int)std::floor(360.0 * std::cos(pole * 3.14159265358979323846 / 180.0));
    if (n < 1) n = 1;
    g.nlon[b] = n;
    g.off[b] = off;
    off += n;
  }
  g.off[kNB] = off;
  ncell = off;
}

}  // namespace

extern "C" {

int lgpu_create(int device, lgpu_handle **out) {
  if (!out) return LGPU_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= 0) return LGPU_ERR_CUDA;
  if (device < 0 || device >= n) return LGPU_ERR_ARG;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return LGPU_ERR_CUDA;
  lgpu_handle *h = new lgpu_handle();
  h->device = device;
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&h->dst, cudaStreamNonBlocking) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev_upc)
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  if (cudaEventCreateWithFlags(&h->ev_gram_done, cudaEventDisableTiming) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev)
    if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev_in)   // also time the background upload
    if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev_tune)
    if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev_cull)
    if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &row : h->ev_chunk)
    for (auto &ev : row)
      if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev_obs)
    if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &ev : h->ev_up)
    if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  for (auto &row : h->ev_down)
    for (auto &ev : row)
      if (cudaEventCreate(&ev) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  if (cudaMallocHost(&h->pin_scr, 64 * sizeof(int)) != cudaSuccess) { delete h; return LGPU_ERR_CUDA; }
  build_geom(h->geom, h->ncell);
  if (h->buf[B_GEOM].ensure(sizeof(IndexGeom)) != cudaSuccess ||
      cudaMemcpy(h->buf[B_GEOM].p, &h->geom, sizeof(IndexGeom), cudaMemcpyHostToDevice) != cudaSuccess) {
    delete h;
    return LGPU_ERR_CUDA;
  }
  *out = h;
  return LGPU_OK;
}

void lgpu_destroy(lgpu_handle *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->cst) cudaStreamSynchronize(h->cst);
  if (h->dst) cudaStreamSynchronize(h->dst);
  for (auto &b : h->buf) b.release();
  learn_free(h);
  if (h->pin_off) cudaFreeHost(h->pin_off);
  if (h->pin_scr) cudaFreeHost(h->pin_scr);
  for (auto &ev : h->ev) if (ev) cudaEventDestroy(ev);
  for (auto &ev : h->ev_in) if (ev) cudaEventDestroy(ev);
  for (auto &ev : h->ev_tune) if (ev) cudaEventDestroy(ev);
  for (auto &ev : h->ev_cull) if (ev) cudaEventDestroy(ev);
  for (auto &row : h->ev_chunk)
    for (auto &ev : row) if (ev) cudaEventDestroy(ev);
  for (auto &ev : h->ev_obs) if (ev) cudaEventDestroy(ev);
  for (auto &ev : h->ev_up) if (ev) cudaEventDestroy(ev);
  for (auto &row : h->ev_down)
    for (auto &ev : row) if (ev) cudaEventDestroy(ev);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->cst) cudaStreamDestroy(h->cst);
  if (h->dst) cudaStreamDestroy(h->dst);
  for (auto &ev : h->ev_upc) if (ev) cudaEventDestroy(ev);
  if (h->ev_gram_done) cudaEventDestroy(h->ev_gram_done);
  delete h;
}

const char *lgpu_last_error(const lgpu_handle *h) { return h ? h->err.c_str() : "null handle"; }

// letkf_solver_init (src/letkf_solver.F90:73-142)
int lgpu_solver_init(lgpu_handle *h, const lgpu_solver_config *c) {
  if (!h || !c) return LGPU_ERR_ARG;
  if (c->rtps > 1.0f || c->rtps < 0.0f)
    return fail(h, LGPU_ERR_CONFIG, "illegal value for infl_rtps (should be <1.0 and >0.0).");
  if (c->rtpp > 1.0f || c->rtpp < 0.0f)
    return fail(h, LGPU_ERR_CONFIG, "illegal value for infl_rtpp (should be <1.0 and >0.0).");
  if (c->rtpp != 0.0f && c->rtps != 0.0f)
    return fail(h, LGPU_ERR_CONFIG, "cannot have both RTPS and RTPP enabled at the same time. ");
  if (c->mul < 1.0f) return fail(h, LGPU_ERR_CONFIG, "infl_mul must be >=1.0.");
  h->scfg = *c;
  h->solver_ok = true;
  return LGPU_OK;
}

// letkf_loc_init (src/letkf_loc.F90:164-210) + the plugin's init
int lgpu_loc_init(lgpu_handle *h, const lgpu_loc_config *c) {
  if (!h || !c) return LGPU_ERR_ARG;
  h->loc_ok = false;
  const std::string cls = upper(c->cls);
  DevLoc L{};
  L.tloc_prof = -1.0f;
  L.tloc_sat = -1.0f;
  int rc;
  h->sat_obs.clear();
  h->sat_plats.clear();
  h->lev_depth.clear();
  h->bkg_t_var = -1;
  if (cls == "LOC_NOVRT") {
    L.cls = LOC_NOVRT;
    if ((rc = build_interp(h, L.hz, c->n_hz, c->hz, "hzloc")) != LGPU_OK) return rc;
    L.groups = 1;
  } else if (cls == "LOC_OCEAN") {
    L.cls = LOC_OCEAN;
    if ((rc = build_interp(h, L.hz, c->n_hz, c->hz, "hzloc_prof")) != LGPU_OK) return rc;
    if ((rc = build_interp(h, L.hz_sat, c->n_hz_sat, c->hz_sat, "hzloc_sat")) != LGPU_OK) return rc;
    L.tloc_prof = c->tloc_prof;
    L.tloc_sat = c->tloc_sat;
    if (c->n_sat_obs < 0 || c->n_sat_obs > LGPU_MAX_IDS || c->n_sat_plats < 0 || c->n_sat_plats > LGPU_MAX_IDS)
      return fail(h, LGPU_ERR_CAPACITY, "sat_obs / sat_plats lists hold at most 32 ids");
    if (c->n_sat_obs > 0 && !c->sat_obs) return LGPU_ERR_ARG;
    if (c->n_sat_plats > 0 && !c->sat_plats) return LGPU_ERR_ARG;
    h->sat_obs.assign(c->sat_obs, c->sat_obs + c->n_sat_obs);
    h->sat_plats.assign(c->sat_plats, c->sat_plats + c->n_sat_plats);
    if (c->vtloc_surf == 0) {
      L.groups = 1;
    } else if (c->vtloc_surf == 1) {
      if (!(c->bkg_t_delta >= 0.0f)) return fail(h, LGPU_ERR_CONFIG, "vtloc_surf.bkg_t_delta must be >= 0");
      L.groups = 2;
      L.vtloc_surf = 1;
      L.bkg_t_delta = c->bkg_t_delta;
      h->bkg_t_var = c->bkg_t_var;
    } else {
      return fail(h, LGPU_ERR_CONFIG, "illegal vtloc_surf 'type' given: " + std::to_string(c->vtloc_surf));
    }
  } else if (cls == "LOC_VTGC") {
    L.cls = LOC_VTGC;
    if ((rc = build_interp(h, L.hz, c->n_hz, c->hz, "hzloc")) != LGPU_OK) return rc;
    if (!(c->vtloc > 0.0f)) return fail(h, LGPU_ERR_CONFIG, "loc_vtgc needs vtloc > 0");
    if (c->nlev <= 0 || !c->lev_depth) return fail(h, LGPU_ERR_CONFIG, "loc_vtgc needs the level depths");
    if (c->nlev > LGPU_MAX_LEVELS) return fail(h, LGPU_ERR_CAPACITY, "loc_vtgc supports at most 128 levels");
    L.vloc = c->vtloc;
    h->lev_depth.assign(c->lev_depth, c->lev_depth + c->nlev);
    L.groups = c->nlev;
  } else {
    return fail(h, LGPU_ERR_UNSUPPORTED_LOCALIZER, "localizer class " + cls + " not found.");
  }
  if (L.groups <= 0) return fail(h, LGPU_ERR_CONFIG, "localizer class needs to properly define 'maxgroups'");
  h->loc = L;
  h->loc_ok = true;
  h->auto_choice = 0;
  h->tc_cull = -1;
  h->preloaded = false;
  h->ran = false;
  return LGPU_OK;
}

int lgpu_loc_maxgroups(const lgpu_handle *h) { return (h && h->loc_ok) ? h->loc.groups : -1; }

int lgpu_set_precision(lgpu_handle *h, int mode, float gap_threshold) {
  if (!h) return LGPU_ERR_ARG;
  if (mode < LGPU_PREC_FP32 || mode > LGPU_PREC_FP64)
    return fail(h, LGPU_ERR_ARG, "unknown precision mode " + std::to_string(mode));
  if (!(gap_threshold < 1.0f)) return fail(h, LGPU_ERR_ARG, "gap_threshold must be below 1");
  h->prec = mode;
  h->gap_thresh = gap_threshold > 0.0f ? gap_threshold : 1e-6f;
  return LGPU_OK;
}

int lgpu_set_variant(lgpu_handle *h, int variant) {
  if (!h) return LGPU_ERR_ARG;
  if (variant < LGPU_VARIANT_AUTO || variant > LGPU_VARIANT_LEARNED)
    return fail(h, LGPU_ERR_ARG, "unknown variant " + std::to_string(variant));
  h->variant = variant;
  return LGPU_OK;
}

int lgpu_set_grid(lgpu_handle *h, int nij, const float *lat, const float *lon, const int *mask) {
  if (!h) return LGPU_ERR_ARG;
  if (nij <= 0 || !lat || !lon) return fail(h, LGPU_ERR_ARG, "set_grid: bad arguments");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  std::vector<int> m(nij, 0), c2a(nij, -1), act;
  act.reserve(nij);
  for (int i = 0; i < nij; i++) {
    if (!std::isfinite(lat[i]) || !std::isfinite(lon[i]) || lat[i] < -90.0f || lat[i] > 90.0f)
      return fail(h, LGPU_ERR_ARG, "set_grid: latitude out of range at ij=" + std::to_string(i));
    m[i] = mask ? (mask[i] != 0) : 0;
    if (!m[i]) { c2a[i] = (int)act.size(); act.push_back(i); }
  }
  CK(h->buf[B_LAT].ensure(sizeof(float) * nij), "alloc lat");
  CK(h->buf[B_LON].ensure(sizeof(float) * nij), "alloc lon");
  CK(h->buf[B_MASK].ensure(sizeof(int) * nij), "alloc mask");
  CK(h->buf[B_COL2ACT].ensure(sizeof(int) * nij), "alloc col2act");
  CK(h->buf[B_ACTIVE].ensure(sizeof(int) * std::max<size_t>(1, act.size())), "alloc active");
  CK(cudaMemcpyAsync(h->buf[B_LAT].p, lat, sizeof(float) * nij, cudaMemcpyHostToDevice, h->st), "H2D lat");
  CK(cudaMemcpyAsync(h->buf[B_LON].p, lon, sizeof(float) * nij, cudaMemcpyHostToDevice, h->st), "H2D lon");
  CK(cudaMemcpyAsync(h->buf[B_MASK].p, m.data(), sizeof(int) * nij, cudaMemcpyHostToDevice, h->st), "H2D mask");
  CK(cudaMemcpyAsync(h->buf[B_COL2ACT].p, c2a.data(), sizeof(int) * nij, cudaMemcpyHostToDevice, h->st), "H2D c2a");
  if (!act.empty())
    CK(cudaMemcpyAsync(h->buf[B_ACTIVE].p, act.data(), sizeof(int) * act.size(), cudaMemcpyHostToDevice, h->st), "H2D act");
  const std::vector<int> tiles = build_tiles(act, lat, lon);
  CK(h->buf[B_TILECOLS].ensure(sizeof(int) * std::max<size_t>(1, tiles.size())), "alloc tiles");
  CK(h->buf[B_TILEPAR].ensure(sizeof(TilePar) * std::max<size_t>(1, tiles.size() / 128)), "alloc tiles");
  CK(h->buf[B_TILEN].ensure(sizeof(int) * std::max<size_t>(1, tiles.size() / 128)), "alloc tiles");
  CK(h->buf[B_TILEOFF].ensure(sizeof(int) * (tiles.size() / 128 + 1)), "alloc tiles");
  if (!tiles.empty())
    CK(cudaMemcpyAsync(h->buf[B_TILECOLS].p, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice, h->st),
       "H2D tiles");
  CK(cudaStreamSynchronize(h->st), "set_grid sync");
  h->ntiles = (int)(tiles.size() / 128);
  h->auto_choice = 0;
  h->tc_cull = -1;
  h->preloaded = false;
  h->ncol = nij;
  h->nact = (int)act.size();
  h->h_col2act = c2a;
  h->grid_ok = true;
  h->ran = false;
  return LGPU_OK;
}

namespace {

// Validation, device buffers and slab metadata shared by lgpu_set_state and
// lgpu_bind_state; the member data is not copied here.
int prepare_state(lgpu_handle *h, int k, int ns, const float *state, const float *mean, const float *sprd, int nvars,
                  const lgpu_statevar *vars) {
  if (!h->grid_ok) return fail(h, LGPU_ERR_ORDER, "set_state before set_grid");
  if (!state || !mean || !sprd || !vars || nvars <= 0 || ns <= 0) return fail(h, LGPU_ERR_ARG, "set_state: bad arguments");
  if (k < 2) return fail(h, LGPU_ERR_ARG, "ensemble size must be >= 2");
  if (k > kMaxK) return fail(h, LGPU_ERR_UNSUPPORTED, "ensemble size > 128 is not supported by this build");
  if ((size_t)ns * ((k + 3) & ~3) * 8 > 200 * 1024)
    return fail(h, LGPU_ERR_UNSUPPORTED, "a column's state (ns x k) exceeds the 100 KB the update kernel stages");
  // slab -> (variable, level); every slab must belong to exactly one variable
  std::vector<int> sv(ns, -1), sl(ns, -1);
  std::vector<float> inc(nvars), lb(nvars), ub(nvars);
  for (int v = 0; v < nvars; v++) {
    const auto &x = vars[v];
    if (x.levels <= 0 || x.grid_s_idx < 0 || x.grid_s_idx + x.levels > ns)
      return fail(h, LGPU_ERR_ARG, "set_state: variable " + std::to_string(v) + " slab range outside [0, ns)");
    for (int l = 0; l < x.levels; l++) {
      if (sv[x.grid_s_idx + l] >= 0) return fail(h, LGPU_ERR_ARG, "set_state: overlapping variable slabs");
      sv[x.grid_s_idx + l] = v;
      sl[x.grid_s_idx + l] = l;
    }
    inc[v] = x.ana_inc_max;
    lb[v] = x.ana_bounds[0];
    ub[v] = x.ana_bounds[1];
  }
  for (int s = 0; s < ns; s++)
    if (sv[s] < 0) return fail(h, LGPU_ERR_ARG, "set_state: slab " + std::to_string(s) + " belongs to no variable");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t nx = (size_t)h->ncol * ns * k, nm = (size_t)h->ncol * ns;
  CK(h->buf[B_BKG].ensure(nx * 4), "alloc state");
  CK(h->buf[B_ANA].ensure(nx * 4), "alloc analysis");
  CK(h->buf[B_MEANB].ensure(nm * 4), "alloc mean");
  CK(h->buf[B_SPRDB].ensure(nm * 4), "alloc sprd");
  CK(h->buf[B_MEANA].ensure(nm * 4), "alloc mean_a");
  CK(h->buf[B_SPRDA].ensure(nm * 4), "alloc sprd_a");
  CK(h->buf[B_SLABVAR].ensure(ns * 4), "alloc slabvar");
  CK(h->buf[B_SLABLEV].ensure(ns * 4), "alloc slablev");
  CK(h->buf[B_VARINC].ensure(nvars * 4), "alloc varinc");
  CK(h->buf[B_VARLB].ensure(nvars * 4), "alloc varlb");
  CK(h->buf[B_VARUB].ensure(nvars * 4), "alloc varub");
  (void)nx;
  (void)nm;
  CK(cudaMemcpyAsync(h->buf[B_SLABVAR].p, sv.data(), ns * 4, cudaMemcpyHostToDevice, h->st), "H2D sv");
  CK(cudaMemcpyAsync(h->buf[B_SLABLEV].p, sl.data(), ns * 4, cudaMemcpyHostToDevice, h->st), "H2D sl");
  CK(cudaMemcpyAsync(h->buf[B_VARINC].p, inc.data(), nvars * 4, cudaMemcpyHostToDevice, h->st), "H2D inc");
  CK(cudaMemcpyAsync(h->buf[B_VARLB].p, lb.data(), nvars * 4, cudaMemcpyHostToDevice, h->st), "H2D lb");
  CK(cudaMemcpyAsync(h->buf[B_VARUB].p, ub.data(), nvars * 4, cudaMemcpyHostToDevice, h->st), "H2D ub");
  CK(cudaStreamSynchronize(h->st), "set_state sync");
  if (h->k != k) { h->auto_choice = 0; h->tc_cull = -1; }
  h->k = k;
  h->ns = ns;
  h->kp = (k + 3) & ~3;
  h->vars.assign(vars, vars + nvars);
  return LGPU_OK;
}

}  // namespace

int lgpu_set_state(lgpu_handle *h, int k, int ns, const float *state, const float *mean, const float *sprd, int nvars,
                   const lgpu_statevar *vars) {
  if (!h) return LGPU_ERR_ARG;
  h->state_ok = false;
  h->ran = false;
  h->bound_state = h->bound_mean = h->bound_sprd = nullptr;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(cudaStreamSynchronize(h->cst), "copy stream");
  CK(cudaStreamSynchronize(h->dst), "copy stream");
  const int rc = prepare_state(h, k, ns, state, mean, sprd, nvars, vars);
  if (rc != LGPU_OK) return rc;
  const size_t nx = (size_t)h->ncol * ns * k, nm = (size_t)h->ncol * ns;
  CK(cudaMemcpyAsync(h->buf[B_BKG].p, state, nx * 4, cudaMemcpyHostToDevice, h->st), "H2D state");
  CK(cudaMemcpyAsync(h->buf[B_MEANB].p, mean, nm * 4, cudaMemcpyHostToDevice, h->st), "H2D mean");
  CK(cudaMemcpyAsync(h->buf[B_SPRDB].p, sprd, nm * 4, cudaMemcpyHostToDevice, h->st), "H2D sprd");
  CK(cudaStreamSynchronize(h->st), "set_state sync");
  h->state_ok = true;
  return LGPU_OK;
}

// In-place state, the reference's semantics: letkf_solver_run reads the
// background from state_ij / state_mean_ij / state_sprd_ij and overwrites
// them with the analysis (src/letkf_solver.F90:283-330).
int lgpu_bind_state(lgpu_handle *h, int k, int ns, float *state, float *mean, float *sprd, int nvars,
                    const lgpu_statevar *vars) {
  if (!h) return LGPU_ERR_ARG;
  h->state_ok = false;
  h->ran = false;
  h->bound_state = h->bound_mean = h->bound_sprd = nullptr;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(cudaStreamSynchronize(h->cst), "copy stream");
  CK(cudaStreamSynchronize(h->dst), "copy stream");
  const int rc = prepare_state(h, k, ns, state, mean, sprd, nvars, vars);
  if (rc != LGPU_OK) return rc;
  h->bound_state = state;
  h->bound_mean = mean;
  h->bound_sprd = sprd;
  h->state_ok = true;
  return LGPU_OK;
}

int lgpu_set_obs(lgpu_handle *h, int nobs, const lgpu_obs *o, const float *hx, const float *hx_mean) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->state_ok) return fail(h, LGPU_ERR_ORDER, "set_obs before set_state (the ensemble size is needed)");
  if (nobs < 0 || (nobs > 0 && (!o || !hx || !hx_mean || !o->lat || !o->lon || !o->zdim || !o->time || !o->val ||
                                 !o->err || !o->obsid || !o->platid)))
    return fail(h, LGPU_ERR_ARG, "set_obs: bad arguments");
  for (int i = 0; i < nobs; i++)
    if (!(o->err[i] > 0.0f)) return fail(h, LGPU_ERR_ARG, "set_obs: observation error must be > 0 at obs " + std::to_string(i));
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const auto t_host = std::chrono::steady_clock::now();
  const size_t n = std::max(nobs, 1), k = h->k;
  int bi[8] = {B_OLAT, B_OLON, B_OZ, B_OTIME, B_OVAL, B_OERR, B_OOBSID, B_OPLATID};
  const void *src[8] = {o ? o->lat : nullptr, o ? o->lon : nullptr, o ? o->zdim : nullptr, o ? o->time : nullptr,
                        o ? o->val : nullptr, o ? o->err : nullptr, o ? o->obsid : nullptr, o ? o->platid : nullptr};
  for (int q = 0; q < 8; q++) CK(h->buf[bi[q]].ensure(n * 4), "alloc obs");
  CK(h->buf[B_HX].ensure(n * k * 4), "alloc hx");
  CK(h->buf[B_HXM].ensure(n * 4), "alloc hx_mean");
  CK(cudaEventRecord(h->ev_obs[0], h->st), "event");
  for (int q = 0; q < 8; q++) {
    if (nobs > 0) CK(cudaMemcpyAsync(h->buf[bi[q]].p, src[q], (size_t)nobs * 4, cudaMemcpyHostToDevice, h->st), "H2D obs");
  }
  if (nobs > 0) {
    CK(cudaMemcpyAsync(h->buf[B_HX].p, hx, (size_t)nobs * k * 4, cudaMemcpyHostToDevice, h->st), "H2D hx");
    CK(cudaMemcpyAsync(h->buf[B_HXM].p, hx_mean, (size_t)nobs * 4, cudaMemcpyHostToDevice, h->st), "H2D hxm");
  }
  CK(cudaEventRecord(h->ev_obs[1], h->st), "event");
  CK(cudaStreamSynchronize(h->st), "set_obs sync");
  CK(cudaEventElapsedTime(&h->obs_h2d_ms, h->ev_obs[0], h->ev_obs[1]), "timing");
  h->obs_host_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t_host).count();
  h->nobs = nobs;
  h->obs_ok = true;
  h->ran = false;
  return LGPU_OK;
}

// src/letkf_obs.F90:459-488 on the device
int lgpu_set_obs_raw(lgpu_handle *h, int nobs, const lgpu_obs *o, const int *qc, const float *hx_members,
                     int *nobs_kept) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->state_ok) return fail(h, LGPU_ERR_ORDER, "set_obs_raw before set_state (the ensemble size is needed)");
  if (nobs < 0 || (nobs > 0 && (!o || !hx_members || !o->lat || !o->lon || !o->zdim || !o->time || !o->val ||
                                 !o->err || !o->obsid || !o->platid)))
    return fail(h, LGPU_ERR_ARG, "set_obs_raw: bad arguments");
  for (int i = 0; i < nobs; i++)
    if ((!qc || qc[i] <= 0) && !(o->err[i] > 0.0f))
      return fail(h, LGPU_ERR_ARG, "set_obs_raw: observation error must be > 0 at obs " + std::to_string(i));
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t n = std::max(nobs, 1), k = h->k;
  const int raw[8] = {B_RAW0, B_RAW1, B_RAW2, B_RAW3, B_RAW4, B_RAW5, B_RAW6, B_RAW7};
  const int dst[8] = {B_OLAT, B_OLON, B_OZ, B_OTIME, B_OVAL, B_OERR, B_OOBSID, B_OPLATID};
  const void *src[8] = {o ? o->lat : nullptr, o ? o->lon : nullptr, o ? o->zdim : nullptr, o ? o->time : nullptr,
                        o ? o->val : nullptr, o ? o->err : nullptr, o ? o->obsid : nullptr, o ? o->platid : nullptr};
  for (int q = 0; q < 8; q++) {
    CK(h->buf[raw[q]].ensure(n * 4), "alloc raw obs");
    CK(h->buf[dst[q]].ensure(n * 4), "alloc obs");
    if (nobs > 0) CK(cudaMemcpyAsync(h->buf[raw[q]].p, src[q], (size_t)nobs * 4, cudaMemcpyHostToDevice, h->st), "H2D");
  }
  CK(h->buf[B_RAWHX].ensure(n * k * 4), "alloc raw hx");
  CK(h->buf[B_RAWHXM].ensure(n * 4), "alloc");
  CK(h->buf[B_HX].ensure(n * k * 4), "alloc hx");
  CK(h->buf[B_HXM].ensure(n * 4), "alloc hx_mean");
  CK(h->buf[B_RAWQC].ensure(n * 4), "alloc");
  CK(h->buf[B_FLAG].ensure(n * 4), "alloc");
  CK(h->buf[B_POS].ensure(n * 4), "alloc");
  CK(h->buf[B_TOTAL].ensure(16), "alloc");
  CK(h->buf[B_PTRS].ensure(32 * sizeof(void *)), "alloc");
  if (nobs > 0) {
    CK(cudaMemcpyAsync(h->buf[B_RAWHX].p, hx_members, (size_t)nobs * k * 4, cudaMemcpyHostToDevice, h->st), "H2D hx");
    if (qc) CK(cudaMemcpyAsync(h->buf[B_RAWQC].p, qc, (size_t)nobs * 4, cudaMemcpyHostToDevice, h->st), "H2D qc");
  }
  CK(launch_hx_stats(h->st, nobs, (int)k, h->buf[B_RAWHX].as<float>(), h->buf[B_RAWHXM].as<float>(),
                     qc ? h->buf[B_RAWQC].as<int>() : nullptr, h->buf[B_FLAG].as<int>(), h->buf[B_POS].as<int>(),
                     h->buf[B_TOTAL].as<int>()),
     "hx statistics");
  void *ptrs[32];
  for (int q = 0; q < 6; q++) { ptrs[q] = h->buf[raw[q]].p; ptrs[8 + q] = h->buf[dst[q]].p; }
  for (int q = 0; q < 2; q++) { ptrs[16 + q] = h->buf[raw[6 + q]].p; ptrs[24 + q] = h->buf[dst[6 + q]].p; }
  CK(cudaMemcpyAsync(h->buf[B_PTRS].p, ptrs, sizeof(ptrs), cudaMemcpyHostToDevice, h->st), "H2D ptrs");
  void **dp = h->buf[B_PTRS].as<void *>();
  CK(launch_compact(h->st, nobs, (int)k, h->buf[B_FLAG].as<int>(), h->buf[B_POS].as<int>(),
                    reinterpret_cast<const float *const *>(dp), reinterpret_cast<float *const *>(dp + 8), 6,
                    reinterpret_cast<const int *const *>(dp + 16), reinterpret_cast<int *const *>(dp + 24), 2,
                    h->buf[B_RAWHX].as<float>(), h->buf[B_HX].as<float>(), h->buf[B_RAWHXM].as<float>(),
                    h->buf[B_HXM].as<float>()),
     "observation compaction");
  int kept = 0;
  CK(cudaMemcpyAsync(&kept, h->buf[B_TOTAL].p, 4, cudaMemcpyDeviceToHost, h->st), "D2H total");
  CK(cudaStreamSynchronize(h->st), "set_obs_raw");
  h->nobs = kept;
  if (nobs_kept) *nobs_kept = kept;
  h->obs_ok = true;
  h->ran = false;
  return LGPU_OK;
}

// src/letkf_state.F90:326-334 on the device
int lgpu_set_state_members(lgpu_handle *h, int k, int ns, const float *members, int nvars, const lgpu_statevar *vars) {
  if (!h) return LGPU_ERR_ARG;
  if (!members) return fail(h, LGPU_ERR_ARG, "set_state_members: bad arguments");
  // validate and upload exactly as lgpu_set_state, with the members in place of the perturbations
  const size_t nm = (size_t)h->ncol * (ns > 0 ? ns : 1);
  int rc = LGPU_OK;
  {
    // lgpu_set_state copies mean/sprd from the host; give it placeholders and
    // overwrite them with the device statistics below
    std::vector<float> tmp(nm, 0.0f);
    rc = lgpu_set_state(h, k, ns, members, tmp.data(), tmp.data(), nvars, vars);
  }
  if (rc != LGPU_OK) return rc;
  CK(launch_state_stats(h->st, (long long)h->ncol * ns, k, h->buf[B_BKG].as<float>(), h->buf[B_MEANB].as<float>(),
                        h->buf[B_SPRDB].as<float>()),
     "background statistics");
  CK(cudaStreamSynchronize(h->st), "set_state_members");
  return LGPU_OK;
}

int lgpu_get_background(lgpu_handle *h, float *state, float *mean, float *sprd) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->state_ok) return fail(h, LGPU_ERR_ORDER, "get_background before set_state");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t nx = (size_t)h->ncol * h->ns * h->k, nm = (size_t)h->ncol * h->ns;
  if (state) CK(cudaMemcpyAsync(state, h->buf[B_BKG].p, nx * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  if (mean) CK(cudaMemcpyAsync(mean, h->buf[B_MEANB].p, nm * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  if (sprd) CK(cudaMemcpyAsync(sprd, h->buf[B_SPRDB].p, nm * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  CK(cudaStreamSynchronize(h->st), "get_background");
  return LGPU_OK;
}

int lgpu_get_obs_prepared(lgpu_handle *h, float *hx, float *hx_mean, float *lat, float *lon, float *val, float *err) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->obs_ok) return fail(h, LGPU_ERR_ORDER, "get_obs_prepared before set_obs");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t n = h->nobs, k = h->k;
  if (n > 0) {
    if (hx) CK(cudaMemcpyAsync(hx, h->buf[B_HX].p, n * k * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
    if (hx_mean) CK(cudaMemcpyAsync(hx_mean, h->buf[B_HXM].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
    if (lat) CK(cudaMemcpyAsync(lat, h->buf[B_OLAT].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
    if (lon) CK(cudaMemcpyAsync(lon, h->buf[B_OLON].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
    if (val) CK(cudaMemcpyAsync(val, h->buf[B_OVAL].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
    if (err) CK(cudaMemcpyAsync(err, h->buf[B_OERR].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  }
  CK(cudaStreamSynchronize(h->st), "get_obs_prepared");
  return LGPU_OK;
}

// First part of a run: checks, buffers, the observation index and the
// per-column parameters (events ev[0..2]); shared by the exact and the
// learned forms.
static int prepare_run(lgpu_handle *h, ObsSorted &os, int &launches) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->solver_ok) return fail(h, LGPU_ERR_ORDER, "solver_run before solver_init");
  if (!h->loc_ok) return fail(h, LGPU_ERR_ORDER, "solver_run before loc_init");
  if (!h->grid_ok || !h->state_ok || !h->obs_ok) return fail(h, LGPU_ERR_ORDER, "solver_run before grid/state/obs were set");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const int k = h->k, kp = h->kp, ns = h->ns, G = h->loc.groups;
  if (h->loc.cls == LOC_OCEAN && h->loc.vtloc_surf == 1) {
    if (h->bkg_t_var < 0 || h->bkg_t_var >= (int)h->vars.size())
      return fail(h, LGPU_ERR_CONFIG, "vtloc_surf.bkg_t_var does not name a state variable");
    h->loc.bkg_t_idx = h->vars[h->bkg_t_var].grid_s_idx;
    h->loc.bkg_t_len = h->vars[h->bkg_t_var].levels;
  }
  if (h->loc.cls == LOC_VTGC) {
    int maxlev = 0;
    for (auto &v : h->vars) maxlev = std::max(maxlev, v.levels);
    if (maxlev > G) return fail(h, LGPU_ERR_CONFIG, "loc_vtgc: a variable has more levels than level depths given");
    CK(h->buf[B_LEVDEPTH].ensure(sizeof(float) * G), "alloc lev");
    CK(cudaMemcpyAsync(h->buf[B_LEVDEPTH].p, h->lev_depth.data(), sizeof(float) * G, cudaMemcpyHostToDevice, h->st), "H2D lev");
    h->loc.lev_depth = h->buf[B_LEVDEPTH].as<float>();
  }
  const size_t nobs = std::max(h->nobs, 1);
  const long long units = (long long)h->nact * G;
  if (units > 0x7fffffffLL) return fail(h, LGPU_ERR_CAPACITY, "too many (column, group) units");
  h->nunits = (int)units;
  // ---- buffers
  CK(h->buf[B_SATOBS].ensure(sizeof(int) * std::max<size_t>(1, h->sat_obs.size())), "alloc");
  CK(h->buf[B_SATPLATS].ensure(sizeof(int) * std::max<size_t>(1, h->sat_plats.size())), "alloc");
  if (!h->sat_obs.empty())
    CK(cudaMemcpyAsync(h->buf[B_SATOBS].p, h->sat_obs.data(), 4 * h->sat_obs.size(), cudaMemcpyHostToDevice, h->st), "H2D");
  if (!h->sat_plats.empty())
    CK(cudaMemcpyAsync(h->buf[B_SATPLATS].p, h->sat_plats.data(), 4 * h->sat_plats.size(), cudaMemcpyHostToDevice, h->st), "H2D");
  CK(h->buf[B_CELL].ensure(4 * nobs), "alloc");
  CK(h->buf[B_COUNT].ensure(4 * (size_t)h->ncell), "alloc");
  CK(h->buf[B_FILL].ensure(4 * (size_t)h->ncell), "alloc");
  CK(h->buf[B_POSTMP].ensure(4 * nobs), "alloc");
  CK(h->buf[B_ORDER].ensure(4 * nobs), "alloc");
  CK(h->buf[B_ATMP].ensure(16 * nobs), "alloc");
  CK(h->buf[B_BTMP].ensure(16 * nobs), "alloc");
  CK(h->buf[B_SA].ensure(16 * nobs), "alloc");
  CK(h->buf[B_SB].ensure(16 * nobs), "alloc");
  CK(h->buf[B_SHX].ensure(4 * nobs * kp), "alloc sorted hx");
  CK(h->buf[B_SIDX].ensure(4 * nobs), "alloc");
  CK(h->buf[B_CSTART].ensure(4 * ((size_t)h->ncell + 1)), "alloc");
  CK(h->buf[B_CP].ensure(sizeof(ColPar) * (size_t)h->ncol), "alloc");
  CK(h->buf[B_G].ensure(4 * std::max<size_t>(1, (size_t)units) * packed_size(k)), "alloc Gram");
  CK(h->buf[B_T].ensure(4 * std::max<size_t>(1, (size_t)units) * k * k), "alloc transforms");
  CK(h->buf[B_NKEPT].ensure(4 * std::max<size_t>(1, (size_t)units)), "alloc");
  CK(h->buf[B_DMAXHZ].ensure(4 * (size_t)h->ncol), "alloc");
  CK(h->buf[B_DOBSC].ensure(4 * (size_t)h->ncol), "alloc");
  CK(h->buf[B_DLGC].ensure(4 * (size_t)h->ncol * G), "alloc");
  CK(h->buf[B_DLGL].ensure(4 * (size_t)h->ncol * G), "alloc");
  CK(h->buf[B_STATUS].ensure(16), "alloc");
  os.A = h->buf[B_SA].as<float4>();
  os.B = h->buf[B_SB].as<float4>();
  os.hx = h->buf[B_SHX].as<float>();
  os.idx = h->buf[B_SIDX].as<int>();
  os.cell_start = h->buf[B_CSTART].as<int>();
  cudaStream_t st = h->st;
  const bool bound = h->bound_state != nullptr;
  CK(cudaEventRecord(h->ev[0], st), "event");
  if (bound) {
    // the background mean and spread first (the column parameters read the
    // mean); the members follow the Gram (upload_members)
    const size_t nm = (size_t)h->ncol * ns;
    CK(cudaStreamWaitEvent(h->cst, h->ev[0], 0), "stream wait");
    CK(cudaEventRecord(h->ev_up[0], h->cst), "event");
    CK(cudaMemcpyAsync(h->buf[B_MEANB].p, h->bound_mean, nm * 4, cudaMemcpyHostToDevice, h->cst), "H2D mean");
    CK(cudaMemcpyAsync(h->buf[B_SPRDB].p, h->bound_sprd, nm * 4, cudaMemcpyHostToDevice, h->cst), "H2D sprd");
    CK(cudaEventRecord(h->ev_in[0], h->cst), "event");
  }
  // ---- observation index (kd_init counterpart) ----
  CK(launch_obs_index(st, h->nobs, k, kp, h->buf[B_OLAT].as<float>(), h->buf[B_OLON].as<float>(),
                      h->buf[B_OZ].as<float>(), h->buf[B_OTIME].as<float>(), h->buf[B_OVAL].as<float>(),
                      h->buf[B_OERR].as<float>(), h->buf[B_OOBSID].as<int>(), h->buf[B_OPLATID].as<int>(),
                      h->buf[B_HX].as<float>(), h->buf[B_HXM].as<float>(), h->buf[B_SATOBS].as<int>(),
                      (int)h->sat_obs.size(), h->buf[B_SATPLATS].as<int>(), (int)h->sat_plats.size(),
                      h->buf[B_GEOM].as<IndexGeom>(), h->ncell, h->buf[B_CELL].as<int>(), h->buf[B_COUNT].as<int>(),
                      h->buf[B_FILL].as<int>(), h->buf[B_POSTMP].as<int>(), h->buf[B_ORDER].as<int>(),
                      h->buf[B_ATMP].as<float4>(), h->buf[B_BTMP].as<float4>(), os, &launches),
     "observation index");
  CK(cudaEventRecord(h->ev[1], st), "event");
  // ---- per-column parameters (the ocean localizer reads the background mean) ----
  if (bound) CK(cudaStreamWaitEvent(st, h->ev_in[0], 0), "stream wait");
  CK(launch_col_prep(st, h->ncol, h->buf[B_LAT].as<float>(), h->buf[B_LON].as<float>(), h->buf[B_MASK].as<int>(),
                     h->buf[B_MEANB].as<float>(), ns, h->loc, h->buf[B_CP].as<ColPar>(),
                     h->buf[B_DMAXHZ].as<float>(), &launches),
     "column prep");
  CK(cudaMemsetAsync(h->buf[B_DOBSC].p, 0, 4 * (size_t)h->ncol, st), "memset");
  CK(cudaMemsetAsync(h->buf[B_DLGC].p, 0, 4 * (size_t)h->ncol * G, st), "memset");
  CK(cudaMemsetAsync(h->buf[B_DLGL].p, 0, 4 * (size_t)h->ncol * G, st), "memset");
  CK(cudaMemsetAsync(h->buf[B_STATUS].p, 0, 16, st), "memset");
  CK(cudaEventRecord(h->ev[2], st), "event");
  return LGPU_OK;
}

static int learned_run(lgpu_handle *h);
static int eig_scratch(lgpu_handle *h, int units, EigSplit &sp, int &batch);
static UpdateArgs update_args(lgpu_handle *h);

// FP32_RESOLVE: the run's list of units for the FP64 re-solve, counters
// reset; room for every unit of the run twice (an exact run flags a unit at
// most once; the learned form may solve a column in two exact passes)
static int flag_prepare(lgpu_handle *h) {
  if (h->prec != LGPU_PREC_FP32_RESOLVE) return LGPU_OK;
  CK(h->buf[B_FLAGLIST].ensure(16 + 8 * (size_t)std::max(1, h->nunits)), "alloc");
  CK(cudaMemsetAsync(h->buf[B_FLAGLIST].p, 0, 16, h->st), "memset");
  return LGPU_OK;
}

static void flag_args(lgpu_handle *h, EigArgs &ea) {
  ea.gap_thresh = h->gap_thresh;
  ea.flag_list = nullptr;
  ea.flag_n = nullptr;
  ea.flag_cap = 0;
  if (h->prec != LGPU_PREC_FP32_RESOLVE) return;
  ea.flag_n = h->buf[B_FLAGLIST].as<int>();
  ea.flag_list = ea.flag_n + 4;
  ea.flag_cap = 2 * std::max(1, h->nunits);
}

// eigensolve scratch of the split pipeline for `units` units (at most 8 GB,
// units in batches); batch = 0 when it cannot be had (the fused kernel runs)
static int eig_scratch(lgpu_handle *h, int units, EigSplit &sp, int &batch) {
  const int k = h->k;
  const size_t per = eig_split_bytes_per_unit(k);
  const size_t budget = (size_t)8 << 30;
  batch = (int)std::min<size_t>((size_t)std::max(1, units), std::max<size_t>(1024, budget / per));
  const size_t need = per * (size_t)batch + 5 * 256;
  if (h->buf[B_EIGSCR].cap >= need || h->buf[B_EIGSCR].ensure(need) == cudaSuccess) {
    unsigned char *base = h->buf[B_EIGSCR].as<unsigned char>();
    size_t off = 0;
    auto take = [&](size_t bytes) { unsigned char *p = base + off; off += (bytes + 255) & ~(size_t)255; return p; };
    sp.Q = reinterpret_cast<float *>(take((size_t)batch * k * k * 4));
    sp.DE = reinterpret_cast<float *>(take((size_t)batch * 2 * k * 4));
    sp.log = reinterpret_cast<float2 *>(take((size_t)batch * eig_log_cap(k) * 8));
    sp.logn = reinterpret_cast<int *>(take((size_t)batch * 4));
    sp.lam = reinterpret_cast<float *>(take((size_t)batch * k * 4));
    sp.cap = eig_log_cap(k);
  } else {
    cudaGetLastError();   // clear the failed allocation
    batch = 0;
  }
  return LGPU_OK;
}

static UpdateArgs update_args(lgpu_handle *h) {
  UpdateArgs ua;
  ua.ncol = h->ncol;
  ua.ns = h->ns;
  ua.k = h->k;
  ua.groups = h->loc.groups;
  ua.col0 = 0;
  ua.ncols = h->ncol;
  ua.mask = h->buf[B_MASK].as<int>();
  ua.col2act = h->buf[B_COL2ACT].as<int>();
  ua.cp = h->buf[B_CP].as<ColPar>();
  ua.loc_cls = h->loc.cls;
  ua.vtloc_surf = h->loc.vtloc_surf;
  ua.slab_var = h->buf[B_SLABVAR].as<int>();
  ua.slab_lev = h->buf[B_SLABLEV].as<int>();
  ua.var_inc_max = h->buf[B_VARINC].as<float>();
  ua.var_lb = h->buf[B_VARLB].as<float>();
  ua.var_ub = h->buf[B_VARUB].as<float>();
  ua.bkg = h->buf[B_BKG].as<float>();
  ua.mean_b = h->buf[B_MEANB].as<float>();
  ua.sprd_b = h->buf[B_SPRDB].as<float>();
  ua.T = h->buf[B_T].as<float>();
  ua.nkept = h->buf[B_NKEPT].as<int>();
  ua.ana = h->buf[B_ANA].as<float>();
  ua.mean_a = h->buf[B_MEANA].as<float>();
  ua.sprd_a = h->buf[B_SPRDA].as<float>();
  ua.rtps = h->scfg.rtps;
  ua.rtpp = h->scfg.rtpp;
  ua.mul = h->scfg.mul;
  ua.status = h->buf[B_STATUS].as<int>();
  return ua;
}

// The batched tensor-core Gram over a tile set (tiles of 128 columns; the
// records and the weight cache are the handle's scratch): G, nkept and the
// diagnostics of the tiles' units.  Events ev[6] after the tile streams.
struct TileSet {
  int ntiles;
  DevBuf *cols, *par, *n, *off;
};

static int upload_members(lgpu_handle *h, cudaEvent_t after);

// start_upload: a bound state's members start uploading once the tile fill is
// launched (after the tile-stream offsets are read back), beside the Gram
static int run_batched_tiles(lgpu_handle *h, const ObsSorted &os, const TileSet &ts, int &launches,
                             bool start_upload) {
  cudaStream_t st = h->st;
  const int k = h->k, kp = h->kp, G = h->loc.groups;
  CK(launch_tile_prep(st, ts.ntiles, (*ts.cols).as<int>(), h->buf[B_CP].as<ColPar>(),
                      (*ts.par).as<TilePar>(), &launches), "tile prep");
  // tile candidate streams: count, size the record buffer, fill
  CK(launch_tile_count(st, ts.ntiles, (*ts.par).as<TilePar>(), h->buf[B_GEOM].as<IndexGeom>(), os,
                       (*ts.n).as<int>(), (*ts.off).as<int>(), &launches),
     "tile count");
  // the stream offsets size the record buffer and split each tile's stream
  // into accumulation segments
  if (h->pin_off_n < (size_t)ts.ntiles + 1) {
    if (h->pin_off) cudaFreeHost(h->pin_off);
    h->pin_off = nullptr;
    h->pin_off_n = 0;
    CK(cudaMallocHost(&h->pin_off, sizeof(int) * ((size_t)ts.ntiles + 1)), "alloc stream offsets");
    h->pin_off_n = (size_t)ts.ntiles + 1;
  }
  CK(cudaMemcpyAsync(h->pin_off, (*ts.off).as<int>(), sizeof(int) * ((size_t)ts.ntiles + 1), cudaMemcpyDeviceToHost,
                     st),
     "D2H stream offsets");
  CK(cudaStreamSynchronize(st), "stream size sync");
  h->h_tile_off.assign(h->pin_off, h->pin_off + ts.ntiles + 1);
  const int nchunk_total = h->h_tile_off[ts.ntiles];
  CK(h->buf[B_TILEREC].ensure(std::max<size_t>(16, (size_t)nchunk_total * record_bytes(k))), "alloc tile streams");
  CK(launch_tile_fill(st, ts.ntiles, (*ts.par).as<TilePar>(), h->buf[B_GEOM].as<IndexGeom>(), os, k, kp,
                      (*ts.off).as<int>(), h->buf[B_TILEREC].as<unsigned char>(),
                      h->buf[B_STATUS].as<int>(), &launches),
     "tile fill");
  CK(cudaEventRecord(h->ev[6], st), "event");
  if (start_upload) {
    const int rc = upload_members(h, h->ev_gram_done);
    if (rc != LGPU_OK) return rc;
  }
  TcArgs ta;
  ta.ntiles = ts.ntiles;
  ta.groups = G;
  ta.k = k;
  ta.kp = kp;
  gram_tc_passes(k, &ta.npass, &ta.np);
  h->mma_n = ta.np;
  ta.nf = packed_size(k);
  ta.ncol = h->ncol;
  ta.tile_cols = (*ts.cols).as<int>();
  ta.col2act = h->buf[B_COL2ACT].as<int>();
  ta.cp = h->buf[B_CP].as<ColPar>();
  ta.loc = h->loc;
  ta.tp = (*ts.par).as<TilePar>();
  ta.rec = h->buf[B_TILEREC].as<unsigned char>();
  ta.tile_off = (*ts.off).as<int>();
  ta.tile_n = (*ts.n).as<int>();
  ta.G = h->buf[B_G].as<float>();
  ta.nkept = h->buf[B_NKEPT].as<int>();
  ta.diag_obscount = h->buf[B_DOBSC].as<float>();
  ta.diag_lg_obscount = h->buf[B_DLGC].as<float>();
  ta.diag_lg_obsloc = h->buf[B_DLGL].as<float>();
  ta.status = h->buf[B_STATUS].as<int>();
  // weight cache for multi-pass tiles (at most 48 GB; without it every pass
  // recomputes the weights)
  ta.wcache = nullptr;
  ta.nchunk_total = nchunk_total;
  ta.wflag = nullptr;
  if (ta.npass >= 2) {
    const size_t wb = gram_tc_wcache_bytes(G, nchunk_total);
    if (wb <= ((size_t)48 << 30)) {
      if (h->buf[B_WCACHE].cap >= wb || h->buf[B_WCACHE].ensure(std::max<size_t>(wb, 256)) == cudaSuccess) {
        ta.wcache = h->buf[B_WCACHE].as<float>();
        ta.wflag = reinterpret_cast<int *>(h->buf[B_WCACHE].as<unsigned char>() +
                                           (wb - (size_t)G * nchunk_total * sizeof(int)));
      } else {
        cudaGetLastError();   // clear the failed allocation
      }
    }
  }
  // accumulation segments: each tile's stream is split into ranges of at most
  // kSegChunks chunks, each its own CTA (which drains its tensor-core
  // accumulator into its result rows every 64 chunks: the FP32 accumulation
  // error grows with the MMAs summed into one accumulator); the partial
  // Grams of a tile's segments are summed in order afterwards; the partials
  // take at most 24 GB (longer segments otherwise)
  ta.units = (long long)h->nact * G;
  ta.nf = packed_size(k);
  ta.Gpart = nullptr;
  ta.cnt = nullptr;
  auto plan = [&](int seg_chunks, int drain) {
    h->h_tc_work.clear();
    h->h_tc_seg.clear();
    int cblk = 0, blk = 0, most = 1;
    for (int t = 0; t < ts.ntiles; t++) {
      const int n = h->h_tile_off[t + 1] - h->h_tile_off[t];
      const int ns_t = std::max(1, (n + seg_chunks - 1) / seg_chunks);
      const int len = (n + ns_t - 1) / ns_t;
      const bool multi = ns_t > 1 || n > drain;   // more than one accumulator for the tile
      most = std::max(most, ns_t);
      int nb = 0;
      for (int q = 0; q < ns_t; q++) {
        TcWork w{};
        w.tile = t;
        w.seg = q;
        w.cs = std::min(n, q * len);
        w.ce = std::min(n, (q + 1) * len);
        w.cblk = multi ? cblk + q : -1;
        w.blk0 = multi ? blk + nb : -1;
        nb += std::max(1, (w.ce - w.cs + drain - 1) / drain);
        h->h_tc_work.push_back(w);
      }
      if (multi) {
        h->h_tc_seg.push_back(TcSegTile{t, ns_t, cblk, nb, blk, 0, 0, 0});
        cblk += ns_t;
        blk += nb;
      }
    }
    return std::make_pair(std::make_pair(cblk, blk), most);
  };
  const double block_bytes = (double)G * 128.0 * ta.nf * 4.0;
  // over 24 GB of partial blocks: longer drain intervals first, then longer
  // segments (one block each); a segment as long as the longest tile stream
  // leaves one accumulator per tile and no blocks
  int longest = 0;
  for (int t = 0; t < ts.ntiles; t++) longest = std::max(longest, h->h_tile_off[t + 1] - h->h_tile_off[t]);
  int drain = kDrainChunks, seg_chunks = kSegChunks;
  auto pl = plan(seg_chunks, drain);
  while (pl.first.second > 0 && pl.first.second * block_bytes > 24.0 * (1ull << 30)) {
    if (drain < seg_chunks) {
      drain *= 2;
    } else if (seg_chunks < longest) {
      seg_chunks *= 2;
      drain = seg_chunks;
    } else {
      break;   // unreachable: one segment per tile with drain >= its length has no blocks
    }
    pl = plan(seg_chunks, drain);
  }
  if (pl.first.second > 0) {
    const size_t gp = (size_t)pl.first.second * (size_t)block_bytes;
    const size_t cn = (size_t)pl.first.first * G * 128 * 3 * 4;
    if ((h->buf[B_GPART].cap >= gp || h->buf[B_GPART].ensure(gp) == cudaSuccess) &&
        (h->buf[B_GCNT].cap >= cn || h->buf[B_GCNT].ensure(cn) == cudaSuccess)) {
      ta.Gpart = h->buf[B_GPART].as<float>();
      ta.cnt = h->buf[B_GCNT].as<float>();
    } else {
      cudaGetLastError();   // clear the failed allocation: one accumulator per tile
      drain = 1 << 30;
      pl = plan(1 << 30, drain);
    }
  }
  ta.drain = drain;
  CK(h->buf[B_TCWORK].ensure(sizeof(TcWork) * std::max<size_t>(1, h->h_tc_work.size())), "alloc segments");
  CK(h->buf[B_TCSEG].ensure(sizeof(TcSegTile) * std::max<size_t>(1, h->h_tc_seg.size())), "alloc segments");
  CK(cudaMemcpyAsync(h->buf[B_TCWORK].p, h->h_tc_work.data(), sizeof(TcWork) * h->h_tc_work.size(),
                     cudaMemcpyHostToDevice, st), "H2D segments");
  if (!h->h_tc_seg.empty())
    CK(cudaMemcpyAsync(h->buf[B_TCSEG].p, h->h_tc_seg.data(), sizeof(TcSegTile) * h->h_tc_seg.size(),
                       cudaMemcpyHostToDevice, st), "H2D segments");
  ta.work = h->buf[B_TCWORK].as<TcWork>();
  ta.nwork = (int)h->h_tc_work.size();
  ta.segtiles = h->buf[B_TCSEG].as<TcSegTile>();
  ta.nsegtiles = (int)h->h_tc_seg.size();
  h->gram_nseg = pl.second;
  if (h->tc_cull < 0) {
    // the first batched Gram of a configuration runs both producer forms,
    // timed, and keeps the faster; their outputs are bit-identical, and every
    // output of the Gram kernels is overwritten by the second run (the
    // executed-MMA counter is reset between them)
    float tm[2] = {0.0f, 0.0f};
    for (int v = 0; v < 2; v++) {
      ta.cull = v;
      if (v == 1) CK(cudaMemsetAsync(h->buf[B_STATUS].as<int>() + 2, 0, sizeof(int), st), "memset");
      CK(cudaEventRecord(h->ev_cull[v], st), "event");
      CK(launch_gram_tc(st, ta, &launches), "tensor-core gram kernel");
    }
    CK(cudaEventRecord(h->ev_cull[2], st), "event");
    CK(cudaEventSynchronize(h->ev_cull[2]), "tune sync");
    CK(cudaEventElapsedTime(&tm[0], h->ev_cull[0], h->ev_cull[1]), "timing");
    CK(cudaEventElapsedTime(&tm[1], h->ev_cull[1], h->ev_cull[2]), "timing");
    h->tc_cull = tm[1] < tm[0] ? 1 : 0;
    h->tc_tune_ms = std::max(tm[0], tm[1]);
  } else {
    ta.cull = h->tc_cull;
    CK(launch_gram_tc(st, ta, &launches), "tensor-core gram kernel");
  }
  CK(launch_gram_segsum(st, ta, h->buf[B_ACTIVE].as<int>(), &launches), "gram segment sum");
  return LGPU_OK;
}

static int solver_run(lgpu_handle *h);

// A bound state's members, uploaded on the copy stream in the column chunks
// of the update (each chunk with its event), once `after` has been reached on
// the compute stream.  They start after the tile streams (batched Gram) or
// after the Gram (plain): a large copy in flight while the run reads back the
// tile-stream offsets delayed that small read, and with it the Gram's launch,
// by 12 to 108 ms at C2; the Gram kernels, the eigensolve and the update ran
// at full speed beside the same copies.
static int upload_members(lgpu_handle *h, cudaEvent_t after) {
  const int ns = h->ns, k = h->k;
  CK(cudaEventRecord(after, h->st), "event");
  CK(cudaStreamWaitEvent(h->cst, after, 0), "stream wait");
  CK(cudaEventRecord(h->ev_in[1], h->cst), "event");
  for (int c = 0; c < kOutChunks; c++) {
    int b0, b1;
    chunk_bounds(h->ncol, kOutChunks, c, &b0, &b1);
    const size_t c0 = (size_t)b0, c1 = (size_t)b1;
    if (c1 > c0)
      CK(cudaMemcpyAsync(h->buf[B_BKG].as<float>() + c0 * ns * k, h->bound_state + c0 * ns * k,
                         (c1 - c0) * ns * k * 4, cudaMemcpyHostToDevice, h->cst), "H2D state");
    CK(cudaEventRecord(h->ev_upc[c], h->cst), "event");
  }
  CK(cudaEventRecord(h->ev_up[1], h->cst), "event");
  return LGPU_OK;
}

// letkf_solver_run (src/letkf_solver.F90:150-389)
int lgpu_solver_run(lgpu_handle *h) {
  if (!h) return LGPU_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  h->tim = lgpu_timings{};
  const int rc = h->variant == LGPU_VARIANT_LEARNED ? learned_run(h) : solver_run(h);
  h->tim.h2d_obs_ms = h->obs_h2d_ms;
  h->tim.host_obs_ms = h->obs_host_ms;
  h->tim.host_run_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

static int solver_run(lgpu_handle *h) {
  ObsSorted os;
  int launches = 0;
  int rc0 = prepare_run(h, os, launches);
  if (rc0 != LGPU_OK) return rc0;
  const int k = h->k, kp = h->kp, ns = h->ns, G = h->loc.groups;
  cudaStream_t st = h->st;
  const bool bound = h->bound_state != nullptr;
  // ---- search + localize + Gram ----
  // ---- Gram: the batched tensor-core form or the plain per-column form ----
  const TileSet grid_tiles{h->ntiles, &h->buf[B_TILECOLS], &h->buf[B_TILEPAR], &h->buf[B_TILEN], &h->buf[B_TILEOFF]};
  bool uploading = false;   // a bound state's members are on their way
  auto run_batched = [&](bool start_upload) -> int {
    uploading = start_upload && bound;
    return run_batched_tiles(h, os, grid_tiles, launches, start_upload && bound);
  };
  auto run_plain = [&]() -> int {
    GramArgs ga;
    ga.nunits = h->nunits;
    ga.groups = G;
    ga.k = k;
    ga.kp = kp;
    ga.active = h->buf[B_ACTIVE].as<int>();
    ga.cp = h->buf[B_CP].as<ColPar>();
    ga.loc = h->loc;
    ga.obs = os;
    ga.geom = h->buf[B_GEOM].as<IndexGeom>();
    ga.G = h->buf[B_G].as<float>();
    ga.nkept = h->buf[B_NKEPT].as<int>();
    ga.diag_obscount = h->buf[B_DOBSC].as<float>();
    ga.diag_lg_obscount = h->buf[B_DLGC].as<float>();
    ga.diag_lg_obsloc = h->buf[B_DLGL].as<float>();
    ga.ncol = h->ncol;
    CK(launch_gram(st, ga, &launches), "gram kernel");
    return LGPU_OK;
  };
  // AUTO: the first analysis of a configuration (grid, localizer, k) runs
  // both forms, timed, and keeps the faster; the plain form wins below k = 8
  int choice = h->variant;
  if (choice == LGPU_VARIANT_AUTO) choice = k < 8 ? LGPU_VARIANT_PLAIN : h->auto_choice;
  int rc = LGPU_OK;
  if (!h->preloaded && (choice == 0 || (choice == LGPU_VARIANT_BATCHED_TC && h->tc_cull < 0))) {
    // the trials below time kernels: load them first
    CK(preload_gram(), "kernel load");
    CK(preload_gram_tc(h->loc.cls), "kernel load");
    h->preloaded = true;
  }
  if (choice == 0) {
    CK(cudaEventRecord(h->ev_tune[0], st), "event");
    if ((rc = run_plain()) != LGPU_OK) return rc;
    CK(cudaEventRecord(h->ev_tune[1], st), "event");
    if ((rc = run_batched(false)) != LGPU_OK) return rc;
    CK(cudaEventRecord(h->ev_tune[2], st), "event");
    CK(cudaEventSynchronize(h->ev_tune[2]), "tune sync");
    float tp = 0.0f, tb = 0.0f;
    CK(cudaEventElapsedTime(&tp, h->ev_tune[0], h->ev_tune[1]), "timing");
    CK(cudaEventElapsedTime(&tb, h->ev_tune[1], h->ev_tune[2]), "timing");
    tb -= h->tc_tune_ms;   // the batched form's producer tuning ran its Gram twice
    h->tc_tune_ms = 0.0f;
    h->auto_choice = tb <= tp ? LGPU_VARIANT_BATCHED_TC : LGPU_VARIANT_PLAIN;
    // the kept result is the chosen form's
    if (h->auto_choice == LGPU_VARIANT_PLAIN && (rc = run_plain()) != LGPU_OK) return rc;
    choice = h->auto_choice;
  } else if (choice == LGPU_VARIANT_BATCHED_TC) {
    // the whole Gram at once (a bound state's members upload meanwhile)
    if ((rc = run_batched(true)) != LGPU_OK) return rc;
  } else {
    if ((rc = run_plain()) != LGPU_OK) return rc;
  }
  h->used_tc = choice == LGPU_VARIANT_BATCHED_TC;
  CK(cudaEventRecord(h->ev[3], st), "event");
  if (bound && !uploading && (rc = upload_members(h, h->ev_gram_done)) != LGPU_OK) return rc;
  // ---- eigensolve + transform, update + epilogue, in column chunks ----
  // A bound state is processed in kOutChunks column chunks: chunk c's
  // analysis is downloaded into the caller's arrays while the eigensolve and
  // update of the following chunks run.
  EigArgs ea;
  ea.wbar = h->learn_wbar;   // mean weights of every unit while training data is collected
  ea.ulist = nullptr;
  ea.nunits = h->nunits;
  ea.k = k;
  ea.infl = 1.0f;   // letkf_core_solve is called with infl = 1.0 (src/letkf_solver.F90:279)
  ea.G = h->buf[B_G].as<float>();
  ea.nkept = h->buf[B_NKEPT].as<int>();
  ea.T = h->buf[B_T].as<float>();
  ea.status = h->buf[B_STATUS].as<int>();
  UpdateArgs ua = update_args(h);
  if ((rc = flag_prepare(h)) != LGPU_OK) return rc;
  flag_args(h, ea);
  const bool fp64 = h->prec == LGPU_PREC_FP64;
  // eigensolve scratch: the split pipeline (at most 8 GB, units in batches);
  // the fused one-warp kernel over all units if the scratch cannot be had
  // (no FP64 re-solve then)
  EigSplit sp;
  int batch = 0;
  if (!fp64) {
    if ((rc = eig_scratch(h, h->nunits, sp, batch)) != LGPU_OK) return rc;
    if (batch == 0) CK(launch_eig(st, ea, &launches), "eigen kernel");
  }
  const int nch = bound ? kOutChunks : 1;
  float eig_ms = 0.0f, upd_ms = 0.0f, fp64_ms = 0.0f;
  int nrec = 0;
  for (int c = 0; c < nch; c++) {
    int c0, c1;
    chunk_bounds(h->ncol, nch, c, &c0, &c1);
    if (c1 <= c0) break;
    // units of the chunk's active columns
    int a0 = -1, a1 = -1;
    for (int j = c0; j < c1 && a0 < 0; j++) if (h->h_col2act[j] >= 0) a0 = h->h_col2act[j];
    for (int j = c1 - 1; j >= c0 && a1 < 0; j--) if (h->h_col2act[j] >= 0) a1 = h->h_col2act[j] + 1;
    CK(cudaEventRecord(h->ev_chunk[c][0], st), "event");
    if (!fp64 && batch > 0 && a0 >= 0)
      CK(launch_eig_split(st, ea, sp, batch, a0 * G, (a1 - a0) * G, &launches), "eigen kernels");
    CK(cudaEventRecord(h->ev_chunk[c][3], st), "event");
    if (fp64 && a0 >= 0) {
      EigArgs e64 = ea;
      e64.nunits = (a1 - a0) * G;
      CK(launch_eig64(st, e64, a0 * G, &launches), "FP64 eigen kernel");
    } else if (batch > 0 && a0 >= 0 && ea.flag_list) {
      CK(launch_eig64_flagged(st, ea, &launches), "FP64 re-solve");
    }
    CK(cudaEventRecord(h->ev_chunk[c][1], st), "event");
    ua.col0 = c0;
    ua.ncols = c1 - c0;
    // the chunk's background (with a bound state the update's time includes
    // any wait for its upload)
    if (bound) CK(cudaStreamWaitEvent(st, h->ev_upc[c], 0), "stream wait");
    CK(launch_update(st, ua, &launches), "update kernel");
    CK(cudaEventRecord(h->ev_chunk[c][2], st), "event");
    nrec = c + 1;
    if (bound) {
      // downloads on their own stream: they run while the uploads of later
      // chunks (other direction of the link) are still in flight
      CK(cudaStreamWaitEvent(h->dst, h->ev_chunk[c][2], 0), "stream wait");
      CK(cudaEventRecord(h->ev_down[c][0], h->dst), "event");
      const size_t xo = (size_t)c0 * ns * k, xn = (size_t)(c1 - c0) * ns * k;
      const size_t mo = (size_t)c0 * ns, mn = (size_t)(c1 - c0) * ns;
      CK(cudaMemcpyAsync(h->bound_state + xo, h->buf[B_ANA].as<float>() + xo, xn * 4, cudaMemcpyDeviceToHost, h->dst),
         "D2H state");
      CK(cudaMemcpyAsync(h->bound_mean + mo, h->buf[B_MEANA].as<float>() + mo, mn * 4, cudaMemcpyDeviceToHost, h->dst),
         "D2H mean");
      CK(cudaMemcpyAsync(h->bound_sprd + mo, h->buf[B_SPRDA].as<float>() + mo, mn * 4, cudaMemcpyDeviceToHost, h->dst),
         "D2H sprd");
      CK(cudaEventRecord(h->ev_down[c][1], h->dst), "event");
    }
  }
  CK(cudaEventRecord(h->ev[5], st), "event");
  int *stat4 = h->pin_scr;
  stat4[4] = 0;
  CK(cudaMemcpyAsync(stat4, h->buf[B_STATUS].p, 16, cudaMemcpyDeviceToHost, st), "D2H status");
  if (ea.flag_n) CK(cudaMemcpyAsync(stat4 + 4, ea.flag_n, 4, cudaMemcpyDeviceToHost, st), "D2H flag count");
  CK(cudaStreamSynchronize(st), "solver_run");
  const int nflag = stat4[4];
  if (bound) CK(cudaStreamSynchronize(h->cst), "solver_run copies");
  if (bound) CK(cudaStreamSynchronize(h->dst), "solver_run copies");
  float ms[3];
  for (int i = 0; i < 3; i++) CK(cudaEventElapsedTime(&ms[i], h->ev[i], h->ev[i + 1]), "timing");
  for (int c = 0; c < nrec; c++) {
    float te = 0.0f, tu = 0.0f;
    float tf = 0.0f;
    CK(cudaEventElapsedTime(&te, h->ev_chunk[c][0], h->ev_chunk[c][1]), "timing");
    CK(cudaEventElapsedTime(&tu, h->ev_chunk[c][1], h->ev_chunk[c][2]), "timing");
    CK(cudaEventElapsedTime(&tf, h->ev_chunk[c][3], h->ev_chunk[c][1]), "timing");
    eig_ms += te;
    upd_ms += tu;
    fp64_ms += tf;
  }
  h->tim.index_ms = ms[0];
  h->tim.prep_ms = ms[1];
  h->tim.gram_ms = ms[2];
  h->tim.tiles_ms = 0.0f;
  if (h->used_tc) CK(cudaEventElapsedTime(&h->tim.tiles_ms, h->ev[2], h->ev[6]), "timing");
  h->tim.eig_ms = eig_ms;
  h->tim.update_ms = upd_ms;
  CK(cudaEventElapsedTime(&h->tim.total_ms, h->ev[0], h->ev[5]), "timing");
  h->tim.launches = launches;
  h->tim.variant = h->used_tc ? LGPU_VARIANT_BATCHED_TC : LGPU_VARIANT_PLAIN;
  h->tim.units = h->nunits;
  h->tim.kept_pairs = -1;
  h->tim.mma_chunks = h->used_tc ? stat4[2] : 0;
  h->tim.mma_n = h->used_tc ? h->mma_n : 0;
  h->tim.precision = h->prec;
  h->tim.fp64_units = fp64 ? h->nunits : std::min(nflag, ea.flag_cap);   // with a fused-kernel fallback: 0
  h->tim.fp64_ms = fp64_ms;
  h->tim.span_ms = h->tim.total_ms;
  if (bound) {
    const long long nx = (long long)h->ncol * ns * k, nm = (long long)h->ncol * ns;
    float tms = 0.0f, tmm = 0.0f;   // mean and spread, then the members
    CK(cudaEventElapsedTime(&tms, h->ev_up[0], h->ev_in[0]), "timing");
    CK(cudaEventElapsedTime(&tmm, h->ev_in[1], h->ev_up[1]), "timing");
    h->tim.h2d_state_ms = tms + tmm;
    for (int c = 0; c < nrec; c++) {
      float td = 0.0f;
      CK(cudaEventElapsedTime(&td, h->ev_down[c][0], h->ev_down[c][1]), "timing");
      h->tim.d2h_state_ms += td;
    }
    if (nrec > 0) CK(cudaEventElapsedTime(&h->tim.span_ms, h->ev[0], h->ev_down[nrec - 1][1]), "timing");
    h->tim.h2d_state_bytes = 4 * (nx + 2 * nm);
    h->tim.d2h_state_bytes = 4 * (nx + 2 * nm);
  }
  const int status = stat4[0];
  h->ran = true;
  if (status & 1) return fail(h, LGPU_ERR_EIG, "eigensolver did not converge for at least one unit");
  if (status & 2) return fail(h, LGPU_ERR_EIG, "non-positive eigenvalue in at least one unit");
  if (status & 4) return fail(h, LGPU_ERR_NONFINITE, "non-finite analysis mean or spread");
  if (status & 16) return fail(h, LGPU_ERR_CUDA, "tensor-core pipeline wait timed out");
  if (status & 32) return fail(h, LGPU_ERR_CUDA, "internal: malformed eigensolver rotation log");
  if (status & 64) return fail(h, LGPU_ERR_CUDA, "update stage copy wait timed out");
  return LGPU_OK;
}

int lgpu_get_state(lgpu_handle *h, float *state, float *mean, float *sprd) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->ran) return fail(h, LGPU_ERR_ORDER, "get_state before a successful solver_run");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t nx = (size_t)h->ncol * h->ns * h->k, nm = (size_t)h->ncol * h->ns;
  if (state) CK(cudaMemcpyAsync(state, h->buf[B_ANA].p, nx * 4, cudaMemcpyDeviceToHost, h->st), "D2H state");
  if (mean) CK(cudaMemcpyAsync(mean, h->buf[B_MEANA].p, nm * 4, cudaMemcpyDeviceToHost, h->st), "D2H mean");
  if (sprd) CK(cudaMemcpyAsync(sprd, h->buf[B_SPRDA].p, nm * 4, cudaMemcpyDeviceToHost, h->st), "D2H sprd");
  CK(cudaStreamSynchronize(h->st), "get_state");
  return LGPU_OK;
}

int lgpu_get_diag(lgpu_handle *h, float *maxhz, float *obscount, float *lg_obscount, float *lg_obsloc) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->ran) return fail(h, LGPU_ERR_ORDER, "get_diag before a successful solver_run");
  if (!h->scfg.save_diag) return fail(h, LGPU_ERR_CONFIG, "save_diag is off");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t n = h->ncol, ng = (size_t)h->ncol * h->loc.groups;
  if (maxhz) CK(cudaMemcpyAsync(maxhz, h->buf[B_DMAXHZ].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  if (obscount) CK(cudaMemcpyAsync(obscount, h->buf[B_DOBSC].p, n * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  if (lg_obscount) CK(cudaMemcpyAsync(lg_obscount, h->buf[B_DLGC].p, ng * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  if (lg_obsloc) CK(cudaMemcpyAsync(lg_obsloc, h->buf[B_DLGL].p, ng * 4, cudaMemcpyDeviceToHost, h->st), "D2H");
  CK(cudaStreamSynchronize(h->st), "get_diag");
  return LGPU_OK;
}

// loc_ocean's per-column diagnostic (src/subclass.letkf_localizer/
// letkf_loc_ocean.F90:353-358): the level count of the surface localisation
// group (calc_mldlvl_bkgt) of each column of the last run, 0 on masked
// columns (the reference's solver loop skips them before localizer%groups)
int lgpu_get_loc_diag(lgpu_handle *h, float *surf_lvl) {
  if (!h || !surf_lvl) return LGPU_ERR_ARG;
  if (!h->ran) return fail(h, LGPU_ERR_ORDER, "get_loc_diag before a successful solver_run");
  if (h->loc.cls != LOC_OCEAN || h->loc.vtloc_surf != 1)
    return fail(h, LGPU_ERR_CONFIG, "get_loc_diag: the localizer is not loc_ocean with vtloc_surf");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  std::vector<ColPar> cp((size_t)h->ncol);
  CK(cudaMemcpyAsync(cp.data(), h->buf[B_CP].p, sizeof(ColPar) * (size_t)h->ncol, cudaMemcpyDeviceToHost, h->st),
     "D2H column parameters");
  CK(cudaStreamSynchronize(h->st), "get_loc_diag");
  for (int c = 0; c < h->ncol; c++) surf_lvl[c] = h->h_col2act[c] >= 0 ? (float)cp[(size_t)c].mld : 0.0f;
  return LGPU_OK;
}

// letkf_solver_final's diagnostics file (src/letkf_solver.F90:397-527) for a
// grid of nx * ny columns (column ij = i + nx * j)
int lgpu_write_diag(lgpu_handle *h, const char *path, int nx, int ny, const float *lat_nom, const float *lon_nom) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->ran) return fail(h, LGPU_ERR_ORDER, "write_diag before a successful solver_run");
  if (nx <= 0 || ny <= 0 || (long long)nx * ny != h->ncol)
    return fail(h, LGPU_ERR_ARG, "write_diag: nx * ny must equal the column count");
  const size_t n = (size_t)h->ncol, G = (size_t)h->loc.groups;
  std::vector<float> maxhz(n), obsc(n), lgc(n * G), lgl(n * G);
  int rc = lgpu_get_diag(h, maxhz.data(), obsc.data(), lgc.data(), lgl.data());
  if (rc != LGPU_OK) return rc;
  rc = lgpu_write_diag_nc(path, nx, ny, (int)G, lat_nom, lon_nom, maxhz.data(), obsc.data(), lgc.data(), lgl.data());
  if (rc != LGPU_OK) return fail(h, rc, lgpu_io_last_error());
  return LGPU_OK;
}

// loc_ocean_final's diagnostics file (letkf_loc_ocean.F90:249-322):
// vtloc_surf_lvl and its depth vert_nom(vtloc_surf_lvl) per column
int lgpu_write_loc_diag(lgpu_handle *h, const char *path, int nx, int ny, const float *lat_nom, const float *lon_nom,
                        int nz, const float *vert_nom) {
  if (!h) return LGPU_ERR_ARG;
  if (nx <= 0 || ny <= 0 || (long long)nx * ny != h->ncol || nz <= 0 || !vert_nom)
    return fail(h, LGPU_ERR_ARG, "write_loc_diag: nx * ny must equal the column count and vert_nom hold nz depths");
  std::vector<float> lvl((size_t)h->ncol), dep((size_t)h->ncol, 0.0f);
  int rc = lgpu_get_loc_diag(h, lvl.data());
  if (rc != LGPU_OK) return rc;
  for (int c = 0; c < h->ncol; c++) {
    const int l = (int)lvl[(size_t)c];
    if (l > nz) return fail(h, LGPU_ERR_ARG, "write_loc_diag: vert_nom has fewer levels than the surface group");
    dep[(size_t)c] = l >= 1 ? vert_nom[l - 1] : 0.0f;
  }
  rc = lgpu_write_loc_diag_nc(path, nx, ny, lat_nom, lon_nom, lvl.data(), dep.data());
  if (rc != LGPU_OK) return fail(h, rc, lgpu_io_last_error());
  return LGPU_OK;
}

int lgpu_get_timings(const lgpu_handle *h, lgpu_timings *t) {
  if (!h || !t) return LGPU_ERR_ARG;
  *t = h->tim;
  return LGPU_OK;
}

// letkf_solver_final (src/letkf_solver.F90:397-527) minus the NetCDF writer:
// release the per-run work buffers.
int lgpu_solver_final(lgpu_handle *h) {
  if (!h) return LGPU_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->st);
  int work[] = {B_CELL, B_COUNT, B_FILL, B_POSTMP, B_ORDER, B_ATMP, B_BTMP, B_G, B_T};
  for (int b : work) h->buf[b].release();
  return LGPU_OK;
}

int lgpu_get_obslist(lgpu_handle *h, int ij, int group, int *idx, float *rloc, int cap, int *n, int *ncand) {
  if (!h || !n) return LGPU_ERR_ARG;
  if (!h->ran) return fail(h, LGPU_ERR_ORDER, "get_obslist before a successful solver_run");
  if (ij < 0 || ij >= h->ncol || group < 0 || group >= h->loc.groups || cap < 0)
    return fail(h, LGPU_ERR_ARG, "get_obslist: index out of range");
  *n = 0;
  if (ncand) *ncand = 0;
  if (h->h_col2act[ij] < 0) return LGPU_OK;   // masked column: no search (src/letkf_solver.F90:207)
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const int lcap = std::max(h->nobs, 1);
  CK(h->buf[B_LIST_IDX].ensure(4 * (size_t)lcap), "alloc");
  CK(h->buf[B_LIST_R].ensure(4 * (size_t)lcap), "alloc");
  CK(h->buf[B_LIST_CNT].ensure(16), "alloc");
  ObsSorted os;
  os.A = h->buf[B_SA].as<float4>();
  os.B = h->buf[B_SB].as<float4>();
  os.hx = h->buf[B_SHX].as<float>();
  os.idx = h->buf[B_SIDX].as<int>();
  os.cell_start = h->buf[B_CSTART].as<int>();
  CK(launch_obslist(h->st, ij, group, group, h->buf[B_CP].as<ColPar>() + ij, h->loc, os,
                    h->buf[B_GEOM].as<IndexGeom>(), lcap, h->buf[B_LIST_IDX].as<int>(), h->buf[B_LIST_R].as<float>(),
                    h->buf[B_LIST_CNT].as<int>()),
     "obslist kernel");
  int cnt[2] = {0, 0};
  CK(cudaMemcpyAsync(cnt, h->buf[B_LIST_CNT].p, 8, cudaMemcpyDeviceToHost, h->st), "D2H");
  CK(cudaStreamSynchronize(h->st), "obslist");
  const int m = std::min(cnt[0], lcap);
  std::vector<int> li(m);
  std::vector<float> lr(m);
  if (m > 0) {
    CK(cudaMemcpy(li.data(), h->buf[B_LIST_IDX].p, 4 * (size_t)m, cudaMemcpyDeviceToHost), "D2H");
    CK(cudaMemcpy(lr.data(), h->buf[B_LIST_R].p, 4 * (size_t)m, cudaMemcpyDeviceToHost), "D2H");
  }
  std::vector<int> ord(m);
  for (int i = 0; i < m; i++) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int a, int b) { return li[a] < li[b]; });
  for (int i = 0; i < m && i < cap; i++) {
    if (idx) idx[i] = li[ord[i]];
    if (rloc) rloc[i] = lr[ord[i]];
  }
  *n = cnt[0];
  if (ncand) *ncand = cnt[1];
  return LGPU_OK;
}

// lgpu_get_obslist without any allocation (see include/letkf_gpu.h).
int lgpu_get_obslist_noalloc(lgpu_handle *h, int ij, int group, int *idx, float *rloc, int cap, int *n, int *ncand) {
  if (!h || !n) return LGPU_ERR_ARG;
  if (!h->ran) return fail(h, LGPU_ERR_ORDER, "get_obslist_noalloc before a successful solver_run");
  if (ij < 0 || ij >= h->ncol || group < 0 || group >= h->loc.groups || cap < 0)
    return fail(h, LGPU_ERR_ARG, "get_obslist_noalloc: index out of range");
  const int nmax = noalloc_max_list();
  if (h->nobs > nmax)
    return fail(h, LGPU_ERR_CAPACITY, "get_obslist_noalloc: " + std::to_string(h->nobs) +
                                          " observations exceed the fixed list scratch of " + std::to_string(nmax));
  *n = 0;
  if (ncand) *ncand = 0;
  if (h->h_col2act[ij] < 0) return LGPU_OK;   // masked column: no search (src/letkf_solver.F90:207)
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  int *scr = nullptr;
  CK(noalloc_scratch(h->device, &scr), "cudaGetSymbolAddress(list scratch)");
  ObsSorted os;
  os.A = h->buf[B_SA].as<float4>();
  os.B = h->buf[B_SB].as<float4>();
  os.hx = h->buf[B_SHX].as<float>();
  os.idx = h->buf[B_SIDX].as<int>();
  os.cell_start = h->buf[B_CSTART].as<int>();
  CK(launch_obslist_noalloc(h->st, group, h->buf[B_CP].as<ColPar>() + ij, h->loc, os, h->buf[B_GEOM].as<IndexGeom>(),
                            h->nobs, scr),
     "obslist kernel (no alloc)");
  int cnt[2] = {0, 0};
  CK(cudaMemcpyAsync(cnt, scr, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->st), "D2H counts");
  CK(cudaStreamSynchronize(h->st), "obslist (no alloc)");
  const int m = std::min(std::min(cnt[0], nmax), cap);
  if (m > 0) {
    if (idx) CK(cudaMemcpyAsync(idx, scr + 64 + 2 * (size_t)nmax, sizeof(int) * (size_t)m, cudaMemcpyDeviceToHost, h->st),
                "D2H idx");
    if (rloc) CK(cudaMemcpyAsync(rloc, scr + 64 + 3 * (size_t)nmax, sizeof(float) * (size_t)m, cudaMemcpyDeviceToHost,
                                 h->st), "D2H rloc");
    CK(cudaStreamSynchronize(h->st), "obslist (no alloc)");
  }
  *n = cnt[0];
  if (ncand) *ncand = cnt[1];
  return LGPU_OK;
}

int lgpu_debug_transform(lgpu_handle *h, int nunits, int k, const float *gram, float *trans) {
  if (!h || nunits < 0 || (nunits > 0 && (!gram || !trans))) return LGPU_ERR_ARG;
  if (k < 2 || k > kMaxK) return fail(h, LGPU_ERR_UNSUPPORTED, "debug_transform: k outside [2, 128]");
  if (nunits == 0) return LGPU_OK;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const size_t nf = packed_size(k), nt = (size_t)k * k;
  float *dG = nullptr, *dT = nullptr;
  int *dn = nullptr;
  CK(cudaMalloc(&dG, 4 * nf * nunits), "alloc");
  cudaError_t e = cudaMalloc(&dT, 4 * nt * nunits);
  if (e == cudaSuccess) e = cudaMalloc(&dn, 4 * ((size_t)nunits + 1));
  if (e == cudaSuccess) e = cudaMemcpyAsync(dG, gram, 4 * nf * nunits, cudaMemcpyHostToDevice, h->st);
  std::vector<int> ones(nunits + 1, 1);
  ones[nunits] = 0;   // status word
  if (e == cudaSuccess) e = cudaMemcpyAsync(dn, ones.data(), 4 * ((size_t)nunits + 1), cudaMemcpyHostToDevice, h->st);
  int nfp64 = 0;
  if (e == cudaSuccess) e = launch_eig_debug(h->st, nunits, k, dG, dn, dT, dn + nunits, h->prec, h->gap_thresh, &nfp64);
  h->tim.precision = h->prec;
  h->tim.fp64_units = nfp64;
  int status = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(trans, dT, 4 * nt * nunits, cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, dn + nunits, 4, cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(dG);
  cudaFree(dT);
  cudaFree(dn);
  if (e != cudaSuccess) return cuda_fail(h, e, "debug_transform");
  if (status & 1) return fail(h, LGPU_ERR_EIG, "eigensolver did not converge for at least one unit");
  if (status & 2) return fail(h, LGPU_ERR_EIG, "non-positive eigenvalue in at least one unit");
  if (status & 32) return fail(h, LGPU_ERR_CUDA, "internal: malformed eigensolver rotation log");
  return LGPU_OK;
}

// Page-locked host memory: an anonymous mapping (2 MiB aligned, transparent
// huge pages requested), touched and registered with CUDA.  Measured on the
// GB300 host: such buffers keep the full host link rate (about 210 GB/s to
// the device, 190 GB/s back) in a process that starts after other processes
// have used and released most of the host memory, where buffers from
// cudaMallocHost fell to 25-100 GB/s.  cudaMallocHost is the fallback.
namespace {
std::mutex g_host_mu;
std::unordered_map<void *, std::pair<void *, size_t>> g_host_maps;   // user pointer -> (mapping, length)
}  // namespace

int lgpu_host_alloc(size_t bytes, void **ptr) {
  if (!ptr) return LGPU_ERR_ARG;
  *ptr = nullptr;
  const size_t al = (size_t)2 << 20;
  const size_t n = (std::max<size_t>(bytes, 16) + al - 1) / al * al;
  void *raw = mmap(nullptr, n + al, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (raw != MAP_FAILED) {
    void *p = reinterpret_cast<void *>((reinterpret_cast<uintptr_t>(raw) + al - 1) & ~(uintptr_t)(al - 1));
    madvise(p, n, MADV_HUGEPAGE);   // advisory; ignored where unsupported
    std::memset(p, 0, n);
    if (cudaHostRegister(p, n, cudaHostRegisterDefault) == cudaSuccess) {
      std::lock_guard<std::mutex> lock(g_host_mu);
      g_host_maps[p] = std::make_pair(raw, n + al);
      *ptr = p;
      return LGPU_OK;
    }
    cudaGetLastError();
    munmap(raw, n + al);
  }
  cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 16);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? LGPU_ERR_NOMEM : LGPU_ERR_CUDA;
  return LGPU_OK;
}

int lgpu_host_free(void *ptr) {
  if (!ptr) return LGPU_OK;
  std::pair<void *, size_t> m(nullptr, 0);
  {
    std::lock_guard<std::mutex> lock(g_host_mu);
    auto it = g_host_maps.find(ptr);
    if (it != g_host_maps.end()) {
      m = it->second;
      g_host_maps.erase(it);
    }
  }
  if (m.first) {
    const cudaError_t e = cudaHostUnregister(ptr);
    munmap(m.first, m.second);
    return e == cudaSuccess ? LGPU_OK : LGPU_ERR_CUDA;
  }
  if (cudaFreeHost(ptr) != cudaSuccess) return LGPU_ERR_CUDA;
  return LGPU_OK;
}

int lgpu_flush_l2(lgpu_handle *h, size_t bytes) {
  if (!h) return LGPU_ERR_ARG;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(h->buf[B_FLUSH].ensure(bytes), "alloc flush buffer");
  static int salt = 0;
  CK(cudaMemsetAsync(h->buf[B_FLUSH].p, (++salt) & 0xff, bytes, h->st), "flush");
  CK(cudaStreamSynchronize(h->st), "flush sync");
  return LGPU_OK;
}

int lgpu_debug_metric(lgpu_handle *h, int n, const float *lat1, const float *lon1, const float *lat2,
                      const float *lon2, float *dist) {
  if (!h || n < 0 || (n > 0 && (!lat1 || !lon1 || !lat2 || !lon2 || !dist))) return LGPU_ERR_ARG;
  if (n == 0) return LGPU_OK;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  float *d = nullptr;
  CK(cudaMalloc(&d, 5 * sizeof(float) * (size_t)n), "alloc");
  const float *srcs[4] = {lat1, lon1, lat2, lon2};
  for (int q = 0; q < 4; q++)
    cudaMemcpyAsync(d + (size_t)q * n, srcs[q], 4 * (size_t)n, cudaMemcpyHostToDevice, h->st);
  cudaError_t e = launch_debug_metric(h->st, n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, d + 4 * (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dist, d + 4 * (size_t)n, 4 * (size_t)n, cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(h, e, "debug_metric");
  return LGPU_OK;
}

int lgpu_debug_weight(lgpu_handle *h, int n, const float *lat1, const float *lon1, const float *lat2,
                      const float *lon2, const float *L, float *out) {
  if (!h || n < 0 || (n > 0 && (!lat1 || !lon1 || !lat2 || !lon2 || !L || !out))) return LGPU_ERR_ARG;
  if (n == 0) return LGPU_OK;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  float *d = nullptr;
  CK(cudaMalloc(&d, 10 * sizeof(float) * (size_t)n), "alloc");
  const float *src[5] = {lat1, lon1, lat2, lon2, L};
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 5 && e == cudaSuccess; q++)
    e = cudaMemcpyAsync(d + q * (size_t)n, src[q], 4 * (size_t)n, cudaMemcpyHostToDevice, h->st);
  if (e == cudaSuccess) e = launch_debug_weight(h->st, n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n,
                                                d + 4 * (size_t)n, d + 5 * (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + 5 * (size_t)n, 20 * (size_t)n, cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(h, e, "debug_weight");
  return LGPU_OK;
}

int lgpu_debug_gc(lgpu_handle *h, int n, const float *z, const float *L, float *gc) {
  if (!h || n < 0 || (n > 0 && (!z || !L || !gc))) return LGPU_ERR_ARG;
  if (n == 0) return LGPU_OK;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  float *d = nullptr;
  CK(cudaMalloc(&d, 4 * sizeof(float) * (size_t)n), "alloc");
  cudaMemcpyAsync(d, z, 4 * (size_t)n, cudaMemcpyHostToDevice, h->st);
  cudaMemcpyAsync(d + n, L, 4 * (size_t)n, cudaMemcpyHostToDevice, h->st);
  cudaError_t e = launch_debug_gc(h->st, n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n);
  // gc receives 2n values: the fast evaluation then the exact REAL(8) one
  if (e == cudaSuccess) e = cudaMemcpyAsync(gc, d + 2 * (size_t)n, 8 * (size_t)n, cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(h, e, "debug_gc");
  return LGPU_OK;
}

}  // extern "C"

// ===========================================================================
// Learned form (no counterpart in the reference, which solves every column:
// src/letkf_solver.F90:203-384)

struct LearnState {
  lgpu_learn_config cfg{};
  MlpShape shape{};
  size_t nparam = 0;
  std::vector<int> coarse, fine_ok, fine_miss;   // active columns by role
  std::vector<int> rank;                         // [ncol] row of a coarse column in the exact set, or -1
  DevBuf d_fine, d_rank, d_cact, d_mark;
  DevBuf P, Pq, Pm, Pv, Pg, Wt;                  // masters, BF16-rounded copy, Adam moments, gradient, tiled weights
  DevBuf mu_in, sd_in, mu_out, sd_out;
  DevBuf feat, nkf, X, Xt, H1, H2, Yn, flag, gate, gate_n, jacc;
  DevBuf ecols, Gsub, nksub, Tsub, wsub;         // exact subsets
  DevBuf store_X, store_Y, wbar_all;
  DevBuf bidx, Xb, Yb, scr, lacc;
  DevBuf wout;                                   // per-output loss weights: 1 for W, k for w-bar
  DevBuf cells;                                  // per-cell observation aggregates (two float4 per cell)
  long long nstore = 0;
  long long hold0 = 0;     // first row of the last collected analysis (held out from training when ncollect >= 2)
  int ncollect = 0;
  bool stats_ok = false, trained = false;
  unsigned long long runs = 0;
  int adam_step = 0;
  float tau = 3.0e38f;
  int use_net = 1;
  lgpu_learn_stats st{};
  cudaEvent_t ev[6] = {};
};

static void learn_free(lgpu_handle *h) {
  if (!h->learn) return;
  LearnState *L = h->learn;
  DevBuf *all[] = {&L->d_fine, &L->d_rank, &L->d_cact, &L->d_mark, &L->P, &L->Pq, &L->Pm, &L->Pv, &L->Pg, &L->Wt,
                   &L->mu_in, &L->sd_in, &L->mu_out, &L->sd_out, &L->feat, &L->nkf, &L->X, &L->Xt, &L->H1, &L->H2,
                   &L->Yn, &L->flag, &L->gate, &L->gate_n, &L->jacc, &L->ecols, &L->Gsub, &L->nksub, &L->Tsub,
                   &L->wsub, &L->store_X, &L->store_Y, &L->wbar_all, &L->bidx, &L->Xb, &L->Yb, &L->scr, &L->lacc,
                   &L->wout, &L->cells};
  for (DevBuf *b : all) b->release();
  for (auto &e : L->ev) if (e) cudaEventDestroy(e);
  delete L;
  h->learn = nullptr;
}

namespace {

unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

double unif01(unsigned long long &s) {
  s = mix64(s);
  return (double)(s >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

int lgpu_learn_init(lgpu_handle *h, const lgpu_learn_config *cfg) {
  if (!h || !cfg) return LGPU_ERR_ARG;
  if (!h->grid_ok || !h->loc_ok || !h->state_ok)
    return fail(h, LGPU_ERR_ORDER, "learn_init before grid, localizer and state were set");
  if (h->loc.cls != LOC_NOVRT || h->loc.groups != 1)
    return fail(h, LGPU_ERR_UNSUPPORTED, "the learned form supports loc_novrt (one group per column) only");
  if (cfg->nx <= 0 || cfg->ny <= 0 || (long long)cfg->nx * cfg->ny != h->ncol)
    return fail(h, LGPU_ERR_ARG, "learn_init: nx * ny must equal the number of grid columns");
  if (cfg->stride < 2 || cfg->nx % cfg->stride != 0)
    return fail(h, LGPU_ERR_ARG, "learn_init: stride must be >= 2 and divide nx");
  if (cfg->hidden < 16 || cfg->hidden % 16 != 0 || cfg->hidden > 2048)
    return fail(h, LGPU_ERR_ARG, "learn_init: hidden must be a multiple of 16 in [16, 2048]");
  if (!(cfg->judge_frac >= 0.0f && cfg->judge_frac <= 1.0f) || !(cfg->gate_frac >= 0.0f && cfg->gate_frac <= 1.0f) ||
      !(cfg->sample_frac > 0.0f && cfg->sample_frac <= 1.0f) || cfg->train_cap <= 0)
    return fail(h, LGPU_ERR_ARG, "learn_init: fractions must lie in [0, 1] and train_cap be positive");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  learn_free(h);
  LearnState *L = new LearnState();
  h->learn = L;
  L->cfg = *cfg;
  const int k = h->k, nx = cfg->nx, ny = cfg->ny, s = cfg->stride;
  L->shape.din = k * k + k + 16;
  L->shape.k1 = (L->shape.din + 15) & ~15;
  L->shape.H = cfg->hidden;
  L->shape.dout = k * k + k;
  L->nparam = mlp_param_count(L->shape);
  // roles of the active columns
  L->rank.assign(h->ncol, -1);
  for (int c = 0; c < h->ncol; c++) {
    if (h->h_col2act[c] < 0) continue;
    const int i = c % nx, j = c / nx;
    if (i % s == 0 && j % s == 0) {
      L->rank[c] = (int)L->coarse.size();
      L->coarse.push_back(c);
    }
  }
  for (int c = 0; c < h->ncol; c++) {
    if (h->h_col2act[c] < 0 || L->rank[c] >= 0) continue;
    const int i = c % nx, j = c / nx;
    const int i0 = (i / s) * s, j0 = (j / s) * s, i1 = (i0 + s) % nx, j1 = j0 + s < ny ? j0 + s : j0;
    const double fx = (double)(i - i0) / s, fy = j1 != j0 ? (double)(j - j0) / s : 0.0;
    const int nb[4] = {i0 + nx * j0, i1 + nx * j0, i0 + nx * j1, i1 + nx * j1};
    const double w[4] = {(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy};
    bool ok = true;
    for (int q = 0; q < 4; q++)
      if (w[q] > 0.0 && L->rank[nb[q]] < 0) ok = false;
    (ok ? L->fine_ok : L->fine_miss).push_back(c);
  }
  const int nf = std::max<int>(1, (int)L->fine_ok.size());
  const int nexact = std::max<int>(1, h->nact);
  std::vector<int> cact(h->ncol, -1);
  for (int c : L->coarse) cact[c] = h->h_col2act[c];
  const MlpShape &S = L->shape;
  const size_t rows_pad = ((size_t)nf + 127) / 128 * 128;
  const size_t cap = (size_t)cfg->train_cap;
  struct { DevBuf *b; size_t bytes; } al[] = {
      {&L->d_fine, 4 * (size_t)nf}, {&L->d_rank, 4 * (size_t)h->ncol}, {&L->d_cact, 4 * (size_t)h->ncol},
      {&L->d_mark, 4 * (size_t)h->ncol},
      {&L->P, 4 * L->nparam}, {&L->Pq, 4 * L->nparam}, {&L->Pm, 4 * L->nparam}, {&L->Pv, 4 * L->nparam},
      {&L->Pg, 4 * L->nparam}, {&L->Wt, mlp_tiled_weight_bytes(S)},
      {&L->mu_in, 4 * (size_t)S.din}, {&L->sd_in, 4 * (size_t)S.din}, {&L->mu_out, 4 * (size_t)S.dout},
      {&L->sd_out, 4 * (size_t)S.dout},
      {&L->feat, 64 * (size_t)nf}, {&L->nkf, 4 * (size_t)nf}, {&L->X, 4 * (size_t)nf * S.din},
      {&L->Xt, rows_pad * (size_t)S.k1 * 2}, {&L->H1, mlp_act_bytes(S, nf)}, {&L->H2, mlp_act_bytes(S, nf)},
      {&L->Yn, 4 * (size_t)nf * S.dout}, {&L->flag, 4 * (size_t)nf}, {&L->gate, 4 * (size_t)nf}, {&L->gate_n, 16},
      {&L->jacc, 16},
      {&L->ecols, 4 * (size_t)nexact}, {&L->Gsub, 4 * (size_t)nexact * packed_size(k)},
      {&L->nksub, 4 * (size_t)nexact}, {&L->Tsub, 4 * (size_t)nexact * k * k}, {&L->wsub, 4 * (size_t)nexact * k},
      {&L->store_X, 4 * cap * S.din}, {&L->store_Y, 4 * cap * S.dout}, {&L->wbar_all, 4 * (size_t)nexact * k},
      {&L->lacc, 16}, {&L->wout, 4 * (size_t)S.dout}};
  for (auto &a : al) CK(a.b->ensure(a.bytes), "alloc learned form");
  {
    // the analysis mean depends on w-bar alone (W 1 = 1): its k outputs
    // weigh as much in the loss as the k*k outputs of W
    std::vector<float> w(S.dout, 1.0f);
    for (int i = 0; i < k; i++) w[(size_t)k * k + i] = (float)k;
    CK(cudaMemcpy(L->wout.p, w.data(), 4 * w.size(), cudaMemcpyHostToDevice), "H2D loss weights");
  }
  for (auto &e : L->ev) CK(cudaEventCreate(&e), "event");
  CK(cudaMemcpyAsync(L->d_fine.p, L->fine_ok.data(), 4 * L->fine_ok.size(), cudaMemcpyHostToDevice, h->st), "H2D");
  CK(cudaMemcpyAsync(L->d_rank.p, L->rank.data(), 4 * (size_t)h->ncol, cudaMemcpyHostToDevice, h->st), "H2D");
  CK(cudaMemcpyAsync(L->d_cact.p, cact.data(), 4 * (size_t)h->ncol, cudaMemcpyHostToDevice, h->st), "H2D");
  CK(cudaMemsetAsync(L->d_mark.p, 0, 4 * (size_t)h->ncol, h->st), "memset");
  // parameters: uniform(-a, a), a = sqrt(6 / (fan_in + fan_out)) (Glorot);
  // the last layer scaled by 0.1 so the first corrections are small; zero biases
  std::vector<float> p(L->nparam, 0.0f);
  size_t off[6];
  mlp_param_offsets(S, off);
  unsigned long long rs = cfg->seed * 0x2545F4914F6CDD1Dull + 7;
  auto fill = [&](size_t o, int nout, int nin, double scale) {
    const double a = scale * std::sqrt(6.0 / (nin + nout));
    for (size_t q = 0; q < (size_t)nout * nin; q++) p[o + q] = (float)((2.0 * unif01(rs) - 1.0) * a);
  };
  fill(off[0], S.H, S.din, 1.0);
  fill(off[2], S.H, S.H, 1.0);
  fill(off[4], S.dout, S.H, 0.1);
  CK(cudaMemcpyAsync(L->P.p, p.data(), 4 * L->nparam, cudaMemcpyHostToDevice, h->st), "H2D params");
  CK(mlp_round(h->st, (long long)L->nparam, L->P.as<float>(), L->Pq.as<float>()), "round params");
  CK(cudaMemsetAsync(L->Pm.p, 0, 4 * L->nparam, h->st), "memset");
  CK(cudaMemsetAsync(L->Pv.p, 0, 4 * L->nparam, h->st), "memset");
  CK(mlp_tile_weights(h->st, S, L->Pq.as<float>(), L->Wt.as<unsigned char>()), "tile weights");
  CK(cudaStreamSynchronize(h->st), "learn_init");
  L->st.coarse = (int)L->coarse.size();
  L->st.fallback = (int)L->fine_miss.size();
  L->st.tau = L->tau;
  return LGPU_OK;
}

int lgpu_learn_set_network(lgpu_handle *h, int use_network) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->learn) return fail(h, LGPU_ERR_ORDER, "learn_set_network before learn_init");
  h->learn->use_net = use_network ? 1 : 0;
  return LGPU_OK;
}

long long lgpu_learn_param_count(lgpu_handle *h) { return (h && h->learn) ? (long long)h->learn->nparam : -1; }

int lgpu_learn_get_params(lgpu_handle *h, float *params, long long n) {
  if (!h || !params) return LGPU_ERR_ARG;
  if (!h->learn) return fail(h, LGPU_ERR_ORDER, "learn_get_params before learn_init");
  if (n != (long long)h->learn->nparam) return fail(h, LGPU_ERR_ARG, "learn_get_params: wrong parameter count");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(params, h->learn->P.p, 4 * (size_t)n, cudaMemcpyDeviceToHost, h->st), "D2H params");
  CK(cudaStreamSynchronize(h->st), "get params");
  return LGPU_OK;
}

int lgpu_learn_set_params(lgpu_handle *h, const float *params, long long n) {
  if (!h || !params) return LGPU_ERR_ARG;
  if (!h->learn) return fail(h, LGPU_ERR_ORDER, "learn_set_params before learn_init");
  LearnState *L = h->learn;
  if (n != (long long)L->nparam) return fail(h, LGPU_ERR_ARG, "learn_set_params: wrong parameter count");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(L->P.p, params, 4 * (size_t)n, cudaMemcpyHostToDevice, h->st), "H2D params");
  CK(mlp_round(h->st, n, L->P.as<float>(), L->Pq.as<float>()), "round params");
  CK(mlp_tile_weights(h->st, L->shape, L->Pq.as<float>(), L->Wt.as<unsigned char>()), "tile weights");
  CK(cudaStreamSynchronize(h->st), "set params");
  return LGPU_OK;
}

int lgpu_learn_stats_get(lgpu_handle *h, lgpu_learn_stats *out) {
  if (!h || !out) return LGPU_ERR_ARG;
  if (!h->learn) return fail(h, LGPU_ERR_ORDER, "learn_stats before learn_init");
  *out = h->learn->st;
  out->tau = h->learn->tau;
  out->train_rows = h->learn->nstore;
  return LGPU_OK;
}

int lgpu_learn_collect(lgpu_handle *h, long long *rows) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->learn) return fail(h, LGPU_ERR_ORDER, "learn_collect before learn_init");
  LearnState *L = h->learn;
  if (h->bound_state) return fail(h, LGPU_ERR_UNSUPPORTED, "learn_collect with a bound state");
  const int k = h->k;
  const MlpShape &S = L->shape;
  // the exact analysis, with the mean weights of every unit
  const int variant = h->variant;
  if (variant == LGPU_VARIANT_LEARNED) h->variant = LGPU_VARIANT_AUTO;
  CK(h->learn->wbar_all.ensure(4 * (size_t)std::max(1, h->nact) * k), "alloc");
  h->learn_wbar = L->wbar_all.as<float>();
  int rc = lgpu_solver_run(h);
  h->learn_wbar = nullptr;
  h->variant = variant;
  if (rc != LGPU_OK) return rc;
  // a sample of the columns with four coarse neighbours
  std::vector<int> sample;
  const double frac = L->cfg.sample_frac;
  unsigned long long rs = mix64(L->cfg.seed ^ (0x51ull + L->runs++));
  for (int c : L->fine_ok)
    if (unif01(rs) < frac) sample.push_back(c);
  const long long room = (long long)L->cfg.train_cap - L->nstore;
  if ((long long)sample.size() > room) sample.resize((size_t)std::max(0LL, room));
  const int n = (int)sample.size();
  if (n > 0) {
    cudaStream_t st = h->st;
    int launches = 0;
    CK(L->ecols.ensure(4 * (size_t)std::max(n, std::max(1, h->nact))), "alloc");
    CK(cudaMemcpyAsync(L->ecols.p, sample.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, st), "H2D sample");
    CK(L->feat.ensure(64 * (size_t)n), "alloc");
    CK(L->nkf.ensure(4 * (size_t)n), "alloc");
    CK(L->flag.ensure(4 * (size_t)n), "alloc");
    ObsSorted os;
    os.A = h->buf[B_SA].as<float4>();
    os.B = h->buf[B_SB].as<float4>();
    os.hx = h->buf[B_SHX].as<float>();
    os.idx = h->buf[B_SIDX].as<int>();
    os.cell_start = h->buf[B_CSTART].as<int>();
    CK(L->cells.ensure(32 * ((size_t)h->ncell + 1)), "alloc");
    float4 *c0 = L->cells.as<float4>(), *c1 = c0 + h->ncell;
    CK(lrn_cellstats(st, h->ncell, os, c0, c1, &launches), "cell aggregates");
    CK(lrn_obsfeat(st, n, L->ecols.as<int>(), h->buf[B_CP].as<ColPar>(), h->loc, os.cell_start, c0, c1,
                   h->buf[B_GEOM].as<IndexGeom>(), L->feat.as<float>(), L->nkf.as<int>(), &launches),
       "learned features");
    LrnInterpArgs ia;
    ia.nfine = n;
    ia.cols = L->ecols.as<int>();
    ia.nx = L->cfg.nx;
    ia.ny = L->cfg.ny;
    ia.s = L->cfg.stride;
    ia.k = k;
    ia.din = S.din;
    ia.dout = S.dout;
    ia.Ts = h->buf[B_T].as<float>();
    ia.ws = L->wbar_all.as<float>();
    ia.src_of_col = L->d_cact.as<int>();   // coarse column -> its unit
    ia.feat = L->feat.as<float>();
    ia.lat = h->buf[B_LAT].as<float>();
    ia.mu = nullptr;
    ia.sd = nullptr;
    ia.X = L->store_X.as<float>() + (size_t)L->nstore * S.din;
    ia.ldx = S.din;
    ia.flag = L->flag.as<int>();
    ia.Tex = h->buf[B_T].as<float>();
    ia.wex = L->wbar_all.as<float>();
    ia.col2act = h->buf[B_COL2ACT].as<int>();
    ia.Yt = L->store_Y.as<float>() + (size_t)L->nstore * S.dout;
    ia.ldy = S.dout;
    CK(lrn_interp(st, ia, &launches), "learned interpolation");
    CK(cudaStreamSynchronize(st), "collect");
    L->hold0 = L->nstore;
    L->ncollect++;
    L->nstore += n;
  }
  if (rows) *rows = L->nstore;
  return LGPU_OK;
}

namespace lgpu {
cudaError_t mlp_loss_accumulate(cudaStream_t st, const float *parts, int n, float *acc);
}

int lgpu_learn_train(lgpu_handle *h, int epochs, int batch, float lr, float *loss) {
  if (!h) return LGPU_ERR_ARG;
  if (!h->learn) return fail(h, LGPU_ERR_ORDER, "learn_train before learn_init");
  LearnState *L = h->learn;
  if (L->nstore <= 0) return fail(h, LGPU_ERR_ORDER, "learn_train before learn_collect stored rows");
  if (epochs < 0 || batch <= 0 || !(lr > 0.0f)) return fail(h, LGPU_ERR_ARG, "learn_train: epochs >= 0, batch > 0, lr > 0");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = h->st;
  const MlpShape &S = L->shape;
  // the rows of the last collected analysis are held out (for the gate's
  // calibration) once two or more analyses were collected
  const bool holdout = L->ncollect >= 2 && L->hold0 > 0 && L->hold0 < L->nstore;
  const long long n = holdout ? L->hold0 : L->nstore;
  const long long cal0 = holdout ? L->hold0 : 0, cal1 = L->nstore;
  batch = (int)std::min<long long>(batch, n);
  if (!L->stats_ok) {
    CK(lrn_colstats(st, L->store_X.as<float>(), n, S.din, S.din, L->mu_in.as<float>(), L->sd_in.as<float>()),
       "input statistics");
    CK(lrn_colstats(st, L->store_Y.as<float>(), n, S.dout, S.dout, L->mu_out.as<float>(), L->sd_out.as<float>()),
       "output statistics");
    L->stats_ok = true;
  }
  CK(L->bidx.ensure(4 * (size_t)n), "alloc");
  CK(L->Xb.ensure(4 * (size_t)batch * S.din), "alloc");
  CK(L->Yb.ensure(4 * (size_t)batch * S.dout), "alloc");
  CK(L->scr.ensure(4 * mlp_train_scratch_floats(S, batch)), "alloc");
  std::vector<int> perm((size_t)n);
  unsigned long long rs = mix64(L->cfg.seed ^ 0xA5A5ull ^ (unsigned long long)L->adam_step);
  float last = 0.0f;
  for (int ep = 0; ep < epochs; ep++) {
    for (long long i = 0; i < n; i++) perm[(size_t)i] = (int)i;
    for (long long i = n - 1; i > 0; i--) {
      const long long j = (long long)(unif01(rs) * (double)(i + 1));
      std::swap(perm[(size_t)i], perm[(size_t)std::min(j, i)]);
    }
    CK(cudaMemcpyAsync(L->bidx.p, perm.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, st), "H2D batch order");
    CK(cudaMemsetAsync(L->lacc.p, 0, 16, st), "memset");
    int steps = 0;
    for (long long b0 = 0; b0 + batch <= n; b0 += batch) {
      CK(lrn_batch(st, batch, L->bidx.as<int>() + b0, L->store_X.as<float>(), S.din, S.din, L->store_Y.as<float>(),
                   S.dout, S.dout, L->mu_in.as<float>(), L->sd_in.as<float>(), L->mu_out.as<float>(),
                   L->sd_out.as<float>(), L->Xb.as<float>(), L->Yb.as<float>()),
         "training batch");
      int np = 0;
      CK(mlp_grad(st, S, L->Pq.as<float>(), L->Xb.as<float>(), L->Yb.as<float>(), batch, L->Pg.as<float>(),
                  L->scr.as<float>(), &np, L->wout.as<float>()),
         "network gradient");
      CK(mlp_loss_accumulate(st, mlp_loss_parts(S, L->scr.as<float>(), batch), np, L->lacc.as<float>()), "loss");
      L->adam_step++;
      CK(mlp_adam(st, (long long)L->nparam, L->P.as<float>(), L->Pq.as<float>(), L->Pg.as<float>(), L->Pm.as<float>(),
                  L->Pv.as<float>(), lr, L->adam_step),
         "adam");
      steps++;
    }
    float acc = 0.0f;
    CK(cudaMemcpyAsync(&acc, L->lacc.p, 4, cudaMemcpyDeviceToHost, st), "D2H loss");
    CK(cudaStreamSynchronize(st), "train epoch");
    last = steps > 0 ? acc / ((float)steps * (float)batch * (float)S.dout) : 0.0f;
  }
  if (loss) *loss = last;
  CK(mlp_tile_weights(st, S, L->Pq.as<float>(), L->Wt.as<unsigned char>()), "tile weights");
  // gate threshold: the (1 - gate_frac) quantile of the RMS network output
  // over (up to) 16,384 held-out rows (training rows when none are held
  // out), through the tensor-core forward
  const int ncal = (int)std::min<long long>(cal1 - cal0, 16384);
  {
    std::vector<int> idx(ncal);
    for (int i = 0; i < ncal; i++) idx[i] = (int)(cal0 + (long long)i * (cal1 - cal0) / ncal);
    CK(L->bidx.ensure(4 * (size_t)std::max<long long>(n, ncal)), "alloc");
    CK(cudaMemcpyAsync(L->bidx.p, idx.data(), 4 * (size_t)ncal, cudaMemcpyHostToDevice, st), "H2D");
    CK(L->X.ensure(4 * (size_t)ncal * S.din), "alloc");
    CK(L->Yn.ensure(4 * (size_t)ncal * S.dout), "alloc");
    CK(L->Xt.ensure(((size_t)ncal + 127) / 128 * 128 * (size_t)S.k1 * 2), "alloc");
    CK(L->H1.ensure(mlp_act_bytes(S, ncal)), "alloc");
    CK(L->H2.ensure(mlp_act_bytes(S, ncal)), "alloc");
    float *Ycal = L->Yn.as<float>();
    CK(L->Yb.ensure(4 * (size_t)std::max(ncal, batch) * S.dout), "alloc");
    CK(lrn_batch(st, ncal, L->bidx.as<int>(), L->store_X.as<float>(), S.din, S.din, L->store_Y.as<float>(), S.dout,
                 S.dout, L->mu_in.as<float>(), L->sd_in.as<float>(), L->mu_out.as<float>(), L->sd_out.as<float>(),
                 L->X.as<float>(), L->Yb.as<float>()),
       "calibration rows");
    CK(mlp_tile_input(st, S, L->X.as<float>(), ncal, S.din, L->Xt.as<unsigned char>()), "tile input");
    int launches = 0;
    CK(cudaMemsetAsync(h->buf[B_STATUS].p, 0, 16, st), "memset");
    CK(mlp_forward_tc(st, S, L->Wt.as<unsigned char>(), L->Pq.as<float>(), L->Xt.as<unsigned char>(), ncal,
                      L->H1.as<unsigned char>(), L->H2.as<unsigned char>(), Ycal, S.dout, h->buf[B_STATUS].as<int>(),
                      &launches),
       "network forward");
    std::vector<float> y((size_t)ncal * S.dout);
    CK(cudaMemcpyAsync(y.data(), Ycal, 4 * y.size(), cudaMemcpyDeviceToHost, st), "D2H");
    int stat = 0;
    CK(cudaMemcpyAsync(&stat, h->buf[B_STATUS].p, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "calibration");
    if (stat & 16) return fail(h, LGPU_ERR_CUDA, "network forward: tensor-core pipeline wait timed out");
    std::vector<float> sc(ncal);
    for (int r = 0; r < ncal; r++) {
      double q = 0.0;
      for (int e = 0; e < S.dout; e++) q += (double)y[(size_t)r * S.dout + e] * y[(size_t)r * S.dout + e];
      sc[r] = (float)std::sqrt(q / S.dout);
    }
    std::sort(sc.begin(), sc.end());
    const double qf = 1.0 - (double)L->cfg.gate_frac;
    L->tau = L->cfg.gate_frac <= 0.0f ? 3.0e38f : sc[(size_t)std::min<double>(ncal - 1, std::floor(qf * (ncal - 1)))];
  }
  L->trained = true;
  L->st.tau = L->tau;
  return LGPU_OK;
}

// exact solves (PLAIN Gram + split eigensolve) of a column list into the
// compact arrays of the learned state (rows 0..n)
static int learned_exact(lgpu_handle *h, const ObsSorted &os, int n, int &launches) {
  LearnState *L = h->learn;
  if (n <= 0) return LGPU_OK;
  cudaStream_t st = h->st;
  const int k = h->k;
  GramArgs ga;
  ga.nunits = n;
  ga.groups = 1;
  ga.k = k;
  ga.kp = h->kp;
  ga.active = L->ecols.as<int>();
  ga.cp = h->buf[B_CP].as<ColPar>();
  ga.loc = h->loc;
  ga.obs = os;
  ga.geom = h->buf[B_GEOM].as<IndexGeom>();
  ga.G = L->Gsub.as<float>();
  ga.nkept = L->nksub.as<int>();
  ga.diag_obscount = h->buf[B_DOBSC].as<float>();
  ga.diag_lg_obscount = h->buf[B_DLGC].as<float>();
  ga.diag_lg_obsloc = h->buf[B_DLGL].as<float>();
  ga.ncol = h->ncol;
  CK(launch_gram(st, ga, &launches), "gram kernel");
  EigArgs ea;
  ea.nunits = n;
  ea.k = k;
  ea.infl = 1.0f;
  ea.G = L->Gsub.as<float>();
  ea.nkept = L->nksub.as<int>();
  ea.T = L->Tsub.as<float>();
  ea.wbar = L->wsub.as<float>();
  ea.ulist = nullptr;
  ea.status = h->buf[B_STATUS].as<int>();
  flag_args(h, ea);
  if (h->prec == LGPU_PREC_FP64) {
    CK(launch_eig64(st, ea, 0, &launches), "FP64 eigen kernel");
    return LGPU_OK;
  }
  EigSplit sp;
  int batch = 0;
  int rc = eig_scratch(h, n, sp, batch);
  if (rc != LGPU_OK) return rc;
  if (batch == 0) {
    CK(launch_eig(st, ea, &launches), "eigen kernel");
  } else {
    CK(launch_eig_split(st, ea, sp, batch, 0, n, &launches), "eigen kernels");
    if (ea.flag_list) CK(launch_eig64_flagged(st, ea, &launches), "FP64 re-solve");
  }
  return LGPU_OK;
}

static int learned_run(lgpu_handle *h) {
  LearnState *L = h->learn;
  if (!L) return fail(h, LGPU_ERR_ORDER, "LEARNED variant before learn_init");
  if (!L->trained) return fail(h, LGPU_ERR_ORDER, "LEARNED variant before learn_train");
  if (h->bound_state) return fail(h, LGPU_ERR_UNSUPPORTED, "the LEARNED variant with a bound state");
  ObsSorted os;
  int launches = 0;
  int rc = prepare_run(h, os, launches);
  if (rc != LGPU_OK) return rc;
  if ((rc = flag_prepare(h)) != LGPU_OK) return rc;
  cudaStream_t st = h->st;
  const int k = h->k;
  const MlpShape &S = L->shape;
  // exact set: coarse lattice, judge sample, columns without four coarse neighbours
  std::vector<int> ex(L->coarse);
  const int ncoarse = (int)ex.size();
  unsigned long long rs = mix64(L->cfg.seed ^ (0x1234567ull + L->runs++));
  std::vector<int> judge;
  for (int c : L->fine_ok)
    if (unif01(rs) < (double)L->cfg.judge_frac) judge.push_back(c);
  ex.insert(ex.end(), judge.begin(), judge.end());
  ex.insert(ex.end(), L->fine_miss.begin(), L->fine_miss.end());
  const int nex = (int)ex.size(), nj = (int)judge.size();
  const int nf = (int)L->fine_ok.size();
  CK(L->ecols.ensure(4 * (size_t)std::max(1, h->nact)), "alloc");
  CK(cudaMemcpyAsync(L->ecols.p, ex.data(), 4 * (size_t)nex, cudaMemcpyHostToDevice, st), "H2D exact set");
  CK(cudaEventRecord(L->ev[0], st), "event");
  if ((rc = learned_exact(h, os, nex, launches)) != LGPU_OK) return rc;
  CK(cudaEventRecord(L->ev[1], st), "event");
  // network inputs of the columns with four coarse neighbours
  CK(L->cells.ensure(32 * ((size_t)h->ncell + 1)), "alloc");
  float4 *c0 = L->cells.as<float4>(), *c1 = c0 + h->ncell;
  CK(lrn_cellstats(st, h->ncell, os, c0, c1, &launches), "cell aggregates");
  CK(lrn_obsfeat(st, nf, L->d_fine.as<int>(), h->buf[B_CP].as<ColPar>(), h->loc, os.cell_start, c0, c1,
                 h->buf[B_GEOM].as<IndexGeom>(), L->feat.as<float>(), L->nkf.as<int>(), &launches),
     "learned features");
  LrnInterpArgs ia;
  ia.nfine = nf;
  ia.cols = L->d_fine.as<int>();
  ia.nx = L->cfg.nx;
  ia.ny = L->cfg.ny;
  ia.s = L->cfg.stride;
  ia.k = k;
  ia.din = S.din;
  ia.dout = S.dout;
  ia.Ts = L->Tsub.as<float>();
  ia.ws = L->wsub.as<float>();
  ia.src_of_col = L->d_rank.as<int>();   // coarse rows come first in the exact set
  ia.feat = L->feat.as<float>();
  ia.lat = h->buf[B_LAT].as<float>();
  ia.mu = L->mu_in.as<float>();
  ia.sd = L->sd_in.as<float>();
  ia.X = L->X.as<float>();
  ia.ldx = S.din;
  ia.flag = L->flag.as<int>();
  ia.Tex = nullptr;
  ia.wex = nullptr;
  ia.col2act = h->buf[B_COL2ACT].as<int>();
  ia.Yt = nullptr;
  ia.ldy = 0;
  CK(L->X.ensure(4 * (size_t)std::max(1, nf) * S.din), "alloc");
  CK(L->Yn.ensure(4 * (size_t)std::max(1, nf) * S.dout), "alloc");
  CK(L->Xt.ensure(((size_t)std::max(1, nf) + 127) / 128 * 128 * (size_t)S.k1 * 2), "alloc");
  CK(L->H1.ensure(mlp_act_bytes(S, std::max(1, nf))), "alloc");
  CK(L->H2.ensure(mlp_act_bytes(S, std::max(1, nf))), "alloc");
  ia.X = L->X.as<float>();
  CK(lrn_interp(st, ia, &launches), "learned interpolation");
  CK(mlp_tile_input(st, S, L->X.as<float>(), nf, S.din, L->Xt.as<unsigned char>()), "tile input");
  CK(cudaEventRecord(L->ev[2], st), "event");
  CK(mlp_forward_tc(st, S, L->Wt.as<unsigned char>(), L->Pq.as<float>(), L->Xt.as<unsigned char>(), nf,
                    L->H1.as<unsigned char>(), L->H2.as<unsigned char>(), L->Yn.as<float>(), S.dout,
                    h->buf[B_STATUS].as<int>(), &launches),
     "network forward");
  CK(cudaEventRecord(L->ev[3], st), "event");
  CK(cudaMemsetAsync(L->gate_n.p, 0, 16, st), "memset");
  LrnApplyArgs aa;
  aa.nfine = nf;
  aa.cols = L->d_fine.as<int>();
  aa.nx = L->cfg.nx;
  aa.ny = L->cfg.ny;
  aa.s = L->cfg.stride;
  aa.k = k;
  aa.dout = S.dout;
  aa.Ts = L->Tsub.as<float>();
  aa.ws = L->wsub.as<float>();
  aa.src_of_col = L->d_rank.as<int>();
  aa.Yn = L->Yn.as<float>();
  aa.ldy = S.dout;
  aa.mu_out = L->mu_out.as<float>();
  aa.sd_out = L->sd_out.as<float>();
  aa.tau = L->tau;
  aa.net = L->use_net;
  aa.flag = L->flag.as<int>();
  aa.nk_fine = L->nkf.as<int>();
  aa.col2act = h->buf[B_COL2ACT].as<int>();
  aa.T = h->buf[B_T].as<float>();
  aa.nkept = h->buf[B_NKEPT].as<int>();
  aa.gate_cols = L->gate.as<int>();
  aa.gate_n = L->gate_n.as<int>();
  aa.score = nullptr;
  CK(lrn_apply(st, aa, &launches), "learned apply");
  // judge the network on the judged columns it did not send back, then put
  // every exact transform in place
  int ngate = 0;
  CK(cudaMemcpyAsync(&ngate, L->gate_n.p, 4, cudaMemcpyDeviceToHost, st), "D2H gate count");
  CK(cudaStreamSynchronize(st), "gate count");
  CK(lrn_mark(st, ngate, L->gate.as<int>(), L->d_mark.as<int>(), 1), "mark");
  CK(cudaMemsetAsync(L->jacc.p, 0, 16, st), "memset");
  std::vector<int> jsub(nj);
  for (int i = 0; i < nj; i++) jsub[i] = ncoarse + i;
  DevBuf &jb = h->buf[B_LIST_IDX];
  CK(jb.ensure(8 * (size_t)std::max(1, nj)), "alloc");
  CK(cudaMemcpyAsync(jb.p, jsub.data(), 4 * (size_t)nj, cudaMemcpyHostToDevice, st), "H2D");
  CK(lrn_judge(st, nj, L->ecols.as<int>() + ncoarse, jb.as<int>(), L->Tsub.as<float>(), h->buf[B_T].as<float>(),
               h->buf[B_COL2ACT].as<int>(), L->d_mark.as<int>(), k, L->jacc.as<float>(), &launches),
     "judge");
  CK(lrn_mark(st, ngate, L->gate.as<int>(), L->d_mark.as<int>(), 0), "unmark");
  CK(lrn_scatter(st, nex, L->ecols.as<int>(), h->buf[B_COL2ACT].as<int>(), L->Tsub.as<float>(), L->nksub.as<int>(), k,
                 h->buf[B_T].as<float>(), h->buf[B_NKEPT].as<int>(), &launches),
     "exact transforms");
  CK(cudaEventRecord(L->ev[4], st), "event");
  // the gate's columns, solved exactly
  if (ngate > 0) {
    CK(cudaMemcpyAsync(L->ecols.p, L->gate.p, 4 * (size_t)ngate, cudaMemcpyDeviceToDevice, st), "D2D");
    if ((rc = learned_exact(h, os, ngate, launches)) != LGPU_OK) return rc;
    CK(lrn_scatter(st, ngate, L->ecols.as<int>(), h->buf[B_COL2ACT].as<int>(), L->Tsub.as<float>(),
                   L->nksub.as<int>(), k, h->buf[B_T].as<float>(), h->buf[B_NKEPT].as<int>(), &launches),
       "exact transforms");
  }
  CK(cudaEventRecord(L->ev[5], st), "event");
  CK(cudaEventRecord(h->ev[3], st), "event");
  // update of every column
  UpdateArgs ua = update_args(h);
  CK(cudaEventRecord(h->ev_chunk[0][1], st), "event");
  CK(launch_update(st, ua, &launches), "update kernel");
  CK(cudaEventRecord(h->ev_chunk[0][2], st), "event");
  CK(cudaEventRecord(h->ev[5], st), "event");
  int *stat4 = h->pin_scr;
  float *jacc = reinterpret_cast<float *>(h->pin_scr + 8);
  stat4[4] = 0;
  CK(cudaMemcpyAsync(stat4, h->buf[B_STATUS].p, 16, cudaMemcpyDeviceToHost, st), "D2H status");
  if (h->prec == LGPU_PREC_FP32_RESOLVE)
    CK(cudaMemcpyAsync(stat4 + 4, h->buf[B_FLAGLIST].p, 4, cudaMemcpyDeviceToHost, st), "D2H flag count");
  CK(cudaMemcpyAsync(jacc, L->jacc.p, 16, cudaMemcpyDeviceToHost, st), "D2H judge");
  CK(cudaStreamSynchronize(st), "solver_run");
  const int nflag = stat4[4];
  float ms[3];
  for (int i = 0; i < 3; i++) CK(cudaEventElapsedTime(&ms[i], h->ev[i], h->ev[i + 1]), "timing");
  float le[5];
  for (int i = 0; i < 5; i++) CK(cudaEventElapsedTime(&le[i], L->ev[i], L->ev[i + 1]), "timing");
  h->tim.index_ms = ms[0];
  h->tim.prep_ms = ms[1];
  CK(cudaEventElapsedTime(&h->tim.gram_ms, h->ev[2], h->ev[3]), "timing");
  h->tim.tiles_ms = 0.0f;
  h->tim.eig_ms = 0.0f;
  CK(cudaEventElapsedTime(&h->tim.update_ms, h->ev_chunk[0][1], h->ev_chunk[0][2]), "timing");
  CK(cudaEventElapsedTime(&h->tim.total_ms, h->ev[0], h->ev[5]), "timing");
  h->tim.launches = launches;
  h->tim.variant = LGPU_VARIANT_LEARNED;
  h->tim.units = h->nunits;
  h->tim.kept_pairs = -1;
  h->tim.mma_chunks = 0;
  h->tim.mma_n = 0;
  h->tim.precision = h->prec;
  h->tim.fp64_units = h->prec == LGPU_PREC_FP64 ? nex + ngate : std::min(nflag, 2 * std::max(1, h->nunits));
  h->tim.fp64_ms = 0.0f;   // inside exact_ms of the learned statistics
  h->tim.span_ms = h->tim.total_ms;
  L->st.coarse = ncoarse;
  L->st.judged = nj;
  L->st.fallback = (int)L->fine_miss.size();
  L->st.gated = ngate;
  L->st.inferred = nf - ngate;
  L->st.judge_rms = jacc[2] > 0.0f ? std::sqrt(jacc[0] / jacc[2]) / (float)k : 0.0f;
  L->st.judge_ref_rms = jacc[2] > 0.0f ? std::sqrt(jacc[1] / jacc[2]) / (float)k : 0.0f;
  L->st.exact_ms = le[0] + le[4];
  L->st.feature_ms = le[1];
  L->st.network_ms = le[2];
  L->st.apply_ms = le[3];
  h->ran = true;
  const int status = stat4[0];
  if (status & 1) return fail(h, LGPU_ERR_EIG, "eigensolver did not converge for at least one unit");
  if (status & 2) return fail(h, LGPU_ERR_EIG, "non-positive eigenvalue in at least one unit");
  if (status & 4) return fail(h, LGPU_ERR_NONFINITE, "non-finite analysis mean or spread");
  if (status & 16) return fail(h, LGPU_ERR_CUDA, "tensor-core pipeline wait timed out");
  if (status & 32) return fail(h, LGPU_ERR_CUDA, "internal: malformed eigensolver rotation log");
  if (status & 64) return fail(h, LGPU_ERR_CUDA, "update stage copy wait timed out");
  return LGPU_OK;
}

// ---- network verification entry (standalone)
int lgpu_mlp_debug(int device, int din, int hidden, int dout, int rows, const float *params, const float *x,
                   const float *t, float *loss, float *grad, float *y_simt, float *y_tc) {
  if (din <= 0 || hidden <= 0 || hidden % 16 || dout <= 0 || rows <= 0 || !params || !x) return LGPU_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return LGPU_ERR_CUDA;
  MlpShape S;
  S.din = din;
  S.k1 = (din + 15) & ~15;
  S.H = hidden;
  S.dout = dout;
  const size_t np = mlp_param_count(S);
  std::vector<void *> bufs;
  auto take = [&](size_t bytes) -> void * {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  auto release = [&]() { for (void *p : bufs) cudaFree(p); };
  float *P = (float *)take(4 * np), *Pq = (float *)take(4 * np), *G = (float *)take(4 * np);
  float *X = (float *)take(4 * (size_t)rows * din), *Xq = (float *)take(4 * (size_t)rows * din);
  float *T = (float *)take(4 * (size_t)rows * dout), *Y = (float *)take(4 * (size_t)rows * dout);
  float *scr = (float *)take(4 * mlp_train_scratch_floats(S, rows));
  unsigned char *Wt = (unsigned char *)take(mlp_tiled_weight_bytes(S));
  unsigned char *Xt = (unsigned char *)take(((size_t)rows + 127) / 128 * 128 * (size_t)S.k1 * 2);
  unsigned char *H1 = (unsigned char *)take(mlp_act_bytes(S, rows)), *H2 = (unsigned char *)take(mlp_act_bytes(S, rows));
  float *acc = (float *)take(16);
  int *status = (int *)take(16);
  for (void *p : bufs)
    if (!p) { release(); return LGPU_ERR_NOMEM; }
  cudaStream_t st = nullptr;
  cudaError_t e = cudaSuccess;
  int rc = LGPU_OK;
  auto ck = [&](cudaError_t x2) { if (e == cudaSuccess && x2 != cudaSuccess) e = x2; };
  ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  ck(cudaMemcpyAsync(P, params, 4 * np, cudaMemcpyHostToDevice, st));
  ck(cudaMemcpyAsync(X, x, 4 * (size_t)rows * din, cudaMemcpyHostToDevice, st));
  if (t) ck(cudaMemcpyAsync(T, t, 4 * (size_t)rows * dout, cudaMemcpyHostToDevice, st));
  else ck(cudaMemsetAsync(T, 0, 4 * (size_t)rows * dout, st));
  ck(mlp_round(st, (long long)np, P, Pq));
  ck(mlp_round(st, (long long)rows * din, X, Xq));
  ck(cudaMemsetAsync(acc, 0, 16, st));
  ck(cudaMemsetAsync(status, 0, 16, st));
  int nparts = 0;
  ck(mlp_grad(st, S, Pq, Xq, T, rows, G, scr, &nparts, nullptr));
  ck(mlp_loss_accumulate(st, mlp_loss_parts(S, scr, rows), nparts, acc));
  // the forward output of the gradient pass is the CUDA-core forward
  const size_t yoff = (size_t)rows * 4 * S.H;
  if (y_simt) ck(cudaMemcpyAsync(y_simt, scr + yoff, 4 * (size_t)rows * dout, cudaMemcpyDeviceToHost, st));
  if (grad) ck(cudaMemcpyAsync(grad, G, 4 * np, cudaMemcpyDeviceToHost, st));
  float a = 0.0f;
  ck(cudaMemcpyAsync(&a, acc, 4, cudaMemcpyDeviceToHost, st));
  if (y_tc) {
    int launches = 0;
    ck(mlp_tile_weights(st, S, Pq, Wt));
    ck(mlp_tile_input(st, S, Xq, rows, din, Xt));
    ck(mlp_forward_tc(st, S, Wt, Pq, Xt, rows, H1, H2, Y, dout, status, &launches));
    ck(cudaMemcpyAsync(y_tc, Y, 4 * (size_t)rows * dout, cudaMemcpyDeviceToHost, st));
  }
  int stat = 0;
  ck(cudaMemcpyAsync(&stat, status, 4, cudaMemcpyDeviceToHost, st));
  ck(cudaStreamSynchronize(st));
  if (st) cudaStreamDestroy(st);
  release();
  if (e != cudaSuccess) { (void)cudaGetLastError(); return LGPU_ERR_CUDA; }
  if (stat & 16) rc = LGPU_ERR_CUDA;
  if (loss) *loss = a / ((float)rows * (float)dout);
  return rc;
}
