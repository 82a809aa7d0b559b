// lgpu_internal.cuh -- shared device definitions of the sm_103a LETKF path:
// the observation metric, latitude interpolation, Gaspari-Cohn weights, the
// spatial-index geometry and the kernel parameter blocks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "letkf_gpu.h"

namespace lgpu {

// ---------------------------------------------------------------- limits --
constexpr int kMaxK = LGPU_MAX_K;          // ensemble size
constexpr int kMaxGroups = LGPU_MAX_LEVELS;
constexpr int kNB = 180;                   // 1-degree latitude bands of the index
constexpr int kMaxInterp = LGPU_MAX_INTERP + 2;

// Localizer classes.
enum LocClass { LOC_NOVRT = 0, LOC_OCEAN = 1, LOC_VTGC = 2 };

// linearinterp_lat table after the reference's 0/90-degree padding
// (src/letkf_loc.F90:251-294).
struct Interp {
  int n;
  float lat[kMaxInterp];
  float dist[kMaxInterp];
};

// Localizer parameters the device needs (the plugin's "device descriptor").
struct DevLoc {
  int cls;
  int groups;          // maxgroups
  Interp hz;           // novrt/vtgc: hzloc; ocean: hzloc_prof
  Interp hz_sat;       // ocean: hzloc_sat
  float tloc_prof, tloc_sat;
  int vtloc_surf;      // ocean: 1 = bkg_t mixed-layer split
  float bkg_t_delta;
  int bkg_t_idx, bkg_t_len;
  float vloc;          // vtgc vertical length scale
  const float *lev_depth;  // vtgc level depths [groups] (device)
};

// ------------------------------------------------------ exact metric -----
// The observation metric is evaluated with explicitly rounded IEEE
// operations (no contraction) so that host and device produce identical
// distances: sin/cos in double by exact reduction to |x| <= pi/4 and Taylor
// polynomials, great-circle angle from the chord in float,
// theta = 2 asin(|a - b| / 2), distance = 6371 km * theta.
__device__ __forceinline__ void sincos_deg_exact(double a, double &s, double &c) {
  double q = floor(__dadd_rn(__ddiv_rn(a, 90.0), 0.5));
  double r = __dsub_rn(a, __dmul_rn(90.0, q));
  double x = __dmul_rn(r, 0.017453292519943295);
  double x2 = __dmul_rn(x, x);
  double p = 2.8114572543455206e-15;
  p = __dadd_rn(__dmul_rn(p, x2), -7.647163731819816e-13);
  p = __dadd_rn(__dmul_rn(p, x2), 1.6059043836821613e-10);
  p = __dadd_rn(__dmul_rn(p, x2), -2.505210838544172e-08);
  p = __dadd_rn(__dmul_rn(p, x2), 2.7557319223985893e-06);
  p = __dadd_rn(__dmul_rn(p, x2), -0.0001984126984126984);
  p = __dadd_rn(__dmul_rn(p, x2), 0.008333333333333333);
  p = __dadd_rn(__dmul_rn(p, x2), -0.16666666666666666);
  double sn = __dadd_rn(x, __dmul_rn(x, __dmul_rn(x2, p)));
  double u = 4.779477332387385e-14;
  u = __dadd_rn(__dmul_rn(u, x2), -1.1470745597729725e-11);
  u = __dadd_rn(__dmul_rn(u, x2), 2.08767569878681e-09);
  u = __dadd_rn(__dmul_rn(u, x2), -2.755731922398589e-07);
  u = __dadd_rn(__dmul_rn(u, x2), 2.48015873015873e-05);
  u = __dadd_rn(__dmul_rn(u, x2), -0.001388888888888889);
  u = __dadd_rn(__dmul_rn(u, x2), 0.041666666666666664);
  u = __dadd_rn(__dmul_rn(u, x2), -0.5);
  double cs = __dadd_rn(1.0, __dmul_rn(x2, u));
  long long qi = (((long long)q % 4) + 4) % 4;
  if (qi == 0) { s = sn; c = cs; }
  else if (qi == 1) { s = cs; c = -sn; }
  else if (qi == 2) { s = -sn; c = -cs; }
  else { s = -cs; c = sn; }
}

__device__ __forceinline__ float3 unitvec_exact(float lat, float lon) {
  double sp, cp, sl, cl;
  sincos_deg_exact((double)lat, sp, cp);
  sincos_deg_exact((double)lon, sl, cl);
  return make_float3((float)__dmul_rn(cp, cl), (float)__dmul_rn(cp, sl), (float)sp);
}

__device__ __forceinline__ float asin_poly_exact(float x) {
  float x2 = __fmul_rn(x, x);
  float p = 0.008390335366129875f;
  p = __fadd_rn(__fmul_rn(p, x2), 0.009761609137058258f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.01155180111527443f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.013964843936264515f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.017352763563394547f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.022372158244252205f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.0303819440305233f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.0446428582072258f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.07500000298023224f);
  p = __fadd_rn(__fmul_rn(p, x2), 0.1666666716337204f);
  return __fadd_rn(x, __fmul_rn(x, __fmul_rn(x2, p)));
}

// squared chord between two unit vectors
__device__ __forceinline__ float chord2_exact(float ax, float ay, float az, float bx, float by, float bz) {
  float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

__device__ __forceinline__ float dist_from_chord2(float c2) {
  float h = __fmul_rn(0.5f, __fsqrt_rn(c2));
  if (h > 1.0f) h = 1.0f;
  float ang;
  if (h <= 0.5f) ang = asin_poly_exact(h);
  else ang = __fsub_rn(1.5707963705062866f,
                       __fmul_rn(2.0f, asin_poly_exact(__fsqrt_rn(__fmul_rn(__fsub_rn(1.0f, h), 0.5f)))));
  return __fmul_rn(12742000.0f, ang);
}

// linearinterp_lat_get_dist (src/letkf_loc.F90:302-320), REAL arithmetic
__device__ __forceinline__ float interp_get(const Interp &t, float lat) {
  float al = fabsf(lat);
  int i = 0;
  while (i < t.n - 1 && al > t.lat[i]) i++;
  if (i == 0) return t.dist[0];
  float d = __fdiv_rn(__fsub_rn(al, t.lat[i - 1]), __fsub_rn(t.lat[i], t.lat[i - 1]));
  return __fadd_rn(__fmul_rn(d, t.dist[i]), __fmul_rn(__fsub_rn(1.0f, d), t.dist[i - 1]));
}

// letkf_loc_gc (src/letkf_loc.F90:348-378) exactly: REAL(8) with the
// reference's truncated coefficients, result rounded to REAL.
__device__ __forceinline__ float gc_exact(float z, float L) {
  double c = __ddiv_rn((double)L, 0.5477225575051661);
  double abs_z = (double)fabsf(z);
  double zc = __ddiv_rn(abs_z, c);
  double z2 = __dmul_rn(zc, zc), z3 = __dmul_rn(z2, zc), z4 = __dmul_rn(z2, z2), z5 = __dmul_rn(z4, zc);
  double res;
  if (abs_z >= __dmul_rn(2.0, c)) {
    res = 0.0;
  } else if (abs_z > c) {
    res = __dsub_rn(__dmul_rn(0.08333, z5), __dmul_rn(0.5, z4));
    res = __dadd_rn(res, __dmul_rn(0.625, z3));
    res = __dadd_rn(res, __dmul_rn(1.66667, z2));
    res = __dsub_rn(res, __dmul_rn(5.0, zc));
    res = __dadd_rn(res, 4.0);
    res = __dsub_rn(res, __ddiv_rn(__dmul_rn(0.66667, c), abs_z));
  } else {
    res = __dadd_rn(__dmul_rn(-0.25, z5), __dmul_rn(0.5, z4));
    res = __dadd_rn(res, __dmul_rn(0.625, z3));
    res = __dsub_rn(res, __dmul_rn(1.66667, z2));
    res = __dadd_rn(res, 1.0);
  }
  return (float)res;
}

// Fast single-precision Gaspari-Cohn with the same truncated coefficients.
// The outer branch is evaluated as Q(t)/zc with t = 2 - zc, where
// Q(z) = z * outer(z) re-expanded about z = 2 (coefficients exact in double,
// rounded to float), which removes the cancellation near the support edge.
// Absolute error against gc_exact is below 4e-7 for all inputs; callers
// re-evaluate with gc_exact when a weight lands near the 1e-4 keep threshold.
__device__ __forceinline__ float gc_fast(float z, float inv_c) {
  float zc = fabsf(z) * inv_c;
  if (zc >= 2.0f) return 0.0f;
  if (zc > 1.0f) {
    float t = 2.0f - zc;
    float q = 0.08333f;
    q = __fmaf_rn(q, t, -0.49996f);
    q = __fmaf_rn(q, t, 0.6248f);
    q = __fmaf_rn(q, t, 0.0005299999999996974f);
    q = __fmaf_rn(q, t, -0.0007799999999991147f);
    q = __fmaf_rn(q, t, 0.0005999999999986017f);
    q = __fmaf_rn(q, t, -0.0001899999999991353f);
    return __fdiv_rn(q, zc);
  }
  float p = -0.25f;
  p = __fmaf_rn(p, zc, 0.5f);
  p = __fmaf_rn(p, zc, 0.625f);
  p = __fmaf_rn(p, zc, -1.66667f);
  return __fmaf_rn(p, zc * zc, 1.0f);
}

__host__ __device__ __forceinline__ float inv_c_of(float L) {
  return (float)(0.5477225575051661 / (double)L);
}

constexpr float kKeep = 1.0e-4f;          // src/letkf_solver.F90:251
constexpr float kGuard1 = 1.0e-6f;        // fast-GC guard band, one factor
constexpr float kGuard2 = 3.0e-6f;        // two-factor products
constexpr float kStdev2Max = 3.65148377f; // SQRT(40.0/3.0) in REAL, src/letkf_solver.F90:47

// ---------------------------------------------- fast weight path -----
// The batched Gram evaluates distance and Gaspari-Cohn in float with fused
// multiply-adds and approximate reciprocals, and falls back to the exact
// metric and the per-column localizer for a pair whose fast distance lies
// within kFastDistBand (relative) of the search radius or whose fast weight
// lies within kGuardFast of the keep threshold.  Against the exact path the
// fast distance is within 1e-6 relative and the fast weight within 2e-8
// absolute near the keep threshold (tests/test_gpu_parity.py); the bands
// hold a 5x margin over those bounds.
constexpr float kFastDistBand = 5.0e-6f;
constexpr float kGuardFast = 1.0e-7f;

// squared chord between unit vectors, fused multiply-adds
__device__ __forceinline__ float chord2_fast(float ax, float ay, float az, float bx, float by, float bz) {
  const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
  return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
}

// asin(x), 0 <= x <= 0.5: Taylor series of asin in Horner form with fused
// multiply-adds (a few ulp).  x <= 0.25: terms to x^13 (truncation below
// 2e-11 relative); otherwise to x^21.
__device__ __forceinline__ float asin_fast(float x, bool short_series = false) {
  const float x2 = x * x;
  float p;
  if (short_series) {
    p = 0.017352763563394547f;
  } else {
    p = 0.008390335366129875f;
    p = __fmaf_rn(p, x2, 0.009761609137058258f);
    p = __fmaf_rn(p, x2, 0.01155180111527443f);
    p = __fmaf_rn(p, x2, 0.013964843936264515f);
    p = __fmaf_rn(p, x2, 0.017352763563394547f);
  }
  p = __fmaf_rn(p, x2, 0.022372158244252205f);
  p = __fmaf_rn(p, x2, 0.0303819440305233f);
  p = __fmaf_rn(p, x2, 0.0446428582072258f);
  p = __fmaf_rn(p, x2, 0.07500000298023224f);
  p = __fmaf_rn(p, x2, 0.1666666716337204f);
  return __fmaf_rn(x * x2, p, x);
}

// Gaspari-Cohn of zc = |z| / c without branches: the same two polynomials as
// gc_fast (outer one in the shifted variable t = 2 - zc, divided by zc with
// the approximate divide); within 1e-6 of gc_exact.
__device__ __forceinline__ float gc_branchless(float zc) {
  const float t = 2.0f - zc;
  float q = 0.08333f;
  q = __fmaf_rn(q, t, -0.49996f);
  q = __fmaf_rn(q, t, 0.6248f);
  q = __fmaf_rn(q, t, 0.0005299999999996974f);
  q = __fmaf_rn(q, t, -0.0007799999999991147f);
  q = __fmaf_rn(q, t, 0.0005999999999986017f);
  q = __fmaf_rn(q, t, -0.0001899999999991353f);
  const float qo = __fdividef(q, zc);
  float p = -0.25f;
  p = __fmaf_rn(p, zc, 0.5f);
  p = __fmaf_rn(p, zc, 0.625f);
  p = __fmaf_rn(p, zc, -1.66667f);
  const float pi = __fmaf_rn(p, zc * zc, 1.0f);
  return zc >= 2.0f ? 0.0f : (zc > 1.0f ? qo : pi);
}

// great-circle distance (m) from the squared chord, fast path (chord <= 1;
// short_series for half-chords up to 0.25)
__device__ __forceinline__ float dist_fast(float c2f, bool short_series = false) {
  const float hf = 0.5f * c2f * rsqrtf(fmaxf(c2f, 1e-30f));
  return 12742000.0f * asin_fast(fminf(hf, 0.5f), short_series);
}

// Packed Gram layout of one unit: the upper triangle of G (i <= j, row-major)
// followed by the right-hand side b; k(k+3)/2 floats.
__host__ __device__ __forceinline__ int tri_off(int i, int k) { return i * k - (i * (i - 1)) / 2; }
__host__ __device__ __forceinline__ int tri_idx(int i, int j, int k) { return tri_off(i, k) + (j - i); }
__host__ __device__ __forceinline__ int packed_size(int k) { return k * (k + 3) / 2; }
// feature f -> (i, j); j == k denotes the right-hand side (y_i * dep)
__host__ __device__ __forceinline__ void packed_ij(int f, int k, int &i, int &j) {
  const int nt = k * (k + 1) / 2;
  if (f >= nt) { i = f - nt; j = k; return; }
  int r = 0;
  while (tri_off(r + 1, k) <= f) r++;
  i = r;
  j = f - tri_off(r, k) + r;
}

// Per-column parameters prepared once per run.
struct ColPar {
  float ux, uy, uz;     // unit vector
  float rmax;           // maxhz * stdev2max (search radius, m)
  float L1, L2;         // horizontal GC length scales (novrt/vtgc: L1; ocean: L1 = prof, L2 = sat)
  float ic1, ic2;       // sqrt(0.3)/L
  float lonn;           // longitude in [0,360)
  float dlon;           // half-width of the longitude window (deg); >= 180 means whole bands
  int b0, b1;           // latitude band range
  int mld;              // ocean: surface-group level count (calc_mldlvl_bkgt)
  int pad;
};

// Localisation weight of one (column, group, observation) with exact keep
// decisions: fast float evaluation, exact REAL(8) re-evaluation in the guard
// band around the keep threshold.  localize_cls is one class; the column's
// parameters are read where the class needs them, so a caller holding c in
// global memory keeps the unused ones out of its registers.
template <int CLS>
__device__ __forceinline__ float localize_cls(const DevLoc &L, const ColPar &c, int gid, float dist, float otime,
                                              float oz, float surf) {
  if (CLS == LOC_OCEAN) {
    // src/subclass.letkf_localizer/letkf_loc_ocean.F90:483-504
    const bool s = surf != 0.0f;
    if (s && gid == 1) return 0.0f;
    const float Lh = s ? c.L2 : c.L1, ic = s ? c.ic2 : c.ic1, tl = s ? L.tloc_sat : L.tloc_prof;
    float r = gc_fast(dist, ic);
    if (tl > 0.0f) {
      float p = r * gc_fast(otime, inv_c_of(tl));
      if (fabsf(p - kKeep) <= kGuard2) p = gc_exact(dist, Lh) * gc_exact(otime, tl);
      return p;
    }
    if (fabsf(r - kKeep) <= kGuard1) r = gc_exact(dist, Lh);
    return r;
  } else if (CLS == LOC_VTGC) {
    const float dz = fabsf(oz - L.lev_depth[gid]);
    float p = gc_fast(dist, c.ic1) * gc_fast(dz, inv_c_of(L.vloc));
    if (fabsf(p - kKeep) <= kGuard2) p = gc_exact(dist, c.L1) * gc_exact(dz, L.vloc);
    return p;
  } else {
    // src/subclass.letkf_localizer/letkf_loc_novrt.F90:181
    float r = gc_fast(dist, c.ic1);
    if (fabsf(r - kKeep) <= kGuard1) r = gc_exact(dist, c.L1);
    return r;
  }
}

__device__ __forceinline__ float localize(const DevLoc &L, const ColPar &c, int gid, float dist,
                                          float otime, float oz, float surf) {
  switch (L.cls) {
  case LOC_OCEAN: return localize_cls<LOC_OCEAN>(L, c, gid, dist, otime, oz, surf);
  case LOC_VTGC: return localize_cls<LOC_VTGC>(L, c, gid, dist, otime, oz, surf);
  default: return localize_cls<LOC_NOVRT>(L, c, gid, dist, otime, oz, surf);
  }
}

// -------------------------------------------------- index geometry -------
// Observations are bucketed in 1-degree latitude bands; band b holds
// nlon[b] equal longitude cells (about 1 degree wide at the band's poleward
// edge).  Cell ids run band-major, so a longitude window of a band is a
// contiguous run of cells and of sorted observations.
struct IndexGeom {
  int nlon[kNB];
  int off[kNB + 1];
};

__host__ __device__ __forceinline__ int band_of(float lat) {
  int b = (int)floorf(lat + 90.0f);
  return b < 0 ? 0 : (b >= kNB ? kNB - 1 : b);
}

__host__ __device__ __forceinline__ float norm_lon(float lon) {
  float l = fmodf(lon, 360.0f);
  if (l < 0.0f) l += 360.0f;
  if (l >= 360.0f) l -= 360.0f;
  return l;
}

// ----------------------------------------------------- kernel launchers --
struct ObsSorted {
  float4 *A;       // (ux, uy, uz, err)
  float4 *B;       // (dep, time, zdim, surf)
  float *hx;       // [nobs][KP] perturbations, zero padded
  int *idx;        // original observation index
  int *cell_start; // [ncell + 1]
};

// The local-observation search of one (column, group), the threads of a
// block striding over the column's index window (kd_search_radius and the
// keep filter of src/letkf_solver.F90:211-263): every observation within the
// search radius adds one to counts[1]; each one whose localisation weight
// passes r > 1e-4 adds one to counts[0] and is handed to emit(p, r), p its
// position in the sorted table.  Entries arrive in no fixed order.  Used by
// the verification queries (lgpu_get_obslist and its no-allocation form).
template <class Emit>
__device__ __forceinline__ void list_search(int gid, const ColPar &cp, const DevLoc &loc, const ObsSorted &obs,
                                            const IndexGeom *geom, int *counts, Emit emit) {
  const float hq = fminf(cp.rmax / 12742000.0f, 1.5707963f);
  const float sh = sinf(hq);
  const float c2max = 4.0f * sh * sh * 1.0001f + 1e-12f;
  for (int b = cp.b0; b <= cp.b1; b++) {
    const int nl = geom->nlon[b], off = geom->off[b];
    int runs[2][2] = {{0, 0}, {0, 0}};
    bool whole = cp.dlon >= 180.0f;
    int clo = 0, chi = nl - 1;
    if (!whole) {
      clo = (int)floorf((cp.lonn - cp.dlon) * (float)nl / 360.0f);
      chi = (int)floorf((cp.lonn + cp.dlon) * (float)nl / 360.0f);
      if (chi - clo + 1 >= nl) whole = true;
    }
    if (whole) { runs[0][0] = obs.cell_start[off]; runs[0][1] = obs.cell_start[off + nl]; }
    else if (clo < 0) {
      runs[0][0] = obs.cell_start[off + clo + nl]; runs[0][1] = obs.cell_start[off + nl];
      runs[1][0] = obs.cell_start[off]; runs[1][1] = obs.cell_start[off + chi + 1];
    } else if (chi >= nl) {
      runs[0][0] = obs.cell_start[off + clo]; runs[0][1] = obs.cell_start[off + nl];
      runs[1][0] = obs.cell_start[off]; runs[1][1] = obs.cell_start[off + chi - nl + 1];
    } else { runs[0][0] = obs.cell_start[off + clo]; runs[0][1] = obs.cell_start[off + chi + 1]; }
    for (int q = 0; q < 2; q++)
      for (int p = runs[q][0] + threadIdx.x; p < runs[q][1]; p += blockDim.x) {
        const float4 A = obs.A[p];
        const float c2 = chord2_exact(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z);
        if (c2 > c2max) continue;
        const float d = dist_from_chord2(c2);
        if (d > cp.rmax) continue;
        atomicAdd(&counts[1], 1);
        const float4 B = obs.B[p];
        const float r = localize(loc, cp, gid, d, B.y, B.z, B.w);
        if (r > kKeep) {
          atomicAdd(&counts[0], 1);
          emit(p, r);
        }
      }
  }
}

cudaError_t launch_obs_index(cudaStream_t st, int nobs, int k, int kp, const float *lat, const float *lon,
                             const float *zdim, const float *time, const float *val, const float *err,
                             const int *obsid, const int *platid, const float *hx, const float *hx_mean,
                             const int *sat_obs, int n_sat_obs, const int *sat_plats, int n_sat_plats,
                             const IndexGeom *geom_d, int ncell, int *d_cell, int *d_count, int *d_fill,
                             int *d_pos_tmp, int *d_order, float4 *Atmp, float4 *Btmp, ObsSorted out,
                             int *launches);

cudaError_t launch_col_prep(cudaStream_t st, int ncol, const float *lat, const float *lon, const int *mask,
                            const float *mean_b, int ns, const DevLoc &loc, ColPar *cp, float *diag_maxhz,
                            int *launches);

struct GramArgs {
  int nunits, groups, k, kp;
  const int *active;      // active (unmasked) columns
  const ColPar *cp;
  DevLoc loc;
  ObsSorted obs;
  const IndexGeom *geom;  // device copy
  float *G;               // [unit][packed_size(k)]  (upper triangle of G, then b)
  int *nkept;             // [unit]
  float *diag_obscount;   // [ncol]
  float *diag_lg_obscount;// [group][ncol]
  float *diag_lg_obsloc;  // [group][ncol]
  int ncol;
};
cudaError_t launch_gram(cudaStream_t st, const GramArgs &a, int *launches);

// Batched (tile) Gram on the tensor cores.
struct TilePar {
  float lonn, dlon;  // longitude window of the tile's search cap (deg)
  int b0, b1;        // latitude band range
  float cx, cy, cz;  // cap centre (unit vector)
  float c2cap;       // squared chord of the cap radius, with margin
  float hmax;        // largest half-chord of a candidate pair of the tile
};
// One accumulation segment of a tile's chunk stream, one CTA: chunks [cs, ce)
// of the tile's stream.  The CTA drains its tensor-core accumulator every
// `drain` chunks; when the tile's stream holds more than one drain interval,
// drain j of this segment goes to partial block blk0 + j and the segment's
// counts to count block cblk (both -1 when the whole stream is one interval:
// the CTA writes G and the counts directly).
struct TcWork {
  int tile, seg, cs, ce, cblk, blk0, pad0, pad1;
};
// A tile whose stream spans more than one drain interval: count blocks
// cblk0 .. cblk0 + nseg - 1 (one per segment), partial blocks blk0 .. blk0 +
// nblk - 1 (one per drain interval, in stream order).
struct TcSegTile {
  int tile, nseg, cblk0, nblk, blk0, pad0, pad1, pad2;
};

struct TcArgs {
  int ntiles, groups, k, kp, npass, np, nf, ncol;
  const int *tile_cols;   // [ntiles][128] column index or -1
  const int *col2act;
  const ColPar *cp;
  DevLoc loc;
  const TilePar *tp;         // per-tile cap parameters
  const unsigned char *rec;  // tile candidate streams (chunk records)
  const int *tile_off;       // [ntiles + 1] first chunk of each tile's stream
  const int *tile_n;         // [ntiles] candidates of each tile
  int cb;                    // bytes per chunk record (set by the launcher)
  uint32_t tmem_cols;        // TMEM columns per CTA (set by the launcher)
  float *wcache;             // weight cache [groups][chunks] TF32 hi | lo operand blocks, or null
  int *wflag;                // [groups][chunks]: the chunk has a kept pair (MMA issued)
  int nchunk_total;          // chunks over all tiles (weight cache indexing)
  int pass0, npl;            // feature passes of one launch: [pass0, pass0 + npl) (set by the launcher)
  // accumulation segments and drains: each tile's chunk stream is split into
  // segments (one CTA each), and each CTA moves its tensor-core accumulator
  // out every `drain` chunks (the FP32 accumulation error of the tensor core
  // grows with the MMAs summed into one accumulator); launch_gram_segsum sums
  // a tile's drained partials in stream order, compensated (doubled precision)
  const TcWork *work;     // [nwork] work items (tile order, then segment)
  int nwork;
  int drain;              // chunks per drain interval
  int cull;               // 1: a warp skips the distance and localizer of four records none of its columns can reach
  long long units;
  float *Gpart;              // [partial block][group][nf][128] (feature-major: coalesced drains)
  float *cnt;                // [count block][group][128][3]: kept, candidates, sum rho
  const TcSegTile *segtiles; // [nsegtiles] tiles with more than one segment
  int nsegtiles;
  float *G;
  int *nkept;
  float *diag_obscount, *diag_lg_obscount, *diag_lg_obsloc;
  int *status;
};
// G += the partial Grams of segments 1..nseg-1; kept counts and diagnostics
// from the per-segment counts
cudaError_t launch_gram_segsum(cudaStream_t st, const TcArgs &a, const int *active, int *launches);
cudaError_t launch_tile_prep(cudaStream_t st, int ntiles, const int *tile_cols, const ColPar *cp, TilePar *tp,
                             int *launches);
// tile candidate streams: counts + chunk offsets (tile_off[ntiles] = total
// chunks), then the records (record_bytes(k) per chunk of 16)
size_t record_bytes(int k);
cudaError_t launch_tile_count(cudaStream_t st, int ntiles, const TilePar *tp, const IndexGeom *geom,
                              const ObsSorted &obs, int *tile_n, int *tile_off, int *launches);
cudaError_t launch_tile_fill(cudaStream_t st, int ntiles, const TilePar *tp, const IndexGeom *geom,
                             const ObsSorted &obs, int k, int kp, const int *tile_off, unsigned char *rec,
                             int *status, int *launches);
cudaError_t launch_gram_tc(cudaStream_t st, const TcArgs &a, int *launches);
// CUDA loads a kernel at its first use: these load the plain and the batched
// (for one localizer class) Gram kernels ahead of a timed trial
cudaError_t preload_gram(void);
cudaError_t preload_gram_tc(int loc_cls);
size_t gram_tc_wcache_bytes(int groups, int nchunk_total);
void gram_tc_passes(int k, int *npass, int *np);

struct EigArgs {
  int nunits, k;
  float infl;
  const float *G;
  const int *nkept;
  float *T;               // [unit][k][k]
  float *wbar;            // [unit][k] mean weights, or null
  const int *ulist;       // units to solve (the i-th is ulist[i]), or null: units 0..nunits-1
  int *status;            // [1] accumulated error bits
  // FP64 re-solve (split pipeline): a unit whose FP32 solve failed (no
  // convergence, a non-positive or non-finite eigenvalue) or whose relevant
  // FP32 eigenvalues (those above the (k-1)/infl floor by more than the
  // rounding level) have a relative gap min|l_i - l_j| / max l <= gap_thresh
  // is appended to flag_list (flag_n[0] = entries written, at most
  // flag_cap; flag_n[1] = entries already re-solved); null: no flagging
  int *flag_list, *flag_n;
  int flag_cap;
  float gap_thresh;
};
// FP64 eigensolve + transform (a team of warps per unit): units ulist[0..nunits) or
// ubase + 0..nunits; T (and w-bar) written in FP32
cudaError_t launch_eig64(cudaStream_t st, const EigArgs &a, int ubase, int *launches);
// FP64 re-solve of the flagged units not yet re-solved (flag_list entries
// flag_n[1] .. flag_n[0]); the count stays on the device
cudaError_t launch_eig64_flagged(cudaStream_t st, const EigArgs &a, int *launches);
cudaError_t launch_eig(cudaStream_t st, const EigArgs &a, int *launches);
// scratch of the split eigensolve pipeline, for `batch` units
struct EigSplit {
  float *Q;        // [batch][k][k] Householder Q, row-major
  float *DE;       // [batch][2k] diagonal, off-diagonal
  float2 *log;     // [batch][cap] sweep headers (start, count) and rotations (c, s)
  int *logn;       // [batch] log entries, -1 no convergence, -2 overflow
  float *lam;      // [batch][k] eigenvalues
  int cap;
};
int eig_log_cap(int k);
size_t eig_split_bytes_per_unit(int k);
// units [ustart, ustart + ucount), in batches of at most `batch`
cudaError_t launch_eig_split(cudaStream_t st, const EigArgs &a, const EigSplit &sp, int batch, int ustart, int ucount,
                             int *launches);

struct UpdateArgs {
  int ncol, ns, k, groups;
  int col0, ncols;        // columns [col0, col0 + ncols) of this launch
  const int *mask;        // [ncol] device
  const int *col2act;     // [ncol] active index or -1
  const ColPar *cp;
  int loc_cls, vtloc_surf;
  const int *slab_var;    // [ns] variable of each slab
  const int *slab_lev;    // [ns] level of each slab within its variable
  const float *var_inc_max, *var_lb, *var_ub;  // per variable
  const float *bkg, *mean_b, *sprd_b;
  const float *T;
  const int *nkept;
  float *ana, *mean_a, *sprd_a;
  float rtps, rtpp, mul;
  int *status;
};
cudaError_t launch_update(cudaStream_t st, const UpdateArgs &a, int *launches);
// the same update on the tensor cores (lgpu_update_tc.cu): k a multiple of
// 4 with 64 < k <= 128, ns <= 128, at most 2 groups; cudaErrorNotSupported
// otherwise
cudaError_t launch_update_tc(cudaStream_t st, const UpdateArgs &a, int *launches);

// ---- weight-correction network of the learned form (lgpu_mlp.cu) ----
struct MlpShape {
  int din, k1, H, dout;   // k1 = din rounded up to 16
};
size_t mlp_param_count(const MlpShape &s);
void mlp_param_offsets(const MlpShape &s, size_t off[6]);   // W1 b1 W2 b2 W3 b3
size_t mlp_tiled_weight_bytes(const MlpShape &s);
size_t mlp_act_bytes(const MlpShape &s, int rows);
size_t mlp_train_scratch_floats(const MlpShape &s, int rows);
float *mlp_loss_parts(const MlpShape &s, float *scr, int rows);
__host__ __device__ size_t mlp_tile_off(int r, int kk, int K, int rb);
cudaError_t mlp_tile_weights(cudaStream_t st, const MlpShape &s, const float *wq, unsigned char *tiled);
cudaError_t mlp_tile_input(cudaStream_t st, const MlpShape &s, const float *x, int rows, int ld, unsigned char *tiled);
cudaError_t mlp_forward_tc(cudaStream_t st, const MlpShape &s, const unsigned char *wtiled, const float *bias_base,
                           const unsigned char *x, int rows, unsigned char *h1, unsigned char *h2, float *y, int ldy,
                           int *status, int *launches);
cudaError_t mlp_forward_simt(cudaStream_t st, const MlpShape &s, const float *wq, const float *x, int rows, float *y,
                             float *scr);
cudaError_t mlp_grad(cudaStream_t st, const MlpShape &s, const float *wq, const float *x, const float *t, int rows,
                     float *grad, float *scr, int *nparts, const float *wout);
cudaError_t mlp_adam(cudaStream_t st, long long n, float *w, float *wq, const float *g, float *m, float *v, float lr,
                     int step);
cudaError_t mlp_round(cudaStream_t st, long long n, const float *w, float *wq);

// ---- learned analysis form (lgpu_learn.cu) ----
struct LrnInterpArgs {
  int nfine;
  const int *cols;
  int nx, ny, s, k, din, dout;
  const float *Ts, *ws;       // coarse solutions: T = W + w-bar 1^T [src][k][k], w-bar [src][k]
  const int *src_of_col;      // [ncol] row of the coarse solution or -1
  const float *feat;          // [nfine][16] (0..9 from k_lrn_obsfeat)
  const float *lat;
  const float *mu, *sd;       // input standardisation [din], or null (raw rows)
  float *X;                   // [nfine][din] network input rows (row f at X + f * ldx)
  long long ldx;
  int *flag;                  // [nfine] 1 = a coarse neighbour has no solution
  const float *Tex, *wex;     // collecting: exact T / w-bar of every unit
  const int *col2act;
  float *Yt;                  // collecting: residual targets [nfine][dout] (row f at Yt + f * ldy), or null
  long long ldy;
};

struct LrnApplyArgs {
  int nfine;
  const int *cols;
  int nx, ny, s, k, dout;
  const float *Ts, *ws;
  const int *src_of_col;
  const float *Yn;            // network outputs [nfine][ldy] (standardised residuals)
  long long ldy;
  const float *mu_out, *sd_out;
  float tau;                  // gate: RMS of the standardised output above tau -> exact
  int net;                    // 0: interpolation only (zero correction, no score gate)
  const int *flag;
  const int *nk_fine;         // [nfine] kept count
  const int *col2act;
  float *T;                   // [unit][k][k]
  int *nkept;                 // [unit]
  int *gate_cols, *gate_n;    // exact fallback list
  float *score;               // [nfine] or null
};

cudaError_t lrn_cellstats(cudaStream_t st, int ncell, const ObsSorted &obs, float4 *c0, float4 *c1, int *launches);
cudaError_t lrn_obsfeat(cudaStream_t st, int nfine, const int *cols, const ColPar *cp, const DevLoc &loc,
                        const int *cell_start, const float4 *c0, const float4 *c1, const IndexGeom *geom,
                        float *feat, int *nkept, int *launches);
cudaError_t lrn_interp(cudaStream_t st, const LrnInterpArgs &a, int *launches);
cudaError_t lrn_apply(cudaStream_t st, const LrnApplyArgs &a, int *launches);
cudaError_t lrn_judge(cudaStream_t st, int nj, const int *jcols, const int *jsub, const float *Tsub, const float *T,
                      const int *col2act, const int *gate_mark, int k, float *acc, int *launches);
cudaError_t lrn_mark(cudaStream_t st, int n, const int *cols, int *mark, int v);
cudaError_t lrn_scatter(cudaStream_t st, int n, const int *cols, const int *col2act, const float *Tsub,
                        const int *nk_sub, int k, float *T, int *nkept, int *launches);
cudaError_t lrn_colstats(cudaStream_t st, const float *M, long long rows, int n, long long ld, float *mu, float *sd);
cudaError_t lrn_batch(cudaStream_t st, int b, const int *idx, const float *X, long long ldx, int din, const float *Y,
                      long long ldy, int dout, const float *mu, const float *sd, const float *muo, const float *sdo,
                      float *Xb, float *Yb);

// list emission for verification
cudaError_t launch_obslist(cudaStream_t st, int col, int gid, int group_slot, const ColPar *cp_col, const DevLoc &loc,
                           ObsSorted obs, const IndexGeom *geom, int cap, int *d_idx, float *d_r, int *d_counts);

cudaError_t launch_debug_metric(cudaStream_t st, int n, const float *lat1, const float *lon1,
                                const float *lat2, const float *lon2, float *dist);
cudaError_t launch_debug_gc(cudaStream_t st, int n, const float *z, const float *L, float *fast, float *exact);
cudaError_t launch_debug_weight(cudaStream_t st, int n, const float *lat1, const float *lon1, const float *lat2,
                                const float *lon2, const float *L, float *out);

}  // namespace lgpu
