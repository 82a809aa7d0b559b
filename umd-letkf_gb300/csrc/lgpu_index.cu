// lgpu_index.cu -- observation preparation and the spatial index that
// replaces the geoKdTree radius search (src/letkf_obs.F90:492-503 builds
// the tree, :560-573 queries it), plus the per-column localisation
// parameters (localizer%maxhz, search radius, mixed-layer level).
//
// Index: observations bucketed into latitude-band x longitude cells, cells
// band-major; a stable order inside each cell (ascending observation index)
// makes every later reduction deterministic.  The sorted copy holds what the
// Gram kernel streams: unit vector + error (16 B), departure/time/depth/
// surface flag (16 B) and the hx perturbation row padded to KP floats.
#include "lgpu_internal.cuh"

namespace lgpu {

namespace {

__global__ void k_obs_prep(int nobs, const float *lat, const float *lon, const float *zdim, const float *time,
                           const float *val, const float *err, const int *obsid, const int *platid,
                           const float *hx_mean, const int *sat_obs, int n_sat_obs, const int *sat_plats,
                           int n_sat_plats, const IndexGeom *geom, int *cell, int *count, float4 *Atmp,
                           float4 *Btmp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nobs) return;
  float la = lat[i], lo = lon[i];
  float3 u = unitvec_exact(la, lo);
  // dep = val - hx_mean (src/letkf_solver.F90:228)
  float dep = __fsub_rn(val[i], hx_mean[i]);
  // surface classification (src/subclass.letkf_localizer/letkf_loc_ocean.F90:467-479):
  // TRUE unless a non-empty id list misses this observation's id
  float surf = 1.0f;
  if (n_sat_obs > 0) {
    bool f = false;
    for (int j = 0; j < n_sat_obs; j++) f |= (obsid[i] == sat_obs[j]);
    if (!f) surf = 0.0f;
  }
  if (n_sat_plats > 0) {
    bool f = false;
    for (int j = 0; j < n_sat_plats; j++) f |= (platid[i] == sat_plats[j]);
    if (!f) surf = 0.0f;
  }
  int b = band_of(la);
  int nl = geom->nlon[b];
  float ln = norm_lon(lo);
  int c = (int)floorf(ln * (float)nl / 360.0f);
  c = c < 0 ? 0 : (c >= nl ? nl - 1 : c);
  int id = geom->off[b] + c;
  cell[i] = id;
  atomicAdd(&count[id], 1);
  Atmp[i] = make_float4(u.x, u.y, u.z, err[i]);
  Btmp[i] = make_float4(dep, time[i], zdim[i], surf);
}

// exclusive scan of cell counts, one block
__global__ void k_scan(int n, const int *count, int *start) {
  __shared__ int wsum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < n; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < n ? count[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int s = lane < nw ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    int excl = carry + (w > 0 ? wsum[w - 1] : 0) + x - v;
    if (i < n) start[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) start[n] = carry;
}

__global__ void k_scatter(int nobs, const int *cell, const int *start, int *fill, int *pos_tmp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nobs) return;
  int c = cell[i];
  int p = start[c] + atomicAdd(&fill[c], 1);
  pos_tmp[p] = i;
}

// Sort each cell's observation ids ascending (ids are unique: rank sort).
// Small cells in shared memory, very dense cells straight from global.
constexpr int kSortSmem = 4096;
__global__ void k_cell_sort(int ncell, const int *start, const int *in, int *out) {
  __shared__ int s[kSortSmem];
  for (int c = blockIdx.x; c < ncell; c += gridDim.x) {
    int b = start[c], n = start[c + 1] - b;
    if (n == 0) continue;
    if (n == 1) { if (threadIdx.x == 0) out[b] = in[b]; continue; }
    const int *src = in + b;
    if (n <= kSortSmem) {
      for (int t = threadIdx.x; t < n; t += blockDim.x) s[t] = in[b + t];
      __syncthreads();
      src = s;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      int v = src[t], r = 0;
      for (int j = 0; j < n; j++) r += (src[j] < v);
      out[b + r] = v;
    }
    __syncthreads();
  }
}

__global__ void k_gather(int nobs, int k, int kp, const int *order, const float4 *Atmp, const float4 *Btmp,
                         const float *hx, ObsSorted o) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)nobs * kp;
  if (t >= total) return;
  int p = (int)(t / kp), m = (int)(t % kp);
  int i = order[p];
  o.hx[t] = m < k ? hx[(size_t)i * k + m] : 0.0f;
  if (m == 0) {
    o.A[p] = Atmp[i];
    o.B[p] = Btmp[i];
    o.idx[p] = i;
  }
}

// Per-column localisation parameters: localizer%maxhz (loc_novrt :155-161,
// loc_ocean :435-443 = MAX(prof, sat)), max_search_dist = maxhz*stdev2max
// (src/letkf_solver.F90:210-212), the index window of the search circle, and
// for loc_ocean with bkg_t vertical localisation calc_mldlvl_bkgt
// (letkf_loc_ocean.F90:408-427) on the background mean.
__global__ void k_col_prep(int ncol, const float *lat, const float *lon, const int *mask, const float *mean_b,
                           int ns, DevLoc loc, ColPar *cp, float *diag_maxhz) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  float la = lat[c], lo = lon[c];
  float3 u = unitvec_exact(la, lo);
  ColPar p;
  p.ux = u.x; p.uy = u.y; p.uz = u.z;
  float L1 = interp_get(loc.hz, la), L2 = L1, maxhz = L1;
  if (loc.cls == LOC_OCEAN) {
    L2 = interp_get(loc.hz_sat, la);
    maxhz = L1 > L2 ? L1 : L2;
  }
  p.L1 = L1; p.L2 = L2;
  p.ic1 = inv_c_of(L1); p.ic2 = inv_c_of(L2);
  p.rmax = __fmul_rn(maxhz, kStdev2Max);
  if (diag_maxhz) diag_maxhz[c] = mask[c] ? 0.0f : maxhz;
  // conservative index window of the search circle
  float alpha = p.rmax / 6371000.0f;
  float adeg = alpha * 57.29577951308232f * 1.0001f + 0.05f;
  bool full = (la + adeg >= 90.0f) || (la - adeg <= -90.0f) || alpha >= 1.5f;
  float dl = 180.0f;
  if (!full) {
    float s = sinf(alpha) / cosf(la * 0.017453292519943295f);
    dl = s >= 1.0f ? 180.0f : asinf(s) * 57.29577951308232f * 1.0001f + 0.05f;
  }
  p.lonn = norm_lon(lo);
  p.dlon = dl;
  p.b0 = band_of(la - adeg);
  p.b1 = band_of(la + adeg);
  int mld = 0;
  if (loc.cls == LOC_OCEAN && loc.vtloc_surf == 1) {
    const float *m = mean_b + (size_t)c * ns;
    float t0 = m[loc.bkg_t_idx];
    mld = loc.bkg_t_len;
    for (int i = 1; i <= loc.bkg_t_len - 1; i++) {
      float t1 = m[loc.bkg_t_idx + i];
      if (fabsf(__fsub_rn(t0, t1)) > loc.bkg_t_delta) { mld = i; break; }
    }
  }
  p.mld = mld;
  p.pad = 0;
  cp[c] = p;
}

}  // namespace

cudaError_t launch_obs_index(cudaStream_t st, int nobs, int k, int kp, const float *lat, const float *lon,
                             const float *zdim, const float *time, const float *val, const float *err,
                             const int *obsid, const int *platid, const float *hx, const float *hx_mean,
                             const int *sat_obs, int n_sat_obs, const int *sat_plats, int n_sat_plats,
                             const IndexGeom *geom_d, int ncell, int *d_cell, int *d_count, int *d_fill,
                             int *d_pos_tmp, int *d_order, float4 *Atmp, float4 *Btmp, ObsSorted out,
                             int *launches) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(d_count, 0, sizeof(int) * ncell, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(d_fill, 0, sizeof(int) * ncell, st)) != cudaSuccess) return e;
  if (nobs > 0) {
    int nb = (nobs + 255) / 256;
    k_obs_prep<<<nb, 256, 0, st>>>(nobs, lat, lon, zdim, time, val, err, obsid, platid, hx_mean, sat_obs,
                                   n_sat_obs, sat_plats, n_sat_plats, geom_d, d_cell, d_count, Atmp, Btmp);
    (*launches)++;
  }
  k_scan<<<1, 1024, 0, st>>>(ncell, d_count, out.cell_start);
  (*launches)++;
  if (nobs > 0) {
    int nb = (nobs + 255) / 256;
    k_scatter<<<nb, 256, 0, st>>>(nobs, d_cell, out.cell_start, d_fill, d_pos_tmp);
    (*launches)++;
    k_cell_sort<<<4 * 152 * 4, 128, 0, st>>>(ncell, out.cell_start, d_pos_tmp, d_order);
    (*launches)++;
    long long total = (long long)nobs * kp;
    int gb = (int)((total + 255) / 256);
    k_gather<<<gb, 256, 0, st>>>(nobs, k, kp, d_order, Atmp, Btmp, hx, out);
    (*launches)++;
  }
  return cudaGetLastError();
}

cudaError_t launch_col_prep(cudaStream_t st, int ncol, const float *lat, const float *lon, const int *mask,
                            const float *mean_b, int ns, const DevLoc &loc, ColPar *cp, float *diag_maxhz,
                            int *launches) {
  if (ncol <= 0) return cudaSuccess;
  k_col_prep<<<(ncol + 127) / 128, 128, 0, st>>>(ncol, lat, lon, mask, mean_b, ns, loc, cp, diag_maxhz);
  (*launches)++;
  return cudaGetLastError();
}

}  // namespace lgpu
