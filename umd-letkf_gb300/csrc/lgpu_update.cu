// lgpu_update.cu -- ensemble update and analysis epilogue, one CTA per
// column, one warp per slab.
//
// Replaces src/letkf_solver.F90:282-379 for one column:
//   x_a(1 x k) = x_b(1 x k) * T_g for every slab of every group g with local
//   observations (:285-289); other slabs keep the background perturbation;
//   recenter on the new mean (:299-303); clip the mean increment by
//   ana_inc_max and ana_bounds (:308-318); RTPS (:322-335), RTPP (:339-344),
//   multiplicative inflation (:347-349); member bounds and re-mean
//   (:357-371); final spread and add the mean back (:375-379).
// Masked columns are skipped by the reference (:207): their state stays the
// background perturbation and their mean/spread stay the background values.
// Member sums use a fixed butterfly order across the warp.
#include "lgpu_internal.cuh"

namespace lgpu {

namespace {

constexpr int UT = 256;  // 8 warps per column

__device__ __forceinline__ float bsum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(UT) k_update(UpdateArgs a, int tsm_groups) {
  extern __shared__ __align__(16) float Ts[];   // [tsm_groups][k][k] transforms of this column
  const int col = blockIdx.x;
  const int k = a.k, ns = a.ns;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const size_t cbase = (size_t)col * ns * k;
  const int act = a.col2act[col];
  if (a.mask[col] || act < 0) {
    for (int t = threadIdx.x; t < ns * k; t += blockDim.x) a.ana[cbase + t] = a.bkg[cbase + t];
    for (int s = threadIdx.x; s < ns; s += blockDim.x) {
      a.mean_a[(size_t)col * ns + s] = a.mean_b[(size_t)col * ns + s];
      a.sprd_a[(size_t)col * ns + s] = a.sprd_b[(size_t)col * ns + s];
    }
    return;
  }
  const int G = a.groups;
  const size_t ubase = (size_t)act * G;
  // stage the transforms of groups that have observations
  for (int g = 0; g < tsm_groups; g++) {
    if (a.nkept[ubase + g] <= 0) continue;
    if ((k & 1) == 0) {   // k*k and every T offset are multiples of 4 floats
      const float4 *src = reinterpret_cast<const float4 *>(a.T + (ubase + g) * k * k);
      float4 *dst = reinterpret_cast<float4 *>(Ts + (size_t)g * k * k);
      for (int t = threadIdx.x; t < (k * k) / 4; t += blockDim.x) dst[t] = src[t];
    } else {
      for (int t = threadIdx.x; t < k * k; t += blockDim.x) Ts[(size_t)g * k * k + t] = a.T[(ubase + g) * k * k + t];
    }
  }
  __syncthreads();
  const int mld = a.cp[col].mld;
  const float kf = (float)k, km1 = (float)(k - 1);
  for (int s = warp; s < ns; s += nw) {
    const int v = a.slab_var[s], lev = a.slab_lev[s];
    int g = 0;
    if (a.loc_cls == LOC_VTGC) g = lev;
    else if (a.loc_cls == LOC_OCEAN && a.vtloc_surf == 1) g = (lev + 1 <= mld) ? 0 : 1;
    const bool has = g < G && a.nkept[ubase + g] > 0;
    const float *xbp = a.bkg + cbase + (size_t)s * k;
    const int j0 = lane, j1 = lane + 32;
    const float xb0 = j0 < k ? xbp[j0] : 0.0f;
    const float xb1 = j1 < k ? xbp[j1] : 0.0f;
    float x0 = xb0, x1 = xb1;
    if (has) {
      const float *T = (g < tsm_groups) ? Ts + (size_t)g * k * k : a.T + (ubase + g) * k * k;
      float acc0 = 0.0f, acc1 = 0.0f;
      const int i1max = k < 32 ? k : 32;
      for (int i = 0; i < i1max; i++) {
        const float xi = __shfl_sync(0xffffffffu, xb0, i);
        if (j0 < k) acc0 = __fmaf_rn(xi, T[i * k + j0], acc0);
        if (j1 < k) acc1 = __fmaf_rn(xi, T[i * k + j1], acc1);
      }
      for (int i = 32; i < k; i++) {
        const float xi = __shfl_sync(0xffffffffu, xb1, i - 32);
        if (j0 < k) acc0 = __fmaf_rn(xi, T[i * k + j0], acc0);
        if (j1 < k) acc1 = __fmaf_rn(xi, T[i * k + j1], acc1);
      }
      x0 = j0 < k ? acc0 : 0.0f;
      x1 = j1 < k ? acc1 : 0.0f;
    }
    const float mb = a.mean_b[(size_t)col * ns + s], sb = a.sprd_b[(size_t)col * ns + s];
    // recenter
    if (j0 < k) x0 = x0 + mb;
    if (j1 < k) x1 = x1 + mb;
    float m = bsum(x0 + x1) / kf;
    if (j0 < k) x0 = x0 - m;
    if (j1 < k) x1 = x1 - m;
    // clip the increment of the mean
    const float inc = a.var_inc_max[v], lb = a.var_lb[v], ub = a.var_ub[v];
    {
      float r = m - mb;
      r = fmaxf(r, -inc); r = fminf(r, inc);
      r = fmaxf(r, lb - mb); r = fminf(r, ub - mb);
      m = r + mb;
    }
    // RTPS
    if (a.rtps > 0.0f) {
      const float sa = sqrtf(bsum(x0 * x0 + x1 * x1) / km1);
      if (sa > 0.0f) {
        const float f = a.rtps * (sb - sa) / sa + 1.0f;
        x0 = x0 * f; x1 = x1 * f;
      }
    }
    // RTPP
    if (a.rtpp > 0.0f) {
      x0 = a.rtpp * xb0 + (1.0f - a.rtpp) * x0;
      x1 = a.rtpp * xb1 + (1.0f - a.rtpp) * x1;
    }
    // multiplicative
    if (a.mul != 1.0f) { x0 = x0 * a.mul; x1 = x1 * a.mul; }
    // member bounds and re-mean
    {
      if (j0 < k) { x0 = fmaxf(x0, lb - m); x0 = fminf(x0, ub - m); }
      if (j1 < k) { x1 = fmaxf(x1, lb - m); x1 = fminf(x1, ub - m); }
      const float r = bsum(x0 + x1) / kf;
      if (j0 < k) x0 = x0 - r;
      if (j1 < k) x1 = x1 - r;
      m = m + r;
    }
    // spread, add the mean
    const float sa = sqrtf(bsum(x0 * x0 + x1 * x1) / km1);
    float *xa = a.ana + cbase + (size_t)s * k;
    if (j0 < k) xa[j0] = x0 + m;
    if (j1 < k) xa[j1] = x1 + m;
    if (lane == 0) {
      a.mean_a[(size_t)col * ns + s] = m;
      a.sprd_a[(size_t)col * ns + s] = sa;
      if (!isfinite(m) || !isfinite(sa)) atomicOr(a.status, 4);
    }
  }
}

}  // namespace

cudaError_t launch_update(cudaStream_t st, const UpdateArgs &a, int *launches) {
  if (a.ncol <= 0) return cudaSuccess;
  const size_t per = (size_t)a.k * a.k * sizeof(float);
  int tg = a.groups;
  while (tg > 0 && tg * per > 64 * 1024) tg--;
  const size_t smem = tg * per;
  cudaError_t e = cudaFuncSetAttribute(k_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem > 0 ? smem : 16));
  if (e != cudaSuccess) return e;
  k_update<<<a.ncol, UT, smem, st>>>(a, tg);
  (*launches)++;
  return cudaGetLastError();
}

}  // namespace lgpu
