// lgpu_update.cu -- ensemble update and analysis epilogue, one CTA per column.
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
//
// The column's background perturbations (ns x k, contiguous) and its group
// transforms are staged in shared memory with 16-byte loads; X_b T is formed
// four members per thread from float4 rows of T; the epilogue runs one warp
// per slab with a fixed butterfly order for the member sums.
#include "lgpu_internal.cuh"
#include "lgpu_tc.cuh"

namespace lgpu {

namespace {

constexpr int UT = 128;  // 4 warps per column

__device__ __forceinline__ float bsum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int slab_group(const UpdateArgs &a, int lev, int mld) {
  if (a.loc_cls == LOC_VTGC) return lev;
  if (a.loc_cls == LOC_OCEAN && a.vtloc_surf == 1) return (lev + 1 <= mld) ? 0 : 1;
  return 0;
}

// Epilogue of one slab, one warp (lane owns members lane + 32 q, q < NQ:
// NQ = 2 for k <= 64, 4 for k <= 128): recenter, mean-increment clip, RTPS,
// RTPP, multiplicative inflation, member bounds and re-mean, spread; writes
// the analysis members, mean and spread of (col, s).  xr: X_b T row, br:
// background perturbation row.
template <int NQ>
__device__ __forceinline__ void slab_epilogue(const UpdateArgs &a, int col, int s, const float *xr, const float *br,
                                              int lane) {
  const int k = a.k, ns = a.ns;
  const float kf = (float)k, km1 = (float)(k - 1);
  const size_t cbase = (size_t)col * ns * k;
  const int v = a.slab_var[s];
  float x[NQ], xb[NQ];
  bool on[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int j = lane + 32 * q;
    on[q] = j < k;
    x[q] = on[q] ? xr[j] : 0.0f;
    xb[q] = on[q] ? br[j] : 0.0f;
  }
  auto lsum = [&](auto f) {
    float t = f(0);
#pragma unroll
    for (int q = 1; q < NQ; q++) t = t + f(q);
    return bsum(t);
  };
  const float mb = a.mean_b[(size_t)col * ns + s], sb = a.sprd_b[(size_t)col * ns + s];
#pragma unroll
  for (int q = 0; q < NQ; q++)
    if (on[q]) x[q] = x[q] + mb;
  float m = lsum([&](int q) { return x[q]; }) / kf;
#pragma unroll
  for (int q = 0; q < NQ; q++)
    if (on[q]) x[q] = x[q] - m;
  const float inc = a.var_inc_max[v], lb = a.var_lb[v], ub = a.var_ub[v];
  {
    float r = m - mb;
    r = fmaxf(r, -inc); r = fminf(r, inc);
    r = fmaxf(r, lb - mb); r = fminf(r, ub - mb);
    m = r + mb;
  }
  if (a.rtps > 0.0f) {
    const float sa = sqrtf(lsum([&](int q) { return x[q] * x[q]; }) / km1);
    if (sa > 0.0f) {
      const float f = a.rtps * (sb - sa) / sa + 1.0f;
#pragma unroll
      for (int q = 0; q < NQ; q++) x[q] = x[q] * f;
    }
  }
  if (a.rtpp > 0.0f) {
#pragma unroll
    for (int q = 0; q < NQ; q++) x[q] = a.rtpp * xb[q] + (1.0f - a.rtpp) * x[q];
  }
  if (a.mul != 1.0f) {
#pragma unroll
    for (int q = 0; q < NQ; q++) x[q] = x[q] * a.mul;
  }
  {
#pragma unroll
    for (int q = 0; q < NQ; q++)
      if (on[q]) { x[q] = fmaxf(x[q], lb - m); x[q] = fminf(x[q], ub - m); }
    const float r = lsum([&](int q) { return x[q]; }) / kf;
#pragma unroll
    for (int q = 0; q < NQ; q++)
      if (on[q]) x[q] = x[q] - r;
    m = m + r;
  }
  const float sa = sqrtf(lsum([&](int q) { return x[q] * x[q]; }) / km1);
  float *out = a.ana + cbase + (size_t)s * k;
#pragma unroll
  for (int q = 0; q < NQ; q++)
    if (on[q]) out[lane + 32 * q] = x[q] + m;
  if (lane == 0) {
    a.mean_a[(size_t)col * ns + s] = m;
    a.sprd_a[(size_t)col * ns + s] = sa;
    if (!isfinite(m) || !isfinite(sa)) atomicOr(a.status, 4);
  }
}

// smem: xb [ns][kp], xa [ns][kp], T [tg][k][kp]
template <int NQ>
__global__ void __launch_bounds__(UT) k_update(UpdateArgs a, int tsm_groups, int kp) {
  extern __shared__ __align__(16) float sm[];
  const int col = a.col0 + blockIdx.x;
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
  float *xb = sm;
  float *xa = xb + (size_t)ns * kp;
  float *Ts = xa + (size_t)ns * kp;
  const int G = a.groups;
  const size_t ubase = (size_t)act * G;
  const int mld = a.cp[col].mld;
  // ---- stage X_b (rows padded to kp) and the transforms
  if (kp == k) {   // k a multiple of 4: rows are already 16-byte aligned and unpadded
    const float4 *src = reinterpret_cast<const float4 *>(a.bkg + cbase);
    float4 *dst = reinterpret_cast<float4 *>(xb);
    for (int t = threadIdx.x; t < (ns * k) >> 2; t += blockDim.x) dst[t] = src[t];
  } else {
    for (int s = warp; s < ns; s += nw)
      for (int j = lane; j < kp; j += 32) xb[s * kp + j] = j < k ? a.bkg[cbase + (size_t)s * k + j] : 0.0f;
  }
  for (int g = 0; g < tsm_groups; g++) {
    if (a.nkept[ubase + g] <= 0) continue;
    const float *T = a.T + (ubase + g) * k * k;
    float *dst = Ts + (size_t)g * k * kp;
    if (kp == k) {
      const float4 *src4 = reinterpret_cast<const float4 *>(T);
      float4 *dst4 = reinterpret_cast<float4 *>(dst);
      for (int t = threadIdx.x; t < (k * k) >> 2; t += blockDim.x) dst4[t] = src4[t];
    } else {
      for (int i = warp; i < k; i += nw)
        for (int j = lane; j < kp; j += 32) dst[i * kp + j] = j < k ? T[i * k + j] : 0.0f;
    }
  }
  __syncthreads();
  // ---- X_a = X_b T_g: a warp covers spl slabs per pass, a lane one quad of members
  const int q4 = kp >> 2;
  const int spl = 32 / q4;
  const int my_s = lane / q4, jq = lane - my_s * q4;
  const bool lane_on = my_s < spl;
  for (int s0 = warp * spl; s0 < ns; s0 += nw * spl) {
    const int s = s0 + my_s;
    if (!lane_on || s >= ns) continue;
    const int g = slab_group(a, a.slab_lev[s], mld);
    const bool has = g < G && a.nkept[ubase + g] > 0;
    float4 acc;
    if (has) {
      const float *T = (g < tsm_groups) ? Ts + (size_t)g * k * kp : nullptr;
      const float *Tg = a.T + (ubase + g) * k * k;
      const float *xr = xb + (size_t)s * kp;
      acc = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int i = 0; i < k; i++) {
        const float xi = xr[i];
        float4 tv;
        if (T) {
          tv = reinterpret_cast<const float4 *>(T + (size_t)i * kp)[jq];
        } else {
          const int j = 4 * jq;
          tv.x = j < k ? Tg[i * k + j] : 0.f;
          tv.y = j + 1 < k ? Tg[i * k + j + 1] : 0.f;
          tv.z = j + 2 < k ? Tg[i * k + j + 2] : 0.f;
          tv.w = j + 3 < k ? Tg[i * k + j + 3] : 0.f;
        }
        acc.x = __fmaf_rn(xi, tv.x, acc.x);
        acc.y = __fmaf_rn(xi, tv.y, acc.y);
        acc.z = __fmaf_rn(xi, tv.z, acc.z);
        acc.w = __fmaf_rn(xi, tv.w, acc.w);
      }
    } else {
      acc = reinterpret_cast<const float4 *>(xb + (size_t)s * kp)[jq];
    }
    reinterpret_cast<float4 *>(xa + (size_t)s * kp)[jq] = acc;
  }
  __syncthreads();
  // ---- epilogue, one warp per slab
  for (int s = warp; s < ns; s += nw) slab_epilogue<NQ>(a, col, s, xa + (size_t)s * kp, xb + (size_t)s * kp, lane);
}

// Thread-per-slab form for k a multiple of 4 (k <= KMAX): one CTA per
// column, TPS threads per slab (1, or 2 for large k, where the k member
// accumulators of one thread would limit the CTAs per SM by registers).  The
// column's background block (ns x k floats, contiguous) and its group
// transforms arrive in shared memory by two bulk async copies completing on
// one mbarrier; the slab's analysis members stay in registers (with TPS = 2
// the even thread holds members [0, sp), the odd one [sp, k)).  The
// epilogue's member sums run sequentially in member order (the reference's
// SUM): with TPS = 2 the odd thread continues the even thread's partial sum,
// so the order and the result are those of one thread.  The analysis block is
// written back over the background block in shared memory and leaves by one
// bulk async store.  A copy wait that runs out sets status bit 64.
template <int KMAX, int TPS>
__global__ void __launch_bounds__(256, TPS) k_update_rows(UpdateArgs a) {
  extern __shared__ __align__(128) float usm[];   // X [ns][k] | T [groups][k][k]
  __shared__ __align__(8) uint64_t bar;
  constexpr int KH = KMAX / TPS;   // members per thread (a multiple of 4)
  const int col = a.col0 + blockIdx.x;
  const int k = a.k, ns = a.ns, G = a.groups, kk = k * k;
  const int s = threadIdx.x / TPS, half = TPS == 2 ? (threadIdx.x & 1) : 0;
  const int lane = threadIdx.x & 31;
  // this thread's members [jb, jb + nj)
  const int sp = TPS == 2 ? ((k + 7) / 8) * 4 : k;
  const int jb = half ? sp : 0, nj = half ? k - sp : sp, nj4 = nj >> 2;
  const size_t cbase = (size_t)col * ns * k;
  const int act = a.col2act[col];
  const bool skip = a.mask[col] || act < 0;
  float *Xs = usm;
  const float *Tsm = usm + (size_t)ns * k;
  const uint32_t xbytes = (uint32_t)(ns * k * 4), tbytes = skip ? 0u : (uint32_t)(G * kk * 4);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(&bar)),
                 "r"(xbytes + tbytes) : "memory");
    tc::bulk_copy_g2s(Xs, a.bkg + cbase, xbytes, &bar);
    if (tbytes) tc::bulk_copy_g2s(usm + (size_t)ns * k, a.T + (size_t)act * G * kk, tbytes, &bar);
  }
  const bool landed = __syncthreads_and(tc::mbar_wait(&bar, 0));
  if (!landed) {
    if (threadIdx.x == 0) {
      atomicOr(a.status, 64);
      tc::mbar_wait(&bar, 0);   // the copies in flight land before the CTA exits
    }
    return;
  }
  // lanes whose slab exists (both threads of a slab share it)
  const unsigned amask = __ballot_sync(0xffffffffu, s < ns);
  // sequential member reduction acc = step(acc, j) over [0, k) from 0: the
  // even thread's partial is continued by the odd thread, whose total both
  // receive (step is written as the reference's expression, e.g. acc + x*x)
  auto msum = [&](auto step) -> float {
    float acc = 0.0f;
    if (TPS == 1) {
#pragma unroll
      for (int j = 0; j < KH; j++)
        if (j < nj) acc = step(acc, j);
      return acc;
    }
    if (half == 0) {
#pragma unroll
      for (int j = 0; j < KH; j++)
        if (j < nj) acc = step(acc, j);
    }
    const float from0 = __shfl_sync(amask, acc, lane & ~1);
    if (half == 1) {
      acc = from0;
#pragma unroll
      for (int j = 0; j < KH; j++)
        if (j < nj) acc = step(acc, j);
    }
    return __shfl_sync(amask, acc, lane | 1);
  };
  const size_t ms = (size_t)col * ns + s;
  if (s < ns) {
    const float4 *xb4 = reinterpret_cast<const float4 *>(Xs + (size_t)s * k + jb);
    float4 *out4 = reinterpret_cast<float4 *>(Xs + (size_t)s * k + jb);
    if (skip) {   // src/letkf_solver.F90:207: the block leaves unchanged
      if (half == 0) {
        a.mean_a[ms] = a.mean_b[ms];
        a.sprd_a[ms] = a.sprd_b[ms];
      }
    } else {
      const int g = slab_group(a, a.slab_lev[s], a.cp[col].mld);
      const bool has = g < G && a.nkept[(size_t)act * G + g] > 0;
      float x[KH];
#pragma unroll
      for (int j = 0; j < KH; j++) x[j] = 0.0f;
      if (has) {
        // x_a = x_b T_g (src/letkf_solver.F90:285-289), members accumulated in i order
        const float *T = Tsm + (size_t)g * kk + jb;
        const float4 *xr4 = reinterpret_cast<const float4 *>(Xs + (size_t)s * k);
        for (int i4 = 0; i4 < (k >> 2); i4++) {
          const float4 xv = xr4[i4];
          const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const float4 *Tr = reinterpret_cast<const float4 *>(T + (size_t)(4 * i4 + u) * k);
#pragma unroll
            for (int q = 0; q < KH / 4; q++) {
              if (q < nj4) {
                const float4 t = Tr[q];
                x[4 * q + 0] = __fmaf_rn(xs[u], t.x, x[4 * q + 0]);
                x[4 * q + 1] = __fmaf_rn(xs[u], t.y, x[4 * q + 1]);
                x[4 * q + 2] = __fmaf_rn(xs[u], t.z, x[4 * q + 2]);
                x[4 * q + 3] = __fmaf_rn(xs[u], t.w, x[4 * q + 3]);
              }
            }
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < KH / 4; q++)
          if (q < nj4) {
            const float4 v = xb4[q];
            x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
          }
      }
      const float kf = (float)k, km1 = (float)(k - 1);
      const int v = a.slab_var[s];
      const float mb = a.mean_b[ms], sb = a.sprd_b[ms];
      // recenter (:299-303)
#pragma unroll
      for (int j = 0; j < KH; j++)
        if (j < nj) x[j] = x[j] + mb;
      float m = msum([&](float acc, int j) { return acc + x[j]; });
      m = m / kf;
#pragma unroll
      for (int j = 0; j < KH; j++) x[j] = x[j] - m;
      // mean increment clip and bounds (:308-318)
      const float inc = a.var_inc_max[v], lb = a.var_lb[v], ub = a.var_ub[v];
      {
        float r = m - mb;
        r = fmaxf(r, -inc); r = fminf(r, inc);
        r = fmaxf(r, lb - mb); r = fminf(r, ub - mb);
        m = r + mb;
      }
      if (a.rtps > 0.0f) {   // (:322-335)
        const float q2 = msum([&](float acc, int j) { return acc + x[j] * x[j]; });
        const float sa = sqrtf(q2 / km1);
        if (sa > 0.0f) {
          const float f = a.rtps * (sb - sa) / sa + 1.0f;
#pragma unroll
          for (int j = 0; j < KH; j++) x[j] = x[j] * f;
        }
      }
      if (a.rtpp > 0.0f) {   // (:339-344)
#pragma unroll
        for (int q = 0; q < KH / 4; q++)
          if (q < nj4) {
            const float4 b = xb4[q];
            x[4 * q + 0] = a.rtpp * b.x + (1.0f - a.rtpp) * x[4 * q + 0];
            x[4 * q + 1] = a.rtpp * b.y + (1.0f - a.rtpp) * x[4 * q + 1];
            x[4 * q + 2] = a.rtpp * b.z + (1.0f - a.rtpp) * x[4 * q + 2];
            x[4 * q + 3] = a.rtpp * b.w + (1.0f - a.rtpp) * x[4 * q + 3];
          }
      }
      if (a.mul != 1.0f) {   // (:347-349)
#pragma unroll
        for (int j = 0; j < KH; j++) x[j] = x[j] * a.mul;
      }
      {   // member bounds and re-mean (:357-371)
#pragma unroll
        for (int j = 0; j < KH; j++)
          if (j < nj) x[j] = fminf(fmaxf(x[j], lb - m), ub - m);
        float r = msum([&](float acc, int j) { return acc + x[j]; });
        r = r / kf;
#pragma unroll
        for (int j = 0; j < KH; j++) x[j] = x[j] - r;
        m = m + r;
      }
      // spread (:375-379)
      const float q2 = msum([&](float acc, int j) { return acc + x[j] * x[j]; });
      const float sa = sqrtf(q2 / km1);
#pragma unroll
      for (int q = 0; q < KH / 4; q++)
        if (q < nj4) out4[q] = make_float4(x[4 * q] + m, x[4 * q + 1] + m, x[4 * q + 2] + m, x[4 * q + 3] + m);
      if (half == 0) {
        a.mean_a[ms] = m;
        a.sprd_a[ms] = sa;
        if (!isfinite(m) || !isfinite(sa)) atomicOr(a.status, 4);
      }
    }
  }
  // the analysis block (generic-proxy writes) -> global by the async proxy
  tc::fence_proxy_async();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::bulk_store_s2g(a.ana + cbase, Xs, xbytes);
    tc::bulk_commit();
    tc::bulk_wait_all();
  }
}

}  // namespace

cudaError_t launch_update(cudaStream_t st, const UpdateArgs &a, int *launches) {
  if (a.ncol <= 0 || a.ncols <= 0) return cudaSuccess;
  {
    const cudaError_t e = launch_update_tc(st, a, launches);   // the tensor-core form where it applies
    if (e != cudaErrorNotSupported) return e;
  }
  const size_t rbytes = ((size_t)a.ns * a.k + (size_t)a.groups * a.k * a.k) * sizeof(float);
  if (a.k % 4 == 0 && a.ns <= 256 && rbytes <= 200 * 1024) {
    const int k = a.k;
    // above k = 64 two threads per slab (when the slabs fit one CTA)
    const int tps = k > 64 && 2 * a.ns <= 256 ? 2 : 1;
    const int nt = (tps * a.ns + 31) & ~31;
    auto kern = k <= 8    ? k_update_rows<8, 1>
                : k <= 16 ? k_update_rows<16, 1>
                : k <= 24 ? k_update_rows<24, 1>
                : k <= 32 ? k_update_rows<32, 1>
                : k <= 40 ? k_update_rows<40, 1>
                : k <= 48 ? k_update_rows<48, 1>
                : k <= 56 ? k_update_rows<56, 1>
                : k <= 64 ? k_update_rows<64, 1>
                : k <= 80 ? (tps == 2 ? k_update_rows<80, 2> : k_update_rows<80, 1>)
                : k <= 96 ? (tps == 2 ? k_update_rows<96, 2> : k_update_rows<96, 1>)
                : k <= 112 ? (tps == 2 ? k_update_rows<112, 2> : k_update_rows<112, 1>)
                           : (tps == 2 ? k_update_rows<128, 2> : k_update_rows<128, 1>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rbytes);
    if (e != cudaSuccess) return e;
    kern<<<a.ncols, nt, rbytes, st>>>(a);
    (*launches)++;
    return cudaGetLastError();
  }
  const int kp = (a.k + 3) & ~3;
  const size_t xbytes = 2 * (size_t)a.ns * kp * sizeof(float);
  const size_t per = (size_t)a.k * kp * sizeof(float);
  const size_t budget = 200 * 1024;
  if (xbytes > budget) return cudaErrorInvalidValue;   // checked by the caller
  int tg = a.groups;
  while (tg > 0 && xbytes + tg * per > budget) tg--;
  const size_t smem = xbytes + tg * per;
  auto kern = a.k > 64 ? k_update<4> : k_update<2>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<a.ncols, UT, smem, st>>>(a, tg, kp);
  (*launches)++;
  return cudaGetLastError();
}

}  // namespace lgpu
