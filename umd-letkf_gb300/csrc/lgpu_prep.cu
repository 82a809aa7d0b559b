// lgpu_prep.cu -- the pre-processing immediately upstream of the analysis,
// on the device:
//   src/letkf_obs.F90:459-488   hx_mean = SUM(hx,1)/k, hx' = hx - hx_mean,
//                               then drop qc > 0 observations keeping order
//   src/letkf_state.F90:326-334 mean = SUM(x,1)/k, x' = x - mean,
//                               sprd = SQRT(DOT(x',x')/(k-1))
// Sums run over members in order with explicitly rounded float operations,
// the reference's REAL arithmetic.
#include "lgpu_internal.cuh"

namespace lgpu {

namespace {

// per observation: member mean and perturbations in place; keep flag
__global__ void k_hx_stats(int nobs, int k, float *hx, float *hx_mean, const int *qc, int *flag) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nobs) return;
  float *h = hx + (size_t)o * k;
  float sum = 0.0f;
  for (int m = 0; m < k; m++) sum = __fadd_rn(sum, h[m]);
  const float mean = __fdiv_rn(sum, (float)k);
  for (int m = 0; m < k; m++) h[m] = __fsub_rn(h[m], mean);
  hx_mean[o] = mean;
  flag[o] = qc ? (qc[o] > 0 ? 0 : 1) : 1;   // obs_def(i)%qc > 0 is dropped
}

// exclusive scan of the keep flags, one block (order preserving)
__global__ void k_flag_scan(int n, const int *flag, int *pos, int *total) {
  __shared__ int wsum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < n ? flag[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int s = lane < nw ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    const int excl = carry + (w > 0 ? wsum[w - 1] : 0) + x - v;
    if (i < n) pos[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// compaction: i -> pos[i] for kept observations (pos[i] <= i, so the
// destination arrays are separate)
__global__ void k_compact(int nobs, int k, const int *flag, const int *pos, const float *const *src_f, float *const *dst_f,
                          int nf, const int *const *src_i, int *const *dst_i, int ni, const float *hx, float *hx_out,
                          const float *hxm, float *hxm_out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nobs * (k + 1)) return;
  const int o = (int)(t / (k + 1)), m = (int)(t % (k + 1));
  if (!flag[o]) return;
  const int p = pos[o];
  if (m < k) {
    hx_out[(size_t)p * k + m] = hx[(size_t)o * k + m];
  } else {
    hxm_out[p] = hxm[o];
    for (int q = 0; q < nf; q++) dst_f[q][p] = src_f[q][o];
    for (int q = 0; q < ni; q++) dst_i[q][p] = src_i[q][o];
  }
}

// per (column, slab): background mean, perturbations in place, spread
__global__ void k_state_stats(long long ncs, int k, float *x, float *mean, float *sprd) {
  const long long cs = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cs >= ncs) return;
  float *v = x + cs * k;
  float sum = 0.0f;
  for (int m = 0; m < k; m++) sum = __fadd_rn(sum, v[m]);
  const float mu = __fdiv_rn(sum, (float)k);
  float dot = 0.0f;
  for (int m = 0; m < k; m++) {
    const float p = __fsub_rn(v[m], mu);
    v[m] = p;
    dot = __fadd_rn(dot, __fmul_rn(p, p));
  }
  mean[cs] = mu;
  sprd[cs] = __fsqrt_rn(__fdiv_rn(dot, (float)(k - 1)));
}

}  // namespace

cudaError_t launch_hx_stats(cudaStream_t st, int nobs, int k, float *hx, float *hx_mean, const int *qc, int *flag,
                            int *pos, int *total) {
  if (nobs <= 0) return cudaMemsetAsync(total, 0, sizeof(int), st);
  k_hx_stats<<<(nobs + 255) / 256, 256, 0, st>>>(nobs, k, hx, hx_mean, qc, flag);
  k_flag_scan<<<1, 1024, 0, st>>>(nobs, flag, pos, total);
  return cudaGetLastError();
}

cudaError_t launch_compact(cudaStream_t st, int nobs, int k, const int *flag, const int *pos, const float *const *src_f,
                           float *const *dst_f, int nf, const int *const *src_i, int *const *dst_i, int ni,
                           const float *hx, float *hx_out, const float *hxm, float *hxm_out) {
  if (nobs <= 0) return cudaSuccess;
  const long long n = (long long)nobs * (k + 1);
  k_compact<<<(int)((n + 255) / 256), 256, 0, st>>>(nobs, k, flag, pos, src_f, dst_f, nf, src_i, dst_i, ni, hx, hx_out,
                                                      hxm, hxm_out);
  return cudaGetLastError();
}

cudaError_t launch_state_stats(cudaStream_t st, long long ncs, int k, float *x, float *mean, float *sprd) {
  if (ncs <= 0) return cudaSuccess;
  k_state_stats<<<(int)((ncs + 255) / 256), 256, 0, st>>>(ncs, k, x, mean, sprd);
  return cudaGetLastError();
}

}  // namespace lgpu
