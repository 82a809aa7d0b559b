// lgpu_learn.cu -- kernels of the learned analysis form.
//
// The reference solves every grid column exactly (src/letkf_solver.F90:
// 203-384, one letkf_core_solve per column and group).  The learned form
// solves exactly only the columns of a coarse lattice (every s-th column in
// longitude and latitude), a random judge sample and the columns its
// confidence gate sends back; every other column gets the bilinear
// interpolation of the coarse solutions (W, w-bar) plus a correction from
// the network of lgpu_mlp.cu.  The analysis update itself is unchanged.
//
//   k_lrn_cellstats, k_lrn_obsfeat  per column: the observation-geometry
//                  features (local count, sums of localisation weights,
//                  nearest distance, innovation moments) from per-cell
//                  aggregates of the observation index and the same
//                  localizer as the exact path
//   k_lrn_interp   per column: the bilinear (W, w-bar) of the four coarse
//                  neighbours, the network input row and, while collecting
//                  training data, the residual target exact - interpolated
//   k_lrn_apply    per column: interpolation + de-standardised correction ->
//                  T = W + w-bar 1^T, the gate score, the fallback list
//   k_lrn_judge, k_lrn_scatter  judge errors; exact transforms into place
//   k_lrn_colstats, k_lrn_batch  training-set standardisation and batches
#include "lgpu_internal.cuh"
#include <cuda_bf16.h>

namespace lgpu {

namespace {

constexpr int FT = 128;   // threads of the per-column kernels

__device__ __forceinline__ float bsum128(float v, float *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  return red[0] + red[1] + red[2] + red[3];
}

__device__ __forceinline__ float bmax128(float v, float *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  return fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
}

__device__ __forceinline__ float bmin128(float v, float *red) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  return fminf(fminf(red[0], red[1]), fminf(red[2], red[3]));
}

// Per-cell aggregates of the cell-sorted observation table: centroid
// direction (sum of unit vectors) and count; sums of dep, dep^2, 1/err,
// dep/err.  One thread per cell.
__global__ void k_lrn_cellstats(int ncell, ObsSorted obs, float4 *c0, float4 *c1) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int b = obs.cell_start[c], e = obs.cell_start[c + 1];
  float sx = 0.f, sy = 0.f, sz = 0.f, sd = 0.f, sd2 = 0.f, si = 0.f, sdi = 0.f;
  for (int p = b; p < e; p++) {
    const float4 A = obs.A[p];
    const float dep = obs.B[p].x, ie = 1.0f / A.w;
    sx += A.x; sy += A.y; sz += A.z;
    sd += dep; sd2 += dep * dep; si += ie; sdi += dep * ie;
  }
  c0[c] = make_float4(sx, sy, sz, (float)(e - b));
  c1[c] = make_float4(sd, sd2, si, sdi);
}

// Observation-geometry features of column cols[f] from the cell aggregates
// of its search window (one warp per column; a cell's observations are
// taken at the cell's centroid):
//   0 count within the search radius / 100   1 sum rho / 100
//   2 sum rho/err / 1000   3 nearest centroid distance / search radius (1 if none)
//   4 mean dep   5 variance of dep   6 rho-weighted mean dep
//   7 (rho/err)-weighted mean dep   8 max rho   9 mean rho
// (features 10-15 are filled by k_lrn_interp)
__global__ void __launch_bounds__(FT) k_lrn_obsfeat(int nfine, const int *cols, const ColPar *cps, DevLoc loc,
                                                    const int *cell_start, const float4 *c0, const float4 *c1,
                                                    const IndexGeom *geom, float *feat, int *nkept) {
  const int lane = threadIdx.x & 31;
  const int f = blockIdx.x * (FT / 32) + (threadIdx.x >> 5);
  if (f >= nfine) return;   // whole warps
  const int col = cols[f];
  const ColPar cp = cps[col];
  float n = 0.f, sr = 0.f, sre = 0.f, dmin = 3.0e38f, sd = 0.f, sd2 = 0.f, srd = 0.f, sred = 0.f, rmx = 0.f;
  for (int b = cp.b0; b <= cp.b1; b++) {
    const int nl = geom->nlon[b], off = geom->off[b];
    int lo = 0, cnt = nl;
    if (cp.dlon < 180.0f) {
      const int clo = (int)floorf((cp.lonn - cp.dlon) * (float)nl / 360.0f);
      const int chi = (int)floorf((cp.lonn + cp.dlon) * (float)nl / 360.0f);
      if (chi - clo + 1 < nl) { lo = clo; cnt = chi - clo + 1; }
    }
    for (int q = lane; q < cnt; q += 32) {
      const int cell = off + (((lo + q) % nl) + nl) % nl;
      const float4 A = c0[cell];
      if (A.w <= 0.0f) continue;
      const float inv = rsqrtf(A.x * A.x + A.y * A.y + A.z * A.z);
      const float d = dist_from_chord2(chord2_exact(cp.ux, cp.uy, cp.uz, A.x * inv, A.y * inv, A.z * inv));
      if (d > cp.rmax) continue;
      const float r = localize(loc, cp, 0, d, 0.0f, 0.0f, 0.0f);
      if (!(r > kKeep)) continue;
      const float4 B = c1[cell];
      n += A.w;
      sr += r * A.w;
      sre += r * B.z;
      dmin = fminf(dmin, d);
      sd += B.x;
      sd2 += B.y;
      srd += r * B.x;
      sred += r * B.w;
      rmx = fmaxf(rmx, r);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    n += __shfl_xor_sync(0xffffffffu, n, o);
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    sre += __shfl_xor_sync(0xffffffffu, sre, o);
    sd += __shfl_xor_sync(0xffffffffu, sd, o);
    sd2 += __shfl_xor_sync(0xffffffffu, sd2, o);
    srd += __shfl_xor_sync(0xffffffffu, srd, o);
    sred += __shfl_xor_sync(0xffffffffu, sred, o);
    dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    rmx = fmaxf(rmx, __shfl_xor_sync(0xffffffffu, rmx, o));
  }
  if (lane == 0) {
    float *o = feat + (size_t)f * 16;
    const float nn = fmaxf(n, 1.0f);
    const float m = sd / nn;
    o[0] = n / 100.0f;
    o[1] = sr / 100.0f;
    o[2] = sre / 1000.0f;
    o[3] = n > 0.0f ? dmin / cp.rmax : 1.0f;
    o[4] = m;
    o[5] = fmaxf(sd2 / nn - m * m, 0.0f);
    o[6] = sr > 0.0f ? srd / sr : 0.0f;
    o[7] = sre > 0.0f ? sred / sre : 0.0f;
    o[8] = rmx;
    o[9] = sr / nn;
    nkept[f] = (int)n;
  }
}

struct Nb {
  int src[4];
  float w[4];
  int missing;
  float fx, fy;
};

// the four coarse neighbours of column (i, j) on the lattice of stride s
// (periodic in longitude, clamped at the last coarse latitude row) and
// their bilinear weights; src = row of the coarse solution or -1
__device__ __forceinline__ Nb neighbours(int col, int nx, int ny, int s, const int *src_of_col) {
  Nb nb;
  const int i = col % nx, j = col / nx;
  const int i0 = (i / s) * s, j0 = (j / s) * s;
  const int i1 = (i0 + s) % nx;
  const int j1 = j0 + s < ny ? j0 + s : j0;
  nb.fx = (float)(i - i0) / (float)s;
  nb.fy = j1 != j0 ? (float)(j - j0) / (float)s : 0.0f;
  const int c[4] = {i0 + nx * j0, i1 + nx * j0, i0 + nx * j1, i1 + nx * j1};
  const float w[4] = {(1.0f - nb.fx) * (1.0f - nb.fy), nb.fx * (1.0f - nb.fy), (1.0f - nb.fx) * nb.fy, nb.fx * nb.fy};
  nb.missing = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    nb.src[q] = src_of_col[c[q]];
    nb.w[q] = w[q];
    if (w[q] > 0.0f && nb.src[q] < 0) nb.missing = 1;
  }
  return nb;
}

// interpolated W_ij (i < k, j < k) or w-bar_i (j == k) of the neighbours
__device__ __forceinline__ float interp_at(const Nb &nb, const float *Ts, const float *ws, int k, int i, int j) {
  float v = 0.0f;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (nb.w[q] == 0.0f || nb.src[q] < 0) continue;
    const float wb = ws[(size_t)nb.src[q] * k + i];
    const float t = j < k ? Ts[(size_t)nb.src[q] * k * k + (size_t)i * k + j] - wb : wb;
    v += nb.w[q] * t;
  }
  return v;
}

}  // namespace

namespace {

__global__ void __launch_bounds__(FT) k_lrn_interp(LrnInterpArgs a) {
  __shared__ float red[4];
  const int f = blockIdx.x;
  if (f >= a.nfine) return;
  const int col = a.cols[f], k = a.k, kk = k * k;
  const Nb nb = neighbours(col, a.nx, a.ny, a.s, a.src_of_col);
  float *x = a.X + (size_t)f * a.ldx;
  // interpolated W (row-major) and w-bar; spread of the neighbours around it
  float spread = 0.0f;
  for (int e = threadIdx.x; e < kk + k; e += FT) {
    const int i = e < kk ? e / k : e - kk, j = e < kk ? e % k : k;
    const float v = interp_at(nb, a.Ts, a.ws, k, i, j);
    if (e < kk) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (nb.w[q] == 0.0f || nb.src[q] < 0) continue;
        const float wb = a.ws[(size_t)nb.src[q] * k + i];
        const float d = a.Ts[(size_t)nb.src[q] * kk + (size_t)i * k + j] - wb - v;
        spread += nb.w[q] * d * d;
      }
    }
    x[e] = a.mu ? (v - a.mu[e]) / a.sd[e] : v;
    if (a.Yt) {
      const int act = a.col2act[col];
      const float ex = a.wex[(size_t)act * k + i];
      const float t = j < k ? a.Tex[(size_t)act * kk + (size_t)i * k + j] - ex : ex;
      a.Yt[(size_t)f * a.ldy + e] = t - v;
    }
  }
  spread = bsum128(spread, red);
  if (threadIdx.x < 16) {
    const int q = threadIdx.x;
    const float *fo = a.feat + (size_t)f * 16;
    float v;
    if (q < 10) v = fo[q];
    else if (q == 10) v = sinf(a.lat[col] * 0.017453292519943295f);
    else if (q == 11) v = cosf(a.lat[col] * 0.017453292519943295f);
    else if (q == 12) v = nb.fx;
    else if (q == 13) v = nb.fy;
    else if (q == 14) v = log1pf(100.0f * fo[0]);
    else v = sqrtf(spread) / (float)k;
    const int e = kk + k + q;
    x[e] = a.mu ? (v - a.mu[e]) / a.sd[e] : v;
  }
  if (threadIdx.x == 0) a.flag[f] = nb.missing;
}


__global__ void __launch_bounds__(FT) k_lrn_apply(LrnApplyArgs a) {
  __shared__ float red[4];
  __shared__ float wb_s[128];
  const int f = blockIdx.x;
  if (f >= a.nfine) return;
  const int col = a.cols[f], k = a.k, kk = k * k;
  const float *y = a.Yn + (size_t)f * a.ldy;
  float q2 = 0.0f;
  if (a.net)
    for (int e = threadIdx.x; e < a.dout; e += FT) q2 += y[e] * y[e];
  const float score = sqrtf(bsum128(q2, red) / (float)a.dout);
  const bool gated = a.flag[f] || (a.net && !(score <= a.tau));
  if (threadIdx.x == 0) {
    if (a.score) a.score[f] = score;
    if (gated) a.gate_cols[atomicAdd(a.gate_n, 1)] = col;
  }
  if (gated) return;   // CTA-uniform
  const Nb nb = neighbours(col, a.nx, a.ny, a.s, a.src_of_col);
  const int unit = a.col2act[col];
  // w-bar first (T's rows need it)
  for (int i = threadIdx.x; i < k; i += FT) {
    const int e = kk + i;
    wb_s[i] = interp_at(nb, a.Ts, a.ws, k, i, k) + (a.net ? a.mu_out[e] + a.sd_out[e] * y[e] : 0.0f);
  }
  __syncthreads();
  float *T = a.T + (size_t)unit * kk;
  for (int e = threadIdx.x; e < kk; e += FT) {
    const int i = e / k, j = e % k;
    const float w = interp_at(nb, a.Ts, a.ws, k, i, j) + (a.net ? a.mu_out[e] + a.sd_out[e] * y[e] : 0.0f);
    T[e] = w + wb_s[i];
  }
  if (threadIdx.x == 0) a.nkept[unit] = a.nk_fine[f];
}

// judge: squared error of the inferred T against the exact one, and the
// squared norm of the exact T - I, summed over judged columns (not gated)
__global__ void __launch_bounds__(FT) k_lrn_judge(int nj, const int *jcols, const int *jsub, const float *Tsub,
                                                  const float *T, const int *col2act, const int *gate_mark, int k,
                                                  float *acc) {
  __shared__ float red[4];
  const int f = blockIdx.x;
  if (f >= nj) return;
  const int col = jcols[f];
  if (gate_mark[col]) return;
  const int unit = col2act[col], kk = k * k;
  const float *te = Tsub + (size_t)jsub[f] * kk, *ti = T + (size_t)unit * kk;
  float e2 = 0.0f, r2 = 0.0f;
  for (int e = threadIdx.x; e < kk; e += FT) {
    const float d = ti[e] - te[e];
    const float r = te[e] - ((e / k) == (e % k) ? 1.0f : 0.0f);
    e2 += d * d;
    r2 += r * r;
  }
  e2 = bsum128(e2, red);
  r2 = bsum128(r2, red);
  if (threadIdx.x == 0) {
    atomicAdd(acc + 0, e2);
    atomicAdd(acc + 1, r2);
    atomicAdd(acc + 2, 1.0f);
  }
}

__global__ void k_lrn_mark(int n, const int *cols, int *mark, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mark[cols[i]] = v;
}

// exact transforms of a column list into the per-unit arrays
__global__ void k_lrn_scatter(int n, const int *cols, const int *col2act, const float *Tsub, const int *nk_sub, int k,
                              float *T, int *nkept) {
  const int kk = k * k;
  const long long total = (long long)n * kk;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int e = (int)(t / kk), q = (int)(t % kk);
    const int unit = col2act[cols[e]];
    T[(size_t)unit * kk + q] = Tsub[(size_t)e * kk + q];
    if (q == 0) nkept[unit] = nk_sub[e];
  }
}

// column means and standard deviations of a [rows][n] matrix (n columns,
// leading dimension ld), FP64 sums; sd floored at 1e-6 (and at 1e-3 of the
// largest sd of the matrix, so that constant inputs stay near zero)
__global__ void k_lrn_colstats(const float *M, long long rows, int n, long long ld, float *mu, float *sd) {
  __shared__ double s1[256], s2[256];
  const int c = blockIdx.x;
  double a = 0.0, b = 0.0;
  for (long long r = threadIdx.x; r < rows; r += blockDim.x) {
    const double v = M[r * ld + c];
    a += v;
    b += v * v;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      s1[threadIdx.x] += s1[threadIdx.x + o];
      s2[threadIdx.x] += s2[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = s1[0] / (double)(rows > 0 ? rows : 1);
    const double var = s2[0] / (double)(rows > 0 ? rows : 1) - m * m;
    mu[c] = (float)m;
    sd[c] = (float)sqrt(var > 0.0 ? var : 0.0);
  }
}

__global__ void k_lrn_sdfloor(float *sd, int n) {
  __shared__ float red[256];
  float m = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, sd[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  const float fl = fmaxf(1e-6f, 1e-3f * red[0]);
  for (int i = threadIdx.x; i < n; i += blockDim.x) sd[i] = fmaxf(sd[i], fl);
}

// training batch: rows idx[0..b) of the store, standardised; inputs rounded
// to BF16 (the network's input precision)
__global__ void k_lrn_batch(int b, const int *idx, const float *X, long long ldx, int din, const float *Y,
                            long long ldy, int dout, const float *mu, const float *sd, const float *muo,
                            const float *sdo, float *Xb, float *Yb) {
  const long long total = (long long)b * (din + dout);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / (din + dout)), c = (int)(t % (din + dout));
    const long long src = idx[r];
    if (c < din) {
      const float v = (X[src * ldx + c] - mu[c]) / sd[c];
      Xb[(size_t)r * din + c] = __bfloat162float(__float2bfloat16_rn(v));
    } else {
      const int o = c - din;
      Yb[(size_t)r * dout + o] = (Y[src * ldy + o] - muo[o]) / sdo[o];
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers

cudaError_t lrn_cellstats(cudaStream_t st, int ncell, const ObsSorted &obs, float4 *c0, float4 *c1, int *launches) {
  if (ncell <= 0) return cudaSuccess;
  k_lrn_cellstats<<<(ncell + 255) / 256, 256, 0, st>>>(ncell, obs, c0, c1);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t lrn_obsfeat(cudaStream_t st, int nfine, const int *cols, const ColPar *cp, const DevLoc &loc,
                        const int *cell_start, const float4 *c0, const float4 *c1, const IndexGeom *geom,
                        float *feat, int *nkept, int *launches) {
  if (nfine <= 0) return cudaSuccess;
  const int per = FT / 32;
  k_lrn_obsfeat<<<(nfine + per - 1) / per, FT, 0, st>>>(nfine, cols, cp, loc, cell_start, c0, c1, geom, feat, nkept);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t lrn_interp(cudaStream_t st, const LrnInterpArgs &a, int *launches) {
  if (a.nfine <= 0) return cudaSuccess;
  k_lrn_interp<<<a.nfine, FT, 0, st>>>(a);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t lrn_apply(cudaStream_t st, const LrnApplyArgs &a, int *launches) {
  if (a.nfine <= 0) return cudaSuccess;
  if (a.k > 128) return cudaErrorInvalidValue;
  k_lrn_apply<<<a.nfine, FT, 0, st>>>(a);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t lrn_judge(cudaStream_t st, int nj, const int *jcols, const int *jsub, const float *Tsub, const float *T,
                      const int *col2act, const int *gate_mark, int k, float *acc, int *launches) {
  if (nj <= 0) return cudaSuccess;
  k_lrn_judge<<<nj, FT, 0, st>>>(nj, jcols, jsub, Tsub, T, col2act, gate_mark, k, acc);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t lrn_mark(cudaStream_t st, int n, const int *cols, int *mark, int v) {
  if (n <= 0) return cudaSuccess;
  k_lrn_mark<<<(n + 255) / 256, 256, 0, st>>>(n, cols, mark, v);
  return cudaGetLastError();
}

cudaError_t lrn_scatter(cudaStream_t st, int n, const int *cols, const int *col2act, const float *Tsub,
                        const int *nk_sub, int k, float *T, int *nkept, int *launches) {
  if (n <= 0) return cudaSuccess;
  const long long total = (long long)n * k * k;
  const int grid = (int)std::min<long long>(4096, (total + 255) / 256);
  k_lrn_scatter<<<grid, 256, 0, st>>>(n, cols, col2act, Tsub, nk_sub, k, T, nkept);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t lrn_colstats(cudaStream_t st, const float *M, long long rows, int n, long long ld, float *mu, float *sd) {
  if (n <= 0) return cudaSuccess;
  k_lrn_colstats<<<n, 256, 0, st>>>(M, rows, n, ld, mu, sd);
  k_lrn_sdfloor<<<1, 256, 0, st>>>(sd, n);
  return cudaGetLastError();
}

cudaError_t lrn_batch(cudaStream_t st, int b, const int *idx, const float *X, long long ldx, int din, const float *Y,
                      long long ldy, int dout, const float *mu, const float *sd, const float *muo, const float *sdo,
                      float *Xb, float *Yb) {
  if (b <= 0) return cudaSuccess;
  const long long total = (long long)b * (din + dout);
  const int grid = (int)std::min<long long>(4096, (total + 255) / 256);
  k_lrn_batch<<<grid, 256, 0, st>>>(b, idx, X, ldx, din, Y, ldy, dout, mu, sd, muo, sdo, Xb, Yb);
  return cudaGetLastError();
}

}  // namespace lgpu
