// lgpu_eig.cu -- batched symmetric eigensolve and LETKF transform, one warp
// per (column, group) unit, FP32.
//
// Replaces src/letkf_core.F90:100-141: with A = G + (k-1)/infl I (G from
// the Gram stage, upper triangle as ssyev('V','U') reads it),
//   Pa   = V diag(1/lambda) V^T
//   W    = V diag(sqrt((k-1)/lambda)) V^T
//   wbar = Pa b               (b = Yb^T R^-1 rho dep, computed in the Gram stage)
//   T    = W + wbar 1^T
// The eigendecomposition is Householder tridiagonalisation (Golub & Van Loan,
// Matrix Computations, 4th ed., Alg. 8.3.1) followed by the implicit-shift
// QL iteration with Wilkinson shifts on the tridiagonal matrix (the
// tql2 scheme of Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11,
// 1968), accumulating the rotations into Z, and back-transformation
// V = Q Z.  Rows of the k x k work matrices are spread over the 32 lanes;
// the QL scalar recurrence is evaluated redundantly by every lane (shared
// memory broadcasts) with lane 0 as the only writer.
#include "lgpu_internal.cuh"

namespace lgpu {

namespace {

__device__ __forceinline__ float wsum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__host__ __device__ __forceinline__ int eig_floats_per_warp(int k) {
  const int ld = k + 1;
  return k * ld + 8 * k + 8;
}

__global__ void k_eig(EigArgs a, int wpb) {
  extern __shared__ __align__(16) float sm[];
  const int k = a.k, ld = k + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int unit = blockIdx.x * wpb + warp;
  if (unit >= a.nunits) return;           // whole warps exit; no block-level barriers below
  if (a.nkept[unit] <= 0) return;         // no local observations: the update keeps the background
  float *A = sm + (size_t)warp * eig_floats_per_warp(k);   // A, then Q, then V (one k x k matrix)
  float *d = A + k * ld;
  float *e = d + k;
  float *tau = e + k;
  float *bv = tau + k;
  float *p = bv + k;
  float *w = p + k;
  float *fl = w + k;
  float *gl = fl + k;
  const float *G = a.G + (size_t)unit * packed_size(k);
  // (k-1)/infl on the diagonal, src/letkf_core.F90:101-104
  const float shift = (float)(k - 1) * 1.0f / a.infl;
  for (int t = lane; t < k * k; t += 32) {
    const int i = t / k, j = t % k;
    float v = (i <= j) ? G[tri_idx(i, j, k)] : G[tri_idx(j, i, k)];
    if (i == j) v += shift;
    A[i * ld + j] = v;
  }
  for (int i = lane; i < k; i += 32) bv[i] = G[k * (k + 1) / 2 + i];
  __syncwarp();

  // ---- Householder tridiagonalisation: column j's reflector zeroes A[j+2:, j];
  // its vector v_j = A[j+1:, j] stays in column j
  for (int j = 0; j < k - 2; j++) {
    const int m = k - j - 1;                 // length of x = A[j+1:, j]
    float s = 0.0f;
    for (int r = lane; r < m; r += 32) { float x = A[(j + 1 + r) * ld + j]; s += x * x; }
    const float sig = wsum(s);
    const float x0 = A[(j + 1) * ld + j];
    const float s1 = sig - x0 * x0;
    if (!(s1 > 1e-30f * sig) || sig == 0.0f) {
      if (lane == 0) { tau[j] = 0.0f; e[j] = x0; d[j] = A[j * ld + j]; }
      __syncwarp();
      continue;
    }
    const float alpha = -copysignf(sqrtf(sig), x0);
    const float v0 = x0 - alpha;
    const float t = 2.0f / (v0 * v0 + s1);
    __syncwarp();
    if (lane == 0) { A[(j + 1) * ld + j] = v0; tau[j] = t; e[j] = alpha; d[j] = A[j * ld + j]; }
    __syncwarp();
    // p = t * A22 v
    for (int r = lane; r < m; r += 32) {
      const float *row = A + (j + 1 + r) * ld + (j + 1);
      float acc = 0.0f;
      for (int c = 0; c < m; c++) acc = __fmaf_rn(row[c], A[(j + 1 + c) * ld + j], acc);
      p[r] = t * acc;
    }
    __syncwarp();
    float pv = 0.0f;
    for (int r = lane; r < m; r += 32) pv = __fmaf_rn(p[r], A[(j + 1 + r) * ld + j], pv);
    const float beta = 0.5f * t * wsum(pv);
    for (int r = lane; r < m; r += 32) w[r] = p[r] - beta * A[(j + 1 + r) * ld + j];
    __syncwarp();
    // A22 -= v w^T + w v^T
    for (int r = lane; r < m; r += 32) {
      float *row = A + (j + 1 + r) * ld + (j + 1);
      const float vr = A[(j + 1 + r) * ld + j], wr = w[r];
      for (int c = 0; c < m; c++) {
        const float vc = A[(j + 1 + c) * ld + j], wc = w[c];
        row[c] = row[c] - __fmaf_rn(vr, wc, wr * vc);
      }
    }
    __syncwarp();
  }
  if (lane == 0) {
    if (k >= 2) {
      d[k - 2] = A[(k - 2) * ld + (k - 2)];
      e[k - 2] = A[(k - 1) * ld + (k - 2)];
    }
    d[k - 1] = A[(k - 1) * ld + (k - 1)];
    e[k - 1] = 0.0f;
  }
  __syncwarp();

  // ---- Q = H_0 H_1 ... H_{k-3} formed in place, last reflector first: the
  // trailing block [j+1:, j+1:] holds H_{j+1}..H_{k-3} (identity on row and
  // column j+1); v_j is still in column j, outside the block.  Each lane owns
  // columns lane and lane + 32.
  {
    const bool two = lane + 32 < k;
    const int c0 = lane, c1 = two ? lane + 32 : lane;
    for (int j = k - 2; j >= 0; j--) {
      // identity on row and column j + 1 of the block
      if (c0 > j + 1 && c0 < k) { A[(j + 1) * ld + c0] = 0.0f; A[c0 * ld + (j + 1)] = 0.0f; }
      if (two && c1 > j + 1) { A[(j + 1) * ld + c1] = 0.0f; A[c1 * ld + (j + 1)] = 0.0f; }
      if (lane == 0) A[(j + 1) * ld + (j + 1)] = 1.0f;
      __syncwarp();
      if (j > k - 3) continue;                 // the last block (2 x 2) has no reflector
      const float t = tau[j];
      if (t == 0.0f) continue;
      const int m = k - j - 1;
      // w_c = t * sum_r v_r Q[r][c]; Q[r][c] -= v_r w_c  (rows, columns j+1..k-1)
      float w0 = 0.0f, w1 = 0.0f;
      const bool in0 = c0 > j && c0 < k, in1 = two && c1 > j;
      for (int r = 0; r < m; r++) {
        const float v = A[(j + 1 + r) * ld + j];
        if (in0) w0 = __fmaf_rn(v, A[(j + 1 + r) * ld + c0], w0);
        if (in1) w1 = __fmaf_rn(v, A[(j + 1 + r) * ld + c1], w1);
      }
      w0 *= t;
      w1 *= t;
      __syncwarp();
      for (int r = 0; r < m; r++) {
        const float v = A[(j + 1 + r) * ld + j];
        if (in0) A[(j + 1 + r) * ld + c0] -= v * w0;
        if (in1) A[(j + 1 + r) * ld + c1] -= v * w1;
      }
      __syncwarp();
    }
    // row and column 0: Q e_0 = e_0
    if (c0 > 0 && c0 < k) { A[c0] = 0.0f; A[c0 * ld] = 0.0f; }
    if (two) { A[c1] = 0.0f; A[c1 * ld] = 0.0f; }
    if (lane == 0) A[0] = 1.0f;
    __syncwarp();
  }

  // ---- implicit-shift QL on (d, e), rotations applied at once to the
  // columns (i, i+1) of Q (V = Q Z).  The scalar recurrence is evaluated
  // redundantly by every lane: d[i+1] is carried in a register and only e[i],
  // d[i] (not yet written in this sweep) are read, so lane 0 alone writes
  // results, without barriers inside the sweep.  Each lane owns rows lane and
  // lane + 32 of Q and carries the pending column i+1 of its rows.
  int bad = 0;
  {
    const bool two = lane + 32 < k;
    const bool own = lane < k;
    float *q0 = A + (own ? lane : 0) * ld, *q1 = A + (two ? lane + 32 : 0) * ld;
    for (int l = 0; l < k; l++) {
      int iter = 0;
      for (;;) {
        // first m >= l with a negligible e[m] (m = k-1 if none): lanes test
        // 32 consecutive candidates at a time
        int m = k - 1;
        for (int base = l; base < k - 1; base += 32) {
          const int mm = base + lane;
          bool small = false;
          if (mm < k - 1) small = fabsf(e[mm]) <= 1.1920929e-7f * (fabsf(d[mm]) + fabsf(d[mm + 1]));
          const unsigned bal = __ballot_sync(0xffffffffu, small);
          if (bal) { m = base + __ffs(bal) - 1; break; }
        }
        if (m == l) break;
        if (++iter > 60) { bad = 1; break; }
        const float dl = d[l], el = e[l];
        float g = (d[l + 1] - dl) / (2.0f * el);
        float r = sqrtf(g * g + 1.0f);
        g = d[m] - dl + el / (g + copysignf(r, g));
        float s = 1.0f, c = 1.0f, pp = 0.0f;
        float di1 = d[m];
        float z0 = own ? q0[m] : 0.0f, z1 = two ? q1[m] : 0.0f;   // pending column i+1
        float ei = e[m - 1], di = d[m - 1];
        int i = m - 1;
        bool deflate = false;
        for (; i >= l; i--) {
          const int in = i > 0 ? i - 1 : 0;
          const float ei_n = e[in], di_n = d[in];           // next step's operands
          const float a0 = own ? q0[i] : 0.0f, a1 = two ? q1[i] : 0.0f;
          const float f = s * ei, b = c * ei;
          r = sqrtf(f * f + g * g);
          if (lane == 0) e[i + 1] = r;
          if (r == 0.0f) {
            if (lane == 0) { d[i + 1] = di1 - pp; e[m] = 0.0f; }
            deflate = true;
            break;
          }
          const float ir = __frcp_rn(r);
          s = f * ir;
          c = g * ir;
          g = di1 - pp;
          const float rr = (di - g) * s + 2.0f * c * b;
          pp = s * rr;
          if (lane == 0) d[i + 1] = g + pp;
          g = c * rr - b;
          di1 = di;
          // rotation (c, s) on columns (i, i+1) of the lane's rows
          if (own) { q0[i + 1] = s * a0 + c * z0; z0 = c * a0 - s * z0; }
          if (two) { q1[i + 1] = s * a1 + c * z1; z1 = c * a1 - s * z1; }
          ei = ei_n;
          di = di_n;
        }
        const int ilo = deflate ? i + 1 : l;
        if (own) q0[ilo] = z0;
        if (two) q1[ilo] = z1;
        if (!deflate && lane == 0) { d[l] = d[l] - pp; e[l] = g; e[m] = 0.0f; }
        __syncwarp();
      }
      if (bad) break;
    }
  }
  __syncwarp();

  // ---- spectral functions: f = sqrt((k-1)/lambda), g = 1/lambda
  //      (src/letkf_core.F90:111-113, :128-131); fl holds sqrt(f)
  for (int l = lane; l < k; l += 32) {
    const float lam = d[l];
    if (!(lam > 0.0f)) bad |= 2;
    fl[l] = sqrtf(sqrtf((float)(k - 1) / lam));
    gl[l] = 1.0f / lam;
  }
  __syncwarp();
  // s_l = g_l * (V^T b)_l
  for (int l = lane; l < k; l += 32) {
    float acc = 0.0f;
    for (int q = 0; q < k; q++) acc = __fmaf_rn(A[q * ld + l], bv[q], acc);
    p[l] = gl[l] * acc;
  }
  __syncwarp();
  // wbar_i = sum_l V[i][l] s_l
  for (int i = lane; i < k; i += 32) {
    float acc = 0.0f;
    for (int l = 0; l < k; l++) acc = __fmaf_rn(A[i * ld + l], p[l], acc);
    w[i] = acc;
  }
  __syncwarp();
  // U = V diag(sqrt f) in place: T = U U^T + wbar 1^T
  for (int t = lane; t < k * k; t += 32) { const int i = t / k, l = t % k; A[i * ld + l] *= fl[l]; }
  __syncwarp();
  // T_ij = sum_l U[i][l] U[j][l] + wbar_i ; lane owns columns lane, lane + 32
  float *T = a.T + (size_t)unit * k * k;
  if (lane < k) {
    const bool two = lane + 32 < k;
    const int j0 = lane, j1 = two ? lane + 32 : lane;
    const float *u0 = A + j0 * ld, *u1 = A + j1 * ld;
    for (int i = 0; i < k; i++) {
      const float *ur = A + i * ld;
      float acc0 = 0.0f, acc1 = 0.0f;
      for (int l = 0; l < k; l++) {
        const float y = ur[l];
        acc0 = __fmaf_rn(y, u0[l], acc0);
        acc1 = __fmaf_rn(y, u1[l], acc1);
      }
      T[i * k + j0] = acc0 + w[i];
      if (two) T[i * k + j1] = acc1 + w[i];
    }
  }
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && lane == 0) atomicOr(a.status, bad);
}

}  // namespace

cudaError_t launch_eig(cudaStream_t st, const EigArgs &a, int *launches);

cudaError_t launch_eig_debug(cudaStream_t st, int nunits, int k, const float *G, const int *nkept, float *T,
                             int *status) {
  EigArgs a;
  a.nunits = nunits;
  a.k = k;
  a.infl = 1.0f;
  a.G = G;
  a.nkept = nkept;
  a.T = T;
  a.status = status;
  int l = 0;
  return launch_eig(st, a, &l);
}

cudaError_t launch_eig(cudaStream_t st, const EigArgs &a, int *launches) {
  if (a.nunits <= 0) return cudaSuccess;
  // warps per block: the most resident warps per SM for this unit size
  const size_t per = (size_t)eig_floats_per_warp(a.k) * sizeof(float);
  const size_t sm_bytes = 227 * 1024;
  int wpb = 1, best = 0;
  for (int c = 1; c <= 8; c++) {
    if ((size_t)c * per > sm_bytes) break;
    int blocks = (int)(sm_bytes / ((size_t)c * per + 1024));   // 1 KB reserved per block
    if (blocks > 32) blocks = 32;
    int warps = blocks * c;
    if (warps > 64) warps = 64;
    if (warps > best) { best = warps; wpb = c; }
  }
  const size_t smem = (size_t)wpb * per;
  cudaError_t e = cudaFuncSetAttribute(k_eig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = (a.nunits + wpb - 1) / wpb;
  k_eig<<<grid, 32 * wpb, smem, st>>>(a, wpb);
  (*launches)++;
  return cudaGetLastError();
}

}  // namespace lgpu
