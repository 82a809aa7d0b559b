// lgpu_eig.cu -- batched symmetric eigensolve and LETKF transform per
// (column, group) unit: FP32 (the reference's ssyev precision), with an FP64
// form for the units flagged by the eigenvalue-gap test or for every unit.
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
// V = Q Z.  The split pipeline (used whenever its scratch fits) reduces in
// registers (k_eig_tri_r: a warp per unit up to k = 48; k_eig_tri_t: a team
// of ceil(k / 32) warps, one row per thread, above), runs the QL scalar
// recurrence once per unit (k_eig_ql) and replays the logged rotations on Q's
// rows in shared memory (k_eig_vec: one warp, two rows per lane, up to
// k = 64; four warps, one row per thread, above).  The fused kernel (k_eig,
// the fallback) works on the matrices in shared memory with the rows spread
// over a warp's or team's threads (tt + TS q) and evaluates the QL recurrence
// redundantly on every lane (shared memory broadcasts) with lane 0 as the
// only writer.  The FP64 form (k_eig64) runs the fused phases in double on a
// team of 2 or 4 warps.
#include "lgpu_internal.cuh"
#include <algorithm>

namespace lgpu {

namespace {

__device__ __forceinline__ float fmar(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmar(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float rcpr(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcpr(double x) { return __drcp_rn(x); }
// unit roundoff and the smallest scale treated as zero, per precision
template <class R> struct Lim;
template <> struct Lim<float> {
  static constexpr float eps = 1.1920929e-7f, tiny = 1e-30f;
};
template <> struct Lim<double> {
  static constexpr double eps = 2.220446049250313e-16, tiny = 1e-300;
};

template <class R>
__device__ __forceinline__ R wsum(R v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__host__ __device__ __forceinline__ int eig_floats_per_warp(int k) {
  const int ld = k + 1;
  return k * ld + 8 * k + 8;
}

// A team of NW warps works on one unit: thread tt of TS = 32 NW owns rows /
// columns tt + TS q of the work matrices.  NW = 1 is one warp per unit
// (several units per CTA); NW > 1 is one unit per CTA, so the CTA barrier is
// the team barrier.  Sums run over the warp's butterfly, then over the warps
// in warp order (deterministic).
template <int NW, class R = float>
struct Team {
  static constexpr int TS = 32 * NW;
  int tt, lane, warp;
  R *red;       // NW values in shared memory (NW > 1)
  __device__ __forceinline__ void sync() const {
    if constexpr (NW == 1) __syncwarp();
    else __syncthreads();
  }
  __device__ __forceinline__ R sum(R v) const {
    v = wsum<R>(v);
    if constexpr (NW == 1) {
      return v;
    } else {
      if (lane == 0) red[warp] = v;
      __syncthreads();
      R t = red[0];
#pragma unroll
      for (int q = 1; q < NW; q++) t += red[q];
      __syncthreads();
      return t;
    }
  }
};

// Work arrays of one unit in shared memory: A (k x ld, ld = k + 1) holds A,
// then Q, then V; then d, e, tau, bv, p, w, fl, gl (k each).
template <class R = float>
struct EigWork {
  R *A, *d, *e, *tau, *bv, *p, *w, *fl, *gl;
  __device__ EigWork(R *base, int k) {
    A = base;
    d = A + k * (k + 1);
    e = d + k; tau = e + k; bv = tau + k; p = bv + k; w = p + k; fl = w + k; gl = fl + k;
  }
};

// A = G + (k-1)/infl I from the packed Gram block, b from its tail
template <int NW, class R>
__device__ __forceinline__ void eig_load(const EigArgs &a, int unit, EigWork<R> &W, const Team<NW, R> &T) {
  const int k = a.k, ld = k + 1, tt = T.tt, TS = T.TS;
  R *A = W.A, *bv = W.bv;
  const float *Gin = a.G + (size_t)unit * packed_size(k);
  // (k-1)/infl on the diagonal, src/letkf_core.F90:101-104
  const R shift = (R)(k - 1) * R(1) / (R)a.infl;
  for (int t = tt; t < k * k; t += TS) {
    const int i = t / k, j = t % k;
    R v = (i <= j) ? (R)Gin[tri_idx(i, j, k)] : (R)Gin[tri_idx(j, i, k)];
    if (i == j) v += shift;
    A[i * ld + j] = v;
  }
  for (int i = tt; i < k; i += TS) bv[i] = (R)Gin[k * (k + 1) / 2 + i];
  T.sync();

}

template <int NQ, int NW, class R>
__device__ __forceinline__ void eig_form_q(int k, EigWork<R> &W, const Team<NW, R> &T);

// Householder tridiagonalisation (d, e, tau; reflector vectors in the
// columns of A) and Q formed in place.  NQ: rows / columns per lane
// (tt + TS q, q < NQ).
template <int NQ, int NW, class R>
__device__ __forceinline__ void eig_tridiag_q(int k, EigWork<R> &W, const Team<NW, R> &T) {
  const int ld = k + 1, tt = T.tt, TS = T.TS;
  R *A = W.A, *d = W.d, *e = W.e, *tau = W.tau, *p = W.p, *w = W.w;
  R *vv = W.fl;   // the current reflector, contiguous (fl is free until the transform)
  // ---- Householder tridiagonalisation: column j's reflector zeroes A[j+2:, j];
  // its vector v_j = A[j+1:, j] stays in column j
  for (int j = 0; j < k - 2; j++) {
    const int m = k - j - 1;                 // length of x = A[j+1:, j]
    R s = R(0);
    for (int r = tt; r < m; r += TS) { R x = A[(j + 1 + r) * ld + j]; s += x * x; }
    const R sig = T.sum(s);
    const R x0 = A[(j + 1) * ld + j];
    const R s1 = sig - x0 * x0;
    if (!(s1 > Lim<R>::tiny * sig) || sig == R(0)) {
      if (tt == 0) { tau[j] = R(0); e[j] = x0; d[j] = A[j * ld + j]; }
      T.sync();
      continue;
    }
    const R alpha = -copysign(sqrt(sig), x0);
    const R v0 = x0 - alpha;
    const R t = R(2) / (v0 * v0 + s1);
    T.sync();
    if (tt == 0) { A[(j + 1) * ld + j] = v0; tau[j] = t; e[j] = alpha; d[j] = A[j * ld + j]; }
    for (int r = tt; r < m; r += TS) vv[r] = r == 0 ? v0 : A[(j + 1 + r) * ld + j];
    T.sync();
    // p = t * A22 v
    for (int r = tt; r < m; r += TS) {
      const R *row = A + (j + 1 + r) * ld + (j + 1);
      R acc = R(0);
#pragma unroll 4
      for (int c = 0; c < m; c++) acc = fmar(row[c], vv[c], acc);
      p[r] = t * acc;
    }
    T.sync();
    R pv = R(0);
    for (int r = tt; r < m; r += TS) pv = fmar(p[r], vv[r], pv);
    const R beta = R(0.5) * t * T.sum(pv);
    for (int r = tt; r < m; r += TS) w[r] = p[r] - beta * vv[r];
    T.sync();
    // A22 -= v w^T + w v^T
    for (int r = tt; r < m; r += TS) {
      R *row = A + (j + 1 + r) * ld + (j + 1);
      const R vr = vv[r], wr = w[r];
#pragma unroll 4
      for (int c = 0; c < m; c++) row[c] = row[c] - fmar(vr, w[c], wr * vv[c]);
    }
    T.sync();
  }
  if (tt == 0) {
    if (k >= 2) {
      d[k - 2] = A[(k - 2) * ld + (k - 2)];
      e[k - 2] = A[(k - 1) * ld + (k - 2)];
    }
    d[k - 1] = A[(k - 1) * ld + (k - 1)];
    e[k - 1] = R(0);
  }
  T.sync();
  eig_form_q<NQ>(k, W, T);
}

// Q = H_0 H_1 ... H_{k-3} formed in place from the reflectors in the columns
// of A below the diagonal (v_j in column j, tau[j]), last reflector first:
// the trailing block [j+1:, j+1:] holds H_{j+1}..H_{k-3} (identity on row
// and column j+1); v_j is still in column j, outside the block.  Each thread
// owns columns tt + TS q.  The entries on and above the diagonal are not read
// before they are written.
template <int NQ, int NW, class R>
__device__ __forceinline__ void eig_form_q(int k, EigWork<R> &W, const Team<NW, R> &T) {
  const int ld = k + 1, tt = T.tt, TS = T.TS;
  R *A = W.A, *tau = W.tau;
  R *vv = W.fl;
  {
    for (int j = k - 2; j >= 0; j--) {
      // identity on row and column j + 1 of the block
#pragma unroll
      for (int q = 0; q < NQ; q++) {
        const int c = tt + TS * q;
        if (c > j + 1 && c < k) { A[(j + 1) * ld + c] = R(0); A[c * ld + (j + 1)] = R(0); }
      }
      if (tt == 0) A[(j + 1) * ld + (j + 1)] = R(1);
      T.sync();
      if (j > k - 3) continue;                 // the last block (2 x 2) has no reflector
      const R t = tau[j];
      if (t == R(0)) continue;
      const int m = k - j - 1;
      for (int r = tt; r < m; r += TS) vv[r] = A[(j + 1 + r) * ld + j];
      T.sync();
      // w_c = t * sum_r v_r Q[r][c]; Q[r][c] -= v_r w_c  (rows, columns j+1..k-1)
      R wc[NQ];
      bool in[NQ];
#pragma unroll
      for (int q = 0; q < NQ; q++) {
        const int c = tt + TS * q;
        wc[q] = R(0);
        in[q] = c > j && c < k;
      }
      for (int r = 0; r < m; r++) {
        const R v = vv[r];
#pragma unroll
        for (int q = 0; q < NQ; q++)
          if (in[q]) wc[q] = fmar(v, A[(j + 1 + r) * ld + tt + TS * q], wc[q]);
      }
#pragma unroll
      for (int q = 0; q < NQ; q++) wc[q] *= t;
      for (int r = 0; r < m; r++) {
        const R v = vv[r];
#pragma unroll
        for (int q = 0; q < NQ; q++)
          if (in[q]) A[(j + 1 + r) * ld + tt + TS * q] -= v * wc[q];
      }
      T.sync();
    }
    // row and column 0: Q e_0 = e_0
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int c = tt + TS * q;
      if (c > 0 && c < k) { A[c] = R(0); A[c * ld] = R(0); }
    }
    if (tt == 0) A[0] = R(1);
    T.sync();
  }

}

// spectral functions and T = U U^T + wbar 1^T (A holds V, d the eigenvalues)
template <int NQ, int NW, class R>
__device__ __forceinline__ void eig_transform(const EigArgs &a, int unit, EigWork<R> &W, const Team<NW, R> &TM,
                                              int &bad) {
  const int k = a.k, ld = k + 1, tt = TM.tt, TS = TM.TS;
  R *A = W.A, *d = W.d, *bv = W.bv, *p = W.p, *w = W.w, *fl = W.fl, *gl = W.gl;
  // ---- spectral functions: f = sqrt((k-1)/lambda), g = 1/lambda
  //      (src/letkf_core.F90:111-113, :128-131); fl holds sqrt(f)
  for (int l = tt; l < k; l += TS) {
    const R lam = d[l];
    if (!(lam > R(0))) bad |= 2;
    fl[l] = sqrt(sqrt((R)(k - 1) / lam));
    gl[l] = R(1) / lam;
  }
  TM.sync();
  // s_l = g_l * (V^T b)_l
  for (int l = tt; l < k; l += TS) {
    R acc = R(0);
    for (int q = 0; q < k; q++) acc = fmar(A[q * ld + l], bv[q], acc);
    p[l] = gl[l] * acc;
  }
  TM.sync();
  // wbar_i = sum_l V[i][l] s_l
  for (int i = tt; i < k; i += TS) {
    R acc = R(0);
    for (int l = 0; l < k; l++) acc = fmar(A[i * ld + l], p[l], acc);
    w[i] = acc;
    if (a.wbar) a.wbar[(size_t)unit * k + i] = (float)acc;
  }
  TM.sync();
  // U = V diag(sqrt f) in place: T = U U^T + wbar 1^T
  for (int t = tt; t < k * k; t += TS) { const int i = t / k, l = t % k; A[i * ld + l] *= fl[l]; }
  TM.sync();
  // T_ij = sum_l U[i][l] U[j][l] + wbar_i ; thread owns columns tt + TS q
  // (a column past k repeats the thread's first column and is not stored)
  float *Tout = a.T + (size_t)unit * k * k;
  // rows in blocks of TRB (a row past k repeats row 0 and is not stored);
  // every sum runs over l in ascending order
  if (tt < k) {
    constexpr int TRB = 4;
    const R *u[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) u[q] = A + (tt + TS * q < k ? tt + TS * q : tt) * ld;
    for (int i0 = 0; i0 < k; i0 += TRB) {
      const R *ur[TRB];
#pragma unroll
      for (int b = 0; b < TRB; b++) ur[b] = A + (i0 + b < k ? i0 + b : 0) * ld;
      R acc[TRB][NQ];
#pragma unroll
      for (int b = 0; b < TRB; b++)
#pragma unroll
        for (int q = 0; q < NQ; q++) acc[b][q] = R(0);
      for (int l = 0; l < k; l++) {
        R uq[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++) uq[q] = u[q][l];
#pragma unroll
        for (int b = 0; b < TRB; b++) {
          const R y = ur[b][l];
#pragma unroll
          for (int q = 0; q < NQ; q++) acc[b][q] = fmar(y, uq[q], acc[b][q]);
        }
      }
#pragma unroll
      for (int b = 0; b < TRB; b++)
#pragma unroll
        for (int q = 0; q < NQ; q++)
          if (i0 + b < k && tt + TS * q < k) Tout[(i0 + b) * k + tt + TS * q] = (R)(acc[b][q] + w[i0 + b]);
    }
  }
}

// Deflation test of the QL iteration: e_m is negligible when it is below
// eps32 of its two diagonal neighbours (the local test of LAPACK's ssteqr /
// EISPACK's tql2 family) or, from the kQlAbsIter-th iteration on the current
// eigenvalue, below eps32 times the norm of the whole tridiagonal matrix
// (tql2's absolute test).  The second test ends the iteration where rounding
// at the eps32 ||T|| level keeps a strongly graded block from meeting the
// local test.  Applied from the first iteration it also deflated, at the
// ||T|| level, off-diagonals between near-equal small eigenvalues that the
// local test resolves in a few more sweeps (a rank-one update with k = 100
// and condition ~1e5: those eigenvalues off by ~eps32 ||T||); the delay
// keeps them.
constexpr int kQlAbsIter = 6;

template <class R>
__device__ __forceinline__ bool ql_negligible(R em, R dm, R dm1, R tabs) {
  const R ae = fabs(em);
  return ae <= Lim<R>::eps * (fabs(dm) + fabs(dm1)) || ae <= tabs;
}

// eps32 * max_i (|d_i| + |e_i|), elements at stride `st`
template <class R>
__device__ __forceinline__ R ql_abs_tol(int k, const R *d, const R *e, int st) {
  R an = R(0);
  for (int i = 0; i < k; i++) an = fmax(an, fabs(d[(size_t)i * st]) + fabs(e[(size_t)i * st]));
  return Lim<R>::eps * an;
}

// implicit-shift QL on (d, e) with the rotations applied to the columns of
// A (Q -> V), one warp
template <int NQ, class R>
__device__ __forceinline__ void eig_ql_warp(int k, EigWork<R> &W, int lane, int &bad) {
  const int ld = k + 1;
  R *A = W.A, *d = W.d, *e = W.e;
  // ---- implicit-shift QL on (d, e), rotations applied at once to the
  // columns (i, i+1) of Q (V = Q Z).  The scalar recurrence is evaluated
  // redundantly by every lane: d[i+1] is carried in a register and only e[i],
  // d[i] (not yet written in this sweep) are read, so lane 0 alone writes
  // results, without barriers inside the sweep.  Each lane owns rows
  // lane + 32 q of Q and carries the pending column i+1 of its rows.
  {
    bool own[NQ];
    R *qr[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      own[q] = lane + 32 * q < k;
      qr[q] = A + (own[q] ? lane + 32 * q : 0) * ld;
    }
    const R tabs = ql_abs_tol(k, d, e, 1);
    for (int l = 0; l < k; l++) {
      int iter = 0;
      for (;;) {
        // first m >= l with a negligible e[m] (m = k-1 if none): lanes test
        // 32 consecutive candidates at a time
        int m = k - 1;
        for (int base = l; base < k - 1; base += 32) {
          const int mm = base + lane;
          bool small = false;
          if (mm < k - 1) small = ql_negligible(e[mm], d[mm], d[mm + 1], iter >= kQlAbsIter ? tabs : R(0));
          const unsigned bal = __ballot_sync(0xffffffffu, small);
          if (bal) { m = base + __ffs(bal) - 1; break; }
        }
        if (m == l) break;
        if (++iter > 60) { bad = 1; break; }
        const R dl = d[l], el = e[l];
        R g = (d[l + 1] - dl) / (R(2) * el);
        R r = sqrt(g * g + R(1));
        g = d[m] - dl + el / (g + copysign(r, g));
        R s = R(1), c = R(1), pp = R(0);
        R di1 = d[m];
        R z[NQ];   // pending column i+1
#pragma unroll
        for (int q = 0; q < NQ; q++) z[q] = own[q] ? qr[q][m] : R(0);
        R ei = e[m - 1], di = d[m - 1];
        int i = m - 1;
        bool deflate = false;
        for (; i >= l; i--) {
          const int in = i > 0 ? i - 1 : 0;
          const R ei_n = e[in], di_n = d[in];           // next step's operands
          R av[NQ];
#pragma unroll
          for (int q = 0; q < NQ; q++) av[q] = own[q] ? qr[q][i] : R(0);
          const R f = s * ei, b = c * ei;
          r = sqrt(f * f + g * g);
          if (lane == 0) e[i + 1] = r;
          if (r == R(0)) {
            if (lane == 0) { d[i + 1] = di1 - pp; e[m] = R(0); }
            deflate = true;
            break;
          }
          const R ir = rcpr(r);
          s = f * ir;
          c = g * ir;
          g = di1 - pp;
          const R rr = (di - g) * s + R(2) * c * b;
          pp = s * rr;
          if (lane == 0) d[i + 1] = g + pp;
          g = c * rr - b;
          di1 = di;
          // rotation (c, s) on columns (i, i+1) of the lane's rows
#pragma unroll
          for (int q = 0; q < NQ; q++)
            if (own[q]) { qr[q][i + 1] = s * av[q] + c * z[q]; z[q] = c * av[q] - s * z[q]; }
          ei = ei_n;
          di = di_n;
        }
        const int ilo = deflate ? i + 1 : l;
#pragma unroll
        for (int q = 0; q < NQ; q++)
          if (own[q]) qr[q][ilo] = z[q];
        if (!deflate && lane == 0) { d[l] = d[l] - pp; e[l] = g; e[m] = R(0); }
        __syncwarp();
      }
      if (bad) break;
    }
  }
  __syncwarp();

}

template <int NQ>
__global__ void k_eig(EigArgs a, int wpb) {
  extern __shared__ __align__(16) float sm[];
  const int k = a.k;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int un = blockIdx.x * wpb + warp;
  if (un >= a.nunits) return;             // whole warps exit; no block-level barriers below
  const int unit = a.ulist ? a.ulist[un] : un;
  if (a.nkept[unit] <= 0) return;         // no local observations: the update keeps the background
  EigWork W(sm + (size_t)warp * eig_floats_per_warp(k), k);
  const Team<1> T{lane, lane, warp, nullptr};
  eig_load(a, unit, W, T);
  eig_tridiag_q<NQ>(k, W, T);
  int bad = 0;
  eig_ql_warp<NQ>(k, W, lane, bad);
  eig_transform<NQ>(a, unit, W, T, bad);
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && lane == 0) atomicOr(a.status, bad);
}

// ---------------------------------------------------------------------------
// Split pipeline (the arithmetic of k_eig):
//   k_eig_tri_r / k_eig_tri_t  the Householder reduction and Q with the work
//              matrix in registers (a warp per unit up to k = 48, a team of
//              ceil(k / 32) warps with one row per thread above); Q, d and e
//              to global
//   k_eig_ql   thread per unit: the QL recurrence on (d, e) alone, logging
//              every sweep (start index, rotation count) and rotation (c, s)
//   k_eig_vec  team per unit: the logged rotations applied to Q's columns
//              (V = Q Z), then the spectral functions and T
//   k_eig_flag (FP32_RESOLVE) warp per unit: units for the FP64 re-solve
// The scalar recurrence, which the fused kernel evaluates redundantly on all
// 32 lanes, runs once per unit.

// The first stage for k <= 48 with the work matrix in registers: one warp
// per unit, lane l holds rows l and l + 32 of A (K = k rounded up to 8
// columns, zero beyond k).  Step j of the Householder reduction: the lane
// owning row j publishes x = A[j][j+1:] (= A[j+1:][j]) as the reflector
// row VH[j] in shared memory (zeros outside j+1..k-1); p = t A v and the
// rank-two update A -= v w^T + w v^T run on every lane's rows over the full
// row width (columns and rows outside the trailing block meet zeros in v and
// w and are left exactly unchanged), in column groups of four skipped while
// they lie left of the block.  The dot products run over the columns in
// ascending order as the shared-memory form does.  Q = H_0 ... H_{k-3} is
// then formed with lane l holding columns l and l + 32 in the same registers
// (reflectors applied from the last to the first).  Output: Q
// row-major and (d, e) to the scratch.
constexpr int RWPB = 4;   // warps (units) per block

template <int K>
__global__ void __launch_bounds__(32 * RWPB, 4) k_eig_tri_r(EigArgs a, EigSplit sp, int u0, int nb) {
  constexpr int NQ = (K + 31) / 32;
  constexpr int NR = K > 2 ? K - 2 : 1;   // reflector rows
  constexpr int K4 = K / 4;
  __shared__ __align__(16) float sv[RWPB][NR * K + 4 * K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ub = blockIdx.x * RWPB + warp;
  if (ub >= nb) return;
  const int unit = a.ulist ? a.ulist[u0 + ub] : u0 + ub;
  if (a.nkept[unit] <= 0) return;
  const int k = a.k;
  float *VH = sv[warp];            // reflector j in row j
  float *ww = VH + NR * K;         // w of the current step
  float *dd = ww + K, *ee = dd + K, *tau = ee + K;
  // A = G + (k-1)/infl I (src/letkf_core.F90:101-104), upper triangle packed
  const float *Gin = a.G + (size_t)unit * packed_size(k);
  const float shift = (float)(k - 1) * 1.0f / a.infl;
  float A[NQ][K];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int r = lane + 32 * q;
#pragma unroll
    for (int c = 0; c < K; c++) {
      float v = 0.0f;
      if (r < k && c < k) {
        v = r <= c ? Gin[tri_idx(r, c, k)] : Gin[tri_idx(c, r, k)];
        if (r == c) v += shift;
      }
      A[q][c] = v;
    }
  }
  for (int j = 0; j < k - 2; j++) {
    float *vj = VH + j * K;
    __syncwarp();
    // the owner of row j stores it whole (columns past k are zero in A);
    // then d_j is taken and columns 0..j are cleared, one per lane
    if (lane == (j & 31)) {
      if (NQ == 1 || (j >> 5) == 0) {
#pragma unroll
        for (int c4 = 0; c4 < K4; c4++)
          *reinterpret_cast<float4 *>(vj + 4 * c4) =
              make_float4(A[0][4 * c4], A[0][4 * c4 + 1], A[0][4 * c4 + 2], A[0][4 * c4 + 3]);
      } else {
#pragma unroll
        for (int c4 = 0; c4 < K4; c4++)
          *reinterpret_cast<float4 *>(vj + 4 * c4) = make_float4(A[NQ - 1][4 * c4], A[NQ - 1][4 * c4 + 1],
                                                                 A[NQ - 1][4 * c4 + 2], A[NQ - 1][4 * c4 + 3]);
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int c = lane + 32 * q;
      if (c <= j) {
        if (c == j) dd[j] = vj[j];
        vj[c] = 0.0f;
      }
    }
    __syncwarp();
    float s = 0.0f;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int c = lane + 32 * q;
      if (c < K) { const float x = vj[c]; s += x * x; }
    }
    const float sig = wsum<float>(s);
    const float x0 = vj[j + 1];
    const float s1 = sig - x0 * x0;
    if (!(s1 > Lim<float>::tiny * sig) || sig == 0.0f) {
      if (lane == 0) { tau[j] = 0.0f; ee[j] = x0; }
      continue;
    }
    const float alpha = -copysignf(sqrtf(sig), x0);
    const float v0 = x0 - alpha;
    const float t = 2.0f / (v0 * v0 + s1);
    __syncwarp();
    if (lane == 0) { vj[j + 1] = v0; tau[j] = t; ee[j] = alpha; }
    __syncwarp();
    // p = t A v
    float p[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      float acc = 0.0f;
#pragma unroll
      for (int c4 = 0; c4 < K4; c4++) {
        if (4 * c4 + 3 <= j) continue;
        const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * c4);
        acc = __fmaf_rn(A[q][4 * c4 + 0], v4.x, acc);
        acc = __fmaf_rn(A[q][4 * c4 + 1], v4.y, acc);
        acc = __fmaf_rn(A[q][4 * c4 + 2], v4.z, acc);
        acc = __fmaf_rn(A[q][4 * c4 + 3], v4.w, acc);
      }
      p[q] = t * acc;
    }
    float pv = 0.0f;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int r = lane + 32 * q;
      if (r < K) pv = __fmaf_rn(p[q], vj[r], pv);
    }
    const float beta = 0.5f * t * wsum<float>(pv);
    float w[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int r = lane + 32 * q;
      w[q] = (r > j && r < k) ? p[q] - beta * vj[r] : 0.0f;
      if (r < K) ww[r] = w[q];
    }
    __syncwarp();
    // A -= v w^T + w v^T
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int r = lane + 32 * q;
      const float vr = r < K ? vj[r] : 0.0f, wr = w[q];
#pragma unroll
      for (int c4 = 0; c4 < K4; c4++) {
        if (4 * c4 + 3 <= j) continue;
        const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * c4);
        const float4 w4 = *reinterpret_cast<const float4 *>(ww + 4 * c4);
        A[q][4 * c4 + 0] = A[q][4 * c4 + 0] - __fmaf_rn(vr, w4.x, wr * v4.x);
        A[q][4 * c4 + 1] = A[q][4 * c4 + 1] - __fmaf_rn(vr, w4.y, wr * v4.y);
        A[q][4 * c4 + 2] = A[q][4 * c4 + 2] - __fmaf_rn(vr, w4.z, wr * v4.z);
        A[q][4 * c4 + 3] = A[q][4 * c4 + 3] - __fmaf_rn(vr, w4.w, wr * v4.w);
      }
    }
  }
  __syncwarp();
  // the last 2 x 2 block: d[k-2], d[k-1], e[k-2]
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int r = lane + 32 * q;
    if (r == k - 2 || r == k - 1) {
#pragma unroll
      for (int c = 0; c < K; c++) {
        if (c == r) dd[r] = A[q][c];
        if (r == k - 1 && c == k - 2) ee[k - 2] = A[q][c];
      }
    }
  }
  if (lane == 0) ee[k - 1] = 0.0f;
  __syncwarp();
  // Q = H_0 H_1 ... H_{k-3} I, reflectors from the last to the first; lane l
  // holds columns l and l + 32
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int c = lane + 32 * q;
#pragma unroll
    for (int r = 0; r < K; r++) A[q][r] = (r == c && c < k) ? 1.0f : 0.0f;
  }
  for (int j = k - 3; j >= 0; j--) {
    const float t = tau[j];
    if (t == 0.0f) continue;
    const float *vj = VH + j * K;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      float s = 0.0f;
#pragma unroll
      for (int r4 = 0; r4 < K4; r4++) {
        if (4 * r4 + 3 <= j) continue;
        const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * r4);
        s = __fmaf_rn(v4.x, A[q][4 * r4 + 0], s);
        s = __fmaf_rn(v4.y, A[q][4 * r4 + 1], s);
        s = __fmaf_rn(v4.z, A[q][4 * r4 + 2], s);
        s = __fmaf_rn(v4.w, A[q][4 * r4 + 3], s);
      }
      s *= t;
#pragma unroll
      for (int r4 = 0; r4 < K4; r4++) {
        if (4 * r4 + 3 <= j) continue;
        const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * r4);
        A[q][4 * r4 + 0] -= v4.x * s;
        A[q][4 * r4 + 1] -= v4.y * s;
        A[q][4 * r4 + 2] -= v4.z * s;
        A[q][4 * r4 + 3] -= v4.w * s;
      }
    }
  }
  float *Q = sp.Q + (size_t)ub * k * k;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int c = lane + 32 * q;
    if (c < k) {
#pragma unroll
      for (int r = 0; r < K; r++)
        if (r < k) Q[(size_t)r * k + c] = A[q][r];
    }
  }
  float *de = sp.DE + (size_t)ub * 2 * k;
  for (int i = lane; i < k; i += 32) { de[i] = dd[i]; de[k + i] = ee[i]; }
}

// k_eig_tri_t<K, NW>: k_eig_tri_r for 48 < k <= K <= 64 with a team of NW
// warps per unit (one unit per CTA, 32 NW >= K): thread t holds row t of the
// work matrix in registers; the reflector row VH[j] is written by thread j,
// the sums over the rows run through the team in warp order, and Q is formed
// with thread t holding column t.  Shared memory (dynamic): the reflectors
// (K - 2) x K, then w, d, e, tau (K each).  Same arithmetic as k_eig_tri_r,
// one row per thread instead of two per lane.
template <int K, int NW>
__global__ void __launch_bounds__(32 * NW) k_eig_tri_t(EigArgs a, EigSplit sp, int u0, int nb) {
  constexpr int NR = K - 2;
  constexpr int K4 = K / 4;
  static_assert(32 * NW >= K, "one row per thread");
  extern __shared__ __align__(16) float tsm[];
  __shared__ float red[NW];
  float *VH = tsm;                 // reflector j in row j
  float *ww = VH + NR * K;         // w of the current step
  float *dd = ww + K, *ee = dd + K, *tau = ee + K;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int ub = blockIdx.x;
  if (ub >= nb) return;
  const int unit = a.ulist ? a.ulist[u0 + ub] : u0 + ub;
  if (a.nkept[unit] <= 0) return;
  const int k = a.k;
  // the team's sum (butterfly in each warp, then the warps in order)
  auto tsum = [&](float v) -> float {
    v = wsum<float>(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float r = red[0];
#pragma unroll
    for (int q = 1; q < NW; q++) r += red[q];
    __syncthreads();
    return r;
  };
  // A = G + (k-1)/infl I (src/letkf_core.F90:101-104), row t
  const float *Gin = a.G + (size_t)unit * packed_size(k);
  const float shift = (float)(k - 1) * 1.0f / a.infl;
  float A[K];
#pragma unroll
  for (int c = 0; c < K; c++) {
    float v = 0.0f;
    if (t < k && c < k) {
      v = t <= c ? Gin[tri_idx(t, c, k)] : Gin[tri_idx(c, t, k)];
      if (t == c) v += shift;
    }
    A[c] = v;
  }
  for (int j = 0; j < k - 2; j++) {
    float *vj = VH + j * K;
    __syncthreads();
    // thread j stores its row whole (columns past k are zero in A); then d_j
    // is taken and columns 0..j are cleared, one per thread
    if (t == j) {
#pragma unroll
      for (int c4 = 0; c4 < K4; c4++)
        *reinterpret_cast<float4 *>(vj + 4 * c4) = make_float4(A[4 * c4], A[4 * c4 + 1], A[4 * c4 + 2], A[4 * c4 + 3]);
    }
    __syncthreads();
    if (t <= j) {
      if (t == j) dd[j] = vj[j];
      vj[t] = 0.0f;
    }
    __syncthreads();
    const float xt = t < K ? vj[t] : 0.0f;
    const float sig = tsum(xt * xt);
    const float x0 = vj[j + 1];
    const float s1 = sig - x0 * x0;
    if (!(s1 > Lim<float>::tiny * sig) || sig == 0.0f) {
      if (t == 0) { tau[j] = 0.0f; ee[j] = x0; }
      continue;
    }
    const float alpha = -copysignf(sqrtf(sig), x0);
    const float v0 = x0 - alpha;
    const float tt = 2.0f / (v0 * v0 + s1);
    __syncthreads();
    if (t == 0) { vj[j + 1] = v0; tau[j] = tt; ee[j] = alpha; }
    __syncthreads();
    // p = t A v
    float acc = 0.0f;
#pragma unroll
    for (int c4 = 0; c4 < K4; c4++) {
      if (4 * c4 + 3 <= j) continue;
      const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * c4);
      acc = __fmaf_rn(A[4 * c4 + 0], v4.x, acc);
      acc = __fmaf_rn(A[4 * c4 + 1], v4.y, acc);
      acc = __fmaf_rn(A[4 * c4 + 2], v4.z, acc);
      acc = __fmaf_rn(A[4 * c4 + 3], v4.w, acc);
    }
    const float p = tt * acc;
    const float vt = t < K ? vj[t] : 0.0f;
    const float beta = 0.5f * tt * tsum(t < K ? __fmaf_rn(p, vt, 0.0f) : 0.0f);
    const float w = (t > j && t < k) ? p - beta * vt : 0.0f;
    if (t < K) ww[t] = w;
    __syncthreads();
    // A -= v w^T + w v^T
#pragma unroll
    for (int c4 = 0; c4 < K4; c4++) {
      if (4 * c4 + 3 <= j) continue;
      const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * c4);
      const float4 w4 = *reinterpret_cast<const float4 *>(ww + 4 * c4);
      A[4 * c4 + 0] = A[4 * c4 + 0] - __fmaf_rn(vt, w4.x, w * v4.x);
      A[4 * c4 + 1] = A[4 * c4 + 1] - __fmaf_rn(vt, w4.y, w * v4.y);
      A[4 * c4 + 2] = A[4 * c4 + 2] - __fmaf_rn(vt, w4.z, w * v4.z);
      A[4 * c4 + 3] = A[4 * c4 + 3] - __fmaf_rn(vt, w4.w, w * v4.w);
    }
  }
  __syncthreads();
  // the last 2 x 2 block: d[k-2], d[k-1], e[k-2]
  if (t == k - 2 || t == k - 1) {
#pragma unroll
    for (int c = 0; c < K; c++) {
      if (c == t) dd[t] = A[c];
      if (t == k - 1 && c == k - 2) ee[k - 2] = A[c];
    }
  }
  if (t == 0) ee[k - 1] = 0.0f;
  __syncthreads();
  // Q = H_0 H_1 ... H_{k-3} I, reflectors from the last to the first; thread
  // t holds column t
#pragma unroll
  for (int r = 0; r < K; r++) A[r] = (r == t && t < k) ? 1.0f : 0.0f;
  for (int j = k - 3; j >= 0; j--) {
    const float tj = tau[j];
    if (tj == 0.0f) continue;
    const float *vj = VH + j * K;
    float s = 0.0f;
#pragma unroll
    for (int r4 = 0; r4 < K4; r4++) {
      if (4 * r4 + 3 <= j) continue;
      const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * r4);
      s = __fmaf_rn(v4.x, A[4 * r4 + 0], s);
      s = __fmaf_rn(v4.y, A[4 * r4 + 1], s);
      s = __fmaf_rn(v4.z, A[4 * r4 + 2], s);
      s = __fmaf_rn(v4.w, A[4 * r4 + 3], s);
    }
    s *= tj;
#pragma unroll
    for (int r4 = 0; r4 < K4; r4++) {
      if (4 * r4 + 3 <= j) continue;
      const float4 v4 = *reinterpret_cast<const float4 *>(vj + 4 * r4);
      A[4 * r4 + 0] -= v4.x * s;
      A[4 * r4 + 1] -= v4.y * s;
      A[4 * r4 + 2] -= v4.z * s;
      A[4 * r4 + 3] -= v4.w * s;
    }
  }
  float *Q = sp.Q + (size_t)ub * k * k;
  if (t < k) {
#pragma unroll
    for (int r = 0; r < K; r++)
      if (r < k) Q[(size_t)r * k + t] = A[r];
  }
  float *de = sp.DE + (size_t)ub * 2 * k;
  for (int i = t; i < k; i += 32 * NW) { de[i] = dd[i]; de[k + i] = ee[i]; }
}

template <int K, int NW>
static size_t tri_t_smem() { return ((size_t)(K - 2) * K + 4 * K) * sizeof(float); }

constexpr int QLT = 64;   // threads (units) per block of k_eig_ql

__global__ void __launch_bounds__(QLT) k_eig_ql(EigArgs a, EigSplit sp, int u0, int nb) {
  extern __shared__ __align__(16) float qs[];   // d[k][QLT], e[k][QLT]
  const int k = a.k, t = threadIdx.x;
  const int ub = blockIdx.x * QLT + t;
  float *d = qs + t, *e = qs + (size_t)k * QLT + t;   // element i at [i * QLT]
#define D(i) d[(size_t)(i) * QLT]
#define E(i) e[(size_t)(i) * QLT]
  if (ub >= nb) return;
  const int unit = a.ulist ? a.ulist[u0 + ub] : u0 + ub;
  if (a.nkept[unit] <= 0) return;
  const float *de = sp.DE + (size_t)ub * 2 * k;
  for (int i = 0; i < k; i++) { D(i) = de[i]; E(i) = de[k + i]; }
  const float tabs = ql_abs_tol(k, d, e, QLT);
  float2 *lg = sp.log + (size_t)ub * sp.cap;
  int pos = 0, bad = 0;
  for (int l = 0; l < k; l++) {
    int iter = 0;
    for (;;) {
      int m = l;
      const float tab = iter >= kQlAbsIter ? tabs : 0.0f;
      while (m < k - 1 && !ql_negligible(E(m), D(m), D(m + 1), tab)) m++;
      if (m == l) break;
      if (++iter > 60) { bad |= 1; break; }
      const float dl = D(l), el = E(l);
      float g = (D(l + 1) - dl) / (2.0f * el);
      float r = sqrtf(g * g + 1.0f);
      g = D(m) - dl + el / (g + copysignf(r, g));
      float s = 1.0f, c = 1.0f, pp = 0.0f;
      float di1 = D(m);
      const int hdr = pos++;
      int cnt = 0;
      bool deflate = false;
      for (int i = m - 1; i >= l; i--) {
        const float ei = E(i), di = D(i);
        const float f = s * ei, b = c * ei;
        r = sqrtf(f * f + g * g);
        E(i + 1) = r;
        if (r == 0.0f) {
          D(i + 1) = di1 - pp;
          E(m) = 0.0f;
          deflate = true;
          break;
        }
        const float ir = __frcp_rn(r);
        s = f * ir;
        c = g * ir;
        g = di1 - pp;
        const float rr = (di - g) * s + 2.0f * c * b;
        pp = s * rr;
        D(i + 1) = g + pp;
        g = c * rr - b;
        di1 = di;
        if (pos < sp.cap) lg[pos] = make_float2(c, s);
        pos++;
        cnt++;
      }
      if (hdr < sp.cap) lg[hdr] = make_float2(__int_as_float(m), __int_as_float(cnt));
      if (!deflate) { D(l) = D(l) - pp; E(l) = g; E(m) = 0.0f; }
    }
    if (bad) break;
  }
#undef D
#undef E
  // -1: no convergence (status bit 1); -2: log overflow (k_eig_vec reruns the QL)
  sp.logn[ub] = bad ? -1 : (pos > sp.cap ? -2 : pos);
  float *lam = sp.lam + (size_t)ub * k;
  for (int i = 0; i < k; i++) lam[i] = d[(size_t)i * QLT];
  if (bad && !a.flag_list) atomicOr(a.status, bad);   // with flagging, the FP64 re-solve takes the unit
}

template <int NQ, int NW>
__global__ void k_eig_vec(EigArgs a, EigSplit sp, int wpb, int u0, int nb) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float tred[NW];
  const int k = a.k, ld = k + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = NW == 1 ? warp : 0;
  const int ub = blockIdx.x * wpb + slot;
  if (ub >= nb) return;
  const int unit = a.ulist ? a.ulist[u0 + ub] : u0 + ub;
  if (a.nkept[unit] <= 0) return;
  const int total = sp.logn[ub];
  if (total == -1) return;                // no convergence: status set by k_eig_ql
  EigWork W(sm + (size_t)slot * eig_floats_per_warp(k), k);
  const Team<NW> T{NW == 1 ? lane : (int)threadIdx.x, lane, warp, tred};
  const int tt = T.tt, TS = T.TS;
  float *A = W.A;
  const float *Q = sp.Q + (size_t)ub * k * k;
  for (int t = tt; t < k * k; t += TS) A[(t / k) * ld + (t % k)] = Q[t];
  const float *lam = sp.lam + (size_t)ub * k;
  for (int t = tt; t < k; t += TS) W.d[t] = lam[t];
  const float *G = a.G + (size_t)unit * packed_size(k);
  T.sync();
  int bad = 0;
  if (total < 0) {
    // the rotation log overflowed: the first warp runs the QL here from the
    // tridiagonal form, on all rows
    const float *de = sp.DE + (size_t)ub * 2 * k;
    for (int t = tt; t < k; t += TS) { W.d[t] = de[t]; W.e[t] = de[k + t]; }
    T.sync();
    constexpr int NQW = 32 * NW * NQ <= 64 ? 2 : 4;
    if (warp == 0 || NW == 1) eig_ql_warp<NQW>(k, W, lane, bad);
  } else {
    // replay the rotations on the thread's rows (tt + TS q).  The log passes
    // through a window in the scratch vectors e .. gl (free until the
    // transform; 8-byte aligned), refilled by the team at a sweep boundary
    // whenever the next sweep (header + cnt <= k entries) would not fit, so
    // that a sweep's rotations are read with one broadcast load each
    const float2 *lg = sp.log + (size_t)ub * sp.cap;
    const int wofs = (k * (k + 2)) & 1;   // e sits k (k + 2) floats into the unit's scratch
    float2 *win = reinterpret_cast<float2 *>(W.e + wofs);
    const int WN = (7 * k + 8 - wofs) / 2;   // e, tau, bv, p, w, fl, gl and the 8 spare floats
    bool own[NQ];
    float *qr[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      own[q] = tt + TS * q < k;
      qr[q] = A + (own[q] ? tt + TS * q : 0) * ld;
    }
    int base = 0;
    auto refill = [&](int from) {   // team-uniform
      T.sync();
      base = from;
      const int n = total - from < WN ? total - from : WN;
      for (int t = tt; t < n; t += TS) win[t] = lg[from + t];
      T.sync();
    };
    refill(0);
    int pidx = 0;
    while (pidx < total) {
      if (pidx >= base + WN) refill(pidx);
      const float2 h = win[pidx - base];
      const int m = __float_as_int(h.x), cnt = __float_as_int(h.y);
      if (m < 1 || m >= k || cnt < 0 || cnt > m || pidx + 1 + cnt > total) { bad |= 32; break; }   // malformed log
      if (pidx + 1 + cnt > base + WN) refill(pidx);
      const float2 *rot = win + (pidx + 1 - base);
      pidx += 1 + cnt;
      float z[NQ];
#pragma unroll
      for (int q = 0; q < NQ; q++) z[q] = own[q] ? qr[q][m] : 0.0f;
#pragma unroll 2
      for (int r = 0; r < cnt; r++) {
        const float2 cs = rot[r];
        const float c = cs.x, s = cs.y;
        const int i = m - 1 - r;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
          const float av = own[q] ? qr[q][i] : 0.0f;
          if (own[q]) { qr[q][i + 1] = s * av + c * z[q]; z[q] = c * av - s * z[q]; }
        }
      }
#pragma unroll
      for (int q = 0; q < NQ; q++)
        if (own[q]) qr[q][m - cnt] = z[q];
    }
  }
  // b after the replay: its slot is part of the log window
  T.sync();
  for (int i = tt; i < k; i += TS) W.bv[i] = G[k * (k + 1) / 2 + i];
  T.sync();
  eig_transform<NQ>(a, unit, W, T, bad);
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && a.flag_list) {
    if (lane == 0) sp.logn[ub] = -1;   // k_eig_flag hands the unit to the FP64 re-solve
  } else if (bad && lane == 0) {
    atomicOr(a.status, bad);
  }
}

// FP64 re-solve candidates of a batch (warp per unit, after k_eig_vec):
// the FP32 solve failed, or two relevant eigenvalues lie within
// gap_thresh * max l of each other.  The eigenvalues at the (k-1)/infl floor
// (the null space of the Gram, k - n of them when n < k) are exactly
// degenerate and harmless, since T is a function of the matrix and not of
// the basis chosen in an eigenspace; they are left out of the test.
__global__ void k_eig_flag(EigArgs a, EigSplit sp, int u0, int nb) {
  const int lane = threadIdx.x & 31;
  const int ub = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (ub >= nb) return;
  const int unit = a.ulist ? a.ulist[u0 + ub] : u0 + ub;
  if (a.nkept[unit] <= 0) return;
  const int k = a.k;
  bool flag = sp.logn[ub] == -1;
  if (!flag) {
    const float *lam = sp.lam + (size_t)ub * k;
    float lmax = 0.0f;
    for (int i = lane; i < k; i += 32) lmax = fmaxf(lmax, lam[i]);
    for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    // rounding level of the FP32 eigenvalues: a few k eps of the largest
    const float floor_v = (float)(k - 1) / a.infl;
    const float tol = 4.0f * (float)k * 1.1920929e-7f * lmax;
    float gap = 3.0e38f;
    for (int i = lane; i < k; i += 32) {
      const float li = lam[i];
      if (li - floor_v <= tol) continue;
      for (int j = 0; j < k; j++) {
        const float lj = lam[j];
        if (j != i && lj - floor_v > tol) gap = fminf(gap, fabsf(li - lj));
      }
    }
    for (int o = 16; o > 0; o >>= 1) gap = fminf(gap, __shfl_xor_sync(0xffffffffu, gap, o));
    flag = gap <= a.gap_thresh * lmax;
  }
  if (flag && lane == 0) {
    const int pos = atomicAdd(a.flag_n, 1);
    if (pos < a.flag_cap) a.flag_list[pos] = unit;
    else atomicOr(a.status, 128);   // list full: the unit keeps its FP32 solve
  }
}

// Implicit-shift QL for a team of NW warps: per sweep, warp 0 evaluates the
// scalar recurrence (as eig_ql_warp: redundantly on its lanes, lane 0
// writing d, e and the rotations (c, s) of the sweep into cs_c / cs_s), then
// every thread of the team applies the sweep's rotations to its own rows of
// Q (rows tt + TS q) in the same order and arithmetic as eig_ql_warp.
// ctl[0]: the sweep's m (-1: l converged, -2: no convergence), ctl[1]: the
// lowest rotated column.
template <int NQ, int NW, class R>
__device__ __forceinline__ void eig_ql_team(int k, EigWork<R> &W, const Team<NW, R> &T, R *cs_c, R *cs_s,
                                            int *ctl, int &bad) {
  const int ld = k + 1, tt = T.tt, TS = T.TS, lane = T.lane;
  R *A = W.A, *d = W.d, *e = W.e;
  bool own[NQ];
  R *qr[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    own[q] = tt + TS * q < k;
    qr[q] = A + (own[q] ? tt + TS * q : 0) * ld;
  }
  const R tabs = ql_abs_tol(k, d, e, 1);
  for (int l = 0; l < k; l++) {
    int iter = 0;
    for (;;) {
      if (T.warp == 0) {
        int m = k - 1;
        for (int base = l; base < k - 1; base += 32) {
          const int mm = base + lane;
          bool small = false;
          if (mm < k - 1) small = ql_negligible(e[mm], d[mm], d[mm + 1], iter >= kQlAbsIter ? tabs : R(0));
          const unsigned bal = __ballot_sync(0xffffffffu, small);
          if (bal) { m = base + __ffs(bal) - 1; break; }
        }
        int c0 = m, c1 = l;
        if (m == l) {
          c0 = -1;
        } else if (++iter > 60) {
          c0 = -2;
        } else {
          const R dl = d[l], el = e[l];
          R g = (d[l + 1] - dl) / (R(2) * el);
          R r = sqrt(g * g + R(1));
          g = d[m] - dl + el / (g + copysign(r, g));
          R s = R(1), c = R(1), pp = R(0);
          R di1 = d[m];
          R ei = e[m - 1], di = d[m - 1];
          int i = m - 1;
          bool deflate = false;
          for (; i >= l; i--) {
            const int in = i > 0 ? i - 1 : 0;
            const R ei_n = e[in], di_n = d[in];
            const R f = s * ei, b = c * ei;
            r = sqrt(f * f + g * g);
            if (lane == 0) e[i + 1] = r;
            if (r == R(0)) {
              if (lane == 0) { d[i + 1] = di1 - pp; e[m] = R(0); }
              deflate = true;
              break;
            }
            const R ir = rcpr(r);
            s = f * ir;
            c = g * ir;
            g = di1 - pp;
            const R rr = (di - g) * s + R(2) * c * b;
            pp = s * rr;
            if (lane == 0) { d[i + 1] = g + pp; cs_c[i] = c; cs_s[i] = s; }
            g = c * rr - b;
            di1 = di;
            ei = ei_n;
            di = di_n;
          }
          c1 = deflate ? i + 1 : l;
          if (!deflate && lane == 0) { d[l] = d[l] - pp; e[l] = g; e[m] = R(0); }
        }
        if (lane == 0) { ctl[0] = c0; ctl[1] = c1; }
      }
      T.sync();
      const int m = ctl[0], ilo = ctl[1];
      if (m < 0) {
        if (m == -2) bad = 1;
        T.sync();   // ctl is read by every thread before warp 0 writes it again
        break;
      }
      R z[NQ];
#pragma unroll
      for (int q = 0; q < NQ; q++) z[q] = own[q] ? qr[q][m] : R(0);
      for (int i = m - 1; i >= ilo; i--) {
        const R c = cs_c[i], s = cs_s[i];
#pragma unroll
        for (int q = 0; q < NQ; q++)
          if (own[q]) {
            const R av = qr[q][i];
            qr[q][i + 1] = s * av + c * z[q];
            z[q] = c * av - s * z[q];
          }
      }
#pragma unroll
      for (int q = 0; q < NQ; q++)
        if (own[q]) qr[q][ilo] = z[q];
      T.sync();
    }
    if (bad) break;
  }
  T.sync();
}

// FP64 eigensolve + transform, a team of NW warps per unit (one unit per
// block at a time), grid-stride over the units: ulist / ubase + 0..nunits,
// or (range != null) the flagged entries flag_list[range[1] ..
// min(range[0], flag_cap)).  GB300 runs FP64 at 1/64 of the FP32 rate, so a
// single unit's latency (the re-solve of a few flagged units) is spread over
// the SM's four schedulers.
template <int NW>
__global__ void k_eig64(EigArgs a, int ubase, const int *range) {
  extern __shared__ __align__(16) double smd[];
  __shared__ double tred[NW];
  __shared__ int ctl[2];
  const int k = a.k;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int beg = 0, end = a.nunits;
  const int *list = a.ulist;
  if (range) {
    beg = range[1];
    end = min(range[0], a.flag_cap);
    list = a.flag_list;
  }
  EigWork<double> W(smd, k);
  const Team<NW, double> T{(int)threadIdx.x, lane, warp, tred};
  for (int un = beg + blockIdx.x; un < end; un += gridDim.x) {
    const int unit = list ? list[un] : ubase + un;
    if (a.nkept[unit] <= 0) continue;
    __syncthreads();   // the previous unit's transform has read the work arrays
    eig_load(a, unit, W, T);
    eig_tridiag_q<1>(k, W, T);
    int bad = 0;
    eig_ql_team<1>(k, W, T, W.p, W.w, ctl, bad);
    eig_transform<1>(a, unit, W, T, bad);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && lane == 0) atomicOr(a.status, bad);
  }
}

}  // namespace

namespace {
// warps per unit of the FP64 kernel: every row of Q on its own thread
int eig64_team(int k) { return k <= 64 ? 2 : 4; }

template <int NW>
cudaError_t eig64_go_t(cudaStream_t st, const EigArgs &a, int ubase, const int *range, int blocks, int *launches) {
  const size_t smem = (size_t)eig_floats_per_warp(a.k) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_eig64<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_eig64<NW><<<blocks, 32 * NW, smem, st>>>(a, ubase, range);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t eig64_go(cudaStream_t st, const EigArgs &a, int ubase, const int *range, int blocks, int *launches) {
  return eig64_team(a.k) == 2 ? eig64_go_t<2>(st, a, ubase, range, blocks, launches)
                              : eig64_go_t<4>(st, a, ubase, range, blocks, launches);
}

// resident units per SM (one per block), from the shared memory of one unit
int eig64_per_sm(int k) {
  const size_t per = (size_t)eig_floats_per_warp(k) * sizeof(double) + 1024;
  return std::max(1, std::min(16, (int)((227 * 1024) / per)));
}
}  // namespace

cudaError_t launch_eig64(cudaStream_t st, const EigArgs &a, int ubase, int *launches) {
  if (a.nunits <= 0) return cudaSuccess;
  return eig64_go(st, a, ubase, nullptr, std::min(a.nunits, 152 * eig64_per_sm(a.k)), launches);
}

cudaError_t launch_eig64_flagged(cudaStream_t st, const EigArgs &a, int *launches) {
  if (!a.flag_list || a.flag_cap <= 0) return cudaSuccess;
  // one block per flagged unit up to the resident limit; the count stays on the device
  cudaError_t e = eig64_go(st, a, 0, a.flag_n, std::min(a.flag_cap, 152 * eig64_per_sm(a.k)), launches);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(a.flag_n + 1, a.flag_n, sizeof(int), cudaMemcpyDeviceToDevice, st);
}

cudaError_t launch_eig(cudaStream_t st, const EigArgs &a, int *launches);

static int eig_wpb_floats(int floats) {
  // warps per block: the most resident warps per SM for this unit size
  const size_t per = (size_t)floats * sizeof(float);
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
  return wpb;
}

static int eig_wpb(int k) { return eig_wpb_floats(eig_floats_per_warp(k)); }

// warps per unit of k_eig_vec, measured on GB300: k <= 64 one warp (two
// rows per lane; C2, k = 40: 26 ms against 33 with two warps), k > 64 four
// warps (one row per thread; C4, k = 100: eigensolve 693 ms against 717 with
// two warps of two rows per thread, whose 64-thread teams left 15% of the
// warp slots filled)
static int eig_team(int k) { return k <= 64 ? 1 : 4; }

// The first stage, in registers with Q formed there: one warp up to k = 48
// (k_eig_tri_r), above a team of ceil(k / 32) warps with one row per thread
// (k_eig_tri_t).  Measured on GB300 (eigensolve ms): k = 40 shared-memory
// full matrix 25.8, packed lower triangle 26.6, registers 23.7; k = 64 full
// 57.2, packed 53.8, team registers 38.4; C4 (k = 100) full 1057, packed
// (Q formed in k_eig_vec) 855, four-warp team registers 718.  The shared-memory
// and packed forms are not built.

// the register-resident first stage (k <= 48)
static cudaError_t launch_tri_r(cudaStream_t st, const EigArgs &a, const EigSplit &sp, int u0, int nb) {
  const int grid = (nb + RWPB - 1) / RWPB;
  switch ((a.k + 7) & ~7) {
  case 8: k_eig_tri_r<8><<<grid, 32 * RWPB, 0, st>>>(a, sp, u0, nb); break;
  case 16: k_eig_tri_r<16><<<grid, 32 * RWPB, 0, st>>>(a, sp, u0, nb); break;
  case 24: k_eig_tri_r<24><<<grid, 32 * RWPB, 0, st>>>(a, sp, u0, nb); break;
  case 32: k_eig_tri_r<32><<<grid, 32 * RWPB, 0, st>>>(a, sp, u0, nb); break;
  case 40: k_eig_tri_r<40><<<grid, 32 * RWPB, 0, st>>>(a, sp, u0, nb); break;
  case 48: k_eig_tri_r<48><<<grid, 32 * RWPB, 0, st>>>(a, sp, u0, nb); break;
  default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// the register-resident first stage with a two-warp team per unit (48 < k <= 64)
template <int K, int NW>
static cudaError_t launch_tri_t_k(cudaStream_t st, const EigArgs &a, const EigSplit &sp, int u0, int nb) {
  const size_t smem = tri_t_smem<K, NW>();
  cudaError_t e = cudaFuncSetAttribute(k_eig_tri_t<K, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_eig_tri_t<K, NW><<<nb, 32 * NW, smem, st>>>(a, sp, u0, nb);
  return cudaGetLastError();
}

static cudaError_t launch_tri_t(cudaStream_t st, const EigArgs &a, const EigSplit &sp, int u0, int nb) {
  switch ((a.k + 7) & ~7) {
  case 56: return launch_tri_t_k<56, 2>(st, a, sp, u0, nb);
  case 64: return launch_tri_t_k<64, 2>(st, a, sp, u0, nb);
  case 72: return launch_tri_t_k<72, 3>(st, a, sp, u0, nb);
  case 80: return launch_tri_t_k<80, 3>(st, a, sp, u0, nb);
  case 88: return launch_tri_t_k<88, 3>(st, a, sp, u0, nb);
  case 96: return launch_tri_t_k<96, 3>(st, a, sp, u0, nb);
  case 104: return launch_tri_t_k<104, 4>(st, a, sp, u0, nb);
  case 112: return launch_tri_t_k<112, 4>(st, a, sp, u0, nb);
  case 120: return launch_tri_t_k<120, 4>(st, a, sp, u0, nb);
  case 128: return launch_tri_t_k<128, 4>(st, a, sp, u0, nb);
  default: return cudaErrorInvalidValue;
  }
}

template <int NQ, int NW>
static cudaError_t launch_split_t(cudaStream_t st, const EigArgs &a, const EigSplit &sp, int batch, int ustart,
                                  int ucount, int *launches) {
  // k_eig_vec: its own warps per block from its shared memory
  const int wpb = NW == 1 ? eig_wpb(a.k) : 1;
  const size_t smem = (size_t)wpb * eig_floats_per_warp(a.k) * sizeof(float);
  const int threads = NW == 1 ? 32 * wpb : 32 * NW;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_eig_vec<NQ, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
      cudaSuccess)
    return e;
  const size_t qsm = (size_t)2 * a.k * QLT * sizeof(float);
  if ((e = cudaFuncSetAttribute(k_eig_ql, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)qsm)) != cudaSuccess)
    return e;
  const int uend = ustart + ucount;
  for (int u0 = ustart; u0 < uend; u0 += batch) {
    const int nb = uend - u0 < batch ? uend - u0 : batch;
    if ((e = a.k <= 48 ? launch_tri_r(st, a, sp, u0, nb) : launch_tri_t(st, a, sp, u0, nb)) != cudaSuccess) return e;
    k_eig_ql<<<(nb + QLT - 1) / QLT, QLT, qsm, st>>>(a, sp, u0, nb);
    k_eig_vec<NQ, NW><<<(nb + wpb - 1) / wpb, threads, smem, st>>>(a, sp, wpb, u0, nb);
    (*launches) += 3;
    if (a.flag_list) {
      k_eig_flag<<<(nb + 7) / 8, 256, 0, st>>>(a, sp, u0, nb);
      (*launches)++;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int eig_log_cap(int k) { return 2 * k * k + 4 * k + 64; }

size_t eig_split_bytes_per_unit(int k) {
  return (size_t)k * k * 4 + (size_t)2 * k * 4 + (size_t)eig_log_cap(k) * 8 + 4 + (size_t)k * 4;
}

cudaError_t launch_eig_split(cudaStream_t st, const EigArgs &a, const EigSplit &sp, int batch, int ustart, int ucount,
                             int *launches) {
  if (ucount <= 0) return cudaSuccess;
  if (eig_team(a.k) == 1) return launch_split_t<2, 1>(st, a, sp, batch, ustart, ucount, launches);   // k <= 64
  return launch_split_t<1, 4>(st, a, sp, batch, ustart, ucount, launches);                            // k <= 128
}

cudaError_t launch_eig_debug(cudaStream_t st, int nunits, int k, const float *G, const int *nkept, float *T,
                             int *status, int prec, float gap_thresh, int *nfp64) {
  EigArgs a;
  a.wbar = nullptr;
  a.ulist = nullptr;
  a.flag_list = nullptr;
  a.flag_n = nullptr;
  a.flag_cap = 0;
  a.gap_thresh = gap_thresh;
  a.nunits = nunits;
  a.k = k;
  a.infl = 1.0f;
  a.G = G;
  a.nkept = nkept;
  a.T = T;
  a.status = status;
  *nfp64 = 0;
  int l = 0;
  if (prec == LGPU_PREC_FP64) {
    cudaError_t e = launch_eig64(st, a, 0, &l);
    cudaError_t e2 = cudaStreamSynchronize(st);
    *nfp64 = nunits;
    return e != cudaSuccess ? e : e2;
  }
  // the split pipeline, as lgpu_solver_run uses it
  const size_t per = eig_split_bytes_per_unit(k);
  const size_t n = nunits > 0 ? nunits : 1;
  unsigned char *buf = nullptr;
  // six arrays, each start rounded up to 256 bytes (at most 5 * 255 bytes of padding)
  cudaError_t e = cudaMalloc(&buf, per * n + 16 + 4 * n + 6 * 256);
  if (e != cudaSuccess) return e;
  EigSplit sp;
  size_t off = 0;
  auto take = [&](size_t bytes) { unsigned char *p = buf + off; off += (bytes + 255) & ~(size_t)255; return p; };
  sp.Q = reinterpret_cast<float *>(take(n * k * k * 4));
  sp.DE = reinterpret_cast<float *>(take(n * 2 * k * 4));
  sp.log = reinterpret_cast<float2 *>(take(n * (size_t)eig_log_cap(k) * 8));
  sp.logn = reinterpret_cast<int *>(take(n * 4));
  sp.lam = reinterpret_cast<float *>(take(n * k * 4));
  sp.cap = eig_log_cap(k);
  if (prec == LGPU_PREC_FP32_RESOLVE) {
    a.flag_n = reinterpret_cast<int *>(take(16 + 4 * n));
    a.flag_list = a.flag_n + 4;
    a.flag_cap = (int)n;
    e = cudaMemsetAsync(a.flag_n, 0, 16, st);
  }
  if (e == cudaSuccess) e = launch_eig_split(st, a, sp, nunits, 0, nunits, &l);
  if (e == cudaSuccess && a.flag_list) e = launch_eig64_flagged(st, a, &l);
  if (e == cudaSuccess && a.flag_n) e = cudaMemcpyAsync(nfp64, a.flag_n, 4, cudaMemcpyDeviceToHost, st);
  cudaError_t e2 = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (*nfp64 > (int)n) *nfp64 = (int)n;
  return e != cudaSuccess ? e : e2;
}

cudaError_t launch_eig(cudaStream_t st, const EigArgs &a, int *launches) {
  if (a.nunits <= 0) return cudaSuccess;
  const int wpb = eig_wpb(a.k);
  const size_t per = (size_t)eig_floats_per_warp(a.k) * sizeof(float);
  const size_t smem = (size_t)wpb * per;
  auto fused = a.k > 64 ? k_eig<4> : k_eig<2>;
  cudaError_t e = cudaFuncSetAttribute(fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = (a.nunits + wpb - 1) / wpb;
  fused<<<grid, 32 * wpb, smem, st>>>(a, wpb);
  (*launches)++;
  return cudaGetLastError();
}

}  // namespace lgpu
