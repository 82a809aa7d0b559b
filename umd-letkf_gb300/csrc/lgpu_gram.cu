// lgpu_gram.cu -- fused local-observation search, localisation and Gram
// product, one CTA per (column, localisation group) unit.
//
// Replaces, per unit, src/letkf_solver.F90:210-263 (search, gather,
// localize, keep r > 1e-4) and the data-heavy half of letkf_core_solve
// (src/letkf_core.F90:92-98): G = (Yb diag(rloc/err)) Yb^T and the
// right-hand side b = (Yb diag(rloc/err)) dep, which the reference forms
// later as Pa * hdxb_rinv * dep (:118-125).  The upper triangle of G and b
// are written packed per unit; the eigensolve stage consumes them.
//
// Data flow per CTA: the search circle's index window is a list of
// contiguous runs of the cell-sorted observation table; threads stream
// candidates (32 B records, coalesced), apply the exact distance test and
// the localizer, compact the kept observations into a ring of staging
// slots, and every 64 kept observations load their hx rows into shared
// memory (scaled copy A = y*rloc/err and plain copy B = [y, dep]) and
// accumulate the k x (k+1) block with 4x4 register tiles.
#include "lgpu_internal.cuh"

namespace lgpu {

namespace {

constexpr int GT = 256;     // threads per CTA = candidates per chunk
constexpr int BUF = 64;     // kept observations per Gram flush
constexpr int RING = 512;   // staging ring (>= GT + BUF, power of two)
constexpr int MAXSEG = 2 * kNB;

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct __align__(16) GramSmem {
  int seg_start[MAXSEG];
  int seg_pref[MAXSEG + 1];
  int ring_pos[RING];
  float ring_w[RING];
  float ring_d[RING];
  int wcnt[GT / 32];
  int wcnt2[GT / 32];
  float wred[GT / 32];
  int total;
  int nkept_chunk;
  int ncand_chunk;
};

// NSET register tile sets per thread: 1 while the k x (k+1) block has at most
// GT 4x4 tiles (k <= 60), else ceil(tiles / GT) with thread t owning tiles
// t, t + GT, ... (k <= 128: at most 5 sets)
template <int NSET>
__global__ void __launch_bounds__(GT) k_gram(GramArgs a) {
  extern __shared__ __align__(16) float dyn[];
  __shared__ GramSmem S;
  const int k = a.k, kp = a.kp;
  const int ntn = (k + 1 + 3) / 4;       // column tiles incl. RHS column
  const int ntm = kp / 4;                // row tiles
  const int kb = 4 * ntn > kp ? 4 * ntn : kp;  // B row width
  float *As = dyn;                       // [BUF][kp]
  float *Bs = As + BUF * kp;             // [BUF][kb]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ntiles = ntm * ntn;
  const int nslice = ntiles >= GT ? 1 : GT / ntiles;
  const bool gram_thread = tid < ntiles * nslice;
  const int tile = gram_thread ? tid % ntiles : 0;
  const int slice = gram_thread ? tid / ntiles : 0;
  const int mi = tile / ntn, ni = tile % ntn;
  // more tiles than threads (k > 60): threads also own tiles tid + s GT
  int mix[NSET > 1 ? NSET : 1], nix[NSET > 1 ? NSET : 1];
  bool tset[NSET > 1 ? NSET : 1];
#pragma unroll
  for (int q = 1; q < NSET; q++) {
    tset[q] = ntiles > GT && tid + q * GT < ntiles;
    mix[q] = tset[q] ? (tid + q * GT) / ntn : 0;
    nix[q] = tset[q] ? (tid + q * GT) % ntn : 0;
  }

  for (int unit = blockIdx.x; unit < a.nunits; unit += gridDim.x) {
    const int act = unit / a.groups, g = unit % a.groups;
    const int col = a.active[act];
    const ColPar cp = a.cp[col];

    // ---- 1. index window -> runs of the sorted observation table
    const int nb = cp.b1 - cp.b0 + 1;
    if (tid < nb) {
      int b = cp.b0 + tid;
      int nl = a.geom->nlon[b], off = a.geom->off[b];
      int s0 = 0, l0 = 0, s1 = 0, l1 = 0;
      bool whole = cp.dlon >= 180.0f;
      int clo = 0, chi = nl - 1;
      if (!whole) {
        clo = (int)floorf((cp.lonn - cp.dlon) * (float)nl / 360.0f);
        chi = (int)floorf((cp.lonn + cp.dlon) * (float)nl / 360.0f);
        if (chi - clo + 1 >= nl) whole = true;
      }
      if (whole) {
        s0 = a.obs.cell_start[off];
        l0 = a.obs.cell_start[off + nl] - s0;
      } else {
        int lo = clo, hi = chi;
        if (lo < 0) {            // wraps below 0
          int w0 = lo + nl;
          s0 = a.obs.cell_start[off + w0];
          l0 = a.obs.cell_start[off + nl] - s0;
          s1 = a.obs.cell_start[off];
          l1 = a.obs.cell_start[off + hi + 1] - s1;
        } else if (hi >= nl) {   // wraps above nl-1
          s0 = a.obs.cell_start[off + lo];
          l0 = a.obs.cell_start[off + nl] - s0;
          s1 = a.obs.cell_start[off];
          l1 = a.obs.cell_start[off + (hi - nl) + 1] - s1;
        } else {
          s0 = a.obs.cell_start[off + lo];
          l0 = a.obs.cell_start[off + hi + 1] - s0;
        }
      }
      S.seg_start[2 * tid] = s0;
      S.seg_start[2 * tid + 1] = s1;
      S.seg_pref[2 * tid] = l0;        // lengths for now
      S.seg_pref[2 * tid + 1] = l1;
    }
    __syncthreads();
    // exclusive scan of the 2*nb run lengths (<= 360): two per thread
    {
      const int nseg = 2 * nb;
      int i0 = 2 * tid, i1 = 2 * tid + 1;
      int v0 = i0 < nseg ? S.seg_pref[i0] : 0;
      int v1 = i1 < nseg ? S.seg_pref[i1] : 0;
      int x = v0 + v1, incl = x;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) S.wcnt[wid] = incl;
      __syncthreads();
      if (wid == 0) {
        int s = lane < GT / 32 ? S.wcnt[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, s, o);
          if (lane >= o) s += y;
        }
        if (lane < GT / 32) S.wcnt[lane] = s;
      }
      __syncthreads();
      int base = (wid > 0 ? S.wcnt[wid - 1] : 0) + incl - x;
      __syncthreads();
      if (i0 < nseg) S.seg_pref[i0] = base;
      if (i1 < nseg) S.seg_pref[i1] = base + v0;
      if (tid == 0) {
        S.total = S.wcnt[GT / 32 - 1];
        S.seg_pref[nseg] = S.total;
      }
      __syncthreads();
    }
    const int nseg = 2 * nb;
    const int total = S.total;

    // ---- 2. stream candidates, localize, compact, accumulate
    float acc[4][4], accx[NSET > 1 ? NSET : 1][4][4];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[r][c] = 0.0f;
#pragma unroll
    for (int q = 1; q < NSET; q++)
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) accx[q][r][c] = 0.0f;
    int head = 0, tail = 0;          // ring indices (monotone)
    int ncand = 0, nkept = 0;        // block totals
    float rsum = 0.0f;               // per-thread partial sum of kept weights

    const float rmax = cp.rmax;
    // chord^2 bound of the search radius with a relative margin (quick reject)
    const float hq = fminf(rmax / 12742000.0f, 1.5707963f);
    const float sh = sinf(hq);
    const float c2max = 4.0f * sh * sh * 1.0001f + 1e-12f;

    for (int base = 0; base < total; base += GT) {
      const int j = base + tid;
      bool cand = false, keep = false;
      int pos = 0;
      float w = 0.0f, dep = 0.0f, r = 0.0f;
      if (j < total) {
        // locate the run holding candidate j (binary search over <= 361 prefixes)
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (S.seg_pref[mid] <= j) lo = mid; else hi = mid - 1;
        }
        pos = S.seg_start[lo] + (j - S.seg_pref[lo]);
        const float4 A = a.obs.A[pos];
        const float c2 = chord2_exact(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z);
        if (c2 <= c2max) {
          const float d = dist_from_chord2(c2);
          if (d <= rmax) {
            cand = true;
            const float4 B = a.obs.B[pos];
            r = localize(a.loc, cp, g, d, B.y, B.z, B.w);
            if (r > kKeep) {
              keep = true;
              w = __fdiv_rn(r, A.w);
              dep = B.x;
              rsum += r;
            }
          }
        }
      }
      // block-wide ordered compaction of kept candidates
      const unsigned bk = __ballot_sync(0xffffffffu, keep);
      const unsigned bc = __ballot_sync(0xffffffffu, cand);
      if (lane == 0) { S.wcnt[wid] = __popc(bk); S.wcnt2[wid] = __popc(bc); }
      __syncthreads();
      int woff = 0, ktot = 0, ctot = 0;
#pragma unroll
      for (int q = 0; q < GT / 32; q++) {
        int v = S.wcnt[q];
        woff += (q < wid) ? v : 0;
        ktot += v;
        ctot += S.wcnt2[q];
      }
      if (keep) {
        int slot = (tail + woff + __popc(bk & ((1u << lane) - 1u))) & (RING - 1);
        S.ring_pos[slot] = pos;
        S.ring_w[slot] = w;
        S.ring_d[slot] = dep;
      }
      tail += ktot;
      nkept += ktot;
      ncand += ctot;
      __syncthreads();

      // flush full batches
      while (tail - head >= BUF || (base + GT >= total && tail > head)) {
        const int cnt = min(BUF, tail - head);
        // stage hx rows: A = y * w, B = [y, dep, 0...]
        const int q4 = kp / 4, qb = kb / 4;
        const float4 *hx4 = reinterpret_cast<const float4 *>(a.obs.hx);
        for (int t = tid; t < BUF * qb; t += GT) {
          const int e = t / qb, q = t % qb;
          float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
          float we = 0.0f, de = 0.0f;
          if (e < cnt) {
            const int slot = (head + e) & (RING - 1);
            we = S.ring_w[slot];
            de = S.ring_d[slot];
            if (q < q4) y = hx4[(size_t)S.ring_pos[slot] * q4 + q];
          }
          if (q < q4) {
            reinterpret_cast<float4 *>(As + e * kp)[q] = make_float4(y.x * we, y.y * we, y.z * we, y.w * we);
          }
          float4 yb = y;
          if (q == (k >> 2)) {
            const int c = k & 3;
            if (c == 0) yb.x = de; else if (c == 1) yb.y = de; else if (c == 2) yb.z = de; else yb.w = de;
          }
          reinterpret_cast<float4 *>(Bs + e * kb)[q] = yb;
        }
        __syncthreads();
        if (gram_thread) {
          const float *ap = As + 4 * mi;
          const float *bp = Bs + 4 * ni;
          for (int e = slice; e < cnt; e += nslice) {
            const float4 av = *reinterpret_cast<const float4 *>(ap + e * kp);
            const float4 bv = *reinterpret_cast<const float4 *>(bp + e * kb);
            const float ar[4] = {av.x, av.y, av.z, av.w};
            const float br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
            for (int r2 = 0; r2 < 4; r2++)
#pragma unroll
              for (int c = 0; c < 4; c++) acc[r2][c] = __fmaf_rn(ar[r2], br[c], acc[r2][c]);
          }
#pragma unroll
          for (int q = 1; q < NSET; q++) {
            if (!tset[q]) continue;
            const float *ap2 = As + 4 * mix[q];
            const float *bp2 = Bs + 4 * nix[q];
            for (int e = 0; e < cnt; e++) {
              const float4 av = *reinterpret_cast<const float4 *>(ap2 + e * kp);
              const float4 bv = *reinterpret_cast<const float4 *>(bp2 + e * kb);
              const float ar[4] = {av.x, av.y, av.z, av.w};
              const float br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
              for (int r2 = 0; r2 < 4; r2++)
#pragma unroll
                for (int c = 0; c < 4; c++) accx[q][r2][c] = __fmaf_rn(ar[r2], br[c], accx[q][r2][c]);
            }
          }
        }
        head += cnt;
        __syncthreads();
      }
    }

    // ---- 3. reduce the K-split partial tiles and write G | b
    float *red = As;   // ntiles*16 floats (fits in the A/B staging area)
    for (int s = 0; s < nslice; s++) {
      if (gram_thread && slice == s) {
#pragma unroll
        for (int r2 = 0; r2 < 4; r2++)
#pragma unroll
          for (int c = 0; c < 4; c++) {
            float *dst = red + tile * 16 + r2 * 4 + c;
            *dst = (s == 0) ? acc[r2][c] : *dst + acc[r2][c];
          }
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 1; q < NSET; q++) {
      if (!tset[q]) continue;
#pragma unroll
      for (int r2 = 0; r2 < 4; r2++)
#pragma unroll
        for (int c = 0; c < 4; c++) red[(tid + q * GT) * 16 + r2 * 4 + c] = accx[q][r2][c];
    }
    __syncthreads();
    float *G = a.G + (size_t)unit * packed_size(k);
    for (int t = tid; t < packed_size(k); t += GT) {
      int i, jj;
      packed_ij(t, k, i, jj);
      const int tl = (i >> 2) * ntn + (jj >> 2);
      G[t] = red[tl * 16 + (i & 3) * 4 + (jj & 3)];
    }
    // diagnostics: src/letkf_solver.F90:220, :266-267
    float rs = warp_sum(rsum);
    if (lane == 0) S.wred[wid] = rs;
    __syncthreads();
    if (tid == 0) {
      float t = 0.0f;
      for (int q = 0; q < GT / 32; q++) t += S.wred[q];
      a.nkept[unit] = nkept;
      if (a.diag_lg_obscount) a.diag_lg_obscount[(size_t)g * a.ncol + col] = (float)nkept;
      if (a.diag_lg_obsloc) a.diag_lg_obsloc[(size_t)g * a.ncol + col] = t;
      if (g == 0 && a.diag_obscount) a.diag_obscount[col] = (float)ncand;
    }
    __syncthreads();
  }
}

// Verification: one column/group list, in arrival order; the host sorts it.
// The slot counter is counts[2] (counts[0] counts every kept entry, also
// those beyond cap).
__global__ void k_obslist(int gid, const ColPar *cpp, DevLoc loc, ObsSorted obs, const IndexGeom *geom, int cap,
                          int *out_idx, float *out_r, int *counts) {
  const ColPar cp = *cpp;
  list_search(gid, cp, loc, obs, geom, counts, [&](int p, float r) {
    const int s = atomicAdd(&counts[2], 1);
    if (s < cap) { out_idx[s] = obs.idx[p]; out_r[s] = r; }
  });
}

__global__ void k_debug_metric(int n, const float *lat1, const float *lon1, const float *lat2, const float *lon2,
                               float *dist) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 a = unitvec_exact(lat1[i], lon1[i]), b = unitvec_exact(lat2[i], lon2[i]);
  dist[i] = dist_from_chord2(chord2_exact(a.x, a.y, a.z, b.x, b.y, b.z));
}

__global__ void k_debug_gc(int n, const float *z, const float *L, float *fast, float *exact) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fast[i] = gc_fast(z[i], inv_c_of(L[i]));
  exact[i] = gc_exact(z[i], L[i]);
}

// exact and fast (batched-path) distance and single-factor weight of point pairs
__global__ void k_debug_weight(int n, const float *lat1, const float *lon1, const float *lat2, const float *lon2,
                               const float *L, float *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 a = unitvec_exact(lat1[i], lon1[i]), b = unitvec_exact(lat2[i], lon2[i]);
  const float de = dist_from_chord2(chord2_exact(a.x, a.y, a.z, b.x, b.y, b.z));
  const float df = dist_fast(chord2_fast(a.x, a.y, a.z, b.x, b.y, b.z));
  out[i] = de;
  out[n + i] = df;
  out[2 * n + i] = gc_exact(de, L[i]);
  out[3 * n + i] = gc_branchless(df * inv_c_of(L[i]));
  out[4 * n + i] = dist_fast(chord2_fast(a.x, a.y, a.z, b.x, b.y, b.z), true);
}

}  // namespace

size_t gram_smem_bytes(int k) {
  const int kp = (k + 3) & ~3;
  const int ntn = (k + 1 + 3) / 4;
  const int kb = 4 * ntn > kp ? 4 * ntn : kp;
  const size_t stage = (size_t)BUF * (kp + kb);        // A and B staging rows
  const size_t red = (size_t)(kp / 4) * ntn * 16;      // the tile reduction reuses the area
  return sizeof(float) * (stage > red ? stage : red);
}

static int gram_sets(int k) {
  const int kp = (k + 3) & ~3;
  const int ntiles = (kp / 4) * ((k + 1 + 3) / 4);
  return ntiles <= GT ? 1 : (ntiles + GT - 1) / GT;
}

template <int NSET>
static cudaError_t launch_gram_t(cudaStream_t st, const GramArgs &a, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(k_gram<NSET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_gram<NSET><<<a.nunits, GT, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_gram(cudaStream_t st, const GramArgs &a, int *launches) {
  if (a.nunits <= 0) return cudaSuccess;
  const size_t smem = gram_smem_bytes(a.k);
  (*launches)++;
  switch (gram_sets(a.k)) {
  case 1: return launch_gram_t<1>(st, a, smem);
  case 2: return launch_gram_t<2>(st, a, smem);
  case 3: return launch_gram_t<3>(st, a, smem);
  case 4: return launch_gram_t<4>(st, a, smem);
  case 5: return launch_gram_t<5>(st, a, smem);
  default: return cudaErrorInvalidValue;   // k > 128 is rejected at set-up
  }
}

// loads the plain Gram kernels (CUDA loads a kernel at its first use, which
// must not fall inside a timed trial)
cudaError_t preload_gram(void) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k_gram<1>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_gram<2>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_gram<3>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_gram<4>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_gram<5>);
  return e;
}

cudaError_t launch_obslist(cudaStream_t st, int col, int gid, int group_slot, const ColPar *cp_col, const DevLoc &loc,
                           ObsSorted obs, const IndexGeom *geom, int cap, int *d_idx, float *d_r, int *d_counts) {
  (void)col; (void)group_slot;
  cudaError_t e = cudaMemsetAsync(d_counts, 0, 3 * sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_obslist<<<1, 256, 0, st>>>(gid, cp_col, loc, obs, geom, cap, d_idx, d_r, d_counts);
  return cudaGetLastError();
}

cudaError_t launch_debug_metric(cudaStream_t st, int n, const float *lat1, const float *lon1, const float *lat2,
                                const float *lon2, float *dist) {
  if (n <= 0) return cudaSuccess;
  k_debug_metric<<<(n + 255) / 256, 256, 0, st>>>(n, lat1, lon1, lat2, lon2, dist);
  return cudaGetLastError();
}

cudaError_t launch_debug_gc(cudaStream_t st, int n, const float *z, const float *L, float *fast, float *exact) {
  if (n <= 0) return cudaSuccess;
  k_debug_gc<<<(n + 255) / 256, 256, 0, st>>>(n, z, L, fast, exact);
  return cudaGetLastError();
}

cudaError_t launch_debug_weight(cudaStream_t st, int n, const float *lat1, const float *lon1, const float *lat2,
                                const float *lon2, const float *L, float *out) {
  if (n <= 0) return cudaSuccess;
  k_debug_weight<<<(n + 255) / 256, 256, 0, st>>>(n, lat1, lon1, lat2, lon2, L, out);
  return cudaGetLastError();
}

}  // namespace lgpu
