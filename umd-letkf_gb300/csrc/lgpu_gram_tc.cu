// lgpu_gram_tc.cu -- batched Gram on the tensor cores: one CTA per
// (tile of 128 neighbouring columns, localisation group, feature pass).
//
// Same result as k_gram (src/letkf_solver.F90:210-268 and the Gram / RHS half
// of src/letkf_core.F90:92-125), reorganised so that neighbouring columns
// share their observations.  For a tile the Gram entries of every column form
// one GEMM over the tile's candidate observations o:
//
//   G[c, f] = sum_o W[c, o] * P[o, f],   W[c, o] = rloc_c(o) / err_o
//                                        P[o, f] = y_i(o) * y_j(o)   f = (i <= j)
//                                                = y_i(o) * dep(o)   f = (i, rhs)
//
// M = 128 columns, N = the k(k+3)/2 packed features (split into passes of at
// most 432 so the accumulator fits TMEM), K = candidate observations in
// chunks of 16.
//
// Candidate streams.  Before the GEMM, three small kernels turn each tile's
// search window (latitude bands x longitude range of its cap) into a record
// stream: every observation inside the tile's cap, in window order, packed
// per chunk of 16 as [16 x (ux,uy,uz,1/err)] [16 x (dep,time,zdim,surf)]
// [member-major y: (k+1 rounded to 4) rows x 16] -- one contiguous block per
// chunk, read once per (group, pass) CTA with one bulk async copy.
//
// GEMM CTA roles (17 warps):
//   warps 0-15  producers; thread t owns column t % 128 for observations
//               [4 (t / 128), +4) of each chunk and feature t:
//               weights: the distance (fast float path without branches;
//               the exact metric and the per-column localizer where the
//               fast value lies near the search radius or the keep
//               threshold: bit-identical keep decisions to the per-column
//               path), W = rloc / err;
//               features: y_i * y_j, y_i * dep over the chunk;
//               both operands are split into tf32 hi + lo parts and stored
//               in the no-swizzle K-major core-matrix layout of an operand
//               stage;
//   warp 16     one thread keeps the record ring filled (cp.async.bulk, one
//               per chunk, mbarrier transaction counts; a slot is refilled
//               once every producer has finished the chunk in it), issues
//               tcgen05.mma kind::tf32 for hi*hi + hi*lo + lo*hi (FP32
//               accumulation in TMEM, relative error ~2^-21 per product) and
//               frees the stage with tcgen05.commit; chunks in which no
//               column keeps an observation issue no MMA.
// The epilogue reads TMEM lane c = column c and writes the packed Gram block
// of each unit.  Every wait is bounded; a wait that runs out sets status bit
// 16, the MMA thread waits (bounded) for its copies in flight and TMEM is
// freed.
//
// Long tile streams are split into up to 4 accumulation segments, each its
// own CTA, summed in order by k_gram_segsum.  The producers come in two forms
// with bit-identical output (with and without a warp-level cull of records
// out of every column's reach); the first analysis of a configuration times
// both and keeps the faster.
#include "lgpu_internal.cuh"
#include "lgpu_tc.cuh"

namespace lgpu {

namespace {

constexpr int TM = 128;        // columns per tile = MMA M = TMEM lanes
constexpr int KC = 16;         // observations per chunk (two K=8 MMA steps)
constexpr int NPW = 16;        // producer warps: 0-7 weights, 8-15 features
constexpr int MMA_WARP = NPW;
constexpr int NT = 32 * (NPW + 1);
constexpr int NPMAX = 432;     // features per pass
constexpr int NSMAX = 2, NRMAX = 6;
constexpr uint32_t CMB = 128;                 // bytes per core matrix (8 rows x 16 B)
constexpr uint32_t SBO = (KC / 4) * CMB;      // bytes per 8-row group (all K of the chunk)
constexpr uint32_t WB = (TM / 8) * SBO;       // bytes per W operand copy
constexpr size_t kSmemBudget = 227 * 1024 - 4096;   // dynamic shared memory (static part below 4 KB)
constexpr int WT = 256;        // threads of the stream kernels
constexpr int WCB = 2 * WB;   // bytes of one chunk's cached weight operand block (hi | lo)
constexpr int YS = 20;         // floats per member row of a chunk record (16 observations + 4: conflict-free rows)
__device__ __forceinline__ uint32_t kmaj(int row, int kk) {
  return (uint32_t)(row >> 3) * SBO + (uint32_t)(kk >> 2) * CMB + (uint32_t)(row & 7) * 16u + (uint32_t)(kk & 3) * 4u;
}

__device__ __forceinline__ bool in_cap(const TilePar &t, float4 A) {
  const float dx = __fsub_rn(t.cx, A.x), dy = __fsub_rn(t.cy, A.y), dz = __fsub_rn(t.cz, A.z);
  return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz)) <= t.c2cap;
}

// ---------------------------------------------------------------------------
// Search window of a tile as runs of the cell-sorted observation table
// (per latitude band at most two runs, the second for a window across 0/360),
// concatenated: candidate j of the window lives at seg_start[s] + j -
// seg_pref[s] for the last s with seg_pref[s] <= j.  Block of WT threads.
struct Window {
  int seg_start[2 * kNB];
  int seg_pref[2 * kNB + 1];
  int wsc[WT / 32];
  int nseg, total;
};

__device__ void build_window(Window &W, const TilePar &tp, const IndexGeom *geom, const int *cell_start) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nb = tp.b1 - tp.b0 + 1;
  int l0 = 0, l1 = 0;
  if (tid < nb) {
    const int b = tp.b0 + tid;
    const int nl = geom->nlon[b], off = geom->off[b];
    int s0 = 0, s1 = 0;
    bool whole = tp.dlon >= 180.0f;
    int clo = 0, chi = nl - 1;
    if (!whole) {
      clo = (int)floorf((tp.lonn - tp.dlon) * (float)nl / 360.0f);
      chi = (int)floorf((tp.lonn + tp.dlon) * (float)nl / 360.0f);
      if (chi - clo + 1 >= nl) whole = true;
    }
    if (whole) {
      s0 = cell_start[off];
      l0 = cell_start[off + nl] - s0;
    } else if (clo < 0) {
      s0 = cell_start[off + clo + nl];
      l0 = cell_start[off + nl] - s0;
      s1 = cell_start[off];
      l1 = cell_start[off + chi + 1] - s1;
    } else if (chi >= nl) {
      s0 = cell_start[off + clo];
      l0 = cell_start[off + nl] - s0;
      s1 = cell_start[off];
      l1 = cell_start[off + (chi - nl) + 1] - s1;
    } else {
      s0 = cell_start[off + clo];
      l0 = cell_start[off + chi + 1] - s0;
    }
    W.seg_start[2 * tid] = s0;
    W.seg_start[2 * tid + 1] = s1;
  }
  const int x = l0 + l1;
  int incl = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) W.wsc[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int sv = lane < WT / 32 ? W.wsc[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, sv, o);
      if (lane >= o) sv += y;
    }
    if (lane < WT / 32) W.wsc[lane] = sv;
  }
  __syncthreads();
  const int base = (wid > 0 ? W.wsc[wid - 1] : 0) + incl - x;
  if (tid < nb) {
    W.seg_pref[2 * tid] = base;
    W.seg_pref[2 * tid + 1] = base + l0;
  }
  if (tid == 0) {
    W.nseg = 2 * nb;
    W.total = W.wsc[WT / 32 - 1];
    W.seg_pref[2 * nb] = W.total;
  }
  __syncthreads();
}

__device__ __forceinline__ int window_pos(const Window &W, int j) {
  int lo = 0, hi = W.nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (W.seg_pref[mid] <= j) lo = mid; else hi = mid - 1;
  }
  return W.seg_start[lo] + (j - W.seg_pref[lo]);
}

// candidates per tile: observations of the window inside the tile's cap
__global__ void __launch_bounds__(WT) k_tile_count(int ntiles, const TilePar *tps, const IndexGeom *geom,
                                                   const float4 *obsA, const int *cell_start, int *tile_n) {
  __shared__ Window W;
  __shared__ int red[WT / 32];
  const int tile = blockIdx.x;
  const TilePar tp = tps[tile];
  build_window(W, tp, geom, cell_start);
  int cnt = 0;
#pragma unroll 4
  for (int j = threadIdx.x; j < W.total; j += WT) cnt += in_cap(tp, __ldg(obsA + window_pos(W, j)));
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < WT / 32; w++) t += red[w];
    tile_n[tile] = t;
  }
}

// chunk offsets of the tile streams: tile_off[t] = sum over earlier tiles of
// ceil(n / 16); tile_off[ntiles] = total chunks.  One block.
__global__ void k_tile_scan(int ntiles, const int *tile_n, int *tile_off) {
  __shared__ int wsum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < ntiles; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < ntiles ? (tile_n[i] + KC - 1) / KC : 0;
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
    if (i < ntiles) tile_off[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_off[ntiles] = carry;
}

// one record entry: slot e of chunk c of the tile stream
__device__ __forceinline__ void put_record(unsigned char *rec0, int cb, int k, int kp, int kr, int q, const float4 &A,
                                           const float4 &B, const float *hx) {
  unsigned char *r = rec0 + (size_t)(q >> 4) * cb;
  const int e = q & 15;
  reinterpret_cast<float4 *>(r)[e] = A;
  reinterpret_cast<float4 *>(r + 256)[e] = B;
  float *yT = reinterpret_cast<float *>(r + 512);
  if (hx) {
    // the member row through the read-only path, four 16-byte loads in
    // flight before their stores
    const float4 *h4 = reinterpret_cast<const float4 *>(hx);
    const int n4 = kp >> 2;
    for (int q0 = 0; q0 < n4; q0 += 4) {
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; u++) v[u] = q0 + u < n4 ? __ldg(h4 + q0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int i = 4 * (q0 + u);
        if (i + 0 < k) yT[(i + 0) * YS + e] = v[u].x;
        if (i + 1 < k) yT[(i + 1) * YS + e] = v[u].y;
        if (i + 2 < k) yT[(i + 2) * YS + e] = v[u].z;
        if (i + 3 < k) yT[(i + 3) * YS + e] = v[u].w;
      }
    }
    yT[k * YS + e] = B.x;
  } else {
    for (int i = 0; i <= k; i++) yT[i * YS + e] = 0.0f;
  }
  for (int i = k + 1; i < kr; i++) yT[i * YS + e] = 0.0f;
  if (e < YS - 16)
    for (int i = 0; i < kr; i++) yT[i * YS + 16 + e] = 0.0f;
}

// tile streams: the window scanned again in order, cap members compacted
// (order preserving) into the tile's chunk records; the last chunk padded
// with zero entries
__global__ void __launch_bounds__(WT) k_tile_fill(int ntiles, const TilePar *tps, const IndexGeom *geom, ObsSorted obs,
                                                  int k, int kp, int kr, int cb, const int *tile_off,
                                                  unsigned char *rec, int *status) {
  __shared__ Window W;
  __shared__ int wsc[WT / 32];
  __shared__ int qpos[2 * WT];   // in-cap window positions not yet written, in window order
  const int tile = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const TilePar tp = tps[tile];
  build_window(W, tp, geom, obs.cell_start);
  const int c0 = tile_off[tile];
  const int cap = (tile_off[tile + 1] - c0) * KC;
  unsigned char *rec0 = rec + (size_t)c0 * cb;
  // the in-cap observations are queued in window order and written WT at a
  // time by the whole block (about a third of a window is in the cap)
  auto write = [&](int q, int p) {
    if (q < cap) {
      const float4 A = obs.A[p];
      put_record(rec0, cb, k, kp, kr, q, make_float4(A.x, A.y, A.z, __frcp_rn(A.w)), obs.B[p],
                 obs.hx + (size_t)p * kp);
    } else {
      atomicOr(status, 16);
    }
  };
  int base = 0, pend = 0;
  // the thread's next window candidate (position and record) is loaded one
  // iteration ahead, so that its latency overlaps the current compaction
  int p_nx = 0;
  float4 a_nx = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid < W.total) {
    p_nx = window_pos(W, tid);
    a_nx = __ldg(obs.A + p_nx);
  }
  for (int jb = 0; jb < W.total; jb += WT) {
    const int j = jb + tid;
    const int p = p_nx;
    const bool ok = j < W.total && in_cap(tp, a_nx);
    if (j + WT < W.total) {
      p_nx = window_pos(W, j + WT);
      a_nx = __ldg(obs.A + p_nx);
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) wsc[wid] = __popc(m);
    __syncthreads();
    int before = 0, cnt = 0;
    for (int w = 0; w < WT / 32; w++) {
      before += w < wid ? wsc[w] : 0;
      cnt += wsc[w];
    }
    if (ok) qpos[pend + before + __popc(m & ((1u << lane) - 1u))] = p;
    pend += cnt;
    __syncthreads();
    if (pend >= WT) {
      write(base + tid, qpos[tid]);
      base += WT;
      pend -= WT;
      __syncthreads();
      if (tid < pend) qpos[tid] = qpos[WT + tid];
      __syncthreads();
    }
  }
  if (tid < pend) write(base + tid, qpos[tid]);
  base += pend;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int q = base + tid; q < cap; q += WT) put_record(rec0, cb, k, kp, kr, q, z, z, nullptr);
  if (tid == 0 && (base > cap || cap - base >= KC)) atomicOr(status, 16);   // count and fill disagree
}

struct TcSmem {
  unsigned long long full[NSMAX], empty[NSMAX], rfull[NRMAX], done;
  unsigned long long accf;   // drain: the accumulation so far is complete in TMEM (commit + MMA thread)
  unsigned long long acce;   // drain: the producer warps have read TMEM (one arrival per warp)
  int anyk[NSMAX];           // chunk index + 1 of the last chunk of the stage with a kept pair
  uint32_t tmem;
  int issued;                // MMAs were issued since the last drain
  int sub_issued;            // the same, for the accumulation a drain hands over
  int fault;
  unsigned char fi[NPMAX];
  unsigned char fj[NPMAX];
};

// per-CTA constants of the localizer's fast path
struct LocK {
  float icv, levg;            // vtgc: vertical 1/c, depth of the group's level
  float tprof, tsat;          // ocean: time scales (0 = off)
  float ictp, icts;           // ocean: their 1/c
};

// fast localisation weight (no branches); LOC selects the localizer class
template <int LOC>
__device__ __forceinline__ float loc_fast(const LocK &lk, const ColPar &cp, int g, float d, const float4 &B) {
  if (LOC == LOC_VTGC) {
    return gc_branchless(d * cp.ic1) * gc_branchless(fabsf(B.z - lk.levg) * lk.icv);
  } else if (LOC == LOC_OCEAN) {
    const bool sat = B.w != 0.0f;
    const float rh = gc_branchless(d * (sat ? cp.ic2 : cp.ic1));
    const float tl = sat ? lk.tsat : lk.tprof;
    const float rt = tl > 0.0f ? gc_branchless(fabsf(B.y) * (sat ? lk.icts : lk.ictp)) : 1.0f;
    return (sat && g == 1) ? 0.0f : rh * rt;
  } else {
    return gc_branchless(d * cp.ic1);
  }
}

__device__ __forceinline__ void bar_arrive(unsigned long long *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(b)) : "memory");
}

// WMODE: 0 = weights computed; 1 = weights computed and written to the
// weight cache as the stage's TF32 hi/lo operand block, with the chunk's
// MMA flag (first feature pass of a tile); 2 = the operand block is
// bulk-copied from the cache into the stage (later passes: the producers
// form only the feature products).  CULL (WMODE 0, 1): a warp whose 32
// columns have none of its four records within their search chords skips
// the distance and localizer evaluation (their weights are zero either way;
// results are bit-identical); pays where search radii are small next to the
// tile caps, costs registers where they are not
template <int LOC, int NS, int NR, int WMODE, bool CULL>
__global__ void __launch_bounds__(NT, 1) k_gram_tc(TcArgs a) {
  static_assert(NS <= NSMAX && NR <= NRMAX, "operand stages / record slots beyond the barrier arrays");
  extern __shared__ __align__(1024) unsigned char dsm[];
  __shared__ __align__(16) TcSmem S;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  // block = (work item, group, pass of this launch), pass fastest
  const int pass = a.pass0 + blockIdx.x % a.npl;
  const int g = (blockIdx.x / a.npl) % a.groups;
  const TcWork wk = a.work[blockIdx.x / (a.npl * a.groups)];
  const int tile = wk.tile;
  const int k = a.k, NP = a.np, nf = a.nf, cb = a.cb;
  const int slotb = cb;   // ring slot: one chunk record
  const uint32_t PB = (uint32_t)(NP / 8) * SBO;
  const uint32_t stage_bytes = 2 * WB + 2 * PB;
  auto stage_ptr = [&](int s) { return dsm + (size_t)s * stage_bytes; };
  unsigned char *ring = dsm + (size_t)NS * stage_bytes;
  // this CTA's segment of the tile's chunk stream
  const int t0 = a.tile_off[tile], tn = a.tile_off[tile + 1] - t0;
  const int cs = min(tn, wk.cs), ce = min(tn, wk.ce);
  const int c0 = t0 + cs;
  float *wcache = WMODE != 0 ? a.wcache + (size_t)g * a.nchunk_total * (WCB / 4) : nullptr;
  int *wflag = WMODE != 0 ? a.wflag + (size_t)g * a.nchunk_total : nullptr;
  const int nchunks = ce - cs;
  const int ntile = a.tile_n[tile] - cs * KC;   // candidates from the segment's first chunk on
  const uint32_t tmem_cols = a.tmem_cols;

  // ---- setup: TMEM, barriers, feature table
  if (wid == 0) tc::tmem_alloc(&S.tmem, tmem_cols);
  if (tid == 0) {
    for (int s = 0; s < NS; s++) {
      tc::mbar_init(reinterpret_cast<uint64_t *>(&S.full[s]), WMODE == 2 ? NPW + 1 : NPW);
      tc::mbar_init(reinterpret_cast<uint64_t *>(&S.empty[s]), 1);
      S.anyk[s] = 0;
    }
    for (int r = 0; r < NR; r++) tc::mbar_init(reinterpret_cast<uint64_t *>(&S.rfull[r]), 1);
    tc::mbar_init(reinterpret_cast<uint64_t *>(&S.done), 1);
    tc::mbar_init(reinterpret_cast<uint64_t *>(&S.accf), 2);
    tc::mbar_init(reinterpret_cast<uint64_t *>(&S.acce), NPW);
    S.issued = 0;
    S.sub_issued = 0;
    S.fault = 0;
    tc::mbar_fence_init();
  }
  for (int f = tid; f < NP; f += NT) {
    const int fg = pass * NP + f;
    int i = 255, j = 255;
    if (fg < nf) packed_ij(fg, k, i, j);
    S.fi[f] = (unsigned char)i;
    S.fj[f] = (unsigned char)j;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = S.tmem;

  // producer thread: column wc, observations [4 wq, 4 wq + 4) of each chunk,
  // and feature f = tid
  const int wc = tid & (TM - 1), wq = (tid >> 7) & 3;
  int ncand = 0, nkeep = 0;
  float rsum = 0.0f;

  // The CTA's results: TMEM lane = column wc.  A tile whose stream is one
  // drain interval writes the column's G row (thread tid < TM, warps 0-3);
  // otherwise every drain interval goes to its own partial block,
  // feature-major, so that a warp's stores of one feature are 32 consecutive
  // floats (the 16 producer warps drain, each warp a quarter of the features
  // of its lane quarter).
  const int G = a.groups;
  const int D = a.drain;
  const int nvalid = nf - pass * NP < NP ? nf - pass * NP : NP;
  // the accumulator's lane of this thread (TMEM lane quarter wid % 4; zeros
  // unless from_tmem, which is CTA-uniform), features [16 q, 16 q + 16) for
  // q = q0, q0 + qs, ..., into partial block blk
  auto store_block = [&](int blk, bool from_tmem, int q0, int qs) {
    float *base = a.Gpart + (((size_t)blk * G + g) * nf + (size_t)pass * NP) * TM + wc;
    for (int f0 = 16 * q0; f0 < NP; f0 += 16 * qs) {
      float v[16];
      if (from_tmem) {
        tc::tmem_ld16(tmem + ((uint32_t)((wid & 3) * 32) << 16) + (uint32_t)f0, v);
      } else {
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = 0.0f;
      }
#pragma unroll
      for (int q = 0; q < 16; q++)
        if (f0 + q < nvalid) base[(size_t)(f0 + q) * TM] = v[q];
    }
  };
  // drain j (all 16 producer warps, warp w the features of quarter w / 4):
  // wait until the MMAs before boundary (j + 1) D have completed, move the
  // accumulator to its block, hand TMEM back to the MMA thread
  const int nflush = nchunks > 0 ? (nchunks - 1) / D : 0;
  int nflushed = 0;
  auto flush = [&](int j) {
    if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.accf), j & 1)) S.fault = 1;
    tc::fence_after();
    store_block(wk.blk0 + j, S.sub_issued != 0 && S.fault == 0, wid >> 2, 4);
    tc::fence_before();
    __syncwarp();
    if (lane == 0) bar_arrive(&S.acce);
  };

  if (wid < NPW) {
    const int col = a.tile_cols[(size_t)tile * TM + wc];
    const bool colv = col >= 0;
    ColPar cp;
    if (colv) cp = a.cp[col];
    else { cp.ux = cp.uy = cp.uz = 0.0f; cp.rmax = -1.0f; cp.L1 = cp.L2 = 1.0f; cp.ic1 = cp.ic2 = 1.0f; }
    float c2max = -1.0f;
    if (colv) {
      const float hq = fminf(cp.rmax / 12742000.0f, 1.5707963f);
      const float sh = sinf(hq);
      c2max = 4.0f * sh * sh * 1.0001f + 1e-12f;
    }
    const float rlo = cp.rmax * (1.0f - kFastDistBand), rhi = cp.rmax * (1.0f + kFastDistBand);
    const bool short_asin = a.tp[tile].hmax <= 0.25f;   // CTA-uniform
    LocK lk;
    lk.icv = LOC == LOC_VTGC ? inv_c_of(a.loc.vloc) : 1.0f;
    lk.levg = LOC == LOC_VTGC ? a.loc.lev_depth[g] : 0.0f;
    lk.tprof = a.loc.tloc_prof;
    lk.tsat = a.loc.tloc_sat;
    lk.ictp = (LOC == LOC_OCEAN && lk.tprof > 0.0f) ? inv_c_of(lk.tprof) : 1.0f;
    lk.icts = (LOC == LOC_OCEAN && lk.tsat > 0.0f) ? inv_c_of(lk.tsat) : 1.0f;
    const int f = tid;
    const bool fin = f < NP;
    const int fi = fin ? S.fi[f] : 255, fj = fin ? S.fj[f] : 255;
    const bool fv = fi != 255;
    const int rowi = (fv ? fi : 0) * YS, rowj = (fv ? fj : 0) * YS;

    for (int ch = 0; ch < nchunks; ch++) {
      const int s = ch % NS, r = ch % NR;
      // the producers drain TMEM at boundary b = (j + 1) D once the stages
      // of chunks b .. b + NS - 1 are produced: the MMA of chunk b + NS needs
      // the stage chunk b frees, which waits for the drain
      if (nflushed < nflush && ch == (nflushed + 1) * D + NS) flush(nflushed++);
      if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.rfull[r]), (ch / NR) & 1)) { S.fault = 1; break; }
      if (ch >= NS && !tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.empty[s]), ((ch / NS) - 1) & 1)) {
        S.fault = 1;
        break;
      }
      const unsigned char *rec = ring + (size_t)r * slotb;
      const float4 *RA = reinterpret_cast<const float4 *>(rec);
      unsigned char *Whi = stage_ptr(s), *Wlo = Whi + WB, *Phi = Whi + 2 * WB, *Plo = Phi + PB;
      bool anyk = false;
      if (WMODE == 2) {
        // ---- the chunk's weight operand block (hi | lo) from the cache into
        // the stage, counted on the stage's full barrier (the stage is free:
        // its empty barrier was waited on above)
        if (tid == 0) {
          uint64_t *fb = reinterpret_cast<uint64_t *>(&S.full[s]);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(fb)),
                       "r"((uint32_t)WCB) : "memory");
          tc::bulk_copy_g2s(Whi, wcache + (size_t)(c0 + ch) * (WCB / 4), (uint32_t)WCB, fb);
        }
      } else {
      // ---- weights: four observations, fast path without branches
      float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      unsigned unsure = 0, inr = 0;
      unsigned candm = 0xfu;
      if constexpr (CULL) {
        candm = 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = wq * 4 + u;
          const float4 A = RA[e];
          const float c2f = chord2_fast(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z);
          candm |= ((ch * KC + e < ntile) && (c2f <= c2max) ? 1u : 0u) << u;
        }
      }
      if (!CULL || __any_sync(0xffffffffu, candm != 0)) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = wq * 4 + u;
          const float4 A = RA[e];
          const float4 B = RA[16 + e];
          const float c2f = chord2_fast(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z);
          const bool cand = (ch * KC + e < ntile) && (c2f <= c2max);
          const float hf = 0.5f * c2f * rsqrtf(fmaxf(c2f, 1e-30f));
          const float d = 12742000.0f * asin_fast(fminf(hf, 0.5f), short_asin);
          const float rl = loc_fast<LOC>(lk, cp, g, d, B);
          const bool in = cand && d <= cp.rmax;
          const bool uns = cand && (hf > 0.5f || (d >= rlo && d <= rhi) || (in && fabsf(rl - kKeep) <= kGuardFast));
          const bool kept = in && rl > kKeep;
          w[u] = kept ? rl : 0.0f;
          unsure |= (uns ? 1u : 0u) << u;
          inr |= (in ? 1u : 0u) << u;
        }
      }
      // ---- rare: exact metric and the per-column localizer
      if (__any_sync(0xffffffffu, unsure != 0)) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          if (!((unsure >> u) & 1u)) continue;
          const int e = wq * 4 + u;
          const float4 A = RA[e];
          const float4 B = RA[16 + e];
          const float de = dist_from_chord2(chord2_exact(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z));
          const bool in = de <= cp.rmax;
          // the class's exact localizer with the column's parameters from
          // global memory (keeps them out of the producers' registers)
          float rl = in ? localize_cls<LOC>(a.loc, a.cp[col], g, de, B.y, B.z, B.w) : 0.0f;
          w[u] = (in && rl > kKeep) ? rl : 0.0f;
          inr = (inr & ~(1u << u)) | ((in ? 1u : 0u) << u);
        }
      }
      {
        float h4[4], l4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const float rl = w[u];
          ncand += (inr >> u) & 1u;
          float wv = 0.0f;
          if (rl > 0.0f) {
            nkeep++;
            rsum += rl;
            anyk = true;
            wv = rl * RA[wq * 4 + u].w;   // the record holds 1/err
          }
          tc::split_tf32(wv, h4[u], l4[u]);
        }
        const uint32_t off = kmaj(wc, wq * 4);
        *reinterpret_cast<float4 *>(Whi + off) = make_float4(h4[0], h4[1], h4[2], h4[3]);
        *reinterpret_cast<float4 *>(Wlo + off) = make_float4(l4[0], l4[1], l4[2], l4[3]);
        if (WMODE == 1) {
          float *blk = wcache + (size_t)(c0 + ch) * (WCB / 4);
          *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(blk) + off) =
              make_float4(h4[0], h4[1], h4[2], h4[3]);
          *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(blk) + WB + off) =
              make_float4(l4[0], l4[1], l4[2], l4[3]);
        }
      }
      }
      // ---- feature products: feature f over the 16 observations
      if (fin) {
        const float *yT = reinterpret_cast<const float *>(rec + 512);
        const float4 *yi = reinterpret_cast<const float4 *>(yT + rowi);
        const float4 *yj = reinterpret_cast<const float4 *>(yT + rowj);
#pragma unroll
        for (int grp = 0; grp < 4; grp++) {
          const float4 a4 = yi[grp], b4 = yj[grp];
          const float v[4] = {a4.x * b4.x, a4.y * b4.y, a4.z * b4.z, a4.w * b4.w};
          float h4[4], l4[4];
#pragma unroll
          for (int u = 0; u < 4; u++) tc::split_tf32(fv ? v[u] : 0.0f, h4[u], l4[u]);
          const uint32_t off = kmaj(f, grp * 4);
          *reinterpret_cast<float4 *>(Phi + off) = make_float4(h4[0], h4[1], h4[2], h4[3]);
          *reinterpret_cast<float4 *>(Plo + off) = make_float4(l4[0], l4[1], l4[2], l4[3]);
        }
      }
      if (__any_sync(0xffffffffu, anyk) && lane == 0) S.anyk[s] = ch + 1;
      tc::fence_proxy_async();
      __syncwarp();
      if (lane == 0) bar_arrive(&S.full[s]);
    }
    while (nflushed < nflush) flush(nflushed++);
  } else if (wid == MMA_WARP) {
    // ================================================= MMA issue + record loads (one thread)
    if (lane == 0) {
      const unsigned char *src = a.rec + (size_t)c0 * cb;
      auto load = [&](int ch) {
        unsigned char *dst = ring + (size_t)(ch % NR) * slotb;
        uint64_t *bar = reinterpret_cast<uint64_t *>(&S.rfull[ch % NR]);
        tc::bulk_load(dst, src + (size_t)ch * cb, (uint32_t)cb, bar);
      };
      int n_loaded = nchunks < NR ? nchunks : NR;
      for (int ch = 0; ch < n_loaded; ch++) load(ch);
      const int nb0 = NP < 256 ? NP : 256, nb1 = NP - nb0;
      const uint32_t id0 = tc::idesc_tf32(TM, nb0), id1 = nb1 > 0 ? tc::idesc_tf32(TM, nb1) : 0u;
      bool issued = false;   // since the last drain
      int nmma = 0, fj = 0;
      // later passes: the chunks' MMA flags from pass 0, loaded two chunks
      // ahead into alternating registers (each is read two iterations after
      // its load is issued)
      auto flag_at = [&](int c) { return (WMODE == 2 && c < nchunks) ? wflag[c0 + c] : 0; };
      int flag_even = flag_at(0), flag_odd = flag_at(1);
      for (int ch = 0; ch < nchunks; ch++) {
        const int s = ch % NS;
        if (ch > 0 && ch % a.drain == 0) {
          // boundary: hand the accumulation to the producer warps and wait
          // until they have read TMEM; the next MMA starts a fresh accumulation
          S.sub_issued = issued ? 1 : 0;
          tc::commit(reinterpret_cast<uint64_t *>(&S.accf));
          bar_arrive(&S.accf);
          if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.acce), fj & 1)) { S.fault = 1; break; }
          tc::fence_after();
          fj++;
          issued = false;
        }
        int cached_flag = 0;
        if (WMODE == 2) {
          if (ch & 1) { cached_flag = flag_odd; flag_odd = flag_at(ch + 2); }
          else { cached_flag = flag_even; flag_even = flag_at(ch + 2); }
        }
        if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.full[s]), (ch / NS) & 1)) { S.fault = 1; break; }
        // every producer is done with the records of chunk ch: refill the slot
        if (n_loaded < nchunks) load(n_loaded++);
        const bool mma = WMODE == 2 ? cached_flag != 0 : S.anyk[s] == ch + 1;
        if (WMODE == 1) wflag[c0 + ch] = mma ? 1 : 0;
        if (mma) {
          tc::fence_after();
          const uint32_t whi = tc::smem_u32(stage_ptr(s)), wlo = whi + WB, phi = whi + 2 * WB, plo = phi + PB;
#pragma unroll
          for (int t = 0; t < 3; t++)
#pragma unroll
            for (int ks = 0; ks < KC / 8; ks++) {
              const uint32_t acc = (issued || t > 0 || ks > 0) ? 1u : 0u;
              const uint32_t aw = t == 2 ? wlo : whi, bp = t == 1 ? plo : phi;
              const uint64_t ad = tc::smem_desc(aw + ks * 2 * CMB, CMB, SBO);
              const uint64_t bd0 = tc::smem_desc(bp + ks * 2 * CMB, CMB, SBO);
              tc::mma_tf32(tmem, ad, bd0, id0, acc);
              if (nb1 > 0) {
                const uint64_t bd1 = tc::smem_desc(bp + (uint32_t)(nb0 / 8) * SBO + ks * 2 * CMB, CMB, SBO);
                tc::mma_tf32(tmem + (uint32_t)nb0, ad, bd1, id1, acc);
              }
            }
          tc::commit(reinterpret_cast<uint64_t *>(&S.empty[s]));
          issued = true;
          nmma++;
        } else {
          bar_arrive(&S.empty[s]);
        }
      }
      // every MMA issued by this thread has completed once `done` flips
      tc::commit(reinterpret_cast<uint64_t *>(&S.done));
      if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.done), 0)) S.fault = 1;
      S.issued = issued ? 1 : 0;
      if (nmma) atomicAdd(a.status + 2, nmma);   // chunks whose MMAs ran (executed-work counter)
      // no record copy may still be in flight when the CTA exits
      for (int ch = n_loaded > NR ? n_loaded - NR : 0; ch < n_loaded; ch++)
        if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.rfull[ch % NR]), (ch / NR) & 1)) S.fault = 1;
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const bool fault = S.fault != 0;
  const bool issued = S.issued != 0;
  // per-column partial counts of observation quarters 1-3, in the (now idle)
  // operand stage memory
  int *dcand = reinterpret_cast<int *>(dsm), *dkept = dcand + 3 * TM;
  float *drsum = reinterpret_cast<float *>(dkept + 3 * TM);
  if (wid < NPW && wq > 0) {
    dcand[(wq - 1) * TM + wc] = ncand;
    dkept[(wq - 1) * TM + wc] = nkeep;
    drsum[(wq - 1) * TM + wc] = rsum;
  }
  __syncthreads();

  // ---- per-column diagnostics, kept counts, epilogue (warps 0-3 = TMEM lanes)
  if (tid < TM) {
    for (int q = 0; q < 3; q++) {
      ncand += dcand[q * TM + wc];
      nkeep += dkept[q * TM + wc];
      rsum += drsum[q * TM + wc];
    }
    const int col = a.tile_cols[(size_t)tile * TM + wc];
    const bool colv = col >= 0;
    size_t unit = 0;
    if (colv) unit = (size_t)a.col2act[col] * G + g;
    if (colv && pass == 0) {
      if (wk.cblk < 0) {
        a.nkept[unit] = nkeep;
        if (a.diag_lg_obscount) a.diag_lg_obscount[(size_t)g * a.ncol + col] = (float)nkeep;
        if (a.diag_lg_obsloc) a.diag_lg_obsloc[(size_t)g * a.ncol + col] = rsum;
        if (g == 0 && a.diag_obscount) a.diag_obscount[col] = (float)ncand;
      } else {
        float *cc = a.cnt + (((size_t)wk.cblk * G + g) * TM + wc) * 3;
        cc[0] = (float)nkeep;
        cc[1] = (float)ncand;
        cc[2] = rsum;
      }
    }
    if (wk.blk0 >= 0) {
      // the last drain interval of the segment
      store_block(wk.blk0 + nflush, issued && !fault, 0, 1);
    } else {
      // the whole stream in one accumulator: the column's G row (16-byte
      // aligned: nf and NP are multiples of 4)
      float *Gp = colv ? a.G + unit * (size_t)nf + (size_t)pass * NP : nullptr;
      for (int f0 = 0; f0 < NP; f0 += 16) {
        float v[16];
        if (issued && !fault) {
          tc::tmem_ld16(tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)f0, v);
        } else {
#pragma unroll
          for (int q = 0; q < 16; q++) v[q] = 0.0f;
        }
        if (Gp) {
          if (f0 + 16 <= nvalid && (nf & 3) == 0) {
#pragma unroll
            for (int q = 0; q < 16; q += 4)
              *reinterpret_cast<float4 *>(Gp + f0 + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
          } else {
#pragma unroll
            for (int q = 0; q < 16; q++)
              if (f0 + q < nvalid) Gp[f0 + q] = v[q];
          }
        }
      }
    }
  }
  if (fault && tid == 0) atomicOr(a.status, 16);
  tc::fence_before();
  __syncthreads();
  if (wid == 0) tc::tmem_dealloc(tmem, tmem_cols);
}

// Tile caps: centre = normalised mean of the tile's unit vectors, angular
// radius = max over columns of (angle to centre + search radius / R), then
// the same conservative band / longitude window as a single column.
__global__ void k_tile_prep(int ntiles, const int *tile_cols, const ColPar *cp, TilePar *tp) {
  const int tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (tile >= ntiles) return;
  double sx = 0, sy = 0, sz = 0;
  for (int c = lane; c < TM; c += 32) {
    const int col = tile_cols[(size_t)tile * TM + c];
    if (col < 0) continue;
    sx += cp[col].ux; sy += cp[col].uy; sz += cp[col].uz;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
    sz += __shfl_xor_sync(0xffffffffu, sz, o);
  }
  const double nrm = sqrt(sx * sx + sy * sy + sz * sz);
  const double cx = nrm > 0 ? sx / nrm : 1.0, cy = nrm > 0 ? sy / nrm : 0.0, cz = nrm > 0 ? sz / nrm : 0.0;
  double amax = 0.0;
  for (int c = lane; c < TM; c += 32) {
    const int col = tile_cols[(size_t)tile * TM + c];
    if (col < 0) continue;
    const double dot = fmin(1.0, fmax(-1.0, cx * cp[col].ux + cy * cp[col].uy + cz * cp[col].uz));
    const double ang = acos(dot) + (double)cp[col].rmax / 6371000.0;
    amax = fmax(amax, ang);
  }
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  // largest half-chord sqrt(c2max)/2 of a candidate pair (the weight producers' c2max)
  float hm = 0.0f;
  for (int c = lane; c < TM; c += 32) {
    const int col = tile_cols[(size_t)tile * TM + c];
    if (col < 0) continue;
    const float hq = fminf(cp[col].rmax / 12742000.0f, 1.5707963f);
    const float sh = sinf(hq);
    hm = fmaxf(hm, sqrtf(4.0f * sh * sh * 1.0001f + 1e-12f) * 0.5f);
  }
  for (int o = 16; o > 0; o >>= 1) hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
  if (lane == 0) {
    TilePar t;
    const double lat = asin(fmax(-1.0, fmin(1.0, cz))) * 57.29577951308232;
    double lon = atan2(cy, cx) * 57.29577951308232;
    if (lon < 0) lon += 360.0;
    if (lon >= 360.0) lon -= 360.0;
    const double alpha = amax * 1.0001 + 1e-6;
    const double adeg = alpha * 57.29577951308232 + 0.05;
    const bool full = (lat + adeg >= 90.0) || (lat - adeg <= -90.0) || alpha >= 1.5;
    double dl = 180.0;
    if (!full) {
      const double sr = sin(alpha) / cos(lat * 0.017453292519943295);
      dl = sr >= 1.0 ? 180.0 : asin(sr) * 57.29577951308232 * 1.0001 + 0.05;
    }
    t.lonn = (float)lon;
    t.dlon = (float)dl;
    t.cx = (float)cx;
    t.cy = (float)cy;
    t.cz = (float)cz;
    const double ch = 2.0 * sin(0.5 * fmin(alpha, 3.14159265358979));
    t.c2cap = (float)(ch * ch * 1.00001 + 1e-9);
    t.hmax = hm * 1.0001f;
    t.b0 = band_of((float)(lat - adeg));
    t.b1 = band_of((float)(lat + adeg));
    tp[tile] = t;
  }
}

// Stage / ring depths: two operand stages and six record slots (k <= 128:
// 2 x 70 KB + 6 x 10.8 KB).  At k = 40 they made the Gram 1.8 ms faster than
// three stages with three slots (the producers waited on the record copies);
// twelve slots gained nothing more.
void gram_tc_config(int k, int np, int *ns, int *nr, size_t *smem) {
  const size_t PB = (size_t)(np / 8) * SBO;
  const size_t stage = 2 * WB + 2 * PB;
  const size_t cb = record_bytes(k);

  *ns = 2;
  *nr = 6;
  *smem = (size_t)*ns * stage + (size_t)*nr * cb;
}

}  // namespace

size_t record_bytes(int k) { return 512 + (size_t)(((k + 4) & ~3) * YS) * sizeof(float); }

void gram_tc_passes(int k, int *npass, int *np) {
  const int nf = packed_size(k);
  int p = (nf + NPMAX - 1) / NPMAX;
  int n = (nf + p - 1) / p;
  n = (n + 15) & ~15;
  while (n > NPMAX) { p++; n = ((nf + p - 1) / p + 15) & ~15; }
  *npass = p;
  *np = n;
}

cudaError_t launch_tile_prep(cudaStream_t st, int ntiles, const int *tile_cols, const ColPar *cp, TilePar *tp,
                             int *launches) {
  if (ntiles <= 0) return cudaSuccess;
  k_tile_prep<<<(ntiles + 3) / 4, 128, 0, st>>>(ntiles, tile_cols, cp, tp);
  (*launches)++;
  return cudaGetLastError();
}

cudaError_t launch_tile_count(cudaStream_t st, int ntiles, const TilePar *tp, const IndexGeom *geom,
                              const ObsSorted &obs, int *tile_n, int *tile_off, int *launches) {
  if (ntiles <= 0) return cudaMemsetAsync(tile_off, 0, sizeof(int), st);
  k_tile_count<<<ntiles, WT, 0, st>>>(ntiles, tp, geom, obs.A, obs.cell_start, tile_n);
  k_tile_scan<<<1, 1024, 0, st>>>(ntiles, tile_n, tile_off);
  (*launches) += 2;
  return cudaGetLastError();
}

cudaError_t launch_tile_fill(cudaStream_t st, int ntiles, const TilePar *tp, const IndexGeom *geom,
                             const ObsSorted &obs, int k, int kp, const int *tile_off, unsigned char *rec,
                             int *status, int *launches) {
  if (ntiles <= 0) return cudaSuccess;
  const int kr = (k + 4) & ~3;
  k_tile_fill<<<ntiles, WT, 0, st>>>(ntiles, tp, geom, obs, k, kp, kr, (int)record_bytes(k), tile_off, rec, status);
  (*launches)++;
  return cudaGetLastError();
}

template <int LOC, int NS, int NR, int WMODE, bool CULL>
static cudaError_t launch_gram_tc_c(cudaStream_t st, const TcArgs &a, size_t smem, long long grid) {
  cudaError_t e = cudaFuncSetAttribute(k_gram_tc<LOC, NS, NR, WMODE, CULL>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_gram_tc<LOC, NS, NR, WMODE, CULL><<<(int)grid, NT, smem, st>>>(a);
  return cudaGetLastError();
}

template <int LOC, int NS, int NR, int WMODE>
static cudaError_t launch_gram_tc_t(cudaStream_t st, const TcArgs &a, size_t smem, long long grid) {
  if (WMODE != 2 && a.cull) return launch_gram_tc_c<LOC, NS, NR, WMODE, WMODE != 2>(st, a, smem, grid);
  return launch_gram_tc_c<LOC, NS, NR, WMODE, false>(st, a, smem, grid);
}

template <int LOC>
static cudaError_t launch_gram_tc_loc(cudaStream_t st, TcArgs a, int *launches) {
  int ns, nr;
  size_t smem;
  gram_tc_config(a.k, a.np, &ns, &nr, &smem);   // two stages, six record slots
  (void)ns;
  (void)nr;
  if (smem > kSmemBudget) return cudaErrorInvalidValue;   // k <= 128 fits
  const long long per_pass = (long long)a.nwork * a.groups;
  if (per_pass * a.npass > 0x7fffffffLL) return cudaErrorInvalidValue;
  cudaError_t e;
  if (a.npass >= 2 && a.wcache) {
    // first pass computes the weights and caches them; later passes read them
    a.pass0 = 0;
    a.npl = 1;
    e = launch_gram_tc_t<LOC, 2, 6, 1>(st, a, smem, per_pass);
    if (e != cudaSuccess) return e;
    a.pass0 = 1;
    a.npl = a.npass - 1;
    e = launch_gram_tc_t<LOC, 2, 6, 2>(st, a, smem, per_pass * a.npl);
    (*launches) += 2;
    return e;
  }
  a.pass0 = 0;
  a.npl = a.npass;
  e = launch_gram_tc_t<LOC, 2, 6, 0>(st, a, smem, per_pass * a.npass);
  (*launches)++;
  return e;
}

cudaError_t launch_gram_tc(cudaStream_t st, const TcArgs &a_in, int *launches) {
  if (a_in.ntiles <= 0) return cudaSuccess;
  TcArgs a = a_in;
  a.cb = (int)record_bytes(a.k);
  uint32_t tc = 32;
  while ((int)tc < a.np) tc <<= 1;
  a.tmem_cols = tc;
  switch (a.loc.cls) {
  case LOC_OCEAN: return launch_gram_tc_loc<LOC_OCEAN>(st, a, launches);
  case LOC_VTGC: return launch_gram_tc_loc<LOC_VTGC>(st, a, launches);
  default: return launch_gram_tc_loc<LOC_NOVRT>(st, a, launches);
  }
}

namespace {
// A tile whose stream spans several drain intervals: G = the sum of its
// partial blocks in stream order, compensated in FP32 (Sum2 of Ogita, Rump
// and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6),
// 2005: Knuth's error-free TwoSum carries each addition's rounding error
// into a second accumulator, so the result is as accurate as a sum in twice
// the working precision, rounded once; GB300's FP64 pipe is 1/64 of its FP32
// rate, which an FP64 sum of the partials runs into); kept counts,
// candidate counts and the sums of rho summed over the segments in segment
// order (FP32 for rho, as one CTA accumulates it).  One block per (tile,
// group, 32 features): the sums are formed with threads along the columns
// (coalesced block reads) and written with a warp along a column's row
// (coalesced G writes) through shared memory; the first feature block of a
// (tile, group) also sums the counts.
constexpr int SST = 256;
__global__ void __launch_bounds__(SST) k_gram_segsum(TcArgs a) {
  __shared__ float acc[32][TM + 1];
  const int nfc = (a.nf + 31) / 32;
  const int fc = blockIdx.x % nfc, tg = blockIdx.x / nfc;
  const TcSegTile st = a.segtiles[tg / a.groups];
  const int g = tg % a.groups, G = a.groups, nf = a.nf;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = tid & (TM - 1), fh = tid >> 7;   // column, feature half
  const size_t bstride = (size_t)G * nf * TM;   // between consecutive blocks
  const float *P = a.Gpart + ((size_t)st.blk0 * G + g) * nf * TM;
  {
    const int f0 = 32 * fc;
    // blocks in stream order, the 16 features' loads of a block independent
    float hs[16], ls[16];   // running sum, accumulated rounding errors
#pragma unroll
    for (int i = 0; i < 16; i++) hs[i] = ls[i] = 0.0f;
    const int fb = f0 + fh * 16;
    for (int b = 0; b < st.nblk; b++) {
      const float *Pb = P + b * bstride + (size_t)fb * TM + c;
      float x[16];
#pragma unroll
      for (int i = 0; i < 16; i++) x[i] = fb + i < nf ? Pb[(size_t)i * TM] : 0.0f;
#pragma unroll
      for (int i = 0; i < 16; i++) {
        // TwoSum: s + e == hs + x exactly
        const float s = __fadd_rn(hs[i], x[i]);
        const float z = __fsub_rn(s, hs[i]);
        const float e = __fadd_rn(__fsub_rn(hs[i], __fsub_rn(s, z)), __fsub_rn(x[i], z));
        hs[i] = s;
        ls[i] = __fadd_rn(ls[i], e);
      }
    }
#pragma unroll
    for (int i = 0; i < 16; i++) acc[fh * 16 + i][c] = __fadd_rn(hs[i], ls[i]);
    __syncthreads();
    for (int cc = warp; cc < TM; cc += SST / 32) {
      const int col = a.tile_cols[(size_t)st.tile * TM + cc];
      if (col < 0 || f0 + lane >= nf) continue;
      const size_t unit = (size_t)a.col2act[col] * G + g;
      a.G[unit * nf + f0 + lane] = acc[lane][cc];
    }
  }
  if (fc == 0 && tid < TM) {
    const int col = a.tile_cols[(size_t)st.tile * TM + c];
    if (col >= 0) {
      const size_t unit = (size_t)a.col2act[col] * G + g;
      float kept = 0.0f, cand = 0.0f, rs = 0.0f;
      for (int s = 0; s < st.nseg; s++) {
        const float *cc = a.cnt + (((size_t)(st.cblk0 + s) * G + g) * TM + c) * 3;
        kept += cc[0];
        cand += cc[1];
        rs += cc[2];
      }
      a.nkept[unit] = (int)kept;
      if (a.diag_lg_obscount) a.diag_lg_obscount[(size_t)g * a.ncol + col] = kept;
      if (a.diag_lg_obsloc) a.diag_lg_obsloc[(size_t)g * a.ncol + col] = rs;
      if (g == 0 && a.diag_obscount) a.diag_obscount[col] = cand;
    }
  }
}
}  // namespace

cudaError_t launch_gram_segsum(cudaStream_t st, const TcArgs &a, const int *active, int *launches) {
  (void)active;
  if (a.nsegtiles <= 0) return cudaSuccess;
  const long long grid = (long long)a.nsegtiles * a.groups * ((a.nf + 31) / 32);
  if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_gram_segsum<<<(int)grid, SST, 0, st>>>(a);
  (*launches)++;
  return cudaGetLastError();
}

size_t gram_tc_wcache_bytes(int groups, int nchunk_total) {
  return (size_t)groups * nchunk_total * (WCB + sizeof(int));   // operand blocks, then the MMA flags
}

template <int LOC>
static cudaError_t preload_gram_tc_loc() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaSuccess;
  auto get = [&](const void *f) { if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, f); };
  get((const void *)k_gram_tc<LOC, 2, 6, 0, false>);
  get((const void *)k_gram_tc<LOC, 2, 6, 0, true>);
  get((const void *)k_gram_tc<LOC, 2, 6, 1, false>);
  get((const void *)k_gram_tc<LOC, 2, 6, 1, true>);
  get((const void *)k_gram_tc<LOC, 2, 6, 2, false>);
  get((const void *)k_tile_prep);
  get((const void *)k_tile_count);
  get((const void *)k_tile_scan);
  get((const void *)k_tile_fill);
  get((const void *)k_gram_segsum);
  return e;
}

// loads the batched Gram's kernels for a localizer class (CUDA loads a
// kernel at its first use, which must not fall inside a timed trial)
cudaError_t preload_gram_tc(int loc_cls) {
  switch (loc_cls) {
  case LOC_OCEAN: return preload_gram_tc_loc<LOC_OCEAN>();
  case LOC_VTGC: return preload_gram_tc_loc<LOC_VTGC>();
  default: return preload_gram_tc_loc<LOC_NOVRT>();
  }
}

}  // namespace lgpu
