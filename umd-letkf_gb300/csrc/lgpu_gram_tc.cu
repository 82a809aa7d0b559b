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
// chunks of 16.  Per chunk, CUDA-core threads evaluate the exact distance and
// the localizer for every (column, observation) pair (bit-identical keep
// decisions to the per-column path), form the feature products, split both
// operands into tf32 hi + lo parts and store them in the no-swizzle K-major
// core-matrix layout; one thread issues tcgen05.mma kind::tf32 for the
// three products hi*hi + hi*lo + lo*hi with FP32 accumulation in TMEM
// (relative error ~2^-21 per product, FP32-class).  Two shared-memory stages
// let the tensor cores run while the next chunk is produced; chunks in which
// no column keeps any observation issue no MMA.  The epilogue reads TMEM
// lane c = column c and writes the packed Gram block of each unit.
#include "lgpu_internal.cuh"
#include "lgpu_tc.cuh"

namespace lgpu {

namespace {

constexpr int TM = 128;        // columns per tile = MMA M = TMEM lanes
constexpr int KC = 16;         // observations per chunk (two K=8 MMA steps)
constexpr int NT = 512;        // threads per CTA: warps 0-7 weights, warps 8-15 features
constexpr int NPMAX = 432;     // features per pass
constexpr int TMEM_COLS = 512;
constexpr int MAXSEG = 2 * kNB;
constexpr int YT_LD = 16;      // transposed staging row: 16 observations of one member
constexpr uint32_t CMB = 128;                 // bytes per core matrix (8 rows x 16 B)
constexpr uint32_t SBO = (KC / 4) * CMB;      // bytes per 8-row group (all K of the chunk)
constexpr uint32_t WB = (TM / 8) * SBO;       // bytes per W operand copy

__device__ __forceinline__ uint32_t kmaj(int row, int kk) {
  return (uint32_t)(row >> 3) * SBO + (uint32_t)(kk >> 2) * CMB + (uint32_t)(row & 7) * 16u + (uint32_t)(kk & 3) * 4u;
}

struct TcSmem {
  int seg_start[MAXSEG];
  int seg_pref[MAXSEG + 1];
  int wsc[NT / 32];
  int total;
  uint32_t tmem;
  unsigned long long mbar[2];
  int pos[2][KC];            // sorted positions of the chunk's observations (double buffered)
  float4 obsA[KC];           // ux, uy, uz, 1/err
  float4 obsB[KC];           // dep, time, zdim, surf
  int obsValid[KC];
  unsigned char fi[NPMAX];
  unsigned char fj[NPMAX];
  int dcand[TM], dkept[TM];
  float drsum[TM];
};

__device__ __forceinline__ int run_lookup(const TcSmem &S, int nseg, int jj) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (S.seg_pref[mid] <= jj) lo = mid; else hi = mid - 1;
  }
  return S.seg_start[lo] + (jj - S.seg_pref[lo]);
}

__global__ void __launch_bounds__(NT, 1) k_gram_tc(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char dsm[];
  __shared__ __align__(16) TcSmem S;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int pass = blockIdx.x % a.npass;
  const int g = (blockIdx.x / a.npass) % a.groups;
  const int tile = blockIdx.x / (a.npass * a.groups);
  const int k = a.k, kp = a.kp, NP = a.np, nf = a.nf;
  const uint32_t PB = (uint32_t)(NP / 8) * SBO;
  const uint32_t stage_bytes = 2 * WB + 2 * PB;
  unsigned char *stg[2] = {dsm, dsm + stage_bytes};
  float *yT = reinterpret_cast<float *>(dsm + 2 * stage_bytes);   // [kp + 4][YT_LD]

  // ---- setup: TMEM, barriers, feature table
  if (wid == 0) tc::tmem_alloc(&S.tmem, TMEM_COLS);
  if (tid == 0) {
    tc::mbar_init(reinterpret_cast<uint64_t *>(&S.mbar[0]), 1);
    tc::mbar_init(reinterpret_cast<uint64_t *>(&S.mbar[1]), 1);
    tc::mbar_fence_init();
  }
  for (int f = tid; f < NP; f += NT) {
    const int fg = pass * NP + f;
    int i = 255, j = 255;
    if (fg < nf) packed_ij(fg, k, i, j);
    S.fi[f] = (unsigned char)i;
    S.fj[f] = (unsigned char)j;
  }
  const TilePar tp = a.tp[tile];
  // weight role (warps 0-7): column tid & 127, observations [8*(tid>>7), +8)
  const bool wrole = tid < 256;
  const int wc = tid & (TM - 1), wh = (tid >> 7) & 1;
  const int col = a.tile_cols[(size_t)tile * TM + wc];
  const bool colv = wrole && col >= 0;
  ColPar cp;
  if (colv) cp = a.cp[col];
  else { cp.ux = cp.uy = cp.uz = 0.0f; cp.rmax = -1.0f; cp.L1 = cp.L2 = 1.0f; cp.ic1 = cp.ic2 = 1.0f; }
  float c2max = -1.0f;
  if (colv) {
    const float hq = fminf(cp.rmax / 12742000.0f, 1.5707963f);
    const float sh = sinf(hq);
    c2max = 4.0f * sh * sh * 1.0001f + 1e-12f;
  }
  int ncand = 0, nkeep = 0;
  float rsum = 0.0f;

  // ---- index window of the tile -> runs of the sorted observation table
  const int nb = tp.b1 - tp.b0 + 1;
  if (tid < nb) {
    const int b = tp.b0 + tid;
    const int nl = a.geom->nlon[b], off = a.geom->off[b];
    int s0 = 0, l0 = 0, s1 = 0, l1 = 0;
    bool whole = tp.dlon >= 180.0f;
    int clo = 0, chi = nl - 1;
    if (!whole) {
      clo = (int)floorf((tp.lonn - tp.dlon) * (float)nl / 360.0f);
      chi = (int)floorf((tp.lonn + tp.dlon) * (float)nl / 360.0f);
      if (chi - clo + 1 >= nl) whole = true;
    }
    if (whole) {
      s0 = a.obs.cell_start[off];
      l0 = a.obs.cell_start[off + nl] - s0;
    } else if (clo < 0) {
      s0 = a.obs.cell_start[off + clo + nl];
      l0 = a.obs.cell_start[off + nl] - s0;
      s1 = a.obs.cell_start[off];
      l1 = a.obs.cell_start[off + chi + 1] - s1;
    } else if (chi >= nl) {
      s0 = a.obs.cell_start[off + clo];
      l0 = a.obs.cell_start[off + nl] - s0;
      s1 = a.obs.cell_start[off];
      l1 = a.obs.cell_start[off + (chi - nl) + 1] - s1;
    } else {
      s0 = a.obs.cell_start[off + clo];
      l0 = a.obs.cell_start[off + chi + 1] - s0;
    }
    S.seg_start[2 * tid] = s0;
    S.seg_start[2 * tid + 1] = s1;
    S.seg_pref[2 * tid] = l0;
    S.seg_pref[2 * tid + 1] = l1;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = S.tmem;
  const int nseg = 2 * nb;
  {
    const int i0 = 2 * tid, i1 = 2 * tid + 1;
    const int v0 = i0 < nseg ? S.seg_pref[i0] : 0;
    const int v1 = i1 < nseg ? S.seg_pref[i1] : 0;
    const int x = v0 + v1;
    int incl = x;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) S.wsc[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      int s = lane < NT / 32 ? S.wsc[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (lane < NT / 32) S.wsc[lane] = s;
    }
    __syncthreads();
    const int basev = (wid > 0 ? S.wsc[wid - 1] : 0) + incl - x;
    __syncthreads();
    if (i0 < nseg) S.seg_pref[i0] = basev;
    if (i1 < nseg) S.seg_pref[i1] = basev + v0;
    if (tid == 0) { S.total = S.wsc[NT / 32 - 1]; S.seg_pref[nseg] = S.total; }
    __syncthreads();
  }
  const int total = S.total;
  const int nchunks = (total + KC - 1) / KC;
  if (tid < KC && tid < total) S.pos[0][tid] = run_lookup(S, nseg, tid);
  __syncthreads();

  // MMA N-blocks of this pass: [0, min(NP,256)), [256, NP)
  const int nb0 = NP < 256 ? NP : 256, nb1 = NP - nb0;
  const uint32_t id0 = tc::idesc_tf32(TM, nb0), id1 = nb1 > 0 ? tc::idesc_tf32(TM, nb1) : 0u;
  bool pending0 = false, pending1 = false;
  uint32_t phase0 = 0, phase1 = 0;
  bool issued = false, fault = false;
  const float4 *hx4 = reinterpret_cast<const float4 *>(a.obs.hx);
  const int q4 = kp >> 2;
  // feature role (warps 8-15): features tid-256 and tid (those < NP)
  const int pf0 = tid - 256;

  for (int ch = 0; ch < nchunks; ch++) {
    const int s = ch & 1;
    const int pb = ch & 1;
    // ---- stage: hx transposed to yT[member][obs] (+ dep as member k), obs records
    {
      const int t = tid;
      const int nq = q4 + 1;             // hx quads + the quad holding dep at index k
      if (t < nq * KC) {
        const int qq = t >> 4, e = t & 15;
        const int jj = ch * KC + e;
        const bool v = jj < total;
        const int pos = v ? S.pos[pb][e] : 0;
        float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
        if (v && qq < q4) y = hx4[(size_t)pos * q4 + qq];
        if (qq == (k >> 2)) {
          const float dep = v ? a.obs.B[pos].x : 0.0f;
          const int c = k & 3;
          if (c == 0) y.x = dep; else if (c == 1) y.y = dep; else if (c == 2) y.z = dep; else y.w = dep;
        }
        yT[(4 * qq + 0) * YT_LD + e] = y.x;
        yT[(4 * qq + 1) * YT_LD + e] = y.y;
        yT[(4 * qq + 2) * YT_LD + e] = y.z;
        yT[(4 * qq + 3) * YT_LD + e] = y.w;
      } else if (t >= 480 && t < 480 + KC) {
        const int e = t - 480;
        const int jj = ch * KC + e;
        const bool v = jj < total;
        const int pos = v ? S.pos[pb][e] : 0;
        float4 A = make_float4(0.f, 0.f, 0.f, 1.f), B = make_float4(0.f, 0.f, 0.f, 0.f);
        if (v) { A = a.obs.A[pos]; B = a.obs.B[pos]; A.w = __frcp_rn(A.w); }
        S.obsA[e] = A;
        S.obsB[e] = B;
        S.obsValid[e] = v;
      } else if (t >= 448 && t < 448 + KC) {
        // positions of the next chunk
        const int e = t - 448;
        const int jj = (ch + 1) * KC + e;
        if (jj < total) S.pos[pb ^ 1][e] = run_lookup(S, nseg, jj);
      }
    }
    // ---- stage s must be free (MMAs of chunk ch-2 done): thread 0 waits, the
    // barrier publishes the staged data and the outcome
    {
      bool bad = false;
      if (tid == 0) {
        if (s == 0 && pending0) bad = !tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.mbar[0]), phase0);
        if (s == 1 && pending1) bad = !tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.mbar[1]), phase1);
      }
      if (s == 0 && pending0) { phase0 ^= 1; pending0 = false; }
      if (s == 1 && pending1) { phase1 ^= 1; pending1 = false; }
      if (__syncthreads_or(bad)) { fault = true; break; }
    }
    unsigned char *Whi = stg[s], *Wlo = stg[s] + WB, *Phi = stg[s] + 2 * WB, *Plo = stg[s] + 2 * WB + PB;
    bool anyk = false;
    if (wrole) {
      // ---- W: weights of column wc for 8 observations (exact keep decisions)
#pragma unroll
      for (int grp = 0; grp < 2; grp++) {
        float h4[4], l4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = wh * 8 + grp * 4 + u;
          float w = 0.0f;
          const float4 A = S.obsA[e];
          const float c2 = chord2_exact(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z);
          if (c2 <= c2max && S.obsValid[e]) {
            const float d = dist_from_chord2(c2);
            if (d <= cp.rmax) {
              ncand++;
              const float4 B = S.obsB[e];
              const float r = localize(a.loc, cp, g, d, B.y, B.z, B.w);
              if (r > kKeep) {
                w = r * A.w;
                nkeep++;
                rsum += r;
                anyk = true;
              }
            }
          }
          tc::split_tf32(w, h4[u], l4[u]);
        }
        const uint32_t off = kmaj(wc, wh * 8 + grp * 4);
        *reinterpret_cast<float4 *>(Whi + off) = make_float4(h4[0], h4[1], h4[2], h4[3]);
        *reinterpret_cast<float4 *>(Wlo + off) = make_float4(l4[0], l4[1], l4[2], l4[3]);
      }
    } else {
      // ---- P: feature products y_i * y_j for 16 observations
#pragma unroll
      for (int rep = 0; rep < 2; rep++) {
        const int f = pf0 + 256 * rep;
        if (f < NP) {
          const int i = S.fi[f], j = S.fj[f];
          const bool fv = i != 255;
          const float4 *yi = reinterpret_cast<const float4 *>(yT + (fv ? i : 0) * YT_LD);
          const float4 *yj = reinterpret_cast<const float4 *>(yT + (fv ? j : 0) * YT_LD);
#pragma unroll
          for (int grp = 0; grp < 4; grp++) {
            const float4 a4 = yi[grp], b4 = yj[grp];
            float v[4] = {a4.x * b4.x, a4.y * b4.y, a4.z * b4.z, a4.w * b4.w};
            float h4[4], l4[4];
#pragma unroll
            for (int u = 0; u < 4; u++) tc::split_tf32(fv ? v[u] : 0.0f, h4[u], l4[u]);
            const uint32_t off = kmaj(f, grp * 4);
            *reinterpret_cast<float4 *>(Phi + off) = make_float4(h4[0], h4[1], h4[2], h4[3]);
            *reinterpret_cast<float4 *>(Plo + off) = make_float4(l4[0], l4[1], l4[2], l4[3]);
          }
        }
      }
    }
    tc::fence_proxy_async();
    const bool chunk_keep = __syncthreads_or(anyk) != 0;
    // ---- issue: D += Whi*Phi + Whi*Plo + Wlo*Phi
    if (chunk_keep) {
      if (tid == 0) {
        tc::fence_after();
        const uint32_t aw[3] = {tc::smem_u32(Whi), tc::smem_u32(Whi), tc::smem_u32(Wlo)};
        const uint32_t bp[3] = {tc::smem_u32(Phi), tc::smem_u32(Plo), tc::smem_u32(Phi)};
#pragma unroll
        for (int t = 0; t < 3; t++)
#pragma unroll
          for (int ks = 0; ks < KC / 8; ks++) {
            const uint32_t acc = (issued || t > 0 || ks > 0) ? 1u : 0u;
            const uint64_t ad = tc::smem_desc(aw[t] + ks * 2 * CMB, CMB, SBO);
            const uint64_t bd0 = tc::smem_desc(bp[t] + ks * 2 * CMB, CMB, SBO);
            tc::mma_tf32(tmem, ad, bd0, id0, acc);
            if (nb1 > 0) {
              const uint64_t bd1 = tc::smem_desc(bp[t] + (uint32_t)(nb0 / 8) * SBO + ks * 2 * CMB, CMB, SBO);
              tc::mma_tf32(tmem + (uint32_t)nb0, ad, bd1, id1, acc);
            }
          }
        tc::commit(reinterpret_cast<uint64_t *>(&S.mbar[s]));
      }
      issued = true;
      if (s == 0) pending0 = true; else pending1 = true;
    }
  }
  // ---- drain (thread 0 waits, the barrier publishes the outcome)
  {
    bool bad = false;
    if (tid == 0) {
      if (pending0 && !tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.mbar[0]), phase0)) bad = true;
      if (pending1 && !tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.mbar[1]), phase1)) bad = true;
    }
    if (__syncthreads_or(bad)) fault = true;
  }
  tc::fence_after();

  // ---- per-column diagnostics and kept counts (both halves of a column)
  if (wrole && wh == 1) { S.dcand[wc] = ncand; S.dkept[wc] = nkeep; S.drsum[wc] = rsum; }
  __syncthreads();
  const int G = a.groups;
  if (tid < TM) {
    ncand += S.dcand[wc];
    nkeep += S.dkept[wc];
    rsum += S.drsum[wc];
    size_t unit = 0;
    if (colv) unit = (size_t)a.col2act[col] * G + g;
    if (colv && pass == 0) {
      a.nkept[unit] = nkeep;
      if (a.diag_lg_obscount) a.diag_lg_obscount[(size_t)g * a.ncol + col] = (float)nkeep;
      if (a.diag_lg_obsloc) a.diag_lg_obsloc[(size_t)g * a.ncol + col] = rsum;
      if (g == 0 && a.diag_obscount) a.diag_obscount[col] = (float)ncand;
    }
    // ---- epilogue: TMEM lane tid = column tid, 16 features per load
    float *Gp = a.G + unit * (size_t)nf + (size_t)pass * NP;
    const int nvalid = nf - pass * NP < NP ? nf - pass * NP : NP;
    for (int f0 = 0; f0 < NP; f0 += 16) {
      float v[16];
      if (issued && !fault) {
        tc::tmem_ld16(tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)f0, v);
      } else {
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = 0.0f;
      }
      if (colv) {
#pragma unroll
        for (int q = 0; q < 16; q++)
          if (f0 + q < nvalid) Gp[f0 + q] = v[q];
      }
    }
  }
  if (fault && tid == 0) atomicOr(a.status, 16);
  tc::fence_before();
  __syncthreads();
  if (wid == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
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
    t.b0 = band_of((float)(lat - adeg));
    t.b1 = band_of((float)(lat + adeg));
    tp[tile] = t;
  }
}

}  // namespace

size_t gram_tc_smem_bytes(int k, int np) {
  const int kp = (k + 3) & ~3;
  const size_t PB = (size_t)(np / 8) * SBO;
  return 2 * (2 * WB + 2 * PB) + (size_t)(kp + 4) * YT_LD * sizeof(float);
}

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

cudaError_t launch_gram_tc(cudaStream_t st, const TcArgs &a, int *launches) {
  if (a.ntiles <= 0) return cudaSuccess;
  const size_t smem = gram_tc_smem_bytes(a.k, a.np);
  cudaError_t e = cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long grid = (long long)a.ntiles * a.groups * a.npass;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_gram_tc<<<(int)grid, NT, smem, st>>>(a);
  (*launches)++;
  return cudaGetLastError();
}

}  // namespace lgpu
