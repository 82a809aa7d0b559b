// lgpu_update_tc.cu -- the ensemble update on the tensor cores: for every
// column, X_a = X_b T_g (src/letkf_solver.F90:285-289, one sgemm per slab in
// the reference) as one M = 128 (slabs) x N = k (members) x K = k GEMM per
// localisation group, followed by the analysis epilogue of lgpu_update.cu
// (:299-379) on the accumulator rows.
//
// Persistent CTAs, one per SM, each walking the columns
// blockIdx.x, blockIdx.x + gridDim.x, ...; warp roles:
//   epilogue   4 warps: thread s owns slab s (TMEM lane s); reads its row
//              of X_b T_g from TMEM, runs recenter / mean clip / RTPS / RTPP
//              / multiplicative inflation / member bounds / spread in the
//              order and arithmetic of k_update_rows, writes the analysis
//              row, mean and spread; the column's scalars are loaded before
//              the wait for its products, the slab's own once per CTA;
//   4 warps    operand producers: from the raw column block in shared memory,
//              chunks of 32 members of A = X_b (128 x 32) and B = T_g^T
//              (N x 32 per group) split into TF32 hi + lo parts in the
//              no-swizzle K-major core-matrix layout;
//   1 warp     one thread bulk-copies each column's background block
//              (ns x k floats, contiguous) and its group transforms into a
//              raw stage;
//   1 warp     one thread issues tcgen05.mma kind::tf32 hi*hi + hi*lo + lo*hi
//              into a double-buffered TMEM accumulator (FP32), so that the
//              epilogue of one column overlaps the products of the next.
// Padding (slabs past ns, members past k) is zero in both operands.  Every
// wait is bounded; one that runs out sets status bit 64 and the roles wind
// down (copies in flight land, every MMA completes, TMEM is freed).
#include "lgpu_internal.cuh"
#include "lgpu_tc.cuh"

namespace lgpu {

namespace {

constexpr int UM = 128;                        // MMA M: slabs per column, TMEM lanes
constexpr int UKC = 32;                        // members per K chunk (4 MMA steps of 8)
constexpr uint32_t UCMB = 128;                 // bytes per core matrix (8 rows x 16 B)
constexpr uint32_t USBO = (UKC / 4) * UCMB;    // bytes per 8-row group of a chunk operand
constexpr uint32_t UAB = UM * UKC * 4;         // bytes of one A chunk part (hi or lo)
constexpr int NEPI = 4, NPROD = 4;             // epilogue / producer warps
constexpr int LOAD_WARP = NEPI + NPROD, MMA_WARP = LOAD_WARP + 1;
constexpr int UNT = 32 * (MMA_WARP + 1);
constexpr int URS = 4, UOS = 3;                // most raw / operand stages

struct UtcBars {
  unsigned long long raw_full[URS], raw_empty[URS], op_full[UOS], op_empty[UOS];
  unsigned long long acc_full[2], acc_empty[2], done;
  uint32_t tmem;
  int fault;
};

struct UtcCfg {
  int rs, os, nkc;              // raw stages, operand stages, K chunks per column
  uint32_t xbytes, tbytes;      // raw background block, raw transforms (all groups)
  uint32_t toff, raw_stride;    // transforms' offset in a raw stage, stage size
  uint32_t bbytes, op_stride;   // one B chunk part (hi or lo), operand stage size
  uint32_t tmem_cols;
};

__device__ __forceinline__ uint32_t ukmaj(int row, int kk) {
  return (uint32_t)(row >> 3) * USBO + (uint32_t)(kk >> 2) * UCMB + (uint32_t)(row & 7) * 16u;
}

__device__ __forceinline__ void arrive(unsigned long long *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(b)) : "memory");
}

__device__ __forceinline__ int utc_group(const UpdateArgs &a, int lev, int mld) {
  if (a.loc_cls == LOC_VTGC) return lev;
  if (a.loc_cls == LOC_OCEAN && a.vtloc_surf == 1) return (lev + 1 <= mld) ? 0 : 1;
  return 0;
}

template <int NP>
__global__ void __launch_bounds__(UNT, 1) k_update_tc(UpdateArgs a, UtcCfg cf) {
  extern __shared__ __align__(1024) unsigned char dsm[];
  __shared__ __align__(8) UtcBars S;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int k = a.k, ns = a.ns, G = a.groups;
  unsigned char *raw0 = dsm;
  unsigned char *op0 = dsm + (size_t)cf.rs * cf.raw_stride;
  // every role walks the CTA's columns with the next one's active index
  // (-1: masked, src/letkf_solver.F90:207) loaded one iteration ahead
  auto act_of = [&](int i) { return i < a.ncols ? a.col2act[a.col0 + i] : -1; };
  auto B = [](unsigned long long &b) { return reinterpret_cast<uint64_t *>(&b); };

  if (wid == 0) tc::tmem_alloc(&S.tmem, cf.tmem_cols);
  if (tid == 0) {
    for (int i = 0; i < cf.rs; i++) {
      tc::mbar_init(B(S.raw_full[i]), 1);
      tc::mbar_init(B(S.raw_empty[i]), NPROD);
    }
    for (int i = 0; i < cf.os; i++) {
      tc::mbar_init(B(S.op_full[i]), NPROD);
      tc::mbar_init(B(S.op_empty[i]), 1);
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(B(S.acc_full[i]), 1);
      tc::mbar_init(B(S.acc_empty[i]), NEPI);
    }
    tc::mbar_init(B(S.done), 1);
    S.fault = 0;
    tc::mbar_fence_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = S.tmem;
  const int nk8 = (k + 7) >> 3;   // MMA K steps per column

  if (wid < NEPI) {
    // ============================================================ epilogue
    const int s = tid;
    const float kf = (float)k, km1 = (float)(k - 1);
    // the slab's variable, level and bounds (the same for every column)
    int v = 0, lev = 0;
    float inc = 0.0f, lb = 0.0f, ub = 0.0f;
    if (s < ns) {
      v = a.slab_var[s];
      lev = a.slab_lev[s];
      inc = a.var_inc_max[v];
      lb = a.var_lb[v];
      ub = a.var_ub[v];
    }
    // the per-column scalars run two columns ahead: the active index and
    // mixed-layer level of column j + 2, then the group's kept count and the
    // slab's background mean and spread of column j + 1
    const int stride = gridDim.x;
    auto mld_of = [&](int i) { return i < a.ncols ? a.cp[a.col0 + i].mld : 0; };
    auto ms_of = [&](int i) { return (size_t)(a.col0 + (i < a.ncols ? i : 0)) * ns + (s < ns ? s : 0); };
    auto group_of = [&](int act, int mld) { return act >= 0 ? utc_group(a, lev, mld) : 0; };
    auto kept_of = [&](int act, int g) { return (act >= 0 && s < ns && g < G) ? a.nkept[(size_t)act * G + g] : 0; };
    int act0 = act_of(blockIdx.x), g0 = group_of(act0, mld_of(blockIdx.x));
    int nk0 = kept_of(act0, g0);
    float mb0 = a.mean_b[ms_of(blockIdx.x)], sb0 = a.sprd_b[ms_of(blockIdx.x)];
    int act1 = act_of(blockIdx.x + stride), mld1 = mld_of(blockIdx.x + stride);
    int n = 0;
    for (int i = blockIdx.x; i < a.ncols; i += stride) {
      const int col = a.col0 + i;
      const int act = act0, g = g0;
      const bool has = s < ns && g < G && nk0 > 0;
      const float mb = mb0, sb = sb0;
      // column j + 1: kept count, mean, spread; column j + 2: index, level
      g0 = group_of(act1, mld1);
      nk0 = kept_of(act1, g0);
      mb0 = a.mean_b[ms_of(i + stride)];
      sb0 = a.sprd_b[ms_of(i + stride)];
      act0 = act1;
      act1 = act_of(i + 2 * stride);
      mld1 = mld_of(i + 2 * stride);
      const size_t cbase = (size_t)col * ns * k;
      const size_t ms = (size_t)col * ns + s;
      if (act < 0) {   // src/letkf_solver.F90:207: the block leaves unchanged
        if (s < ns) {
          if (a.ana != a.bkg) {
            const float4 *src = reinterpret_cast<const float4 *>(a.bkg + cbase + (size_t)s * k);
            float4 *dst = reinterpret_cast<float4 *>(a.ana + cbase + (size_t)s * k);
            for (int q = 0; q < (k >> 2); q++) dst[q] = src[q];
          }
          a.mean_a[ms] = mb;
          a.sprd_a[ms] = sb;
        }
        continue;
      }
      const int ab = n & 1;
      const int par = (n >> 1) & 1;
      n++;
      if (!tc::mbar_wait(B(S.acc_full[ab]), par)) { S.fault = 1; break; }
      tc::fence_after();
      // the slab's row of X_b T_g (TMEM loads are warp-wide: every group is
      // read, the thread keeps its own)
      float x[NP];
      const uint32_t tb = tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)(ab * G * NP);
#pragma unroll
      for (int c0 = 0; c0 < NP; c0 += 16) {
        float vv[16];
        tc::tmem_ld16(tb + (uint32_t)c0, vv);
#pragma unroll
        for (int q = 0; q < 16; q++) x[c0 + q] = vv[q];
        if (G > 1) {
          tc::tmem_ld16(tb + (uint32_t)(NP + c0), vv);
#pragma unroll
          for (int q = 0; q < 16; q++)
            if (g == 1) x[c0 + q] = vv[q];
        }
      }
      tc::fence_before();
      __syncwarp();
      if (lane == 0) arrive(&S.acc_empty[ab]);
      if (s >= ns) continue;
      const float *xbr = a.bkg + cbase + (size_t)s * k;
      if (!has) {   // no local observations: the background perturbation
#pragma unroll
        for (int j = 0; j < NP; j++)
          if (j < k) x[j] = xbr[j];
      }
      // recenter (:299-303)
#pragma unroll
      for (int j = 0; j < NP; j++)
        if (j < k) x[j] = x[j] + mb;
      float m = 0.0f;
#pragma unroll
      for (int j = 0; j < NP; j++)
        if (j < k) m = m + x[j];
      m = m / kf;
#pragma unroll
      for (int j = 0; j < NP; j++) x[j] = x[j] - m;
      // mean increment clip and bounds (:308-318)
      {
        float r = m - mb;
        r = fmaxf(r, -inc); r = fminf(r, inc);
        r = fmaxf(r, lb - mb); r = fminf(r, ub - mb);
        m = r + mb;
      }
      if (a.rtps > 0.0f) {   // (:322-335)
        float q2 = 0.0f;
#pragma unroll
        for (int j = 0; j < NP; j++)
          if (j < k) q2 = q2 + x[j] * x[j];
        const float sa = sqrtf(q2 / km1);
        if (sa > 0.0f) {
          const float f = a.rtps * (sb - sa) / sa + 1.0f;
#pragma unroll
          for (int j = 0; j < NP; j++) x[j] = x[j] * f;
        }
      }
      if (a.rtpp > 0.0f) {   // (:339-344)
#pragma unroll
        for (int j = 0; j < NP; j++)
          if (j < k) x[j] = a.rtpp * xbr[j] + (1.0f - a.rtpp) * x[j];
      }
      if (a.mul != 1.0f) {   // (:347-349)
#pragma unroll
        for (int j = 0; j < NP; j++) x[j] = x[j] * a.mul;
      }
      {   // member bounds and re-mean (:357-371)
#pragma unroll
        for (int j = 0; j < NP; j++)
          if (j < k) x[j] = fminf(fmaxf(x[j], lb - m), ub - m);
        float r = 0.0f;
#pragma unroll
        for (int j = 0; j < NP; j++)
          if (j < k) r = r + x[j];
        r = r / kf;
#pragma unroll
        for (int j = 0; j < NP; j++) x[j] = x[j] - r;
        m = m + r;
      }
      // spread, add the mean back (:375-379)
      float q2 = 0.0f;
#pragma unroll
      for (int j = 0; j < NP; j++)
        if (j < k) q2 = q2 + x[j] * x[j];
      const float sa = sqrtf(q2 / km1);
      float4 *out4 = reinterpret_cast<float4 *>(a.ana + cbase + (size_t)s * k);
#pragma unroll
      for (int q = 0; q < NP / 4; q++)
        if (4 * q < k) out4[q] = make_float4(x[4 * q] + m, x[4 * q + 1] + m, x[4 * q + 2] + m, x[4 * q + 3] + m);
      a.mean_a[ms] = m;
      a.sprd_a[ms] = sa;
      if (!isfinite(m) || !isfinite(sa)) atomicOr(a.status, 4);
    }
  } else if (wid < NEPI + NPROD) {
    // ============================================================ producers
    const int p = tid - 32 * NEPI;   // 0 .. 127: row of A; B items p, p + 128, ...
    int n = 0, c = 0;
    bool stop = false;
    int nxt = act_of(blockIdx.x);
    for (int i = blockIdx.x; i < a.ncols && !stop; i += gridDim.x) {
      const int act = nxt;
      nxt = act_of(i + gridDim.x);
      if (act < 0) continue;
      const int rsi = n % cf.rs;
      if (!tc::mbar_wait(B(S.raw_full[rsi]), (n / cf.rs) & 1)) { S.fault = 1; break; }
      const float *X = reinterpret_cast<const float *>(raw0 + (size_t)rsi * cf.raw_stride);
      const float *Tr = reinterpret_cast<const float *>(raw0 + (size_t)rsi * cf.raw_stride + cf.toff);
      for (int kc = 0; kc < cf.nkc; kc++) {
        const int osi = c % cf.os;
        if (c >= cf.os && !tc::mbar_wait(B(S.op_empty[osi]), ((c / cf.os) - 1) & 1)) {
          S.fault = 1;
          stop = true;
          break;
        }
        unsigned char *Ahi = op0 + (size_t)osi * cf.op_stride, *Alo = Ahi + UAB;
        // A: row p (slab), members 32 kc + 4 kq .. + 3
#pragma unroll
        for (int kq = 0; kq < UKC / 4; kq++) {
          const int j = UKC * kc + 4 * kq;
          float4 xv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          if (p < ns && j < k) xv = *reinterpret_cast<const float4 *>(X + (size_t)p * k + j);
          float h[4], l[4];
          tc::split_tf32(xv.x, h[0], l[0]);
          tc::split_tf32(xv.y, h[1], l[1]);
          tc::split_tf32(xv.z, h[2], l[2]);
          tc::split_tf32(xv.w, h[3], l[3]);
          const uint32_t off = ukmaj(p, 4 * kq);
          *reinterpret_cast<float4 *>(Ahi + off) = make_float4(h[0], h[1], h[2], h[3]);
          *reinterpret_cast<float4 *>(Alo + off) = make_float4(l[0], l[1], l[2], l[3]);
        }
        // B_g: row nn (output member), K = input members 32 kc + 4 kq .. + 3:
        // B_g[nn][i] = T_g[i][nn]
        for (int g = 0; g < G; g++) {
          unsigned char *Bhi = Ahi + 2 * UAB + (size_t)g * 2 * cf.bbytes, *Blo = Bhi + cf.bbytes;
          const float *Tg = Tr + (size_t)g * k * k;
          for (int w = p; w < NP * (UKC / 4); w += 32 * NPROD) {
            const int nn = w % NP, kq = w / NP;
            const int i0 = UKC * kc + 4 * kq;
            float h[4], l[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const float t = (nn < k && i0 + u < k) ? Tg[(size_t)(i0 + u) * k + nn] : 0.0f;
              tc::split_tf32(t, h[u], l[u]);
            }
            const uint32_t off = ukmaj(nn, 4 * kq);
            *reinterpret_cast<float4 *>(Bhi + off) = make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4 *>(Blo + off) = make_float4(l[0], l[1], l[2], l[3]);
          }
        }
        tc::fence_proxy_async();   // generic-proxy writes -> the tensor core's reads
        __syncwarp();
        if (lane == 0) arrive(&S.op_full[osi]);
        c++;
      }
      if (stop) break;
      __syncwarp();
      if (lane == 0) arrive(&S.raw_empty[rsi]);   // every read of the raw stage is done
      n++;
    }
  } else if (wid == LOAD_WARP) {
    // ============================================================ loader
    if (lane == 0) {
      int n = 0;
      int nxt = act_of(blockIdx.x);
      for (int i = blockIdx.x; i < a.ncols; i += gridDim.x) {
        const int col = a.col0 + i;
        const int act = nxt;
        nxt = act_of(i + gridDim.x);
        if (act < 0) continue;
        const int rsi = n % cf.rs;
        if (n >= cf.rs && !tc::mbar_wait(B(S.raw_empty[rsi]), ((n / cf.rs) - 1) & 1)) { S.fault = 1; break; }
        unsigned char *dst = raw0 + (size_t)rsi * cf.raw_stride;
        uint64_t *fb = B(S.raw_full[rsi]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(fb)),
                     "r"(cf.xbytes + cf.tbytes) : "memory");
        tc::bulk_copy_g2s(dst, a.bkg + (size_t)col * ns * k, cf.xbytes, fb);
        tc::bulk_copy_g2s(dst + cf.toff, a.T + (size_t)act * G * k * k, cf.tbytes, fb);
        n++;
      }
      // no copy may still be in flight when the CTA exits
      for (int j = n > cf.rs ? n - cf.rs : 0; j < n; j++)
        if (!tc::mbar_wait(B(S.raw_full[j % cf.rs]), (j / cf.rs) & 1)) S.fault = 1;
    }
  } else if (wid == MMA_WARP) {
    // ============================================================ MMA issue
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_tf32(UM, NP);
      int n = 0, c = 0;
      bool stop = false;
      int nxt = act_of(blockIdx.x);
      for (int i = blockIdx.x; i < a.ncols && !stop; i += gridDim.x) {
        const int act = nxt;
        nxt = act_of(i + gridDim.x);
        if (act < 0) continue;
        const int ab = n & 1;
        if (n >= 2 && !tc::mbar_wait(B(S.acc_empty[ab]), ((n >> 1) - 1) & 1)) { S.fault = 1; break; }
        tc::fence_after();
        const uint32_t dacc = tmem + (uint32_t)(ab * G * NP);
        for (int kc = 0; kc < cf.nkc; kc++) {
          const int osi = c % cf.os;
          if (!tc::mbar_wait(B(S.op_full[osi]), (c / cf.os) & 1)) { S.fault = 1; stop = true; break; }
          tc::fence_after();
          const uint32_t ahi = tc::smem_u32(op0 + (size_t)osi * cf.op_stride), alo = ahi + UAB;
          const int nks = nk8 - 4 * kc < 4 ? nk8 - 4 * kc : 4;
          for (int g = 0; g < G; g++) {
            const uint32_t bhi = ahi + 2 * UAB + (uint32_t)g * 2 * cf.bbytes, blo = bhi + cf.bbytes;
            for (int ks = 0; ks < nks; ks++)
#pragma unroll
              for (int t = 0; t < 3; t++) {
                const uint32_t acc = (kc > 0 || ks > 0 || t > 0) ? 1u : 0u;
                const uint32_t aw = t == 2 ? alo : ahi, bw = t == 1 ? blo : bhi;
                const uint64_t ad = tc::smem_desc(aw + (uint32_t)ks * 2 * UCMB, UCMB, USBO);
                const uint64_t bd = tc::smem_desc(bw + (uint32_t)ks * 2 * UCMB, UCMB, USBO);
                tc::mma_tf32(dacc + (uint32_t)(g * NP), ad, bd, idesc, acc);
              }
          }
          tc::commit(B(S.op_empty[osi]));   // the stage is free once these MMAs complete
          c++;
        }
        if (stop) break;
        tc::commit(B(S.acc_full[ab]));
        n++;
      }
      // every MMA issued by this thread has completed once `done` flips
      tc::commit(B(S.done));
      if (!tc::mbar_wait(B(S.done), 0)) S.fault = 1;
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (S.fault && tid == 0) atomicOr(a.status, 64);
  if (wid == 0) tc::tmem_dealloc(tmem, cf.tmem_cols);
}

template <int NP>
cudaError_t launch_np(cudaStream_t st, const UpdateArgs &a, const UtcCfg &cf, size_t smem, int grid) {
  cudaError_t e = cudaFuncSetAttribute(k_update_tc<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_update_tc<NP><<<grid, UNT, smem, st>>>(a, cf);
  return cudaGetLastError();
}

}  // namespace

// Used above k = 64: at k = 40 the CUDA-core form (k_update_rows) streams
// the columns faster (C2: 2.6 against 4.4 ms), at k = 100 this form wins
// (C4: 63 against 70 ms).
bool update_tc_eligible(const UpdateArgs &a, size_t *smem_out) {
  if (a.k <= 64 || a.k > 128 || (a.k & 3) || a.ns < 1 || a.ns > UM || a.groups < 1 || a.groups > 2) return false;
  const int NP = (a.k + 15) & ~15;
  const uint32_t xbytes = (uint32_t)a.ns * a.k * 4, tbytes = (uint32_t)a.groups * a.k * a.k * 4;
  const uint32_t toff = (xbytes + 127) & ~127u;
  const uint32_t raw = (toff + tbytes + 127) & ~127u;
  const uint32_t op = (2 * UAB + (uint32_t)a.groups * 2 * NP * UKC * 4 + 1023) & ~1023u;
  const size_t budget = 227 * 1024 - 1024;
  for (int rs = URS; rs >= 1; rs--)
    for (int os = UOS; os >= 2; os--) {
      const size_t smem = (size_t)rs * raw + (size_t)os * op;
      if (smem <= budget) {
        if (smem_out) *smem_out = smem;
        return true;
      }
    }
  return false;
}

cudaError_t launch_update_tc(cudaStream_t st, const UpdateArgs &a, int *launches) {
  if (a.ncol <= 0 || a.ncols <= 0) return cudaSuccess;
  size_t dummy;
  if (!update_tc_eligible(a, &dummy)) return cudaErrorNotSupported;
  UtcCfg cf;
  const int NP = (a.k + 15) & ~15;
  cf.xbytes = (uint32_t)a.ns * a.k * 4;
  cf.tbytes = (uint32_t)a.groups * a.k * a.k * 4;
  cf.toff = (cf.xbytes + 127) & ~127u;
  cf.raw_stride = (cf.toff + cf.tbytes + 127) & ~127u;
  cf.bbytes = (uint32_t)NP * UKC * 4;
  cf.op_stride = (2 * UAB + (uint32_t)a.groups * 2 * cf.bbytes + 1023) & ~1023u;
  cf.nkc = (a.k + UKC - 1) / UKC;
  const size_t budget = 227 * 1024 - 1024;
  size_t smem = 0;
  cf.rs = 0;
  for (int rs = URS; rs >= 1 && !cf.rs; rs--)
    for (int os = UOS; os >= 2; os--) {
      const size_t sm = (size_t)rs * cf.raw_stride + (size_t)os * cf.op_stride;
      if (sm <= budget) { cf.rs = rs; cf.os = os; smem = sm; break; }
    }
  if (!cf.rs) return cudaErrorNotSupported;
  uint32_t tc = 32;
  while ((int)tc < 2 * a.groups * NP) tc <<= 1;
  cf.tmem_cols = tc;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // one CTA per SM (its registers take most of the register file)
  const int grid = a.ncols < nsm ? a.ncols : nsm;
  cudaError_t e;
  switch (NP) {
  case 80: e = launch_np<80>(st, a, cf, smem, grid); break;
  case 96: e = launch_np<96>(st, a, cf, smem, grid); break;
  case 112: e = launch_np<112>(st, a, cf, smem, grid); break;
  case 128: e = launch_np<128>(st, a, cf, smem, grid); break;
  default: return cudaErrorNotSupported;
  }
  if (e == cudaSuccess) (*launches)++;
  return e;
}

}  // namespace lgpu
