// lgpu_mlp.cu -- the weight-correction network of the learned analysis form.
//
// Three dense layers din -> H -> H -> dout with GELU between them; BF16
// weights and activations, FP32 accumulation.  The network maps the
// interpolated transform of a grid column (W, w-bar) plus observation
// geometry features to a correction of (W, w-bar) (no counterpart in the
// reference: the reference solves every column exactly,
// src/letkf_solver.F90:203-384).
//
//   inference  k_mlp_tc: tcgen05.mma kind::f16 (BF16 x BF16 -> FP32 in TMEM),
//              M = 128 rows of a row block, N <= 256 outputs of an N tile,
//              K = 16 per instruction.  Operands live in global memory
//              already in the no-swizzle K-major core-matrix order, one
//              contiguous block per (row block, 16-wide K slice), so one
//              cp.async.bulk per operand and stage fills shared memory.  The
//              epilogue (TMEM -> registers) adds the bias, applies GELU and
//              writes the next layer's input blocks in the same tiled order,
//              or FP32 rows for the last layer.
//   training   k_mlp_gemm: CUDA-core GEMM over strided operands (any
//              transposition), FP32 accumulation of BF16-rounded values,
//              epilogues for the forward (bias, GELU) and the backward
//              (GELU derivative); k_mlp_adam updates FP32 master weights and
//              their BF16 copies.
#include "lgpu_internal.cuh"
#include "lgpu_tc.cuh"
#include <cuda_bf16.h>

namespace lgpu {

namespace {

constexpr int RB_ACT = 128;   // rows per activation block (MMA M)
constexpr int RB_W = 256;     // rows per weight block (largest MMA N)
constexpr int TC_NS = 8;      // operand stages of k_mlp_tc (96 KB: two CTAs per SM, 2 x 256 TMEM columns)
constexpr int TC_THREADS = 128;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  return cdf + z * pdf;
}

}  // namespace

// byte offset of element (r, kk) of a K-major tiled BF16 matrix: row blocks of
// rb rows, K slices of 16; inside a (row block, K slice) block the core
// matrices (8 rows x 8 elements, 128 B) run along K first (LBO 128 B), then
// along the rows (SBO 256 B)
__host__ __device__ size_t mlp_tile_off(int r, int kk, int K, int rb) {
  const int b = r / rb, rr = r % rb, ks = kk >> 4, k16 = kk & 15;
  return ((size_t)b * (size_t)(K >> 4) + (size_t)ks) * (size_t)(rb * 32) + (size_t)(rr >> 3) * 256 +
         (size_t)(k16 >> 3) * 128 + (size_t)(rr & 7) * 16 + (size_t)(k16 & 7) * 2;
}

namespace {

// ---------------------------------------------------------------------------
// Tensor-core inference layer.
struct MlpTcArgs {
  const unsigned char *A;   // activations, tiled (row blocks of 128)
  const unsigned char *B;   // weights [N x K], tiled (row blocks of 256)
  const float *bias;        // [N]
  int K;                    // multiple of 16
  int N;                    // outputs (real)
  int npad;                 // N rounded up to 16
  int rows;                 // valid rows
  unsigned char *out_t;     // EPI 0: next layer's tiled input, K = kout
  int kout;
  float *out;               // EPI 1: FP32 rows, leading dimension ldo
  int ldo;
  int *status;              // bit 16: a wait ran out
};

struct __align__(8) MlpTcSmem {
  unsigned long long full[TC_NS], empty[TC_NS], done;
  uint32_t tmem;
  int fault;
};

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Instruction descriptor, kind::f16: D f32, A/B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Roles: thread 0 keeps the stages filled (bulk copies, transaction counts),
// thread 32 issues the MMAs and frees stages with tcgen05.commit; then all 4
// warps read the accumulator (warp w: TMEM lanes 32w..32w+31 = rows).
template <int EPI>
__global__ void __launch_bounds__(TC_THREADS) k_mlp_tc(MlpTcArgs a) {
  extern __shared__ __align__(1024) unsigned char dsm[];
  __shared__ MlpTcSmem S;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int rb = blockIdx.x, nt = blockIdx.y;
  const int n0 = nt * RB_W;
  const int NT = min(RB_W, a.npad - n0);              // multiple of 16
  const int ksteps = a.K >> 4;
  const uint32_t abytes = RB_ACT * 32, bbytes = (uint32_t)NT * 32;
  const uint32_t stage = RB_ACT * 32 + RB_W * 32;     // 12 KB
  if (wid == 0) tc::tmem_alloc(&S.tmem, 256);
  if (tid == 0) {
    for (int s = 0; s < TC_NS; s++) {
      tc::mbar_init(reinterpret_cast<uint64_t *>(&S.full[s]), 1);
      tc::mbar_init(reinterpret_cast<uint64_t *>(&S.empty[s]), 1);
    }
    tc::mbar_init(reinterpret_cast<uint64_t *>(&S.done), 1);
    S.fault = 0;
    tc::mbar_fence_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = S.tmem;
  const unsigned char *Ablk = a.A + (size_t)rb * ksteps * (RB_ACT * 32);
  const unsigned char *Bblk = a.B + (size_t)nt * ksteps * (RB_W * 32);
  if (tid == 0) {
    // producer
    for (int q = 0; q < ksteps; q++) {
      const int s = q % TC_NS;
      if (q >= TC_NS &&
          !tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.empty[s]), (uint32_t)(((q / TC_NS) - 1) & 1))) {
        S.fault = 1;
        break;
      }
      unsigned char *st = dsm + (size_t)s * stage;
      uint64_t *fb = reinterpret_cast<uint64_t *>(&S.full[s]);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(fb)),
                   "r"(abytes + bbytes) : "memory");
      tc::bulk_copy_g2s(st, Ablk + (size_t)q * (RB_ACT * 32), abytes, fb);
      tc::bulk_copy_g2s(st + RB_ACT * 32, Bblk + (size_t)q * (RB_W * 32), bbytes, fb);
    }
  } else if (tid == 32) {
    // MMA issue
    const uint32_t idesc = idesc_bf16(128, NT);
    int q = 0;
    for (; q < ksteps; q++) {
      const int s = q % TC_NS;
      if (!tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.full[s]), (uint32_t)((q / TC_NS) & 1))) {
        S.fault = 1;
        break;
      }
      tc::fence_after();
      const uint32_t sa = tc::smem_u32(dsm + (size_t)s * stage);
      const uint64_t ad = tc::smem_desc(sa, 128, 256);
      const uint64_t bd = tc::smem_desc(sa + RB_ACT * 32, 128, 256);
      mma_bf16(tmem, ad, bd, idesc, q > 0 ? 1u : 0u);
      tc::commit(reinterpret_cast<uint64_t *>(&S.empty[s]));
    }
    tc::commit(reinterpret_cast<uint64_t *>(&S.done));
    if (q < ksteps) {
      // a wait ran out: let the copies already issued land before exit
      for (int r = q; r < ksteps && r < q + TC_NS; r++)
        tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.full[r % TC_NS]), (uint32_t)((r / TC_NS) & 1), 1000000L);
    }
  }
  __syncwarp();
  const bool ok = tc::mbar_wait(reinterpret_cast<uint64_t *>(&S.done), 0);
  tc::fence_after();
  if (!ok || S.fault) {
    if (tid == 0) atomicOr(a.status, 16);
  } else {
    // epilogue: row r = 32 wid + lane of the block, 16 columns at a time
    const int row = rb * RB_ACT + wid * 32 + lane;
    for (int c0 = 0; c0 < NT; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)c0, v);
      const int n = n0 + c0;
      if (EPI == 0) {
        __align__(16) __nv_bfloat16 hb[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const float z = v[j] + (n + j < a.N ? a.bias[n + j] : 0.0f);
          hb[j] = __float2bfloat16_rn(n + j < a.N ? gelu(z) : 0.0f);
        }
        unsigned char *dst = a.out_t + mlp_tile_off(row, n, a.kout, RB_ACT);
        reinterpret_cast<uint4 *>(dst)[0] = reinterpret_cast<const uint4 *>(hb)[0];
        *reinterpret_cast<uint4 *>(dst + 128) = reinterpret_cast<const uint4 *>(hb)[1];
      } else if (row < a.rows) {
        float *dst = a.out + (size_t)row * a.ldo + n;
        const float *bn = a.bias + n;
        if (n + 16 <= a.N && ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(bn)) & 15) == 0) {
          // 16-byte stores of the row's 16 outputs
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const float4 b = __ldg(reinterpret_cast<const float4 *>(bn) + q);
            reinterpret_cast<float4 *>(dst)[q] =
                make_float4(v[4 * q] + b.x, v[4 * q + 1] + b.y, v[4 * q + 2] + b.z, v[4 * q + 3] + b.w);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; j++)
            if (n + j < a.N) dst[j] = v[j] + bn[j];
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (wid == 0) tc::tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------------------
// CUDA-core GEMM for training: C(m, n) = sum_k A(m, k) B(k, n) with
// A(m, k) = A[m sam + k sak], B(k, n) = B[k sbk + n sbn]; 64 x 64 tiles, 16-wide
// K slices, 256 threads, 4 x 4 outputs per thread, FP32 accumulation in k order.
struct GemmArgs {
  const float *A, *B;
  long long sam, sak, sbk, sbn;
  int M, N, K;
  float *C;            // [M][ldc]
  int ldc;
  const float *bias;   // EPI 1, 3
  float *H;            // EPI 1: BF16-rounded GELU output [M][ldc]
  const float *Zp;     // EPI 2: pre-activation [M][ldc]
};

// EPI 0: C = acc; 1: C = acc + bias (pre-activation), H = bf16(gelu(C));
// 2: C = acc * gelu'(Zp); 3: C = acc + bias
template <int EPI>
__global__ void __launch_bounds__(256) k_mlp_gemm(GemmArgs g) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
  for (int k0 = 0; k0 < g.K; k0 += 16) {
    for (int t = threadIdx.x; t < 64 * 16; t += 256) {
      const int mm = t / 16, kk = t % 16;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < g.M && k < g.K) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : 0.0f;
      const int nn = t % 64, kb = t / 64;
      const int n = n0 + nn, k2 = k0 + kb;
      Bs[kb][nn] = (n < g.N && k2 < g.K) ? g.B[(long long)k2 * g.sbk + (long long)n * g.sbn] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; i++) av[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m >= g.M || n >= g.N) continue;
      const size_t o = (size_t)m * g.ldc + n;
      float v = acc[i][j];
      if (EPI == 1) {
        v += g.bias[n];
        g.C[o] = v;
        g.H[o] = bf16r(gelu(v));
      } else if (EPI == 2) {
        g.C[o] = v * gelu_grad(g.Zp[o]);
      } else if (EPI == 3) {
        g.C[o] = v + g.bias[n];
      } else {
        g.C[o] = v;
      }
    }
}

// weighted mean squared error: dY = 2 w (Y - T) / (rows * n), per-block
// partial sums of w (Y - T)^2 (w: per-output weights, 1 when null)
__global__ void k_mlp_loss(const float *Y, const float *T, float *dY, int rows, int n, const float *wout,
                           float *partial) {
  __shared__ float red[256];
  float s = 0.0f;
  const long long total = (long long)rows * n;
  const float sc = 2.0f / (float)total;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    const float w = wout ? wout[i % n] : 1.0f;
    dY[i] = sc * w * d;
    s += w * d * d;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// column sums of a [rows][n] matrix (bias gradients), row order fixed
__global__ void k_mlp_colsum(const float *D, int rows, int n, float *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  float s = 0.0f;
  for (int r = 0; r < rows; r++) s += D[(size_t)r * n + c];
  out[c] = s;
}

// Adam on FP32 masters, then the BF16-rounded copy used by the forward
__global__ void k_mlp_adam(float *w, float *wq, const float *g, float *m, float *v, long long n, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wq[i] = bf16r(wi);
  }
}

__global__ void k_mlp_round(const float *w, float *wq, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    wq[i] = bf16r(w[i]);
}

// FP32 [rows][K] matrix -> BF16 tiled blocks (row blocks of rb; rows up to
// nrows_pad and columns up to Kpad are zero-filled)
__global__ void k_mlp_tile(const float *src, int rows, int K, int ld, int nrows_pad, int Kpad, int rb,
                           unsigned char *dst) {
  const long long total = (long long)nrows_pad * (Kpad >> 3);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / (Kpad >> 3)), k8 = (int)(t % (Kpad >> 3)) * 8;
    __align__(16) __nv_bfloat16 v[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int kk = k8 + j;
      v[j] = __float2bfloat16_rn((r < rows && kk < K) ? src[(size_t)r * ld + kk] : 0.0f);
    }
    *reinterpret_cast<uint4 *>(dst + mlp_tile_off(r, k8, Kpad, rb)) = *reinterpret_cast<const uint4 *>(v);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side

size_t mlp_param_count(const MlpShape &s) {
  return (size_t)s.H * s.din + s.H + (size_t)s.H * s.H + s.H + (size_t)s.dout * s.H + s.dout;
}

void mlp_param_offsets(const MlpShape &s, size_t off[6]) {
  off[0] = 0;                                 // W1 [H][din]
  off[1] = off[0] + (size_t)s.H * s.din;      // b1
  off[2] = off[1] + s.H;                      // W2 [H][H]
  off[3] = off[2] + (size_t)s.H * s.H;        // b2
  off[4] = off[3] + s.H;                      // W3 [dout][H]
  off[5] = off[4] + (size_t)s.dout * s.H;     // b3
}

size_t mlp_tiled_weight_bytes(const MlpShape &s) {
  const size_t w1 = (size_t)((s.H + RB_W - 1) / RB_W) * RB_W * s.k1 * 2;
  const size_t w2 = (size_t)((s.H + RB_W - 1) / RB_W) * RB_W * s.H * 2;
  const size_t w3 = (size_t)((s.dout + RB_W - 1) / RB_W) * RB_W * s.H * 2;
  return w1 + w2 + w3;
}

static int grid_for(long long n) { return (int)std::min<long long>(4096, std::max<long long>(1, (n + 255) / 256)); }

// BF16 tiled copies of the three weight matrices (the inference operands)
cudaError_t mlp_tile_weights(cudaStream_t st, const MlpShape &s, const float *wq, unsigned char *tiled) {
  size_t off[6];
  mlp_param_offsets(s, off);
  const int hp = (s.H + RB_W - 1) / RB_W * RB_W, dp = (s.dout + RB_W - 1) / RB_W * RB_W;
  unsigned char *t1 = tiled, *t2 = t1 + (size_t)hp * s.k1 * 2, *t3 = t2 + (size_t)hp * s.H * 2;
  k_mlp_tile<<<grid_for((long long)hp * s.k1 / 8), 256, 0, st>>>(wq + off[0], s.H, s.din, s.din, hp, s.k1, RB_W, t1);
  k_mlp_tile<<<grid_for((long long)hp * s.H / 8), 256, 0, st>>>(wq + off[2], s.H, s.H, s.H, hp, s.H, RB_W, t2);
  k_mlp_tile<<<grid_for((long long)dp * s.H / 8), 256, 0, st>>>(wq + off[4], s.dout, s.H, s.H, dp, s.H, RB_W, t3);
  return cudaGetLastError();
}

// FP32 input rows [rows][din] -> BF16 tiled activations (rows padded to 128)
cudaError_t mlp_tile_input(cudaStream_t st, const MlpShape &s, const float *x, int rows, int ld, unsigned char *tiled) {
  const int rp = (rows + RB_ACT - 1) / RB_ACT * RB_ACT;
  k_mlp_tile<<<grid_for((long long)rp * s.k1 / 8), 256, 0, st>>>(x, rows, s.din, ld, rp, s.k1, RB_ACT, tiled);
  return cudaGetLastError();
}

size_t mlp_act_bytes(const MlpShape &s, int rows) {
  const size_t rp = (size_t)(rows + RB_ACT - 1) / RB_ACT * RB_ACT;
  return rp * (size_t)std::max(s.k1, s.H) * 2;
}

template <int EPI>
static cudaError_t launch_tc_layer(cudaStream_t st, const MlpTcArgs &a, int rows, int *launches) {
  const size_t smem = (size_t)TC_NS * (RB_ACT * 32 + RB_W * 32);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_tc<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((rows + RB_ACT - 1) / RB_ACT, (a.npad + RB_W - 1) / RB_W);
  k_mlp_tc<EPI><<<grid, TC_THREADS, smem, st>>>(a);
  (*launches)++;
  return cudaGetLastError();
}

// Inference on the tensor cores: x (tiled, rows padded to 128) -> y [rows][ldy]
// FP32.  h1, h2: tiled scratch of mlp_act_bytes each.
cudaError_t mlp_forward_tc(cudaStream_t st, const MlpShape &s, const unsigned char *wtiled, const float *bias_base,
                           const unsigned char *x, int rows, unsigned char *h1, unsigned char *h2, float *y, int ldy,
                           int *status, int *launches) {
  if (rows <= 0) return cudaSuccess;
  size_t off[6];
  mlp_param_offsets(s, off);
  const int hp = (s.H + RB_W - 1) / RB_W * RB_W;
  const unsigned char *t1 = wtiled, *t2 = t1 + (size_t)hp * s.k1 * 2, *t3 = t2 + (size_t)hp * s.H * 2;
  MlpTcArgs a;
  a.rows = rows;
  a.status = status;
  a.out = nullptr;
  a.ldo = 0;
  // layer 1
  a.A = x; a.B = t1; a.bias = bias_base + off[1]; a.K = s.k1; a.N = s.H; a.npad = s.H;
  a.out_t = h1; a.kout = s.H;
  cudaError_t e = launch_tc_layer<0>(st, a, rows, launches);
  if (e != cudaSuccess) return e;
  // layer 2
  a.A = h1; a.B = t2; a.bias = bias_base + off[3]; a.K = s.H; a.N = s.H; a.npad = s.H;
  a.out_t = h2; a.kout = s.H;
  if ((e = launch_tc_layer<0>(st, a, rows, launches)) != cudaSuccess) return e;
  // layer 3
  a.A = h2; a.B = t3; a.bias = bias_base + off[5]; a.K = s.H; a.N = s.dout; a.npad = (s.dout + 15) & ~15;
  a.out_t = nullptr; a.kout = 0; a.out = y; a.ldo = ldy;
  return launch_tc_layer<1>(st, a, rows, launches);
}

template <int EPI>
static cudaError_t gemm(cudaStream_t st, const GemmArgs &g) {
  dim3 grid((g.N + 63) / 64, (g.M + 63) / 64);
  k_mlp_gemm<EPI><<<grid, 256, 0, st>>>(g);
  return cudaGetLastError();
}

static GemmArgs gargs(const float *A, long long sam, long long sak, const float *B, long long sbk, long long sbn, int M,
                      int N, int K, float *C, int ldc) {
  GemmArgs g;
  g.A = A; g.sam = sam; g.sak = sak;
  g.B = B; g.sbk = sbk; g.sbn = sbn;
  g.M = M; g.N = N; g.K = K;
  g.C = C; g.ldc = ldc;
  g.bias = nullptr; g.H = nullptr; g.Zp = nullptr;
  return g;
}

size_t mlp_train_scratch_floats(const MlpShape &s, int rows) {
  // Z1, H1, Z2, H2, Y, dY, dZ2 (reused for dH2), dZ1, loss partials
  return (size_t)rows * (4 * s.H + 2 * s.dout + 2 * s.H) + 4096;
}

// Forward on the CUDA cores (BF16-rounded weights wq, input x already
// BF16-rounded): y [rows][dout]; scratch of mlp_train_scratch_floats.
cudaError_t mlp_forward_simt(cudaStream_t st, const MlpShape &s, const float *wq, const float *x, int rows, float *y,
                             float *scr) {
  size_t off[6];
  mlp_param_offsets(s, off);
  float *Z1 = scr, *H1 = Z1 + (size_t)rows * s.H, *Z2 = H1 + (size_t)rows * s.H, *H2 = Z2 + (size_t)rows * s.H;
  GemmArgs g = gargs(x, s.din, 1, wq + off[0], 1, s.din, rows, s.H, s.din, Z1, s.H);
  g.bias = wq + off[1];
  g.H = H1;
  cudaError_t e = gemm<1>(st, g);
  if (e != cudaSuccess) return e;
  g = gargs(H1, s.H, 1, wq + off[2], 1, s.H, rows, s.H, s.H, Z2, s.H);
  g.bias = wq + off[3];
  g.H = H2;
  if ((e = gemm<1>(st, g)) != cudaSuccess) return e;
  g = gargs(H2, s.H, 1, wq + off[4], 1, s.H, rows, s.dout, s.H, y, s.dout);
  g.bias = wq + off[5];
  return gemm<3>(st, g);
}

// One forward + backward over a batch: grads (FP32, the parameter layout) of
// the mean squared error between the output and t (each output weighted by
// wout, or 1); the loss partial sums of
// k_mlp_loss are left at mlp_loss_parts (their count in *nparts).  All
// parameters (wq) and the input x are BF16-rounded; hidden activations are
// rounded to BF16 after GELU; accumulation is FP32.
cudaError_t mlp_grad(cudaStream_t st, const MlpShape &s, const float *wq, const float *x, const float *t, int rows,
                     float *grad, float *scr, int *nparts, const float *wout) {
  size_t off[6];
  mlp_param_offsets(s, off);
  float *Z1 = scr, *H1 = Z1 + (size_t)rows * s.H, *Z2 = H1 + (size_t)rows * s.H, *H2 = Z2 + (size_t)rows * s.H;
  float *Y = H2 + (size_t)rows * s.H, *dY = Y + (size_t)rows * s.dout, *dZ2 = dY + (size_t)rows * s.dout;
  float *dZ1 = dZ2 + (size_t)rows * s.H, *parts = dZ1 + (size_t)rows * s.H;
  cudaError_t e = mlp_forward_simt(st, s, wq, x, rows, Y, scr);
  if (e != cudaSuccess) return e;
  const int nb = std::min(1024, std::max(1, (int)(((long long)rows * s.dout + 255) / 256)));
  k_mlp_loss<<<nb, 256, 0, st>>>(Y, t, dY, rows, s.dout, wout, parts);
  *nparts = nb;
  // layer 3: dW3 = dY^T H2, db3 = colsum dY, dZ2 = (dY W3) * gelu'(Z2)
  if ((e = gemm<0>(st, gargs(dY, 1, s.dout, H2, s.H, 1, s.dout, s.H, rows, grad + off[4], s.H))) != cudaSuccess) return e;
  k_mlp_colsum<<<(s.dout + 255) / 256, 256, 0, st>>>(dY, rows, s.dout, grad + off[5]);
  GemmArgs g = gargs(dY, s.dout, 1, wq + off[4], s.H, 1, rows, s.H, s.dout, dZ2, s.H);
  g.Zp = Z2;
  if ((e = gemm<2>(st, g)) != cudaSuccess) return e;
  // layer 2
  if ((e = gemm<0>(st, gargs(dZ2, 1, s.H, H1, s.H, 1, s.H, s.H, rows, grad + off[2], s.H))) != cudaSuccess) return e;
  k_mlp_colsum<<<(s.H + 255) / 256, 256, 0, st>>>(dZ2, rows, s.H, grad + off[3]);
  g = gargs(dZ2, s.H, 1, wq + off[2], s.H, 1, rows, s.H, s.H, dZ1, s.H);
  g.Zp = Z1;
  if ((e = gemm<2>(st, g)) != cudaSuccess) return e;
  // layer 1
  if ((e = gemm<0>(st, gargs(dZ1, 1, s.H, x, s.din, 1, s.H, s.din, rows, grad + off[0], s.din))) != cudaSuccess)
    return e;
  k_mlp_colsum<<<(s.H + 255) / 256, 256, 0, st>>>(dZ1, rows, s.H, grad + off[1]);
  return cudaGetLastError();
}

float *mlp_loss_parts(const MlpShape &s, float *scr, int rows) {
  return scr + (size_t)rows * (4 * s.H + 2 * s.dout + 2 * s.H);
}

cudaError_t mlp_adam(cudaStream_t st, long long n, float *w, float *wq, const float *g, float *m, float *v, float lr,
                     int step) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_mlp_adam<<<grid_for(n), 256, 0, st>>>(w, wq, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
  return cudaGetLastError();
}

cudaError_t mlp_round(cudaStream_t st, long long n, const float *w, float *wq) {
  k_mlp_round<<<grid_for(n), 256, 0, st>>>(w, wq, n);
  return cudaGetLastError();
}

}  // namespace lgpu

namespace lgpu {
namespace {
__global__ void k_mlp_acc(const float *parts, int n, float *acc) {
  __shared__ float red[256];
  float s = 0.0f;
  for (int i = threadIdx.x; i < n; i += 256) s += parts[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) acc[0] += red[0];
}
}  // namespace

// acc[0] += sum of the loss partial sums (one block, fixed order)
cudaError_t mlp_loss_accumulate(cudaStream_t st, const float *parts, int n, float *acc) {
  k_mlp_acc<<<1, 256, 0, st>>>(parts, n, acc);
  return cudaGetLastError();
}
}  // namespace lgpu
