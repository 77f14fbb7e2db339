// The learned SPR ranking: a BF16 multilayer perceptron 64 -> 256 -> 256 ->
// 256 -> 1 (GELU) with FP32 accumulation, trained by AdamW on (move, dlnL)
// pairs.  phylocaml has no learned component; this is the proposal model that
// orders SPR moves (lib/treeNeighborhoods.ml:27-75 leaves the search itself
// as a TODO).
//
// Every layer runs through one tensor-core GEMM kernel, mlp_gemm_kernel:
// C[M x N] = A[M x K] B[N x K]^T with A, B in BF16 (K contiguous), D in TMEM
// (FP32, 128 lanes x N columns), one tcgen05.mma.kind::f16 (M = 128, N <= 256,
// K = 16) per 32 bytes of K, issued by one thread, operands staged into
// shared memory in the K-major no-swizzle core-matrix layout (8 rows x 16
// bytes).  The epilogue (thread = row, tcgen05.ld) is fused per use:
//   EPI_F32    store C (weight gradients)
//   EPI_GELU   z = C + b, h = gelu(z): store z, bf16 h and bf16 h^T, and for
//              the last hidden layer the output y = h . w4 + b4
//   EPI_DGELU  dz = C * gelu'(z): store bf16 dz and dz^T (back-propagation)
// Forward:  h1 = gelu(W1 xn + b1), h2 = gelu(W2 h1 + b2), h3 = gelu(W3 h2 + b3),
//           y = w4 . h3 + b4, xn = (x - mu) / sd in BF16.
// Backward: dz3 = dy w4 * gelu'(z3); dW3 = dz3^T h2; dz2 = (dz3 W3) * gelu'(z2);
//           dW2 = dz2^T h1; dz1 = (dz2 W2) * gelu'(z1); dW1 = dz1^T xn;
//           db_l = sum over rows of dz_l; dw4 = dy^T h3; db4 = sum dy.
// The transposed products use the bf16 copies W^T and h^T written by the
// previous step, so every GEMM reads K-contiguous rows.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "pgpu_internal.cuh"

namespace {

constexpr int IN = 64, HID = 256;
constexpr int GM = 128;           // rows per CTA tile
constexpr int GK = 64;            // K per staged chunk
constexpr int GEMM_SMEM = 96 * 1024;   // staging uses 48 KB; the rest caps residency at 2 CTAs/SM
constexpr uint32_t TMEM_COLS = 256;

// parameter offsets in the flat FP32 vector
constexpr size_t OFF_W1 = 0, OFF_B1 = OFF_W1 + (size_t)HID * IN, OFF_W2 = OFF_B1 + HID,
                 OFF_B2 = OFF_W2 + (size_t)HID * HID, OFF_W3 = OFF_B2 + HID,
                 OFF_B3 = OFF_W3 + (size_t)HID * HID, OFF_W4 = OFF_B3 + HID, OFF_B4 = OFF_W4 + HID,
                 N_PARAMS = OFF_B4 + 1;

enum { EPI_F32 = 0, EPI_GELU = 1, EPI_DGELU = 2 };

__device__ __forceinline__ uint32_t su32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t smem_desc(const void *base, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((su32(base) >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ void tmem_ld16(uint32_t ta, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(ta));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float dgelu(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

struct GemmArgs {
  const __nv_bfloat16 *A, *B;   // [M][lda], [N][ldb]
  int M, N, K, lda, ldb;
  // epilogue
  float *C;                     // EPI_F32: [M][ldc]
  int ldc;
  const float *bias;            // EPI_GELU: [N]
  float *Z;                     // EPI_GELU out / EPI_DGELU in: [M][ldz] (may be null for GELU)
  int ldz;
  __nv_bfloat16 *H, *HT;        // out [M][ldh], [N][ldt] (either may be null)
  int ldh, ldt;
  const float *w4;              // EPI_GELU: fused output layer (or null)
  float b4;
  float *y;                     // [M]
  int *flag;
};

template <int EPI>
__global__ void __launch_bounds__(128) mlp_gemm_kernel(const GemmArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tbase;
  constexpr uint32_t LBO = 128, SBO = (GK / 8) * 128;   // 1024 bytes per 8-row group
  unsigned char *sA = smem;                             // GM/8 * SBO = 16 KB
  unsigned char *sB = smem + (GM / 8) * SBO;            // up to 256/8 * SBO = 32 KB
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row0 = blockIdx.x * GM;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tbase)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&mbar, 1);
    fence_mbarrier_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tbase;
  uint32_t idesc = 0;
  idesc |= 1u << 4;                          // D f32
  idesc |= 1u << 7;                          // A bf16
  idesc |= 1u << 10;                         // B bf16
  idesc |= (uint32_t)(a.N >> 3) << 17;
  idesc |= (uint32_t)(GM >> 4) << 24;
  bool ok = true;
  const int n_chunks = a.K / GK;
  for (int ch = 0; ch < n_chunks; ++ch) {
    const int k0 = ch * GK;
    // stage: one 16-byte global load -> one core-matrix row
    for (int i = tid; i < GM * (GK / 8); i += 128) {
      const int r = i >> 3, kv = i & 7;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (row0 + r < a.M)
        v = *reinterpret_cast<const uint4 *>(a.A + (size_t)(row0 + r) * a.lda + k0 + kv * 8);
      *reinterpret_cast<uint4 *>(sA + (r >> 3) * SBO + kv * LBO + (r & 7) * 16) = v;
    }
    for (int i = tid; i < a.N * (GK / 8); i += 128) {
      const int r = i >> 3, kv = i & 7;
      const uint4 v = *reinterpret_cast<const uint4 *>(a.B + (size_t)r * a.ldb + k0 + kv * 8);
      *reinterpret_cast<uint4 *>(sB + (r >> 3) * SBO + kv * LBO + (r & 7) * 16) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < GK / 16; ++ks) {
        const uint64_t ad = smem_desc(sA + (size_t)ks * 2 * LBO, LBO, SBO);
        const uint64_t bd = smem_desc(sB + (size_t)ks * 2 * LBO, LBO, SBO);
        const uint32_t acc = (ch > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       su32(&mbar))
                   : "memory");
    }
    // the staging buffers are reused only after the MMAs have read them
    ok = __all_sync(0xffffffffu, mbar_wait_bounded(&mbar, ch & 1, a.flag)) && ok;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (!__syncthreads_and(ok)) break;
  }

  // epilogue: thread = row
  const int row = row0 + tid;
  const bool live = row < a.M && ok;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);
  float ysum = 0.0f;
  for (int c0 = 0; c0 < a.N; c0 += 16) {
    float v[16];
    tmem_ld16(lane_base + (uint32_t)c0, v);
    if (!live) continue;
    if (EPI == EPI_F32) {
#pragma unroll
      for (int j = 0; j < 16; ++j) a.C[(size_t)row * a.ldc + c0 + j] = v[j];
    } else if (EPI == EPI_GELU) {
      __align__(16) __nv_bfloat16 hb[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float z = v[j] + a.bias[c0 + j];
        if (a.Z) a.Z[(size_t)row * a.ldz + c0 + j] = z;
        hb[j] = __float2bfloat16_rn(gelu(z));
        if (a.w4) ysum = fmaf(__bfloat162float(hb[j]), a.w4[c0 + j], ysum);
        if (a.HT) a.HT[(size_t)(c0 + j) * a.ldt + row] = hb[j];
      }
      if (a.H) {
        uint4 *dst = reinterpret_cast<uint4 *>(a.H + (size_t)row * a.ldh + c0);
        dst[0] = reinterpret_cast<const uint4 *>(hb)[0];
        dst[1] = reinterpret_cast<const uint4 *>(hb)[1];
      }
    } else {   // EPI_DGELU
      __align__(16) __nv_bfloat16 db[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float z = a.Z[(size_t)row * a.ldz + c0 + j];
        db[j] = __float2bfloat16_rn(v[j] * dgelu(z));
        if (a.HT) a.HT[(size_t)(c0 + j) * a.ldt + row] = db[j];
      }
      if (a.H) {
        uint4 *dst = reinterpret_cast<uint4 *>(a.H + (size_t)row * a.ldh + c0);
        dst[0] = reinterpret_cast<const uint4 *>(db)[0];
        dst[1] = reinterpret_cast<const uint4 *>(db)[1];
      }
    }
  }
  if (EPI == EPI_GELU && a.w4 && live) a.y[row] = ysum + a.b4;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// xn = bf16((x - mu) * inv_sd), rows >= n zero; optional transpose [64][ldt]
__global__ void mlp_norm_kernel(const float *X, size_t n, size_t n_pad, const float *mu,
                                const float *inv_sd, __nv_bfloat16 *Xn, __nv_bfloat16 *XnT, size_t ldt) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad * IN) return;
  const size_t r = i / IN;
  const int k = (int)(i % IN);
  const float v = r < n ? (X[i] - mu[k]) * inv_sd[k] : 0.0f;
  const __nv_bfloat16 b = __float2bfloat16_rn(v);
  Xn[i] = b;
  if (XnT) XnT[(size_t)k * ldt + r] = b;
}

// column mean and 1/sd of X [n][64] (FP64 sums; sd floored at 1e-6)
__global__ void __launch_bounds__(256) mlp_colstats_kernel(const float *X, size_t n, float *mu,
                                                           float *inv_sd) {
  __shared__ double red[2][8];
  const int k = blockIdx.x;
  double s = 0.0, s2 = 0.0;
  for (size_t r = threadIdx.x; r < n; r += 256) {
    const double v = X[r * IN + k];
    s += v;
    s2 += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s;
    red[1][threadIdx.x >> 5] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0, S2 = 0;
    for (int w = 0; w < 8; ++w) {
      S += red[0][w];
      S2 += red[1][w];
    }
    const double m = n ? S / (double)n : 0.0;
    const double var = n ? fmax(S2 / (double)n - m * m, 0.0) : 1.0;
    mu[k] = (float)m;
    inv_sd[k] = (float)(1.0 / fmax(sqrt(var), 1e-6));
  }
}

// dy = 2 sw (y - t) / sum sw, the weighted squared loss, and db4 = sum dy
// (one CTA; fixed summation order)
__global__ void __launch_bounds__(1024) mlp_loss_kernel(const float *y, const float *t, const float *sw,
                                                        int n, float *dy, float *loss, float *db4) {
  __shared__ double red[3][32];
  double s0 = 0, s1 = 0;
  for (int i = threadIdx.x; i < n; i += 1024) {
    const double w = sw ? sw[i] : 1.0;
    const double e = (double)y[i] - (double)t[i];
    s0 += w;
    s1 += w * e * e;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s0;
    red[1][threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  double W = 0, Ls = 0;
  for (int w = 0; w < 32; ++w) {
    W += red[0][w];
    Ls += red[1][w];
  }
  const double inv = W > 0 ? 1.0 / W : 0.0;
  double sd = 0;
  for (int i = threadIdx.x; i < n; i += 1024) {
    const double w = sw ? sw[i] : 1.0;
    const float g = (float)(2.0 * w * ((double)y[i] - (double)t[i]) * inv);
    dy[i] = g;
    sd += g;
  }
  for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[2][threadIdx.x >> 5] = sd;
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0;
    for (int w = 0; w < 32; ++w) S += red[2][w];
    *db4 = (float)S;
    *loss = (float)(Ls * inv);
  }
}

// dz3 = dy w4 gelu'(z3), rows >= n zero: bf16 [n_pad][256] and [256][ldt]
__global__ void mlp_out_bwd_kernel(const float *dy, const float *w4, const float *Z3, int n, int n_pad,
                                   __nv_bfloat16 *DZ, __nv_bfloat16 *DZT, int ldt) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n_pad * HID) return;
  const int r = (int)(i / HID), c = (int)(i % HID);
  const float g = r < n ? dy[r] * w4[c] * dgelu(Z3[i]) : 0.0f;
  const __nv_bfloat16 b = __float2bfloat16_rn(g);
  DZ[i] = b;
  DZT[(size_t)c * ldt + r] = b;
}

// out[j] = sum_r T[j][r] * (s ? s[r] : 1) over r < n (one warp per j)
__global__ void mlp_rowsum_kernel(const __nv_bfloat16 *T, int ld, int n, const float *s, int rows,
                                  float *out) {
  const int j = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= rows) return;
  float acc = 0.0f;
  for (int r = lane; r < n; r += 32) acc = fmaf(__bfloat162float(T[(size_t)j * ld + r]), s ? s[r] : 1.0f, acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[j] = acc;
}

struct AdamArgs {
  float *p, *m, *v;
  const float *g;
  size_t n;
  float lr, b1, b2, eps, wd, c1, c2;   // c1 = 1 - b1^t, c2 = 1 - b2^t
};

// decoupled weight decay on the matrices only (biases and the output bias
// are not decayed)
__global__ void mlp_adamw_kernel(const AdamArgs a) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float g = a.g[i];
  const float m = a.b1 * a.m[i] + (1.0f - a.b1) * g;
  const float v = a.b2 * a.v[i] + (1.0f - a.b2) * g * g;
  a.m[i] = m;
  a.v[i] = v;
  const bool decay = (i < OFF_B1) || (i >= OFF_W2 && i < OFF_B2) || (i >= OFF_W3 && i < OFF_B3) ||
                     (i >= OFF_W4 && i < OFF_B4);
  float p = a.p[i];
  if (decay) p -= a.lr * a.wd * p;
  p -= a.lr * (m / a.c1) / (sqrtf(v / a.c2) + a.eps);
  a.p[i] = p;
}

// bf16 weights W [out][in] and W^T [in][out] from the FP32 master copy
__global__ void mlp_pack_kernel(const float *p, __nv_bfloat16 *W1, __nv_bfloat16 *W1T, __nv_bfloat16 *W2,
                                __nv_bfloat16 *W2T, __nv_bfloat16 *W3, __nv_bfloat16 *W3T) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (size_t)HID * IN) {
    const int o = (int)(i / IN), k = (int)(i % IN);
    const __nv_bfloat16 b = __float2bfloat16_rn(p[OFF_W1 + i]);
    W1[i] = b;
    W1T[(size_t)k * HID + o] = b;
  }
  if (i < (size_t)HID * HID) {
    const int o = (int)(i / HID), k = (int)(i % HID);
    const __nv_bfloat16 b2 = __float2bfloat16_rn(p[OFF_W2 + i]);
    const __nv_bfloat16 b3 = __float2bfloat16_rn(p[OFF_W3 + i]);
    W2[i] = b2;
    W2T[(size_t)k * HID + o] = b2;
    W3[i] = b3;
    W3T[(size_t)k * HID + o] = b3;
  }
}

size_t pad_to(size_t x, size_t m) { return (x + m - 1) / m * m; }

}  // namespace

struct pgpu_mlp {
  pgpu_ctx *ctx = nullptr;
  int max_batch = 0, bpad = 0;   // bpad: rows padded to 128
  long long step = 0;
  float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;   // flat [N_PARAMS]
  __nv_bfloat16 *W1 = nullptr, *W1T = nullptr, *W2 = nullptr, *W2T = nullptr, *W3 = nullptr, *W3T = nullptr;
  float *mu = nullptr, *inv_sd = nullptr, *scal = nullptr;   // scal: loss, db4
  // training scratch (bpad rows)
  __nv_bfloat16 *Xn = nullptr, *XnT = nullptr, *H[3] = {}, *HT[3] = {}, *DZ = nullptr, *DZT = nullptr,
                *DZ2 = nullptr, *DZ2T = nullptr;
  float *Z[3] = {}, *y = nullptr, *dy = nullptr;
  // inference scratch (grown on demand)
  __nv_bfloat16 *iXn = nullptr, *iH0 = nullptr, *iH1 = nullptr;
  size_t icap = 0;
  std::vector<void *> owned;
};

namespace {

pgpu_status malloc_own(pgpu_mlp *n, size_t bytes, void **p) {
  PGPU_CUDA(n->ctx, cudaMalloc(p, std::max<size_t>(bytes, 16)));
  n->owned.push_back(*p);
  return PGPU_OK;
}
template <typename T>
pgpu_status mo(pgpu_mlp *n, size_t count, T **p) {
  void *v;
  PGPU_TRY(malloc_own(n, count * sizeof(T), &v));
  *p = static_cast<T *>(v);
  return PGPU_OK;
}

template <int EPI>
pgpu_status gemm(pgpu_mlp *nn, const GemmArgs &a) {
  if (a.K % GK || a.N % 16 || a.N < 16 || a.N > 256 || a.lda % 8 || a.ldb % 8)
    return pgpu_set_err(nn->ctx, PGPU_ERR_ARG, "mlp: unsupported GEMM shape M=%d N=%d K=%d", a.M, a.N, a.K);
  PGPU_CUDA(nn->ctx, cudaFuncSetAttribute(mlp_gemm_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          GEMM_SMEM));
  mlp_gemm_kernel<EPI><<<(unsigned)((a.M + GM - 1) / GM), 128, GEMM_SMEM, nn->ctx->stream>>>(a);
  return pgpu_after_launch(nn->ctx, "mlp_gemm_kernel");
}

GemmArgs base_args(pgpu_mlp *nn) {
  GemmArgs a{};
  a.flag = nn->ctx->d_flag;
  return a;
}

pgpu_status pack(pgpu_mlp *nn) {
  mlp_pack_kernel<<<(HID * HID + 255) / 256, 256, 0, nn->ctx->stream>>>(nn->p, nn->W1, nn->W1T, nn->W2,
                                                                        nn->W2T, nn->W3, nn->W3T);
  return pgpu_after_launch(nn->ctx, "mlp_pack_kernel");
}

// forward over n rows of Xn (already normalised, n_pad rows); train mode
// keeps Z, H and H^T of every layer.  y gets h3 . w4; the output bias is
// added by mlp_add_b4_kernel, which reads it on the device.
pgpu_status forward(pgpu_mlp *nn, const __nv_bfloat16 *Xn, int n, int n_pad, bool train,
                    __nv_bfloat16 *h0, __nv_bfloat16 *h1, float *y) {
  const __nv_bfloat16 *Wl[3] = {nn->W1, nn->W2, nn->W3};
  const int Kl[3] = {IN, HID, HID};
  const size_t boff[3] = {OFF_B1, OFF_B2, OFF_B3};
  const __nv_bfloat16 *in = Xn;
  for (int l = 0; l < 3; ++l) {
    GemmArgs a = base_args(nn);
    a.A = in;
    a.B = Wl[l];
    a.M = n;
    a.N = HID;
    a.K = Kl[l];
    a.lda = Kl[l];
    a.ldb = Kl[l];
    a.bias = nn->p + boff[l];
    a.ldh = HID;
    a.ldz = HID;
    a.ldt = n_pad;
    if (train) {
      a.Z = nn->Z[l];
      a.H = nn->H[l];
      a.HT = nn->HT[l];
    } else {
      a.H = l == 2 ? nullptr : (l % 2 == 0 ? h0 : h1);
    }
    if (l == 2) {
      a.w4 = nn->p + OFF_W4;
      a.y = y;
    }
    PGPU_TRY(gemm<EPI_GELU>(nn, a));
    in = a.H;
  }
  return PGPU_OK;
}

}  // namespace

// the output bias is read on the device by a small kernel after the GEMMs
namespace {
__global__ void mlp_add_b4_kernel(float *y, int n, const float *b4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += *b4;
}
}  // namespace

extern "C" {

long long pgpu_mlp_n_params(void) { return (long long)N_PARAMS; }

pgpu_status pgpu_mlp_create(pgpu_ctx *ctx, uint64_t seed, int max_batch, pgpu_mlp **out) {
  if (!ctx || !out || max_batch < 1) return PGPU_ERR_ARG;
  *out = nullptr;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  pgpu_mlp *nn = new pgpu_mlp();
  nn->ctx = ctx;
  nn->max_batch = max_batch;
  nn->bpad = (int)pad_to((size_t)max_batch, GM);
  auto fail = [&](pgpu_status st) {
    pgpu_mlp_destroy(nn);
    return st;
  };
#define MLP_TRY(x)                        \
  do {                                    \
    pgpu_status st_ = (x);                \
    if (st_ != PGPU_OK) return fail(st_); \
  } while (0)
  MLP_TRY(mo(nn, N_PARAMS, &nn->p));
  MLP_TRY(mo(nn, N_PARAMS, &nn->m));
  MLP_TRY(mo(nn, N_PARAMS, &nn->v));
  MLP_TRY(mo(nn, N_PARAMS, &nn->g));
  MLP_TRY(mo(nn, (size_t)HID * IN, &nn->W1));
  MLP_TRY(mo(nn, (size_t)HID * IN, &nn->W1T));
  MLP_TRY(mo(nn, (size_t)HID * HID, &nn->W2));
  MLP_TRY(mo(nn, (size_t)HID * HID, &nn->W2T));
  MLP_TRY(mo(nn, (size_t)HID * HID, &nn->W3));
  MLP_TRY(mo(nn, (size_t)HID * HID, &nn->W3T));
  MLP_TRY(mo(nn, IN, &nn->mu));
  MLP_TRY(mo(nn, IN, &nn->inv_sd));
  MLP_TRY(mo(nn, 8, &nn->scal));
  const size_t B = nn->bpad;
  MLP_TRY(mo(nn, B * IN, &nn->Xn));
  MLP_TRY(mo(nn, B * IN, &nn->XnT));
  for (int l = 0; l < 3; ++l) {
    MLP_TRY(mo(nn, B * HID, &nn->H[l]));
    MLP_TRY(mo(nn, B * HID, &nn->HT[l]));
    MLP_TRY(mo(nn, B * HID, &nn->Z[l]));
  }
  MLP_TRY(mo(nn, B * HID, &nn->DZ));
  MLP_TRY(mo(nn, B * HID, &nn->DZT));
  MLP_TRY(mo(nn, B * HID, &nn->DZ2));
  MLP_TRY(mo(nn, B * HID, &nn->DZ2T));
  MLP_TRY(mo(nn, B, &nn->y));
  MLP_TRY(mo(nn, B, &nn->dy));
  // He-uniform initial weights (seeded host RNG), zero biases
  std::vector<float> h(N_PARAMS, 0.0f);
  std::mt19937_64 rng(seed);
  auto fill = [&](size_t off, int fan_out, int fan_in) {
    const float lim = std::sqrt(6.0f / (float)fan_in);
    std::uniform_real_distribution<float> u(-lim, lim);
    for (size_t i = 0; i < (size_t)fan_out * fan_in; ++i) h[off + i] = u(rng);
  };
  fill(OFF_W1, HID, IN);
  fill(OFF_W2, HID, HID);
  fill(OFF_W3, HID, HID);
  {
    const float lim = std::sqrt(3.0f / (float)HID);
    std::uniform_real_distribution<float> u(-lim, lim);
    for (int i = 0; i < HID; ++i) h[OFF_W4 + i] = u(rng);
  }
  std::vector<float> ones(IN, 1.0f), zeros(IN, 0.0f);
  if (cudaMemcpy(nn->p, h.data(), N_PARAMS * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(nn->m, 0, N_PARAMS * 4) != cudaSuccess || cudaMemset(nn->v, 0, N_PARAMS * 4) != cudaSuccess ||
      cudaMemcpy(nn->mu, zeros.data(), IN * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(nn->inv_sd, ones.data(), IN * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(pgpu_set_err(ctx, PGPU_ERR_CUDA, "mlp: initial copies failed"));
  }
  MLP_TRY(pack(nn));
#undef MLP_TRY
  *out = nn;
  return PGPU_OK;
}

void pgpu_mlp_destroy(pgpu_mlp *nn) {
  if (!nn) return;
  if (nn->ctx) cudaSetDevice(nn->ctx->device);
  for (void *p : nn->owned) cudaFree(p);
  delete nn;
}

pgpu_status pgpu_mlp_get_params(pgpu_mlp *nn, float *host) {
  if (!nn || !host) return PGPU_ERR_ARG;
  PGPU_CUDA(nn->ctx, cudaMemcpyAsync(host, nn->p, N_PARAMS * 4, cudaMemcpyDeviceToHost, nn->ctx->stream));
  PGPU_CUDA(nn->ctx, cudaStreamSynchronize(nn->ctx->stream));
  return PGPU_OK;
}

pgpu_status pgpu_mlp_set_params(pgpu_mlp *nn, const float *host) {
  if (!nn || !host) return PGPU_ERR_ARG;
  PGPU_CUDA(nn->ctx, cudaMemcpyAsync(nn->p, host, N_PARAMS * 4, cudaMemcpyHostToDevice, nn->ctx->stream));
  PGPU_TRY(pack(nn));
  PGPU_CUDA(nn->ctx, cudaStreamSynchronize(nn->ctx->stream));
  return PGPU_OK;
}

pgpu_status pgpu_mlp_get_norm(pgpu_mlp *nn, float *mu, float *inv_sd) {
  if (!nn || !mu || !inv_sd) return PGPU_ERR_ARG;
  PGPU_CUDA(nn->ctx, cudaMemcpyAsync(mu, nn->mu, IN * 4, cudaMemcpyDeviceToHost, nn->ctx->stream));
  PGPU_CUDA(nn->ctx, cudaMemcpyAsync(inv_sd, nn->inv_sd, IN * 4, cudaMemcpyDeviceToHost, nn->ctx->stream));
  PGPU_CUDA(nn->ctx, cudaStreamSynchronize(nn->ctx->stream));
  return PGPU_OK;
}

// feature normalisation from the column statistics of X_dev [n][64]
pgpu_status pgpu_mlp_fit_norm(pgpu_mlp *nn, const float *X_dev, size_t n) {
  if (!nn || !X_dev) return PGPU_ERR_ARG;
  mlp_colstats_kernel<<<IN, 256, 0, nn->ctx->stream>>>(X_dev, n, nn->mu, nn->inv_sd);
  return pgpu_after_launch(nn->ctx, "mlp_colstats_kernel");
}

pgpu_status pgpu_mlp_forward(pgpu_mlp *nn, const float *X_dev, size_t n, float *y_dev) {
  if (!nn || !X_dev || !y_dev) return PGPU_ERR_ARG;
  if (n == 0) return PGPU_OK;
  if (n > (size_t)1 << 30) return pgpu_set_err(nn->ctx, PGPU_ERR_LIMIT, "mlp: too many rows");
  PGPU_CUDA(nn->ctx, cudaSetDevice(nn->ctx->device));
  const size_t np = pad_to(n, GM);
  if (nn->icap < np) {
    for (void *q : {(void *)nn->iXn, (void *)nn->iH0, (void *)nn->iH1})
      if (q) {
        cudaFree(q);
        nn->owned.erase(std::find(nn->owned.begin(), nn->owned.end(), q));
      }
    const size_t cap = np + np / 4;
    PGPU_TRY(mo(nn, cap * IN, &nn->iXn));
    PGPU_TRY(mo(nn, cap * HID, &nn->iH0));
    PGPU_TRY(mo(nn, cap * HID, &nn->iH1));
    nn->icap = cap;
  }
  mlp_norm_kernel<<<(unsigned)((np * IN + 255) / 256), 256, 0, nn->ctx->stream>>>(
      X_dev, n, np, nn->mu, nn->inv_sd, nn->iXn, nullptr, 0);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_norm_kernel"));
  PGPU_TRY(forward(nn, nn->iXn, (int)n, (int)np, false, nn->iH0, nn->iH1, y_dev));
  mlp_add_b4_kernel<<<(unsigned)((n + 255) / 256), 256, 0, nn->ctx->stream>>>(y_dev, (int)n, nn->p + OFF_B4);
  return pgpu_after_launch(nn->ctx, "mlp_add_b4_kernel");
}

// gradients of the weighted squared loss into the flat FP32 gradient vector;
// with grad_host non-null they are copied out (and nothing is updated)
static pgpu_status mlp_backprop(pgpu_mlp *nn, const float *X_dev, const float *t_dev, const float *sw_dev,
                                size_t n, float *loss_host) {
  if (n == 0 || n > (size_t)nn->max_batch)
    return pgpu_set_err(nn->ctx, PGPU_ERR_ARG, "mlp: batch of %zu rows (1..%d)", n, nn->max_batch);
  const int B = nn->bpad, ni = (int)n;
  cudaStream_t st = nn->ctx->stream;
  mlp_norm_kernel<<<(unsigned)(((size_t)B * IN + 255) / 256), 256, 0, st>>>(X_dev, n, B, nn->mu, nn->inv_sd,
                                                                           nn->Xn, nn->XnT, B);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_norm_kernel"));
  PGPU_TRY(forward(nn, nn->Xn, B, B, true, nullptr, nullptr, nn->y));
  mlp_add_b4_kernel<<<(B + 255) / 256, 256, 0, st>>>(nn->y, B, nn->p + OFF_B4);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_add_b4_kernel"));
  mlp_loss_kernel<<<1, 1024, 0, st>>>(nn->y, t_dev, sw_dev, ni, nn->dy, &nn->scal[0], nn->g + OFF_B4);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_loss_kernel"));
  // output layer: dw4 = sum_r dy_r h3_r (rows >= n carry dy = 0)
  PGPU_CUDA(nn->ctx, cudaMemsetAsync(nn->dy + ni, 0, (size_t)(B - ni) * 4, st));
  mlp_rowsum_kernel<<<HID / 8, 256, 0, st>>>(nn->HT[2], B, B, nn->dy, HID, nn->g + OFF_W4);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_rowsum_kernel"));
  mlp_out_bwd_kernel<<<(unsigned)(((size_t)B * HID + 255) / 256), 256, 0, st>>>(
      nn->dy, nn->p + OFF_W4, nn->Z[2], ni, B, nn->DZ, nn->DZT, B);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_out_bwd_kernel"));
  // layers 3, 2, 1
  const size_t woff[3] = {OFF_W1, OFF_W2, OFF_W3}, boff[3] = {OFF_B1, OFF_B2, OFF_B3};
  const __nv_bfloat16 *WT[3] = {nn->W1T, nn->W2T, nn->W3T};
  __nv_bfloat16 *dz = nn->DZ, *dzT = nn->DZT, *dz_next = nn->DZ2, *dzT_next = nn->DZ2T;
  for (int l = 2; l >= 0; --l) {
    const int K_in = l == 0 ? IN : HID;
    // dW_l = dz_l^T h_{l-1}   (h_{-1} = xn)
    GemmArgs a = base_args(nn);
    a.A = dzT;
    a.B = l == 0 ? nn->XnT : nn->HT[l - 1];
    a.M = HID;
    a.N = K_in;
    a.K = B;
    a.lda = B;
    a.ldb = B;
    a.C = nn->g + woff[l];
    a.ldc = K_in;
    PGPU_TRY(gemm<EPI_F32>(nn, a));
    mlp_rowsum_kernel<<<HID / 8, 256, 0, st>>>(dzT, B, B, nullptr, HID, nn->g + boff[l]);
    PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_rowsum_kernel"));
    if (l == 0) break;
    // dz_{l-1} = (dz_l W_l) * gelu'(z_{l-1})
    GemmArgs b = base_args(nn);
    b.A = dz;
    b.B = WT[l];
    b.M = B;
    b.N = HID;
    b.K = HID;
    b.lda = HID;
    b.ldb = HID;
    b.Z = nn->Z[l - 1];
    b.ldz = HID;
    b.H = dz_next;
    b.ldh = HID;
    b.HT = dzT_next;
    b.ldt = B;
    PGPU_TRY(gemm<EPI_DGELU>(nn, b));
    std::swap(dz, dz_next);
    std::swap(dzT, dzT_next);
  }
  if (loss_host) {
    PGPU_CUDA(nn->ctx, cudaMemcpyAsync(loss_host, &nn->scal[0], 4, cudaMemcpyDeviceToHost, st));
  }
  return PGPU_OK;
}

pgpu_status pgpu_mlp_grads(pgpu_mlp *nn, const float *X_dev, const float *t_dev, const float *sw_dev,
                           size_t n, float *grad_host, float *loss_host) {
  if (!nn || !X_dev || !t_dev || !grad_host) return PGPU_ERR_ARG;
  PGPU_CUDA(nn->ctx, cudaSetDevice(nn->ctx->device));
  PGPU_TRY(mlp_backprop(nn, X_dev, t_dev, sw_dev, n, loss_host));
  PGPU_CUDA(nn->ctx, cudaMemcpyAsync(grad_host, nn->g, N_PARAMS * 4, cudaMemcpyDeviceToHost, nn->ctx->stream));
  PGPU_CUDA(nn->ctx, cudaStreamSynchronize(nn->ctx->stream));
  return pgpu_check_flag(nn->ctx, "mlp_grads");
}

pgpu_status pgpu_mlp_train_step(pgpu_mlp *nn, const float *X_dev, const float *t_dev, const float *sw_dev,
                                size_t n, float lr, float weight_decay, float *loss_host) {
  if (!nn || !X_dev || !t_dev) return PGPU_ERR_ARG;
  PGPU_CUDA(nn->ctx, cudaSetDevice(nn->ctx->device));
  PGPU_TRY(mlp_backprop(nn, X_dev, t_dev, sw_dev, n, loss_host));
  nn->step += 1;
  AdamArgs a;
  a.p = nn->p;
  a.m = nn->m;
  a.v = nn->v;
  a.g = nn->g;
  a.n = N_PARAMS;
  a.lr = lr;
  a.b1 = 0.9f;
  a.b2 = 0.999f;
  a.eps = 1e-8f;
  a.wd = weight_decay;
  a.c1 = (float)(1.0 - std::pow(0.9, (double)nn->step));
  a.c2 = (float)(1.0 - std::pow(0.999, (double)nn->step));
  mlp_adamw_kernel<<<(unsigned)((N_PARAMS + 255) / 256), 256, 0, nn->ctx->stream>>>(a);
  PGPU_TRY(pgpu_after_launch(nn->ctx, "mlp_adamw_kernel"));
  PGPU_TRY(pack(nn));
  if (loss_host) {
    PGPU_CUDA(nn->ctx, cudaStreamSynchronize(nn->ctx->stream));
    return pgpu_check_flag(nn->ctx, "mlp_train_step");
  }
  return PGPU_OK;
}

}  // extern "C"
