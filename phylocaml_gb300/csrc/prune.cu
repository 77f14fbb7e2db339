// Felsenstein pruning: the tree log-likelihood of weighted site patterns.
//
// The reference's likelihood character is a stub (Likelihood_c.median_2 is
// `failwith "TODO"`, lib/likelihood_c.ml:15); this is the computation that
// slot exists for, over the transition matrices MlModel.compose builds
// (lib/mlModel.ml:585-587, lib/mlmodel.c:325-342, P[i][j] = Pr(j | i, t)):
//
//   CLV_v[r][i] = (sum_j P_{a,r}[i][j] CLV_a[r][j]) * (sum_j P_{b,r}[i][j] CLV_b[r][j])
//   L_s         = sum_r probs[r] sum_i pi[i] CLV_root[r][i]
//   lnL         = sum_s w_s (log L_s + e_s ln 2)
//
// One kernel scores the whole tree (prune_tree_kernel):
//   warp 0, lane 0   producer: streams each tip's row of pattern codes for the
//                    CTA's tile, in the order the schedule reads them, into a
//                    shared ring with 1-D bulk copies on mbarriers;
//   consumer warps   one pattern per thread; the conditional likelihood
//                    vectors of internal nodes live on a per-thread stack in
//                    shared memory (top entry in registers), so no CLV ever
//                    goes to HBM.  After every node the vector is rescaled by
//                    an exact power of two when its largest entry drops below
//                    2^-32 (FP32) or 2^-256 (FP64) and the exponent is added
//                    to the pattern's integer scaler e_s.
// The root log-likelihoods are weighted and summed in FP64 with error-free
// TwoSum steps (a compensated reduction), one (sum, compensation) pair per
// CTA; prune_finalize_kernel adds the pairs in CTA order with Neumaier's
// method, so the result does not depend on scheduling.
//
// T = float is the FP32 form, T = double the FP64 comparison form; both use
// P matrices built in FP64 on the GPU (pmatrix.cu), the FP32 form rounding
// them once.
#include <algorithm>
#include <cmath>

#include "pgpu_internal.cuh"
#include "pmatrix.cuh"

namespace {

struct PruneArgs {
  const uint8_t *tip_codes;   // [n_tips][ld_pat]
  const void *P;              // [2n-2][R][S][S] of T
  const double *code_tab;     // [n_codes][S]
  const double *pi;           // [S]
  const double *probs;        // [R]
  const double *weights;      // [n_pat] or null
  double *site_lnl;           // [n_pat] or null
  double2 *partials;          // [gridDim.x]
  const int4 *ops;            // schedule
  const int32_t *tip_seq;
  int *flag;
  size_t ld_pat, n_pat;
  int n_tips, n_ops, n_codes, R, NT, stages, depth;
};

template <typename T>
struct ScaleTraits;
template <>
struct ScaleTraits<float> {
  static constexpr float thresh = 0x1p-32f;
  __device__ static float pow2(int k) {  // 2^k for -126 <= k <= 127
    return __int_as_float((127 + k) << 23);
  }
  __device__ static int exponent(float x) {
    int e;
    (void)frexpf(x, &e);
    return e;
  }
};
template <>
struct ScaleTraits<double> {
  static constexpr double thresh = 0x1p-256;
  __device__ static double pow2(int k) {  // 2^k for -1022 <= k <= 1023
    return __longlong_as_double((long long)(1023 + k) << 52);
  }
  __device__ static int exponent(double x) {
    int e;
    (void)frexp(x, &e);
    return e;
  }
};

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// compensated sum of (s, c) pairs over the 32 lanes of a warp
__device__ __forceinline__ void warp_csum(double &s, double &c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, c, o);
    double t, e;
    two_sum(s, s2, t, e);
    s = t;
    c = c + c2 + e;
  }
}

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

template <typename T, int S, int RM>
struct PruneLayout {
  __host__ __device__ static size_t ring_off(int stages) { return 16 * (size_t)stages; }
  __host__ __device__ static size_t tab_off(int stages, int NT) { return align16(ring_off(stages) + (size_t)stages * NT); }
  __host__ __device__ static size_t stk_off(int stages, int NT, int n_codes) {
    return align16(tab_off(stages, NT) + (size_t)n_codes * S * sizeof(T));
  }
  __host__ __device__ static size_t bytes(int stages, int NT, int n_codes, int depth) {
    return stk_off(stages, NT, n_codes) + (size_t)depth * RM * S * NT * sizeof(T);
  }
};

template <typename T, int S, int RM>
__global__ void __launch_bounds__(160) prune_tree_kernel(const PruneArgs p) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double2 red[8];
  using L = PruneLayout<T, S, RM>;
  constexpr int RS = RM * S;
  const int NT = p.NT, ST = p.stages, R = p.R;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + ST;
  uint8_t *ring = smem + L::ring_off(ST);                                  // [ST][NT]
  T *tab = reinterpret_cast<T *>(smem + L::tab_off(ST, NT));               // [n_codes][S]
  T *stk = reinterpret_cast<T *>(smem + L::stk_off(ST, NT, p.n_codes));    // [depth][RS][NT]
  const size_t tile0 = (size_t)blockIdx.x * NT;
  const int tid = threadIdx.x;

  for (int i = tid; i < p.n_codes * S; i += blockDim.x) tab[i] = (T)p.code_tab[i];
  if (tid == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NT / 32);
    }
    fence_mbarrier_init();
  }
  __syncthreads();

  if (tid < 32) {
    if (tid == 0) {
      const size_t span = min((size_t)NT, p.ld_pat - tile0);
      const uint32_t bytes = (uint32_t)span;
      int issued = 0;
      for (int j = 0; j < p.n_tips; ++j) {
        const int slot = j % ST, round = j / ST;
        if (round > 0 && !mbar_wait_bounded(&empty[slot], (round - 1) & 1, p.flag)) break;
        const int32_t tip = __ldg(p.tip_seq + j);
        mbar_arrive_expect_tx(&full[slot], bytes);
        bulk_g2s(ring + (size_t)slot * NT, p.tip_codes + (size_t)tip * p.ld_pat + tile0, bytes,
                 &full[slot]);
        issued = j + 1;
      }
      for (int j = max(0, issued - ST); j < issued; ++j)
        (void)mbar_wait_bounded(&full[j % ST], (j / ST) & 1, p.flag);
    }
    return;
  }

  const int c = tid - 32, lane = tid & 31;
  const size_t pat = tile0 + c;
  const bool active = pat < p.n_pat;
  const T *P = reinterpret_cast<const T *>(p.P);
  const size_t PB = (size_t)R * S * S;   // one branch's block

  T top[RS];
  bool top_valid = false;
  int sp = 0, taken = 0, escale = 0;
  bool ok = true;

  auto take = [&]() -> int {
    const int slot = taken % ST;
    const bool got =
        __all_sync(0xffffffffu, mbar_wait_bounded(&full[slot], (taken / ST) & 1, p.flag));
    if (!got) {
      ok = false;
      return 0;
    }
    int code = ring[(size_t)slot * NT + c];
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[slot]);
    ++taken;
    if (code >= p.n_codes) {
      if (active) atomicOr(p.flag, PGPU_FLAG_BADCODE);
      code = 0;
    }
    return code;
  };
  auto pop = [&](T *dst) {
    if (top_valid) {
#pragma unroll
      for (int e = 0; e < RS; ++e) dst[e] = top[e];
      top_valid = false;
    } else {
      --sp;
#pragma unroll
      for (int e = 0; e < RS; ++e) dst[e] = stk[((size_t)sp * RS + e) * NT + c];
    }
  };
  // acc = (or *=) P_child * x, x from registers or from the tip code table
  auto apply = [&](int child, const T *x, int code, T *acc, bool first) {
    const T *Pc = P + (size_t)child * PB;
#pragma unroll
    for (int r = 0; r < RM; ++r) {
      if (r < R) {
        T xv[S];
#pragma unroll
        for (int j = 0; j < S; ++j) xv[j] = code >= 0 ? tab[code * S + j] : x[r * S + j];
#pragma unroll
        for (int i = 0; i < S; ++i) {
          const T *row = Pc + ((size_t)r * S + i) * S;
          T s = 0;
#pragma unroll
          for (int j = 0; j < S; ++j) s = fma(__ldg(row + j), xv[j], s);
          acc[r * S + i] = first ? s : acc[r * S + i] * s;
        }
      }
    }
  };

  for (int i = 0; i < p.n_ops && ok; ++i) {
    const int4 op = __ldg(p.ops + i);
    const int a = op.y, b = op.z;
    T xa[RS], xb[RS];
    if (b >= p.n_tips) pop(xb);
    if (a >= p.n_tips) pop(xa);
    int ca = -1, cb = -1;
    if (a < p.n_tips) ca = take();
    if (b < p.n_tips && ok) cb = take();
    if (!ok) break;
    T acc[RS];
    apply(a, xa, ca, acc, true);
    apply(b, xb, cb, acc, false);
    // exact power-of-two rescaling
    T mx = 0;
#pragma unroll
    for (int e = 0; e < RS; ++e)
      if (e < R * S) mx = fmax(mx, acc[e]);
    if (mx < ScaleTraits<T>::thresh && mx > (T)0) {
      const int ex = ScaleTraits<T>::exponent(mx);
      escale += ex;
      const T f = ScaleTraits<T>::pow2(-ex);
#pragma unroll
      for (int e = 0; e < RS; ++e) acc[e] *= f;
    }
    // push
    if (top_valid) {
#pragma unroll
      for (int e = 0; e < RS; ++e) stk[((size_t)sp * RS + e) * NT + c] = top[e];
      ++sp;
    }
#pragma unroll
    for (int e = 0; e < RS; ++e) top[e] = acc[e];
    top_valid = true;
  }

  // root likelihood, weighted log, compensated block sum
  double s = 0.0, comp = 0.0;
  if (ok && active) {
    double Ls = 0.0;
#pragma unroll
    for (int r = 0; r < RM; ++r) {
      if (r < R) {
        double lr = 0.0;
#pragma unroll
        for (int i = 0; i < S; ++i) lr += p.pi[i] * (double)top[r * S + i];
        Ls += p.probs[r] * lr;
      }
    }
    const double lnl = log(Ls) + (double)escale * 0.69314718055994530942;
    if (p.site_lnl) p.site_lnl[pat] = lnl;
    s = p.weights ? p.weights[pat] * lnl : lnl;
  }
  warp_csum(s, comp);
  const int cw = c >> 5, ncw = NT / 32;
  if (lane == 0) red[cw] = make_double2(s, comp);
  asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
  if (cw == 0) {
    double2 v = lane < ncw ? red[lane] : make_double2(0.0, 0.0);
    double ss = v.x, cc = v.y;
    warp_csum(ss, cc);
    if (lane == 0) p.partials[blockIdx.x] = make_double2(ss, cc);
  }
}

// Neumaier sum of the per-CTA (sum, compensation) pairs in CTA order.
__global__ void __launch_bounds__(32) prune_finalize_kernel(const double2 *partials, int n,
                                                           double *out) {
  if (threadIdx.x != 0) return;
  double s = 0.0, c = 0.0;
  for (int i = 0; i < n; ++i) {
    const double2 v = partials[i];
    double t, e;
    two_sum(s, v.x, t, e);
    s = t;
    c += e + v.y;
  }
  out[0] = s + c;
}

template <typename T, int S, int RM>
pgpu_status launch_prune(pgpu_ctx *ctx, PruneArgs &a, size_t n_tiles) {
  const size_t smem = PruneLayout<T, S, RM>::bytes(a.stages, a.NT, a.n_codes, a.depth);
  if (smem > ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "prune: %zu bytes of shared memory needed", smem);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(prune_tree_kernel<T, S, RM>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
  prune_tree_kernel<T, S, RM><<<(unsigned)n_tiles, 32 + a.NT, smem, ctx->stream>>>(a);
  return pgpu_after_launch(ctx, "prune_tree_kernel");
}

}  // namespace

// Double-buffered pinned staging for the small per-call parameters, so the
// device-pointer entry points never synchronise the stream.
pgpu_status pgpu_stage(pgpu_ctx *ctx, size_t bytes, void **host, void **dev) {
  const int k = ctx->stage_next;
  ctx->stage_next ^= 1;
  if (ctx->stage_ev[k]) PGPU_CUDA(ctx, cudaEventSynchronize(ctx->stage_ev[k]));
  if (ctx->stage_cap[k] < bytes) {
    if (ctx->stage_h[k]) cudaFreeHost(ctx->stage_h[k]);
    if (ctx->stage_d[k]) cudaFree(ctx->stage_d[k]);
    ctx->stage_h[k] = nullptr;
    ctx->stage_d[k] = nullptr;
    ctx->stage_cap[k] = 0;
    const size_t want = std::max<size_t>(bytes, 64 * 1024);
    PGPU_CUDA(ctx, cudaMallocHost(&ctx->stage_h[k], want));
    PGPU_CUDA(ctx, cudaMalloc(&ctx->stage_d[k], want));
    ctx->stage_cap[k] = want;
  }
  if (!ctx->stage_ev[k]) PGPU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->stage_ev[k], cudaEventDisableTiming));
  *host = ctx->stage_h[k];
  *dev = ctx->stage_d[k];
  ctx->stage_cur = k;
  return PGPU_OK;
}

pgpu_status pgpu_stage_commit(pgpu_ctx *ctx, size_t bytes) {
  const int k = ctx->stage_cur;
  PGPU_CUDA(ctx, cudaMemcpyAsync(ctx->stage_d[k], ctx->stage_h[k], bytes, cudaMemcpyHostToDevice,
                                 ctx->stream));
  PGPU_CUDA(ctx, cudaEventRecord(ctx->stage_ev[k], ctx->stream));
  return PGPU_OK;
}

namespace {

pgpu_status check_model(pgpu_ctx *ctx, const pgpu_model *m, const pgpu_tip_codes *codes) {
  if (!m || !m->Q || !m->pi || !m->rates || !m->probs)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: null model field");
  if (!codes || !codes->table || codes->n_codes < 1 || codes->n_codes > 256)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: tip code table must have 1..256 rows");
  if (m->n_rates < 1 || m->n_rates > 8)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "prune: 1..8 rate classes are supported");
  if (m->n_states != 4)
    return pgpu_set_err(ctx, PGPU_ERR_UNSUPPORTED,
                        "prune: the SIMT pruning kernel is built for 4 states (DNA); use "
                        "pgpu_batch_lnl for 20- and 61-state models");
  return PGPU_OK;
}

// all small per-call parameters in one staged block
struct Staged {
  double *Q, *pi, *rates, *probs, *tab, *brlen;
  size_t bytes;
};

Staged stage_layout(int S, int R, int n_codes, int n_br) {
  Staged s{};
  size_t off = 0;
  auto take = [&](size_t n) {
    const size_t o = off;
    off += align16(n * sizeof(double));
    return o;
  };
  s.Q = (double *)take((size_t)S * S);
  s.pi = (double *)take(S);
  s.rates = (double *)take(R);
  s.probs = (double *)take(R);
  s.tab = (double *)take((size_t)n_codes * S);
  s.brlen = (double *)take(n_br);
  s.bytes = off;
  return s;
}

template <typename Ptr>
Ptr *rebase(void *base, Ptr *off) {
  return reinterpret_cast<Ptr *>(static_cast<char *>(base) + reinterpret_cast<size_t>(off));
}

pgpu_status prune_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *m,
                      const pgpu_tip_codes *codes, const uint8_t *tips, size_t ld_pat,
                      const double *weights, size_t n_pat, int precision, double *lnl_dev,
                      double *site_lnl_dev) {
  PGPU_TRY(check_model(ctx, m, codes));
  if (precision != 32 && precision != 64)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: precision must be 32 or 64");
  if (!tree || !tree->brlen) return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: tree->brlen is required");
  if (!tips || !lnl_dev) return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: null buffer");
  if (ld_pat % 16 != 0 || ld_pat < n_pat || ((uintptr_t)tips & 15))
    return pgpu_set_err(ctx, PGPU_ERR_ARG,
                        "prune: ld_pat (%zu) must be a multiple of 16 and >= n_pat, rows 16-byte aligned",
                        ld_pat);
  const TreeSchedule *sch;
  const int4 *dops;
  const int32_t *dseq;
  PGPU_TRY(pgpu_schedule_device(ctx, tree, &sch, &dops, &dseq));
  const int S = m->n_states, R = m->n_rates, n = tree->n_tips, n_br = 2 * n - 2;
  for (int i = 0; i < n_br; ++i)
    if (!(tree->brlen[i] >= 0.0) || !std::isfinite(tree->brlen[i]))
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: branch length %d is negative or not finite", i);

  // stage Q, pi, rates, probs, the code table and the branch lengths
  Staged lay = stage_layout(S, R, codes->n_codes, n_br);
  void *h, *d;
  PGPU_TRY(pgpu_stage(ctx, lay.bytes, &h, &d));
  std::copy(m->Q, m->Q + S * S, rebase(h, lay.Q));
  std::copy(m->pi, m->pi + S, rebase(h, lay.pi));
  std::copy(m->rates, m->rates + R, rebase(h, lay.rates));
  std::copy(m->probs, m->probs + R, rebase(h, lay.probs));
  std::copy(codes->table, codes->table + (size_t)codes->n_codes * S, rebase(h, lay.tab));
  std::copy(tree->brlen, tree->brlen + n_br, rebase(h, lay.brlen));
  PGPU_TRY(pgpu_stage_commit(ctx, lay.bytes));

  // device scratch: eigen system, P matrices, per-CTA partial sums
  const int NT = precision == 32 ? 128 : 64;
  const size_t n_tiles = (n_pat + NT - 1) / NT;
  const size_t SS = (size_t)S * S;
  const size_t p_bytes = (size_t)n_br * R * SS * (precision == 32 ? 4 : 8);
  void *deig, *dP, *dpart;
  PGPU_TRY(pgpu_buf(ctx, BUF_H, 2 * SS * 8 + S * 8 + 64, &deig));
  PGPU_TRY(pgpu_buf(ctx, BUF_I, p_bytes, &dP));
  PGPU_TRY(pgpu_buf(ctx, BUF_G, std::max<size_t>(n_tiles, 1) * sizeof(double2), &dpart));
  double *dU = (double *)deig, *dUi = dU + SS, *dlam = dUi + SS;
  int *dst = reinterpret_cast<int *>(dlam + S);
  PGPU_TRY(pgpu_launch_eig(ctx, rebase(d, lay.Q), rebase(d, lay.pi), S, 1, dU, dlam, dUi, dst));
  PGPU_TRY(pgpu_launch_compose(ctx, dU, dlam, dUi, S, rebase(d, lay.brlen), n_br,
                               rebase(d, lay.rates), R, precision == 64 ? (double *)dP : nullptr,
                               precision == 32 ? (float *)dP : nullptr, false, dst));
  if (n_pat == 0) {
    PGPU_CUDA(ctx, cudaMemsetAsync(lnl_dev, 0, sizeof(double), ctx->stream));
    return PGPU_OK;
  }
  PruneArgs a;
  a.tip_codes = tips;
  a.P = dP;
  a.code_tab = rebase(d, lay.tab);
  a.pi = rebase(d, lay.pi);
  a.probs = rebase(d, lay.probs);
  a.weights = weights;
  a.site_lnl = site_lnl_dev;
  a.partials = (double2 *)dpart;
  a.ops = dops;
  a.tip_seq = dseq;
  a.flag = ctx->d_flag;
  a.ld_pat = ld_pat;
  a.n_pat = n_pat;
  a.n_tips = n;
  a.n_ops = (int)sch->ops.size();
  a.n_codes = codes->n_codes;
  a.R = R;
  a.NT = NT;
  a.stages = 32;
  a.depth = std::max(sch->max_depth, 1);
  if (precision == 32) {
    if (R <= 4) PGPU_TRY((launch_prune<float, 4, 4>(ctx, a, n_tiles)));
    else PGPU_TRY((launch_prune<float, 4, 8>(ctx, a, n_tiles)));
  } else {
    if (R <= 4) PGPU_TRY((launch_prune<double, 4, 4>(ctx, a, n_tiles)));
    else PGPU_TRY((launch_prune<double, 4, 8>(ctx, a, n_tiles)));
  }
  prune_finalize_kernel<<<1, 32, 0, ctx->stream>>>((const double2 *)dpart, (int)n_tiles, lnl_dev);
  return pgpu_after_launch(ctx, "prune_finalize_kernel");
}

}  // namespace

extern "C" {

pgpu_status pgpu_prune_lnl_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *model,
                               const pgpu_tip_codes *codes, const uint8_t *tip_codes_dev,
                               size_t ld_pat, const double *weights_dev, size_t n_pat,
                               int precision, double *lnl_dev, double *site_lnl_dev) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  return prune_dev(ctx, tree, model, codes, tip_codes_dev, ld_pat, weights_dev, n_pat, precision,
                   lnl_dev, site_lnl_dev);
}

pgpu_status pgpu_prune_lnl(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *model,
                           const pgpu_tip_codes *codes, const uint8_t *tip_codes,
                           const double *weights, size_t n_pat, int precision, double *lnl,
                           double *site_lnl) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!tree || tree->n_tips < 2 || !tip_codes || !lnl)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: null argument or fewer than 2 tips");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t n = (size_t)tree->n_tips;
  const size_t ld = (n_pat + 15) / 16 * 16;
  void *dt, *dw = nullptr, *dl, *dsl = nullptr;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, std::max<size_t>(n * ld, 16), &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dl));
  if (weights) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n_pat * 8, &dw));
  if (site_lnl) PGPU_TRY(pgpu_buf(ctx, BUF_SITECOST, n_pat * 8, &dsl));
  cudaStream_t s = ctx->stream;
  if (n_pat) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(dt, ld, tip_codes, n_pat, n_pat, n, cudaMemcpyHostToDevice, s));
    if (weights) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_pat * 8, cudaMemcpyHostToDevice, s));
  }
  PGPU_TRY(prune_dev(ctx, tree, model, codes, (const uint8_t *)dt, ld, (const double *)dw, n_pat,
                     precision, (double *)dl, (double *)dsl));
  double *hl = reinterpret_cast<double *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(hl, dl, 8, cudaMemcpyDeviceToHost, s));
  if (site_lnl && n_pat)
    PGPU_CUDA(ctx, cudaMemcpyAsync(site_lnl, dsl, n_pat * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  PGPU_TRY(pgpu_check_flag(ctx, "prune"));
  *lnl = *hl;
  return PGPU_OK;
}

}  // extern "C"
