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
// CTA; prune_finalize_kernel adds the pairs in contiguous chunks with Neumaier's
// method, so the result does not depend on scheduling.
//
// T = float is the FP32 form, T = double the FP64 comparison form; both use
// P matrices built in FP64 on the GPU (pmatrix.cu), the FP32 form rounding
// them once.
#include <algorithm>
#include <cmath>

#include "pgpu_internal.cuh"
#include "forms.cuh"
#include "pmatrix.cuh"

namespace {
using namespace pgpu_forms;

struct PruneArgs {
  const uint8_t *tip_codes;   // [n_tips][ld_pat]
  const void *P;              // [2n-2][R][S][S] coefficients of the form (see below)
  const void *tiptab;         // [n_tips][R][n_codes][S] tip rows P(t,r) code_tab[c] (form's values)
  const double *code_tab;     // [n_codes][S]
  const double *pi;           // [S]
  const double *probs;        // [R]
  const double *weights;      // [n_pat] or null
  double *site_lnl;           // [n_pat] or null
  double2 *partials;          // [n_models][n_tiles_total], by tile
  const int4 *ops;            // schedule
  const int32_t *tip_seq;
  int *flag;
  // several models over the same tree and patterns: CTA row blockIdx.y
  // scores model blockIdx.y, whose P blocks and tip rows lie P_stride and
  // tab_stride bytes after the previous model's, pi and probs 4 and R
  // doubles after, and whose partial sums follow the previous model's
  size_t P_stride, tab_stride;
  // a launch may cover tiles tile_base .. tile_base + gridDim.x - 1 of
  // n_tiles_total (the host-buffer entry point launches one per copied chunk)
  size_t tile_base, n_tiles_total;
  size_t ld_pat, n_pat;
  int n_tips, n_ops, n_codes, R, NP, depth;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

constexpr int PR_THREADS = 256;   // consumer threads per CTA

// Ring depth in postorder steps (a power of two) and the CTAs each SM should
// hold.  The pair form's slots and stack are twice the FP32 form's, so its
// ring is shorter to fit three CTAs (27 warps) per SM.  growth: how much
// larger each column chunk of host tip codes is than the one before; a
// chunk's copy must end while the previous chunk is scored, and a wave of
// scoring takes about 2.5 (FP32), 6 (pair) or 30 (FP64) times as long as
// copying its tip codes.
template <typename Pol> struct PruneTune {
  static constexpr int stages = 8, min_ctas = 1, growth = 8;
};
template <> struct PruneTune<pgpu_forms::Ff32> {
  static constexpr int stages = 4, min_ctas = 3, growth = 4;
};
template <> struct PruneTune<pgpu_forms::Fp32> {
  static constexpr int stages = 8, min_ctas = 4, growth = 2;
};
// Steps per ring barrier: the producer stages PR_GROUP consecutive steps
// under one mbarrier phase, so the consumers wait and release once per group.
constexpr int PR_GROUP = 2;

// Shared memory of one CTA: the ring of per-op slots, then the CLV stack.
// A slot holds everything one postorder step reads, staged by the producer:
//   [0, NP)            tip codes of child a (if a is a tip)
//   [NP, 2 NP)         tip codes of child b
//   coef block a       R x 16 coefficients of the branch above a (internal a)
//   coef block b
//   tip block a        R x n_codes x 4 tip rows of the branch above a (tip a)
//   tip block b
template <typename Pol>
struct PruneLayout {
  using V = typename Pol::V;
  using Coef = typename Pol::Coef;
  __host__ __device__ static size_t coef_bytes(int R) { return (size_t)R * 16 * sizeof(Coef); }
  __host__ __device__ static size_t tip_bytes(int R, int n_codes) {
    return (size_t)R * n_codes * 4 * sizeof(V);
  }
  __host__ __device__ static size_t coef_off(int NP) { return 2 * (size_t)NP; }
  __host__ __device__ static size_t tip_off(int NP, int R) { return coef_off(NP) + 2 * coef_bytes(R); }
  __host__ __device__ static size_t slot_bytes(int NP, int R, int n_codes) {
    return (tip_off(NP, R) + 2 * tip_bytes(R, n_codes) + 127) & ~size_t(127);
  }
  __host__ __device__ static size_t ring_off() { return 128; }
  __host__ __device__ static size_t stk_off(int NP, int R, int n_codes) {
    return ring_off() + (size_t)PruneTune<Pol>::stages * slot_bytes(NP, R, n_codes);
  }
  __host__ __device__ static size_t bytes(int NP, int R, int n_codes, int depth) {
    return stk_off(NP, R, n_codes) + (size_t)depth * 4 * PR_THREADS * sizeof(V);
  }
};

// One CTA: 32 producer threads + PR_THREADS consumers.  Consumer warp w
// works on rate class w % RT (R <= RT of them active) for 32 patterns of the
// tile; each thread holds the 4 state values of one (pattern, rate class)
// and its own power-of-two scaler.  All lanes of a warp read the same
// coefficient block (a shared-memory broadcast).
template <typename Pol, int RT>
__global__ void __launch_bounds__(32 + PR_THREADS, PruneTune<Pol>::min_ctas)
    prune_tree_kernel(const PruneArgs p) {
  using V = typename Pol::V;
  using Coef = typename Pol::Coef;
  using L = PruneLayout<Pol>;
  constexpr int ST = PruneTune<Pol>::stages, NT = PR_THREADS, G = PR_GROUP, NB = ST / G;
  static_assert(ST % G == 0 && (NB & (NB - 1)) == 0, "ring depth must be a power-of-two number of groups");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double2 red[NT / 32];
  __shared__ double2 xch[RT][NT / RT];   // per pattern and rate class: (part, scaler)
  __shared__ int step_kind[ST];          // per step slot: which of the consumer's step cases
  const int NP = p.NP, R = p.R, NC = p.n_codes;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);     // [NB]
  uint64_t *empty = full + NB;                              // [NB]
  const size_t SB = L::slot_bytes(NP, R, NC);
  unsigned char *ring = smem + L::ring_off();               // [ST][SB]
  V *stk = reinterpret_cast<V *>(smem + L::stk_off(NP, R, NC));   // [depth][4][NT]
  const size_t tile = p.tile_base + blockIdx.x;
  const size_t tile0 = tile * NP;
  const int tid = threadIdx.x;
  const size_t CB = L::coef_bytes(R), TB = L::tip_bytes(R, NC);

  if (tid == 0) {
    for (int s = 0; s < NB; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NT / 32);
    }
    fence_mbarrier_init();
  }
  __syncthreads();

  if (tid < 32) {
    // producer: everything step i reads goes into slot i % ST
    if (tid == 0) {
      const uint32_t code_bytes = (uint32_t)min((size_t)NP, p.ld_pat - tile0);
      const unsigned char *Pg = static_cast<const unsigned char *>(p.P) + blockIdx.y * p.P_stride;
      const unsigned char *Tg = static_cast<const unsigned char *>(p.tiptab) + blockIdx.y * p.tab_stride;
      // step i goes into step slot i % ST; group q (steps qG .. qG + G - 1)
      // completes barrier q % NB once per pass over the ring
      int groups = 0;
      for (int g0 = 0; g0 < p.n_ops; g0 += G) {
        const int q = g0 / G, b = q & (NB - 1), round = q / NB;
        if (round > 0 && !mbar_wait_bounded(&empty[b], (round - 1) & 1, p.flag)) break;
        const int gn = min(G, p.n_ops - g0);
        int4 ops[G];
        uint32_t tx = 0;
        for (int k = 0; k < gn; ++k) {
          const int4 op = __ldg(p.ops + g0 + k);
          ops[k] = op;
          for (int h = 0; h < 2; ++h) {
            const int ch = h == 0 ? op.y : op.z;
            tx += ch < p.n_tips ? code_bytes + (uint32_t)TB : (uint32_t)CB;
          }
          // bit 0: first child internal, bit 1: second child internal; 4
          // marks the first step, which has no earlier result to set aside.
          // The arrive below releases these stores to the consumers' wait.
          const int kind = (op.y >= p.n_tips ? 1 : 0) | (op.z >= p.n_tips ? 2 : 0);
          step_kind[(g0 + k) & (ST - 1)] = g0 + k == 0 ? 4 : kind;
        }
        mbar_arrive_expect_tx(&full[b], tx);
        for (int k = 0; k < gn; ++k) {
          unsigned char *sl = ring + (size_t)((g0 + k) & (ST - 1)) * SB;
          for (int h = 0; h < 2; ++h) {
            const int ch = h == 0 ? ops[k].y : ops[k].z;
            if (ch < p.n_tips) {
              bulk_g2s(sl + (size_t)h * NP, p.tip_codes + (size_t)ch * p.ld_pat + tile0, code_bytes,
                       &full[b]);
              bulk_g2s(sl + L::tip_off(NP, R) + h * TB, Tg + (size_t)ch * TB, (uint32_t)TB, &full[b]);
            } else {
              bulk_g2s(sl + L::coef_off(NP) + h * CB, Pg + (size_t)ch * CB, (uint32_t)CB, &full[b]);
            }
          }
        }
        groups = q + 1;
      }
      // do not leave while copies into this CTA's shared memory are in flight
      for (int q = max(0, groups - NB); q < groups; ++q)
        (void)mbar_wait_bounded(&full[q & (NB - 1)], (q / NB) & 1, p.flag);
    }
    return;
  }

  // consumer warp w works on rate class w % RT for 32 patterns, so every
  // coefficient read of a warp is a broadcast of one rate's P block
  const int c = tid - 32, lane = tid & 31, cwarp = c >> 5;
  const int r = cwarp % RT, pl = (cwarp / RT) * 32 + lane;
  const size_t pat = tile0 + pl;
  const bool active = pat < p.n_pat;
  const bool rate_on = r < R;
  // warps of a rate class beyond R (R < RT) repeat class R - 1 and are
  // dropped at the root, so the step loop has no branch on the rate
  const int rr = min(r, R - 1);

  // The stack discipline is fixed by the schedule: in postorder the result
  // of step i - 1 is always the second child of step i when that child is
  // internal, else its first child when that one is internal; a step with
  // two tip children leaves it pending (push), and a step with two internal
  // children takes its first child from the stack (pop).  So the top of the
  // stack lives in registers and each step is one of four straight-line
  // cases, chosen by a warp-uniform branch.
  V top[4];
  V *my = stk + c;   // this thread's column of the stack: entry (k, e) at my[(4 k + e) NT]
  int sp = 0, escale = 0;
  uint32_t code_max = 0;
  bool ok = true;
  const size_t tipb = L::tip_off(NP, R) + (size_t)rr * NC * 4 * sizeof(V);
  const size_t coefb = L::coef_off(NP) + (size_t)rr * 16 * sizeof(Coef);

  for (int g0 = 0; g0 < p.n_ops && ok; g0 += G) {
    const int q = g0 / G, b = q & (NB - 1);
    const bool got = __all_sync(0xffffffffu, mbar_wait_bounded(&full[b], (q / NB) & 1, p.flag));
    if (!got) {
      ok = false;
      break;
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
    const int i = g0 + k;
    if (i >= p.n_ops) break;
    const int slot = i & (ST - 1);
    const int kind = step_kind[slot];
    const unsigned char *sl = ring + (size_t)slot * SB;
    V acc[4];
    {
      auto tip = [&](int h, V *y) {
        const uint32_t code = sl[h * NP + pl];
        code_max = max(code_max, code);
        Pol::load_tip(sl + tipb + h * TB, min(code, (uint32_t)NC - 1u), y);
      };
      auto coef = [&](int h) { return reinterpret_cast<const Coef *>(sl + coefb + h * CB); };
      V y0[4], y1[4];
      switch (kind) {
        case 0:   // two tips; the previous result waits on the stack
          if (sp < p.depth) {
#pragma unroll
            for (int e = 0; e < 4; ++e) my[(4 * sp + e) * NT] = top[e];
            ++sp;
          } else {
            ok = false;   // schedule and stack size disagree
          }
          tip(0, y0);
          tip(1, y1);
          break;
        case 4:   // the first step: two tips, nothing to set aside
          tip(0, y0);
          tip(1, y1);
          break;
        case 1:   // internal first child (the previous result), tip second
          Pol::rows(coef(0), top, y0);
          tip(1, y1);
          break;
        case 2:   // tip first, internal second child (the previous result)
          tip(0, y0);
          Pol::rows(coef(1), top, y1);
          break;
        default: {   // 3, both internal: the first from the stack
          V xa[4];
          if (sp > 0) {
            --sp;
#pragma unroll
            for (int e = 0; e < 4; ++e) xa[e] = my[(4 * sp + e) * NT];
          } else {
            ok = false;   // schedule and stack disagree
#pragma unroll
            for (int e = 0; e < 4; ++e) xa[e] = Pol::zero();
          }
          Pol::rows(coef(0), xa, y0);
          Pol::rows(coef(1), top, y1);
        }
      }
      Pol::mul4(y0, y1, acc);
    }
    // exact power-of-two rescaling of this rate class's vector (each rate
    // class keeps its own scaler; the root aligns them); rare, so the warp
    // only enters when some lane needs it.  An all-zero vector (a site the
    // tree cannot produce) rescales to zeros again and ends as log 0 = -inf.
    auto mx = fmax(fmax(Pol::mag(acc[0]), Pol::mag(acc[1])), fmax(Pol::mag(acc[2]), Pol::mag(acc[3])));
    if (__any_sync(0xffffffffu, mx < Pol::thresh)) {
      if (mx < Pol::thresh) {
        const int ex = frexp_exp(mx);
        escale += ex;
        // two steps when the largest entry is subnormal, so each factor
        // stays a normal power of two
        const int k1 = min(-ex, 120), k2 = -ex - k1;
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] = Pol::scale(acc[e], k1);
        if (k2 > 0) {
#pragma unroll
          for (int e = 0; e < 4; ++e) acc[e] = Pol::scale(acc[e], k2);
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) top[e] = acc[e];
    }
    // this warp is done with the group's step slots
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
  if (active && r == 0 && rate_on && code_max >= (uint32_t)NC) atomicOr(p.flag, PGPU_FLAG_BADCODE);

  // root: sum over rate classes of probs[r] 2^e_r sum_i pi_i x_i, in FP64;
  // the rate classes of a pattern meet in shared memory
  double part = 0.0;
  if (ok && rate_on) {
    const double *pi = p.pi + (size_t)blockIdx.y * 4, *probs = p.probs + (size_t)blockIdx.y * R;
    double lr = 0.0;
#pragma unroll
    for (int e = 0; e < 4; ++e) lr += pi[e] * Pol::to_d(top[e]);
    part = probs[r] * lr;
  }
  xch[r][pl] = make_double2(part, (double)escale);
  asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
  double s = 0.0, comp = 0.0;
  if (r == 0) {
    int emax = -0x7fffffff;
    for (int q = 0; q < R; ++q) emax = max(emax, (int)xch[q][pl].y);
    double site = 0.0;
    for (int q = 0; q < R; ++q) {
      const double2 v = xch[q][pl];
      site += ldexp(v.x, (int)v.y - emax);
    }
    if (ok && active) {
      const double lnl = log(site) + (double)emax * 0.69314718055994530942;
      if (p.site_lnl) p.site_lnl[pat] = lnl;
      s = p.weights ? p.weights[pat] * lnl : lnl;
    }
  }
  warp_csum(s, comp);
  const int cw = c >> 5;
  if (lane == 0) red[cw] = make_double2(s, comp);
  asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
  if (cw == 0) {
    double2 v = lane < NT / 32 ? red[lane] : make_double2(0.0, 0.0);
    double ss = v.x, cc = v.y;
    warp_csum(ss, cc);
    if (lane == 0) p.partials[(size_t)blockIdx.y * p.n_tiles_total + tile] = make_double2(ss, cc);
  }
}

// Neumaier sum of the per-CTA (sum, compensation) pairs in CTA order, one
// CTA per model.
__global__ void __launch_bounds__(1024) prune_finalize_kernel(const double2 *partials, int n,
                                                             double *out) {
  const double v = csum_block<1024>(partials + (size_t)blockIdx.x * n, n);
  if (threadIdx.x == 0) out[blockIdx.x] = v;
}

template <typename Pol, int RT>
pgpu_status launch_prune_rt(pgpu_ctx *ctx, PruneArgs &a, size_t n_tiles, size_t smem, int n_models,
                            cudaStream_t stream) {
  PGPU_CUDA(ctx, cudaFuncSetAttribute(prune_tree_kernel<Pol, RT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
  prune_tree_kernel<Pol, RT><<<dim3((unsigned)n_tiles, (unsigned)n_models), 32 + PR_THREADS, smem,
                               stream>>>(a);
  return pgpu_after_launch(ctx, "prune_tree_kernel");
}

// Tip codes still in host memory: copied column chunk by column chunk on
// the context's copy stream, each chunk's launch waiting only for its own
// columns, so the copy of chunk k + 1 overlaps the scoring of chunk k.
struct HostTips {
  const uint8_t *host;   // [n_tips][n_pat]
  uint8_t *dev;          // [n_tips][ld_pat]
  size_t n_tips;
};

// The launches of one scoring: tile ranges [bounds[k], bounds[k + 1]).
struct ChunkPlan {
  size_t bounds[PGPU_COPY_CHUNKS + 1];
  int K;
  size_t smem;
};

// Column chunks for tip codes in host memory: the first chunk is one wave
// of CTAs (the one copy the scoring cannot hide), each next one
// PruneTune::growth times the last, so a chunk's copy ends while the chunk
// before it is scored and few launch boundaries drain the GPU; whole waves
// keep every launch but the last free of a part-filled wave.  Tip codes
// already on the device: one launch.
template <typename Pol, int RT>
pgpu_status plan_chunks_rt(pgpu_ctx *ctx, size_t n_tiles, int n_models, bool host, ChunkPlan &pl) {
  pl.K = 0;
  pl.bounds[0] = 0;
  if (host) {
    PGPU_CUDA(ctx, cudaFuncSetAttribute(prune_tree_kernel<Pol, RT>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)std::max<size_t>(pl.smem, 48 * 1024)));
    int per_sm = 0;
    PGPU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prune_tree_kernel<Pol, RT>,
                                                                 32 + PR_THREADS, pl.smem));
    const size_t wave =
        std::max<size_t>((size_t)std::max(per_sm, 1) * (size_t)ctx->num_sms / (size_t)std::max(n_models, 1), 1);
    size_t t = 0, c = wave;
    while (pl.K < PGPU_COPY_CHUNKS - 1 && n_tiles - t >= c + wave) {
      t += c;
      pl.bounds[++pl.K] = t;
      c *= PruneTune<Pol>::growth;
    }
  }
  pl.bounds[++pl.K] = n_tiles;
  return PGPU_OK;
}

// Sets a's tiling and plans its launches.  With the tip codes in host
// memory it also queues every chunk's copy on the copy stream, chunk k's
// end marked by copy_ev[k], so that the first copy runs beside the model
// setup kernels queued after it.
template <typename Pol>
pgpu_status plan_prune(pgpu_ctx *ctx, PruneArgs &a, int RT, int n_models, const HostTips *ht, ChunkPlan &pl) {
  a.NP = PR_THREADS / RT;
  const size_t n_tiles = (a.n_pat + a.NP - 1) / a.NP;
  a.n_tiles_total = n_tiles;
  a.tile_base = 0;
  pl.smem = PruneLayout<Pol>::bytes(a.NP, a.R, a.n_codes, a.depth);
  if (pl.smem > ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "prune: %zu bytes of shared memory needed (tree too deep)",
                        pl.smem);
  const bool host = ht != nullptr;
  switch (RT) {
    case 1: PGPU_TRY((plan_chunks_rt<Pol, 1>(ctx, n_tiles, n_models, host, pl))); break;
    case 2: PGPU_TRY((plan_chunks_rt<Pol, 2>(ctx, n_tiles, n_models, host, pl))); break;
    case 4: PGPU_TRY((plan_chunks_rt<Pol, 4>(ctx, n_tiles, n_models, host, pl))); break;
    default: PGPU_TRY((plan_chunks_rt<Pol, 8>(ctx, n_tiles, n_models, host, pl))); break;
  }
  if (host)
    for (int k = 0; k < pl.K; ++k) {
      const size_t c0 = pl.bounds[k] * a.NP, c1 = std::min(pl.bounds[k + 1] * a.NP, a.n_pat);
      if (c1 > c0)
        PGPU_CUDA(ctx, cudaMemcpy2DAsync(ht->dev + c0, a.ld_pat, ht->host + c0, a.n_pat, c1 - c0, ht->n_tips,
                                         cudaMemcpyHostToDevice, ctx->copy_stream));
      PGPU_CUDA(ctx, cudaEventRecord(ctx->copy_ev[k], ctx->copy_stream));
    }
  return PGPU_OK;
}

// With several chunks, consecutive launches alternate between the context
// stream and the auxiliary one, so a chunk's CTAs take the SMs the previous
// chunk's CTAs leave instead of waiting for the whole launch to drain (the
// tiles are disjoint; each launch waits only for its own columns).
template <typename Pol, int RT>
pgpu_status launch_prune_chunks(pgpu_ctx *ctx, PruneArgs &a, const ChunkPlan &pl, int n_models, bool host) {
  const bool fork = host && pl.K > 1;
  if (fork) {
    PGPU_CUDA(ctx, cudaEventRecord(ctx->aux_ev[0], ctx->stream));
    PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->aux_ev[0], 0));
  }
  for (int k = 0; k < pl.K; ++k) {
    const cudaStream_t ks = fork && (k & 1) ? ctx->aux_stream : ctx->stream;
    if (host) PGPU_CUDA(ctx, cudaStreamWaitEvent(ks, ctx->copy_ev[k], 0));
    a.tile_base = pl.bounds[k];
    PGPU_TRY((launch_prune_rt<Pol, RT>(ctx, a, pl.bounds[k + 1] - pl.bounds[k], pl.smem, n_models, ks)));
  }
  if (fork) {
    PGPU_CUDA(ctx, cudaEventRecord(ctx->aux_ev[1], ctx->aux_stream));
    PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->aux_ev[1], 0));
  }
  a.tile_base = 0;
  return PGPU_OK;
}

template <typename Pol>
pgpu_status launch_prune(pgpu_ctx *ctx, PruneArgs &a, int RT, int n_models, const ChunkPlan &pl, bool host) {
  switch (RT) {
    case 1: return launch_prune_chunks<Pol, 1>(ctx, a, pl, n_models, host);
    case 2: return launch_prune_chunks<Pol, 2>(ctx, a, pl, n_models, host);
    case 4: return launch_prune_chunks<Pol, 4>(ctx, a, pl, n_models, host);
    default: return launch_prune_chunks<Pol, 8>(ctx, a, pl, n_models, host);
  }
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
using namespace pgpu_forms;

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

Staged stage_layout(int S, int R, int n_codes, int n_br, int V) {
  Staged s{};
  size_t off = 0;
  auto take = [&](size_t n) {
    const size_t o = off;
    off += align16(n * sizeof(double));
    return o;
  };
  s.Q = (double *)take((size_t)V * S * S);
  s.pi = (double *)take((size_t)V * S);
  s.rates = (double *)take((size_t)V * R);
  s.probs = (double *)take((size_t)V * R);
  s.tab = (double *)take((size_t)n_codes * S);
  s.brlen = (double *)take(n_br);
  s.bytes = off;
  return s;
}

template <typename Ptr>
Ptr *rebase(void *base, Ptr *off) {
  return reinterpret_cast<Ptr *>(static_cast<char *>(base) + reinterpret_cast<size_t>(off));
}

// Scores n_models models (same state and rate-class counts) over one tree
// and one set of patterns: lnl_dev[v] for model v.  One eigendecomposition
// launch for all models, a P and a tip-table build per model, then one
// pruning launch whose CTA rows are the models.
// host_tips: the codes are still in host memory (n_pat bytes per row) and
// tips is the device buffer they go to; they are copied in chunks that
// overlap the scoring.
pgpu_status prune_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *models, int n_models,
                      const pgpu_tip_codes *codes, const uint8_t *tips, size_t ld_pat,
                      const double *weights, size_t n_pat, int precision, double *lnl_dev,
                      double *site_lnl_dev, const uint8_t *host_tips = nullptr) {
  if (!models || n_models < 1) return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: no model");
  if (n_models > 65535) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "prune: at most 65,535 models per call");
  for (int v = 0; v < n_models; ++v) {
    PGPU_TRY(check_model(ctx, &models[v], codes));
    if (models[v].n_rates != models[0].n_rates)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: every model needs the same number of rate classes");
  }
  if (n_models > 1 && site_lnl_dev)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: site log-likelihoods are for one model at a time");
  if (precision != 32 && precision != 48 && precision != 64)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: precision must be 32, 48 or 64");
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
  const int V = n_models;
  const int S = models[0].n_states, R = models[0].n_rates, n = tree->n_tips, n_br = 2 * n - 2;
  for (int i = 0; i < n_br; ++i)
    if (!(tree->brlen[i] >= 0.0) || !std::isfinite(tree->brlen[i]))
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: branch length %d is negative or not finite", i);

  // stage every model's Q, pi, rates, probs, then the code table and the
  // branch lengths
  Staged lay = stage_layout(S, R, codes->n_codes, n_br, V);
  void *h, *d;
  PGPU_TRY(pgpu_stage(ctx, lay.bytes, &h, &d));
  for (int v = 0; v < V; ++v) {
    const pgpu_model *m = &models[v];
    std::copy(m->Q, m->Q + S * S, rebase(h, lay.Q) + (size_t)v * S * S);
    std::copy(m->pi, m->pi + S, rebase(h, lay.pi) + (size_t)v * S);
    std::copy(m->rates, m->rates + R, rebase(h, lay.rates) + (size_t)v * R);
    std::copy(m->probs, m->probs + R, rebase(h, lay.probs) + (size_t)v * R);
  }
  std::copy(codes->table, codes->table + (size_t)codes->n_codes * S, rebase(h, lay.tab));
  std::copy(tree->brlen, tree->brlen + n_br, rebase(h, lay.brlen));
  PGPU_TRY(pgpu_stage_commit(ctx, lay.bytes));

  // device scratch: eigen systems, P matrices, tip rows, per-CTA partial sums
  const int RT = R <= 1 ? 1 : R <= 2 ? 2 : R <= 4 ? 4 : 8;
  const size_t n_tiles = (n_pat + (PR_THREADS / RT) - 1) / (PR_THREADS / RT);
  const size_t SS = (size_t)S * S;
  const size_t coef = precision == 32 ? 4 : 8;   // float, double, or float pair
  const size_t p_bytes = align16((size_t)n_br * R * SS * coef);
  const size_t tt_bytes =
      align16((size_t)n * R * codes->n_codes * S * (precision == 32 ? 4 : 8));
  void *deig, *dP, *dpart, *dtt;
  PGPU_TRY(pgpu_buf(ctx, BUF_H, (size_t)V * (2 * SS + S) * 8 + (size_t)V * sizeof(int) + 64, &deig));
  PGPU_TRY(pgpu_buf(ctx, BUF_I, (size_t)V * p_bytes, &dP));
  PGPU_TRY(pgpu_buf(ctx, BUF_G, std::max<size_t>(n_tiles, 1) * V * sizeof(double2), &dpart));
  PGPU_TRY(pgpu_buf(ctx, BUF_J, (size_t)V * tt_bytes, &dtt));
  double *dU = (double *)deig, *dUi = dU + V * SS, *dlam = dUi + V * SS;
  int *dst = reinterpret_cast<int *>(dlam + (size_t)V * S);
  PruneArgs a;
  a.tiptab = dtt;
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
  a.P_stride = p_bytes;
  a.tab_stride = tt_bytes;
  a.ld_pat = ld_pat;
  a.n_pat = n_pat;
  a.n_tips = n;
  a.n_ops = (int)sch->ops.size();
  a.n_codes = codes->n_codes;
  a.R = R;
  a.NP = 0;
  a.depth = std::max(sch->max_depth, 1);
  HostTips ht{host_tips, const_cast<uint8_t *>(tips), (size_t)n};
  const HostTips *htp = host_tips ? &ht : nullptr;
  ChunkPlan pl;
  if (n_pat > 0) {
    if (precision == 32) PGPU_TRY(plan_prune<Fp32>(ctx, a, RT, V, htp, pl));
    else if (precision == 48) PGPU_TRY(plan_prune<Ff32>(ctx, a, RT, V, htp, pl));
    else PGPU_TRY(plan_prune<Fp64>(ctx, a, RT, V, htp, pl));
  }
  PGPU_TRY(pgpu_launch_eig(ctx, rebase(d, lay.Q), rebase(d, lay.pi), S, V, dU, dlam, dUi, dst));
  // every model's P matrices, then every model's tip rows in FP64, stored in
  // the form's value type: one launch each for all V models
  PGPU_TRY(pgpu_launch_compose(ctx, dU, dlam, dUi, S, rebase(d, lay.brlen), n_br,
                               rebase(d, lay.rates), R, precision == 64 ? (double *)dP : nullptr,
                               precision == 64 ? nullptr : (float *)dP, false, dst,
                               precision == 32 ? P32_MINUS_I : precision == 48 ? P32_PAIRS_ROWS4
                                                                               : P32_PLAIN,
                               V, p_bytes));
  PGPU_TRY(pgpu_launch_tip_table(ctx, dU, dlam, dUi, S, rebase(d, lay.brlen), n,
                                 rebase(d, lay.rates), R, rebase(d, lay.tab), codes->n_codes, dtt,
                                 precision == 32 ? 0 : precision == 48 ? 3 : 2, dst, V, tt_bytes));
  if (n_pat == 0) {
    PGPU_CUDA(ctx, cudaMemsetAsync(lnl_dev, 0, (size_t)V * sizeof(double), ctx->stream));
    return PGPU_OK;
  }
  if (precision == 32) PGPU_TRY(launch_prune<Fp32>(ctx, a, RT, V, pl, htp != nullptr));
  else if (precision == 48) PGPU_TRY(launch_prune<Ff32>(ctx, a, RT, V, pl, htp != nullptr));
  else PGPU_TRY(launch_prune<Fp64>(ctx, a, RT, V, pl, htp != nullptr));
  prune_finalize_kernel<<<V, 1024, 0, ctx->stream>>>((const double2 *)dpart, (int)n_tiles, lnl_dev);
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
  return prune_dev(ctx, tree, model, 1, codes, tip_codes_dev, ld_pat, weights_dev, n_pat, precision,
                   lnl_dev, site_lnl_dev);
}

pgpu_status pgpu_prune_lnl_models_dev(pgpu_ctx *ctx, const pgpu_tree *tree,
                                      const pgpu_model *models, int n_models,
                                      const pgpu_tip_codes *codes, const uint8_t *tip_codes_dev,
                                      size_t ld_pat, const double *weights_dev, size_t n_pat,
                                      int precision, double *lnl_dev) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  return prune_dev(ctx, tree, models, n_models, codes, tip_codes_dev, ld_pat, weights_dev, n_pat,
                   precision, lnl_dev, nullptr);
}

pgpu_status pgpu_prune_lnl_models(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *models,
                                  int n_models, const pgpu_tip_codes *codes,
                                  const uint8_t *tip_codes, const double *weights, size_t n_pat,
                                  int precision, double *lnl) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!tree || tree->n_tips < 2 || !tip_codes || !lnl || n_models < 1)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "prune: null argument, no model or fewer than 2 tips");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t n = (size_t)tree->n_tips;
  const size_t ld = (n_pat + 15) / 16 * 16;
  void *dt, *dw = nullptr, *dl;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, std::max<size_t>(n * ld, 16), &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, std::max<size_t>((size_t)n_models * 8, 64), &dl));
  if (weights) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n_pat * 8, &dw));
  cudaStream_t s = ctx->stream;
  if (n_pat) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(dt, ld, tip_codes, n_pat, n_pat, n, cudaMemcpyHostToDevice, s));
    if (weights) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_pat * 8, cudaMemcpyHostToDevice, s));
  }
  PGPU_TRY(prune_dev(ctx, tree, models, n_models, codes, (const uint8_t *)dt, ld,
                     (const double *)dw, n_pat, precision, (double *)dl, nullptr));
  PGPU_CUDA(ctx, cudaMemcpyAsync(lnl, dl, (size_t)n_models * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  PGPU_TRY(pgpu_check_flag(ctx, "prune"));
  return PGPU_OK;
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
  // the tip codes go over in column chunks on the copy stream, after
  // everything already queued on the context's stream (which may still read
  // the device buffer), each chunk's scoring waiting for its own columns
  PGPU_TRY(pgpu_copy_stream(ctx));
  PGPU_CUDA(ctx, cudaEventRecord(ctx->copy_ev[PGPU_COPY_CHUNKS], s));
  PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[PGPU_COPY_CHUNKS], 0));
  // the weights go first on the copy stream: the first chunk's event covers them
  if (n_pat && weights)
    PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_pat * 8, cudaMemcpyHostToDevice, ctx->copy_stream));
  PGPU_TRY(pgpu_settle_copies(ctx, prune_dev(ctx, tree, model, 1, codes, (const uint8_t *)dt, ld,
                                              (const double *)dw, n_pat, precision, (double *)dl,
                                              (double *)dsl, tip_codes)));
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
