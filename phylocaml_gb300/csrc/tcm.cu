// Cost-matrix (TCM) medians of state sets over a tree.
//
// Reference: CostMatrix.Make (lib/costMatrix.ml:124-196) tabulates, for a
// bit-flag alphabet and a transformation cost matrix of its atomic states,
// the median cost and median code of every pair of state-set codes
// (fill_cm, :141-166) with one of three median rules chosen by the matrix's
// declared properties (:145-149): find_median_general (:68-86),
// find_median_metric (:104-122) or find_median_equal (:89-101).  A tree's
// cost under such a character is the postorder of Node.Make1D.median_2
// (lib/node.ml:183-198): each internal node takes the table's median of its
// children's codes and adds the table's cost.  With the unit matrix the
// table is Fitch's rule (test/costMatrixTest.ml:83-108).
//
// GPU layout: DNA-sized alphabets (at most 4 states) as 4-bit lanes, eight
// sites per 32-bit word, like the Fitch kernels.  One thread owns one word
// column and walks the whole postorder; the table is packed
// (cost << 4 | median code, bit 31 = "pair has no median", i.e. an empty or
// out-of-alphabet code) and replicated once per lane in shared memory
// (entry e of lane l at [e][l]), so a warp's 32 lookups never share a bank.
// The top of the node stack stays in a register; pushes and pops follow the
// schedule's fixed discipline (a step with two tip children sets the last
// result aside, one with two internal children takes its first child back).
#include <algorithm>
#include <cstring>

#include "pgpu_internal.cuh"

namespace {

constexpr int TC_THREADS = 256;
constexpr uint32_t TC_NONE = 0x80000000u;      // pair without a median
constexpr uint32_t TC_COST_MASK = 0x07ffffffu;  // cost field (bits 4..30)
constexpr int32_t TC_ENTRY_MAX = 1 << 25;       // per TCM entry, so a pair sum fits the field

struct TcmArgs {
  const uint32_t *tips;      // [n_tips][ld]
  const uint32_t *weights;   // [n_sites] or null
  const uint32_t *table;     // [256] packed entries, index (a << 4) | b
  const int4 *ops;           // schedule (k, first, second, -)
  uint32_t *node_sets;       // [n_tips - 1][ld]
  uint32_t *site_cost;       // [n_sites] or null
  unsigned long long *total;
  int *flag;
  size_t ld, n_words, n_sites;
  int n_tips, n_ops, depth;
};

__device__ __forceinline__ uint32_t valid4(size_t w, size_t n_sites) {
  const size_t first = w * 8;
  if (first + 8 <= n_sites) return 0xffffffffu;
  if (first >= n_sites) return 0u;
  return (1u << (4 * int(n_sites - first))) - 1u;
}

__global__ void __launch_bounds__(TC_THREADS) tcm_tree_kernel(const TcmArgs a) {
  __shared__ uint32_t tab[256 * 32];
  __shared__ unsigned long long red[TC_THREADS / 32];
  extern __shared__ uint32_t stk[];   // [depth][TC_THREADS]
  const int t = threadIdx.x, lane = t & 31;
  for (int i = t; i < 256 * 32; i += TC_THREADS) tab[i] = __ldg(a.table + (i >> 5));
  __syncthreads();
  const size_t w = (size_t)blockIdx.x * TC_THREADS + t;
  const bool on = w < a.n_words;
  const uint32_t valid = on ? valid4(w, a.n_sites) : 0u;
  const uint32_t fill = 0x11111111u & ~valid;   // lanes past the last site read as state 1
  const uint32_t *tb = tab + lane;
  auto tip = [&](int ch) -> uint32_t {
    const uint32_t x = on ? __ldg(a.tips + (size_t)ch * a.ld + w) : 0u;
    return (x & valid) | fill;
  };
  uint32_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t top = 0, none = 0;
  int sp = 0;
  bool ok = true;
  for (int i = 0; i < a.n_ops && ok; ++i) {
    const int4 op = __ldg(a.ops + i);
    const int kind = (op.y >= a.n_tips ? 1 : 0) | (op.z >= a.n_tips ? 2 : 0);
    uint32_t xa, xb;
    if (kind == 0) {   // two tips: the previous result waits on the stack
      if (i > 0) {
        if (sp < a.depth) stk[sp++ * TC_THREADS + t] = top;
        else ok = false;
      }
      xa = tip(op.y);
      xb = tip(op.z);
    } else if (kind == 1) {   // the first child is the previous result
      xa = top;
      xb = tip(op.z);
    } else if (kind == 2) {   // the second child is the previous result
      xa = tip(op.y);
      xb = top;
    } else {                  // both internal: the first from the stack
      if (sp > 0) {
        xa = stk[--sp * TC_THREADS + t];
      } else {
        ok = false;
        xa = 0x11111111u;
      }
      xb = top;
    }
    uint32_t out = 0;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const uint32_t ia = (xa >> (4 * l)) & 15u, ib = (xb >> (4 * l)) & 15u;
      const uint32_t e = tb[((ia << 4) | ib) << 5];
      out |= (e & 15u) << (4 * l);
      cnt[l] += e >> 4;   // a no-median entry fails the call, so its bit 31 never matters
      none |= e;
    }
    if (on) a.node_sets[(size_t)op.x * a.ld + w] = out & valid;
    top = out;
  }
  unsigned long long tot = 0;
  if (on && ok) {
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const size_t s = w * 8 + l;
      if (s < a.n_sites) {
        if (a.site_cost) a.site_cost[s] = cnt[l];
        tot += (unsigned long long)(a.weights ? __ldg(a.weights + s) : 1u) * cnt[l];
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (lane == 0) red[t >> 5] = tot;
  if (__any_sync(0xffffffffu, (none & TC_NONE) != 0) && lane == 0) atomicOr(a.flag, PGPU_FLAG_BADCODE);
  __syncthreads();
  if (t == 0) {
    unsigned long long s = 0;
    for (int k = 0; k < TC_THREADS / 32; ++k) s += red[k];
    if (s) atomicAdd(a.total, s);
  }
}

// ---- wide alphabets: medians formed on the fly ----------------------------
// For alphabets of up to 32 atomic states (codes of 8, 16 or 32 bits, one
// site per lane) a table over every pair of codes no longer fits, so each
// node forms its medians from the TCM itself, held transposed in shared
// memory (tT[k][x] = tcm[x][k]).  find_median_general / _metric
// (lib/costMatrix.ml:68-86, 104-122) take, over every atomic pair (a, b) of
// the two codes, the candidates k minimising tcm[a][k] + tcm[b][k], and keep
// the pairs reaching the overall minimum.  That is the same as
//   best = min_k (C_i[k] + C_j[k]),  C_i[k] = min_{a in i} tcm[a][k],
//   code = OR of the k reaching it,
// over all k (general) or the states of i | j (metric): a pair's minimum is
// never below best, and reaches it exactly where some k does.
// find_median_equal (:89-101) intersects at tcm[0][0] or unites at
// tcm[0][1].  A TCM declared symmetric has its table filled for i <= j and
// mirrored (:150-156), so the codes are ordered first.
struct TcmWideArgs {
  const uint32_t *tips;      // [n_tips][ld] lanes of LB bits
  const uint32_t *weights;   // [n_sites] or null
  const uint32_t *tcmT;      // [S][S] transposed costs
  const int4 *ops;
  uint32_t *node_sets;
  uint32_t *site_cost;
  unsigned long long *total;
  int *flag;
  size_t ld, n_words, n_sites;
  int n_tips, n_ops, depth, S, mode, symmetric;
};

template <int LB>
__device__ __forceinline__ uint32_t wide_median(const uint32_t *tT, int S, int mode, int sym,
                                                uint32_t a, uint32_t b, uint32_t &cost,
                                                bool &none) {
  const uint32_t all = S == 32 ? 0xffffffffu : (1u << S) - 1u;
  if (a == 0u || b == 0u || (a & ~all) || (b & ~all)) {
    none = true;
    cost = 0;
    return 0u;
  }
  if (sym && a > b) {
    const uint32_t t = a;
    a = b;
    b = t;
  }
  if (mode == PGPU_TCM_EQUAL) {
    const uint32_t inter = a & b;
    cost = inter ? tT[0] : tT[1 * S + 0];   // tcm[0][0] or tcm[0][1]
    return inter ? inter : (a | b);
  }
  const uint32_t cand = mode == PGPU_TCM_METRIC ? (a | b) : all;
  uint32_t best = 0xffffffffu, code = 0u;
  for (int k = 0; k < S; ++k) {
    if (!((cand >> k) & 1u)) continue;
    const uint32_t *row = tT + k * S;
    uint32_t ca = 0xffffffffu, cb = 0xffffffffu;
    for (uint32_t m = a; m; m &= m - 1) ca = min(ca, row[__ffs(m) - 1]);
    for (uint32_t m = b; m; m &= m - 1) cb = min(cb, row[__ffs(m) - 1]);
    const uint32_t c = ca + cb;
    if (c < best) {
      best = c;
      code = 1u << k;
    } else if (c == best) {
      code |= 1u << k;
    }
  }
  cost = best;
  return code;
}

template <int LB>
__global__ void __launch_bounds__(TC_THREADS) tcm_wide_kernel(const TcmWideArgs a) {
  constexpr int PER = 32 / LB;
  constexpr uint32_t LMASK = LB == 32 ? 0xffffffffu : (1u << LB) - 1u;
  __shared__ uint32_t tT[32 * 32];
  __shared__ unsigned long long red[TC_THREADS / 32];
  extern __shared__ uint32_t stk[];   // [depth][TC_THREADS]
  const int t = threadIdx.x, lane = t & 31;
  for (int i = t; i < a.S * a.S; i += TC_THREADS) tT[i] = __ldg(a.tcmT + i);
  __syncthreads();
  const size_t w = (size_t)blockIdx.x * TC_THREADS + t;
  const bool on = w < a.n_words;
  // lanes past the last site read as atomic state 0, which always has a
  // median, and are written as zero
  uint32_t valid = 0u;
  if (on) {
#pragma unroll
    for (int l = 0; l < PER; ++l)
      if (w * PER + l < a.n_sites) valid |= LMASK << (l * LB);
  }
  uint32_t fill = 0u;
#pragma unroll
  for (int l = 0; l < PER; ++l) fill |= 1u << (l * LB);
  fill &= ~valid;
  auto tip = [&](int ch) -> uint32_t {
    const uint32_t x = on ? __ldg(a.tips + (size_t)ch * a.ld + w) : 0u;
    return (x & valid) | fill;
  };
  uint32_t cnt[PER];
#pragma unroll
  for (int l = 0; l < PER; ++l) cnt[l] = 0;
  uint32_t top = 0;
  int sp = 0;
  bool ok = true, none = false;
  for (int i = 0; i < a.n_ops && ok; ++i) {
    const int4 op = __ldg(a.ops + i);
    const int kind = (op.y >= a.n_tips ? 1 : 0) | (op.z >= a.n_tips ? 2 : 0);
    uint32_t xa, xb;
    if (kind == 0) {
      if (i > 0) {
        if (sp < a.depth) stk[sp++ * TC_THREADS + t] = top;
        else ok = false;
      }
      xa = tip(op.y);
      xb = tip(op.z);
    } else if (kind == 1) {
      xa = top;
      xb = tip(op.z);
    } else if (kind == 2) {
      xa = tip(op.y);
      xb = top;
    } else {
      if (sp > 0) {
        xa = stk[--sp * TC_THREADS + t];
      } else {
        ok = false;
        xa = fill;
      }
      xb = top;
    }
    uint32_t out = 0;
#pragma unroll
    for (int l = 0; l < PER; ++l) {
      uint32_t c;
      bool nm = false;
      const uint32_t m = wide_median<LB>(tT, a.S, a.mode, a.symmetric, (xa >> (l * LB)) & LMASK,
                                         (xb >> (l * LB)) & LMASK, c, nm);
      out |= m << (l * LB);
      cnt[l] += c;
      none |= nm;
    }
    out = (out & valid) | fill;
    if (on) a.node_sets[(size_t)op.x * a.ld + w] = out & valid;
    top = out;
  }
  unsigned long long tot = 0;
  if (on && ok) {
#pragma unroll
    for (int l = 0; l < PER; ++l) {
      const size_t s = w * PER + l;
      if (s < a.n_sites) {
        if (a.site_cost) a.site_cost[s] = cnt[l];
        tot += (unsigned long long)(a.weights ? __ldg(a.weights + s) : 1u) * cnt[l];
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (lane == 0) red[t >> 5] = tot;
  if (__any_sync(0xffffffffu, none) && lane == 0) atomicOr(a.flag, PGPU_FLAG_BADCODE);
  if (!ok) atomicOr(a.flag, PGPU_FLAG_BADCODE);
  __syncthreads();
  if (t == 0) {
    unsigned long long s2 = 0;
    for (int k = 0; k < TC_THREADS / 32; ++k) s2 += red[k];
    if (s2) atomicAdd(a.total, s2);
  }
}

// ---- the table (host): restates fill_cm and the three median rules ----

int64_t tcm_cost(const int32_t *tcm, int S, uint32_t x, uint32_t y) {   // x, y atomic codes
  return tcm[(31 - __builtin_clz(x)) * S + (31 - __builtin_clz(y))];
}

// find_median_pair (lib/costMatrix.ml:57-66)
void median_pair(const int32_t *tcm, int S, uint32_t i, uint32_t j, uint32_t candidates,
                 int64_t *cost, uint32_t *code) {
  int64_t best = INT64_MAX;
  uint32_t assign = 0;
  for (int b = 0; b < S; ++b) {
    const uint32_t k = 1u << b;
    if (!(candidates & k)) continue;
    const int64_t c = tcm_cost(tcm, S, i, k) + tcm_cost(tcm, S, j, k);
    if (c == best) assign |= k;
    else if (c < best) best = c, assign = k;
  }
  *cost = best;
  *code = assign;
}

// find_median_general / _metric / _equal (lib/costMatrix.ml:68-122), codes
// of up to 32 atomic states
void median(const int32_t *tcm, int S, int mode, uint32_t i, uint32_t j, int64_t *cost,
            uint32_t *code) {
  const uint32_t all = S == 32 ? 0xffffffffu : (1u << S) - 1u;
  if (mode == PGPU_TCM_EQUAL) {
    const int64_t unequal = tcm_cost(tcm, S, 1, 2), equal = tcm_cost(tcm, S, 1, 1);
    if (i & j) *cost = equal, *code = i & j;
    else *cost = unequal, *code = i | j;
    return;
  }
  const uint32_t cand = mode == PGPU_TCM_METRIC ? (i | j) : all;
  int64_t best = INT64_MAX;
  uint32_t assign = 0;
  for (int bi = 0; bi < S; ++bi) {
    if (!(i >> bi & 1u)) continue;
    for (int bj = 0; bj < S; ++bj) {
      if (!(j >> bj & 1u)) continue;
      int64_t c;
      uint32_t k;
      median_pair(tcm, S, 1u << bi, 1u << bj, cand, &c, &k);
      if (c == best) assign |= k;
      else if (c < best) best = c, assign = k;
    }
  }
  *cost = best;
  *code = assign;
}

// io: the rows are still in host memory (see HostRows); the segmented
// kernel copies them in chunks, the single-walk kernel whole.
pgpu_status tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips, size_t ld,
                     const uint32_t *weights, size_t n_sites, const uint32_t *table,
                     uint32_t *node_sets, uint32_t *site_cost, unsigned long long *total,
                     const HostRows *io = nullptr) {
  if (!tree || tree->n_tips < 2) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree: need at least 2 tips");
  if (!tips || !node_sets || !total || !table) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree: null buffer");
  const size_t n_words = (n_sites + 7) / 8;
  if (ld < n_words) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree: ld_words (%zu) < %zu", ld, n_words);
  // every site's cost sum must fit uint32
  uint64_t emax = 0;
  for (int e = 0; e < 256; ++e)
    if (!(table[e] & TC_NONE)) emax = std::max<uint64_t>(emax, (table[e] >> 4) & TC_COST_MASK);
  if (emax * (uint64_t)(tree->n_tips - 1) > 0xffffffffull)
    return pgpu_set_err(ctx, PGPU_ERR_OVERFLOW,
                        "tcm_tree: a site's cost can reach %llu x %d, above 2^32 - 1",
                        (unsigned long long)emax, tree->n_tips - 1);
  const TreeSchedule *sch;
  const int4 *d_ops;
  const int32_t *d_seq;
  PGPU_TRY(pgpu_schedule_device(ctx, tree, &sch, &d_ops, &d_seq));
  void *h, *d;
  PGPU_TRY(pgpu_stage(ctx, 256 * sizeof(uint32_t), &h, &d));
  std::memcpy(h, table, 256 * sizeof(uint32_t));
  PGPU_TRY(pgpu_stage_commit(ctx, 256 * sizeof(uint32_t)));
  PGPU_CUDA(ctx, cudaMemsetAsync(total, 0, sizeof(unsigned long long), ctx->stream));
  if (n_words == 0) return PGPU_OK;
  // the segmented schedule: subtrees walked by four warps per 128-word slice.
  // It sums costs in the low 28 bits of a register under the codes' top 4,
  // flushing every p steps so that a site's sum, at most p * emax, stays
  // below 2^28; below 16 steps between flushes it keeps one sum per register.
  const uint64_t per = ((1ull << 28) - 1) / std::max<uint64_t>(emax, 1);
  const int period = per >= 16 ? (int)std::min<uint64_t>(per, 1u << 30) : 0;
  bool launched = false;
  PGPU_TRY(pgpu_tcm_tree_split(ctx, tree, tips, ld, weights, n_sites,
                               static_cast<const uint32_t *>(d), period, node_sets, site_cost, total,
                               &launched, io));
  if (launched) return PGPU_OK;
  const size_t n = (size_t)tree->n_tips;
  if (io)
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(const_cast<uint32_t *>(tips), ld * 4, io->tips, n_words * 4, n_words * 4,
                                     n, cudaMemcpyHostToDevice, ctx->stream));
  TcmArgs a;
  a.tips = tips;
  a.weights = weights;
  a.table = static_cast<const uint32_t *>(d);
  a.ops = d_ops;
  a.node_sets = node_sets;
  a.site_cost = site_cost;
  a.total = total;
  a.flag = ctx->d_flag;
  a.ld = ld;
  a.n_words = n_words;
  a.n_sites = n_sites;
  a.n_tips = tree->n_tips;
  a.n_ops = (int)sch->ops.size();
  a.depth = std::max(sch->max_depth, 1);
  const size_t smem = (size_t)a.depth * TC_THREADS * sizeof(uint32_t);
  if (smem + sizeof(uint32_t) * 256 * 32 > (size_t)ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "tcm_tree: tree too deep (%d stack entries)", a.depth);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(tcm_tree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const unsigned grid = (unsigned)((n_words + TC_THREADS - 1) / TC_THREADS);
  tcm_tree_kernel<<<grid, TC_THREADS, smem, ctx->stream>>>(a);
  PGPU_TRY(pgpu_after_launch(ctx, "tcm_tree_kernel"));
  if (io)
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(io->node_sets, n_words * 4, node_sets, ld * 4, n_words * 4, n - 1,
                                     cudaMemcpyDeviceToHost, ctx->stream));
  return PGPU_OK;
}

pgpu_status tree_wide_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips, size_t ld,
                          const uint32_t *weights, size_t n_sites, int lb, const int32_t *tcm,
                          int S, int mode, int symmetric, uint32_t *node_sets, uint32_t *site_cost,
                          unsigned long long *total) {
  if (!tree || tree->n_tips < 2)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: need at least 2 tips");
  if (!tips || !node_sets || !total || !tcm)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: null buffer");
  if (lb != 8 && lb != 16 && lb != 32)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: lane_bits must be 8, 16 or 32");
  if (S < 1 || S > lb)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "tcm_tree_wide: 1..%d states fit %d-bit lanes (got %d)",
                        lb, lb, S);
  if (mode != PGPU_TCM_GENERAL && mode != PGPU_TCM_METRIC && mode != PGPU_TCM_EQUAL)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: unknown median rule %d", mode);
  if (mode == PGPU_TCM_EQUAL && S < 2)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: the equal-cost rule needs two states");
  int64_t emax = 0;
  for (int e = 0; e < S * S; ++e) {
    if (tcm[e] < 0 || tcm[e] > TC_ENTRY_MAX)
      return pgpu_set_err(ctx, PGPU_ERR_LIMIT,
                          "tcm_tree_wide: costs must lie in [0, 2^25] (entry %d is %d)", e, tcm[e]);
    emax = std::max<int64_t>(emax, tcm[e]);
  }
  // a node adds at most two entries (one for the equal rule)
  if ((uint64_t)(2 * emax) * (uint64_t)(tree->n_tips - 1) > 0xffffffffull)
    return pgpu_set_err(ctx, PGPU_ERR_OVERFLOW,
                        "tcm_tree_wide: a site's cost can reach 2 x %lld x %d, above 2^32 - 1",
                        (long long)emax, tree->n_tips - 1);
  const int per = 32 / lb;
  const size_t n_words = (n_sites + per - 1) / per;
  if (ld < n_words)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: ld_words (%zu) < %zu", ld, n_words);
  const TreeSchedule *sch;
  const int4 *d_ops;
  const int32_t *d_seq;
  PGPU_TRY(pgpu_schedule_device(ctx, tree, &sch, &d_ops, &d_seq));
  void *h, *d;
  PGPU_TRY(pgpu_stage(ctx, (size_t)S * S * sizeof(uint32_t), &h, &d));
  uint32_t *tT = static_cast<uint32_t *>(h);
  for (int x = 0; x < S; ++x)
    for (int k = 0; k < S; ++k) tT[k * S + x] = (uint32_t)tcm[x * S + k];
  PGPU_TRY(pgpu_stage_commit(ctx, (size_t)S * S * sizeof(uint32_t)));
  PGPU_CUDA(ctx, cudaMemsetAsync(total, 0, sizeof(unsigned long long), ctx->stream));
  if (n_words == 0) return PGPU_OK;
  TcmWideArgs a;
  a.tips = tips;
  a.weights = weights;
  a.tcmT = static_cast<const uint32_t *>(d);
  a.ops = d_ops;
  a.node_sets = node_sets;
  a.site_cost = site_cost;
  a.total = total;
  a.flag = ctx->d_flag;
  a.ld = ld;
  a.n_words = n_words;
  a.n_sites = n_sites;
  a.n_tips = tree->n_tips;
  a.n_ops = (int)sch->ops.size();
  a.depth = std::max(sch->max_depth, 1);
  a.S = S;
  a.mode = mode;
  a.symmetric = symmetric ? 1 : 0;
  const size_t smem = (size_t)a.depth * TC_THREADS * sizeof(uint32_t);
  if (smem + sizeof(uint32_t) * 32 * 32 > (size_t)ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "tcm_tree_wide: tree too deep (%d stack entries)",
                        a.depth);
  const unsigned grid = (unsigned)((n_words + TC_THREADS - 1) / TC_THREADS);
  cudaError_t e = cudaSuccess;
  switch (lb) {
    case 8:
      e = cudaFuncSetAttribute(tcm_wide_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) tcm_wide_kernel<8><<<grid, TC_THREADS, smem, ctx->stream>>>(a);
      break;
    case 16:
      e = cudaFuncSetAttribute(tcm_wide_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) tcm_wide_kernel<16><<<grid, TC_THREADS, smem, ctx->stream>>>(a);
      break;
    default:
      e = cudaFuncSetAttribute(tcm_wide_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) tcm_wide_kernel<32><<<grid, TC_THREADS, smem, ctx->stream>>>(a);
      break;
  }
  PGPU_CUDA(ctx, e);
  return pgpu_after_launch(ctx, "tcm_wide_kernel");
}

}  // namespace

extern "C" {

pgpu_status pgpu_tcm_median(const int32_t *tcm, int n_states, int mode, int symmetric, uint32_t i,
                            uint32_t j, int64_t *cost, uint32_t *code) {
  if (!tcm || !cost || !code) return PGPU_ERR_ARG;
  const int S = n_states;
  if (S < 1 || S > 32) return PGPU_ERR_LIMIT;
  if (mode != PGPU_TCM_GENERAL && mode != PGPU_TCM_METRIC && mode != PGPU_TCM_EQUAL) return PGPU_ERR_ARG;
  if (mode == PGPU_TCM_EQUAL && S < 2) return PGPU_ERR_ARG;
  const uint64_t all = (S == 32 ? 0xffffffffull : (1ull << S) - 1ull);
  if (i == 0 || j == 0 || (i & ~all) || (j & ~all)) {   // the reference's (inf, 0)
    *cost = INT64_MAX;
    *code = 0;
    return PGPU_OK;
  }
  if (symmetric && i > j) std::swap(i, j);
  int64_t c;
  uint32_t k;
  median(tcm, S, mode, i, j, &c, &k);
  *cost = c;
  *code = k;
  return PGPU_OK;
}

pgpu_status pgpu_tcm_tree_wide_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips_dev,
                                   size_t ld_words, const uint32_t *weights_dev, size_t n_sites,
                                   int lane_bits, const int32_t *tcm, int n_states, int mode,
                                   int symmetric, uint32_t *node_sets_dev, uint32_t *site_cost_dev,
                                   uint64_t *total_dev) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  return tree_wide_dev(ctx, tree, tips_dev, ld_words, weights_dev, n_sites, lane_bits, tcm, n_states,
                       mode, symmetric, node_sets_dev, site_cost_dev,
                       reinterpret_cast<unsigned long long *>(total_dev));
}

pgpu_status pgpu_tcm_tree_wide(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                               const uint32_t *weights, size_t n_sites, int lane_bits,
                               const int32_t *tcm, int n_states, int mode, int symmetric,
                               uint32_t *node_sets, uint32_t *site_cost, uint64_t *total) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!tree || !tips || !node_sets || !total || !tcm)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: null argument");
  if (tree->n_tips < 2) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: need at least 2 tips");
  if (lane_bits != 8 && lane_bits != 16 && lane_bits != 32)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree_wide: lane_bits must be 8, 16 or 32");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const int per = 32 / lane_bits;
  const size_t n_words = (n_sites + per - 1) / per;
  const size_t ld = (n_words + 3) / 4 * 4;
  const size_t n = (size_t)tree->n_tips, n_int = n - 1;
  void *dt, *dn, *dw = nullptr, *dsc = nullptr, *dtot;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, std::max<size_t>(n * ld * 4, 16), &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_OUT, std::max<size_t>(n_int * ld * 4, 16), &dn));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dtot));
  if (weights) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, std::max<size_t>(n_sites * 4, 16), &dw));
  if (site_cost) PGPU_TRY(pgpu_buf(ctx, BUF_SITECOST, std::max<size_t>(n_sites * 4, 16), &dsc));
  cudaStream_t s = ctx->stream;
  if (n_words) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(dt, ld * 4, tips, n_words * 4, n_words * 4, n,
                                     cudaMemcpyHostToDevice, s));
    if (weights) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_sites * 4, cudaMemcpyHostToDevice, s));
  }
  PGPU_TRY(tree_wide_dev(ctx, tree, (const uint32_t *)dt, ld, (const uint32_t *)dw, n_sites,
                         lane_bits, tcm, n_states, mode, symmetric, (uint32_t *)dn, (uint32_t *)dsc,
                         (unsigned long long *)dtot));
  if (n_words) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(node_sets, n_words * 4, dn, ld * 4, n_words * 4, n_int,
                                     cudaMemcpyDeviceToHost, s));
    if (site_cost) PGPU_CUDA(ctx, cudaMemcpyAsync(site_cost, dsc, n_sites * 4, cudaMemcpyDeviceToHost, s));
  }
  uint64_t *ht = reinterpret_cast<uint64_t *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(ht, dtot, 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  PGPU_TRY(pgpu_check_flag(ctx, "tcm_tree_wide"));
  *total = *ht;
  return PGPU_OK;
}


pgpu_status pgpu_tcm_tables(pgpu_ctx *ctx, const int32_t *tcm, int n_states, int mode, int symmetric,
                            uint32_t *table, int64_t *cost, int32_t *assign) {
  if (!tcm || !table) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tables: null argument");
  const int S = n_states;
  if (S < 1 || S > 4)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "tcm_tables: 1..4 states fit the 4-bit lanes (got %d)", S);
  if (mode != PGPU_TCM_GENERAL && mode != PGPU_TCM_METRIC && mode != PGPU_TCM_EQUAL)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tables: unknown median rule %d", mode);
  if (mode == PGPU_TCM_EQUAL && S < 2)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tables: the equal-cost rule needs two states");
  for (int e = 0; e < S * S; ++e)
    if (tcm[e] < 0 || tcm[e] > TC_ENTRY_MAX)
      return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "tcm_tables: costs must lie in [0, 2^25] (entry %d is %d)",
                          e, tcm[e]);
  for (int i = 0; i < 16; ++i)
    for (int j = 0; j < 16; ++j) {
      table[i * 16 + j] = TC_NONE;
      if (cost) cost[i * 16 + j] = INT64_MAX;
      if (assign) assign[i * 16 + j] = 0;
    }
  const int size = 1 << S;
  for (int i = 1; i < size; ++i)
    for (int j = symmetric ? i : 1; j < size; ++j) {
      int64_t c;
      uint32_t k;
      median(tcm, S, mode, (uint32_t)i, (uint32_t)j, &c, &k);
      const uint32_t packed = ((uint32_t)c << 4) | k;
      table[i * 16 + j] = packed;
      if (cost) cost[i * 16 + j] = c;
      if (assign) assign[i * 16 + j] = k;
      if (symmetric) {
        table[j * 16 + i] = packed;
        if (cost) cost[j * 16 + i] = c;
        if (assign) assign[j * 16 + i] = k;
      }
    }
  return PGPU_OK;
}

pgpu_status pgpu_tcm_tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips_dev,
                              size_t ld_words, const uint32_t *weights_dev, size_t n_sites,
                              const uint32_t *table, uint32_t *node_sets_dev, uint32_t *site_cost_dev,
                              uint64_t *total_dev) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  return tree_dev(ctx, tree, tips_dev, ld_words, weights_dev, n_sites, table, node_sets_dev,
                  site_cost_dev, reinterpret_cast<unsigned long long *>(total_dev));
}

pgpu_status pgpu_tcm_tree(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                          const uint32_t *weights, size_t n_sites, const uint32_t *table,
                          uint32_t *node_sets, uint32_t *site_cost, uint64_t *total) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!tree || !tips || !node_sets || !total || !table)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tcm_tree: null argument");
  if (tree->n_tips < 2) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: need at least 2 tips");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t n_words = (n_sites + 7) / 8;
  const size_t ld = (n_words + 3) / 4 * 4;
  const size_t n = (size_t)tree->n_tips, n_int = n - 1;
  void *dw = nullptr, *dsc = nullptr, *dtot;
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dtot));
  if (weights) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n_sites * 4, &dw));
  if (site_cost) PGPU_TRY(pgpu_buf(ctx, BUF_SITECOST, n_sites * 4, &dsc));
  cudaStream_t s = ctx->stream;
  // rows in page-locked host memory the device can address, 16-byte aligned
  // and a multiple of 4 words long: read and written by the kernel over the
  // CPU-GPU link, with no staging buffers
  const uint32_t *tv = nullptr;
  uint32_t *nv = nullptr;
  if (n_words > 0 && n_words % 4 == 0) {
    tv = static_cast<const uint32_t *>(pgpu_host_view(tips));
    nv = static_cast<uint32_t *>(pgpu_host_view(node_sets));
    if (((uintptr_t)tv | (uintptr_t)nv) & 15) tv = nullptr;
  }
  if (tv && nv) {
    if (weights) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_sites * 4, cudaMemcpyHostToDevice, s));
    PGPU_TRY(pgpu_settle_copies(ctx, tree_dev(ctx, tree, tv, n_words, (const uint32_t *)dw, n_sites, table,
                                               nv, (uint32_t *)dsc, (unsigned long long *)dtot)));
    if (site_cost)
      PGPU_CUDA(ctx, cudaMemcpyAsync(site_cost, dsc, n_sites * 4, cudaMemcpyDeviceToHost, s));
    uint64_t *ht = reinterpret_cast<uint64_t *>(ctx->h_pinned);
    PGPU_CUDA(ctx, cudaMemcpyAsync(ht, dtot, 8, cudaMemcpyDeviceToHost, s));
    PGPU_CUDA(ctx, cudaStreamSynchronize(s));
    PGPU_TRY(pgpu_check_flag(ctx, "tcm_tree"));
    *total = *ht;
    return PGPU_OK;
  }
  void *dt, *dn;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, n * ld * 4, &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_OUT, n_int * ld * 4, &dn));
  // the rows go over in column chunks on the copy streams (or whole, where
  // the single-walk kernel runs), after everything already queued on the
  // context's stream
  PGPU_TRY(pgpu_copy_stream(ctx));
  PGPU_CUDA(ctx, cudaEventRecord(ctx->copy_ev[PGPU_COPY_CHUNKS], s));
  PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[PGPU_COPY_CHUNKS], 0));
  PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->d2h_stream, ctx->copy_ev[PGPU_COPY_CHUNKS], 0));
  if (n_words && weights)
    PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_sites * 4, cudaMemcpyHostToDevice, s));
  const HostRows io{tips, node_sets};
  PGPU_TRY(pgpu_settle_copies(ctx, tree_dev(ctx, tree, (const uint32_t *)dt, ld, (const uint32_t *)dw,
                                             n_sites, table, (uint32_t *)dn, (uint32_t *)dsc,
                                             (unsigned long long *)dtot, n_words ? &io : nullptr)));
  if (n_words && site_cost)
    PGPU_CUDA(ctx, cudaMemcpyAsync(site_cost, dsc, n_sites * 4, cudaMemcpyDeviceToHost, s));
  uint64_t *ht = reinterpret_cast<uint64_t *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(ht, dtot, 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->d2h_stream));
  PGPU_TRY(pgpu_check_flag(ctx, "tcm_tree"));
  *total = *ht;
  return PGPU_OK;
}

}  // extern "C"
