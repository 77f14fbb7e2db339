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

// ---- the table (host): restates fill_cm and the three median rules ----

int64_t tcm_cost(const int32_t *tcm, int S, int x, int y) {   // x, y atomic codes
  return tcm[(31 - __builtin_clz((unsigned)x)) * S + (31 - __builtin_clz((unsigned)y))];
}

// find_median_pair (lib/costMatrix.ml:57-66)
void median_pair(const int32_t *tcm, int S, int i, int j, int candidates, int64_t *cost, int *code) {
  int64_t best = INT64_MAX;
  int assign = 0;
  for (int b = 0; b < S; ++b) {
    const int k = 1 << b;
    if (!(candidates & k)) continue;
    const int64_t c = tcm_cost(tcm, S, i, k) + tcm_cost(tcm, S, j, k);
    if (c == best) assign |= k;
    else if (c < best) best = c, assign = k;
  }
  *cost = best;
  *code = assign;
}

// find_median_general / _metric / _equal (lib/costMatrix.ml:68-122)
void median(const int32_t *tcm, int S, int mode, int i, int j, int64_t *cost, int *code) {
  const int all = (1 << S) - 1;
  if (mode == PGPU_TCM_EQUAL) {
    const int64_t unequal = tcm_cost(tcm, S, 1, 2), equal = tcm_cost(tcm, S, 1, 1);
    if (i & j) *cost = equal, *code = i & j;
    else *cost = unequal, *code = i | j;
    return;
  }
  const int cand = mode == PGPU_TCM_METRIC ? (i | j) : all;
  int64_t best = INT64_MAX;
  int assign = 0;
  for (int bi = 0; bi < S; ++bi) {
    if (!(i >> bi & 1)) continue;
    for (int bj = 0; bj < S; ++bj) {
      if (!(j >> bj & 1)) continue;
      int64_t c;
      int k;
      median_pair(tcm, S, 1 << bi, 1 << bj, cand, &c, &k);
      if (c == best) assign |= k;
      else if (c < best) best = c, assign = k;
    }
  }
  *cost = best;
  *code = assign;
}

pgpu_status tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips, size_t ld,
                     const uint32_t *weights, size_t n_sites, const uint32_t *table,
                     uint32_t *node_sets, uint32_t *site_cost, unsigned long long *total) {
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
  return pgpu_after_launch(ctx, "tcm_tree_kernel");
}

}  // namespace

extern "C" {

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
      int k;
      median(tcm, S, mode, i, j, &c, &k);
      const uint32_t packed = ((uint32_t)c << 4) | (uint32_t)k;
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
  void *dt, *dn, *dw = nullptr, *dsc = nullptr, *dtot;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, n * ld * 4, &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_OUT, n_int * ld * 4, &dn));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dtot));
  if (weights) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n_sites * 4, &dw));
  if (site_cost) PGPU_TRY(pgpu_buf(ctx, BUF_SITECOST, n_sites * 4, &dsc));
  cudaStream_t s = ctx->stream;
  if (n_words) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(dt, ld * 4, tips, n_words * 4, n_words * 4, n,
                                     cudaMemcpyHostToDevice, s));
    if (weights) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_sites * 4, cudaMemcpyHostToDevice, s));
  }
  PGPU_TRY(tree_dev(ctx, tree, (const uint32_t *)dt, ld, (const uint32_t *)dw, n_sites, table,
                    (uint32_t *)dn, (uint32_t *)dsc, (unsigned long long *)dtot));
  if (n_words) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(node_sets, n_words * 4, dn, ld * 4, n_words * 4, n_int,
                                     cudaMemcpyDeviceToHost, s));
    if (site_cost) PGPU_CUDA(ctx, cudaMemcpyAsync(site_cost, dsc, n_sites * 4, cudaMemcpyDeviceToHost, s));
  }
  uint64_t *ht = reinterpret_cast<uint64_t *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(ht, dtot, 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  PGPU_TRY(pgpu_check_flag(ctx, "tcm_tree"));
  *total = *ht;
  return PGPU_OK;
}

}  // extern "C"
