// Tree validation and the stack-machine postorder shared by the Fitch and
// pruning kernels.
//
// phylocaml walks the tree recursively (Tree.post_order_edges,
// lib/tree.ml:171-187) and materialises every node's data.  On the GPU one
// CTA carries a tile of sites through the whole postorder and keeps the
// intermediate node data in shared memory, so the order matters: evaluating
// the child with the larger stack need first (Sethi-Ullman order) bounds the
// number of live intermediate results by the tree's Strahler number, at most
// log2(n_tips) + 1.  Results do not depend on the order: every node is a
// function of its two children only.
#include <algorithm>
#include <cstring>

#include "pgpu_internal.cuh"

pgpu_status pgpu_build_schedule(pgpu_ctx *ctx, const pgpu_tree *tree, TreeSchedule *out) {
  if (!tree || !tree->left || !tree->right)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: null tree or child arrays");
  const int32_t n = tree->n_tips;
  if (n < 2) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: need at least 2 tips (got %d)", n);
  const int32_t n_int = n - 1, n_nodes = 2 * n - 1;
  std::vector<int32_t> uses(n_nodes, 0);
  for (int32_t k = 0; k < n_int; ++k) {
    const int32_t a = tree->left[k], b = tree->right[k];
    if (a < 0 || b < 0 || a >= n + k || b >= n + k || a == b)
      return pgpu_set_err(ctx, PGPU_ERR_ARG,
                          "tree: internal node %d has children (%d, %d); children must be "
                          "distinct ids below %d (postorder)",
                          n + k, a, b, n + k);
    uses[a]++;
    uses[b]++;
  }
  for (int32_t id = 0; id < n_nodes - 1; ++id)
    if (uses[id] != 1)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: node %d is the child of %d nodes (must be 1)",
                          id, uses[id]);

  // stack need of every internal node and which child to evaluate first
  std::vector<int32_t> need(n_nodes, 0);
  std::vector<uint8_t> swap(n_int, 0);
  for (int32_t k = 0; k < n_int; ++k) {
    const int32_t a = tree->left[k], b = tree->right[k];
    const int32_t na = need[a], nb = need[b];
    const int32_t ha = a >= n ? 1 : 0, hb = b >= n ? 1 : 0;
    const int32_t a_first = std::max(na, ha + nb);
    const int32_t b_first = std::max(nb, hb + na);
    swap[k] = b_first < a_first ? 1 : 0;
    need[n + k] = std::max(std::min(a_first, b_first), 1);
  }

  out->n_tips = n;
  out->ops.clear();
  out->ops.reserve(n_int);
  out->tip_seq.clear();
  out->tip_seq.reserve(n);
  // iterative DFS (a caterpillar tree would overflow a recursive one)
  std::vector<std::pair<int32_t, int32_t>> st;
  st.reserve(2 * n);
  st.push_back({n_nodes - 1, 0});
  while (!st.empty()) {
    auto [v, phase] = st.back();
    st.pop_back();
    const int32_t k = v - n;
    int32_t first = tree->left[k], second = tree->right[k];
    if (swap[k]) std::swap(first, second);
    if (phase == 0) {
      st.push_back({v, 1});
      if (second >= n) st.push_back({second, 0});
      if (first >= n) st.push_back({first, 0});
    } else {
      out->ops.push_back(SchedOp{k, first, second, 0});
    }
  }

  // simulate the stack to check the discipline and size it
  std::vector<int32_t> stack;
  int depth = 0;
  for (const SchedOp &op : out->ops) {
    if (op.b >= n) {
      if (stack.empty() || stack.back() != op.b)
        return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: internal schedule error (stack)");
      stack.pop_back();
    }
    if (op.a >= n) {
      if (stack.empty() || stack.back() != op.a)
        return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: internal schedule error (stack)");
      stack.pop_back();
    }
    if (op.a < n) out->tip_seq.push_back(op.a);
    if (op.b < n) out->tip_seq.push_back(op.b);
    stack.push_back(n + op.k);
    depth = std::max<int>(depth, (int)stack.size());
  }
  if ((int32_t)out->ops.size() != n_int || (int32_t)out->tip_seq.size() != n || stack.size() != 1)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: internal schedule error (size)");
  out->max_depth = depth;
  return PGPU_OK;
}

pgpu_status pgpu_schedule_device(pgpu_ctx *ctx, const pgpu_tree *tree, const TreeSchedule **sch,
                                 const int4 **d_ops, const int32_t **d_tip_seq) {
  if (!tree || !tree->left || !tree->right || tree->n_tips < 2)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: null tree or fewer than 2 tips");
  const size_t n_int = (size_t)tree->n_tips - 1;
  const bool same = ctx->sched_valid && ctx->sched.n_tips == tree->n_tips &&
                    std::memcmp(ctx->sched_left.data(), tree->left, n_int * 4) == 0 &&
                    std::memcmp(ctx->sched_right.data(), tree->right, n_int * 4) == 0;
  void *dops, *dseq;
  if (!same) {
    ctx->sched_valid = false;
    PGPU_TRY(pgpu_build_schedule(ctx, tree, &ctx->sched));
    PGPU_TRY(pgpu_buf(ctx, BUF_OPS, ctx->sched.ops.size() * sizeof(SchedOp), &dops));
    PGPU_TRY(pgpu_buf(ctx, BUF_TIPSEQ, ctx->sched.tip_seq.size() * sizeof(int32_t), &dseq));
    // synchronous copies: the host vectors may change on the next call
    PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    PGPU_CUDA(ctx, cudaMemcpy(dops, ctx->sched.ops.data(), ctx->sched.ops.size() * sizeof(SchedOp),
                              cudaMemcpyHostToDevice));
    PGPU_CUDA(ctx, cudaMemcpy(dseq, ctx->sched.tip_seq.data(),
                              ctx->sched.tip_seq.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    ctx->sched_left.assign(tree->left, tree->left + n_int);
    ctx->sched_right.assign(tree->right, tree->right + n_int);
    ctx->sched_valid = true;
  } else {
    PGPU_TRY(pgpu_buf(ctx, BUF_OPS, ctx->sched.ops.size() * sizeof(SchedOp), &dops));
    PGPU_TRY(pgpu_buf(ctx, BUF_TIPSEQ, ctx->sched.tip_seq.size() * sizeof(int32_t), &dseq));
  }
  *sch = &ctx->sched;
  *d_ops = reinterpret_cast<const int4 *>(dops);
  *d_tip_seq = reinterpret_cast<const int32_t *>(dseq);
  return PGPU_OK;
}

extern "C" pgpu_status pgpu_tree_schedule(pgpu_ctx *ctx, const pgpu_tree *tree, int32_t *ops_out,
                                          int32_t *max_depth) {
  TreeSchedule sch;
  PGPU_TRY(pgpu_build_schedule(ctx, tree, &sch));
  if (ops_out)
    for (size_t i = 0; i < sch.ops.size(); ++i) {
      ops_out[3 * i] = sch.ops[i].k;
      ops_out[3 * i + 1] = sch.ops[i].a;
      ops_out[3 * i + 2] = sch.ops[i].b;
    }
  if (max_depth) *max_depth = sch.max_depth;
  return PGPU_OK;
}
