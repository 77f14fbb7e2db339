// Host side of the SPR engine: unrooted topology, the directed-edge pass
// order, the traversal programs of the scan kernels and move application.
//
// A move carries the subtree on p's side of edge (p,u) away from u, joins
// u's two other neighbours s and g into one edge of length t_us + t_ug, and
// re-inserts u (with the subtree and its branch t_pu) in the middle of
// another edge (y,c): t_yu = t_uc = t_yc / 2.  This is Tree.break followed by
// Tree.join (lib/tree.ml:299-494) with the branch-length rule that the
// reference leaves to its callers.
#include <algorithm>
#include <climits>
#include <cstring>

#include "spr.cuh"

pgpu_status spr_from_rooted(pgpu_ctx *ctx, const pgpu_tree *t, SprTopo *out) {
  if (!t || !t->left || !t->right || !t->brlen)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: tree needs left, right and brlen");
  const int n = t->n_tips;
  if (n < 3) return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: need at least 3 tips (got %d)", n);
  const int n_rooted = 2 * n - 1;
  std::vector<int32_t> parent(n_rooted, -1);
  for (int k = 0; k < n - 1; ++k) {
    const int a = t->left[k], b = t->right[k];
    if (a < 0 || b < 0 || a >= n + k || b >= n + k || a == b || parent[a] >= 0 || parent[b] >= 0)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: internal node %d has invalid children (%d, %d)",
                          n + k, a, b);
    parent[a] = n + k;
    parent[b] = n + k;
  }
  for (int v = 0; v < n_rooted - 1; ++v)
    if (parent[v] < 0) return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: node %d has no parent", v);
  for (int v = 0; v < n_rooted - 1; ++v)
    if (!(t->brlen[v] >= 0.0) || t->brlen[v] > 1e6)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: branch length %d is negative or not finite", v);
  const int root = 2 * n - 2, ra = t->left[n - 2], rb = t->right[n - 2];
  SprTopo T;
  T.n = n;
  T.inc.assign(2 * n - 2, {-1, -1, -1});
  std::vector<int> fill(2 * n - 2, 0);
  auto add = [&](int a, int b, double l) {
    const int e = (int)T.ea.size();
    T.ea.push_back(a);
    T.eb.push_back(b);
    T.len.push_back(l);
    T.inc[a][fill[a]++] = e;
    T.inc[b][fill[b]++] = e;
  };
  for (int v = 0; v < root; ++v)
    if (v != ra && v != rb) add(v, parent[v], t->brlen[v]);
  add(ra, rb, t->brlen[ra] + t->brlen[rb]);
  for (int v = 0; v < 2 * n - 2; ++v)
    if (fill[v] != T.deg(v))
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: node %d has degree %d after unrooting", v, fill[v]);
  *out = std::move(T);
  return PGPU_OK;
}

void spr_to_rooted(const SprTopo &T, int32_t *left, int32_t *right, double *brlen, int32_t *ids) {
  const int n = T.n;
  const int e0 = T.inc[0][0], v0 = T.other(e0, 0);
  // postorder of the tree hanging from v0 away from tip 0, new ids for internals
  std::vector<int32_t> id(2 * n - 2, -1);
  for (int v = 0; v < n; ++v) id[v] = v;
  int next = n;
  struct Fr {
    int v, from_e, phase;
  };
  std::vector<Fr> st;
  st.push_back({v0, e0, 0});
  while (!st.empty()) {
    Fr &f = st.back();
    const int v = f.v;
    if (v < n) {
      brlen[v] = T.len[f.from_e];
      st.pop_back();
      continue;
    }
    int ch[2], ce[2], m = 0;
    for (int j = 0; j < 3; ++j)
      if (T.inc[v][j] != f.from_e) {
        ce[m] = T.inc[v][j];
        ch[m++] = T.other(T.inc[v][j], v);
      }
    if (f.phase == 0) {
      f.phase = 1;
      const int e1 = ce[1], c1 = ch[1], e0c = ce[0], c0 = ch[0];
      st.push_back({c1, e1, 0});
      st.push_back({c0, e0c, 0});
      continue;
    }
    const int k = next - n;
    id[v] = next++;
    left[k] = id[ch[0]];
    right[k] = id[ch[1]];
    brlen[id[v]] = f.from_e == e0 ? 0.5 * T.len[e0] : T.len[f.from_e];
    st.pop_back();
  }
  brlen[0] = 0.5 * T.len[e0];
  left[n - 2] = 0;
  right[n - 2] = id[v0];
  if (ids) std::copy(id.begin(), id.end(), ids);
}

void spr_pool_plan(const SprTopo &T, PoolPlan *out) {
  const int n = T.n;
  const int root = T.other(T.inc[0][0], 0);
  std::vector<int32_t> order, pe(2 * n - 2, -1);
  order.reserve(2 * n - 2);
  order.push_back(root);
  for (size_t i = 0; i < order.size(); ++i) {
    const int v = order[i];
    for (int j = 0; j < T.deg(v); ++j) {
      const int e = T.inc[v][j];
      if (e == pe[v]) continue;
      const int c = T.other(e, v);
      pe[c] = e;
      order.push_back(c);
    }
  }
  out->ops.clear();
  out->tips.clear();
  out->tipcnt.assign(T.n_dedges(), 0);
  for (int x = 0; x < n; ++x) {
    const int e = T.inc[x][0], d = T.dedge(x, e);
    out->tips.push_back(make_int4(d, x, e, 0));
    out->tipcnt[d] = 1;
  }
  auto op = [&](int d, int i1, int i2) {
    out->ops.push_back(make_int4(d, i1, i2, 0));
    out->tipcnt[d] = out->tipcnt[i1] + out->tipcnt[i2];
  };
  // toward the root: x's side seen from its parent
  for (int i = (int)order.size() - 1; i > 0; --i) {
    const int x = order[i];
    if (x < n) continue;
    int in[2], m = 0;
    for (int j = 0; j < 3; ++j) {
      const int e = T.inc[x][j];
      if (e != pe[x]) in[m++] = T.dedge(T.other(e, x), e);
    }
    op(T.dedge(x, pe[x]), in[0], in[1]);
  }
  // away from the root: y's side seen from each child
  for (const int y : order) {
    if (y < n) continue;
    for (int j = 0; j < 3; ++j) {
      const int e = T.inc[y][j];
      if (e == pe[y]) continue;
      int in[2], m = 0;
      for (int q = 0; q < 3; ++q) {
        const int f = T.inc[y][q];
        if (f != e) in[m++] = T.dedge(T.other(f, y), f);
      }
      op(T.dedge(y, e), in[0], in[1]);
    }
  }
}

namespace {

// u's two edges other than e_pu
void other_two(const SprTopo &T, int u, int e_pu, int *es, int *eg) {
  int m = 0;
  for (int j = 0; j < 3; ++j)
    if (T.inc[u][j] != e_pu) (m++ == 0 ? *es : *eg) = T.inc[u][j];
}

struct Pending {
  int y, e_in, depth;
};

// Emits the traversal of one prune.  want(y, d) says whether the move onto
// the edge of directed edge d (= c->y) is wanted; down(y, e) whether the
// walk continues into the node across edge e.
template <typename Want, typename Down>
void emit_prune(const SprTopo &T, const PoolPlan &pp, int prune_idx, int dp, SprPlan *plan,
                Want want, Down down, int max_depth = INT_MAX) {
  const int u = T.ddst(dp), e_pu = dp >> 1;
  int es = -1, eg = -1;
  other_two(T, u, e_pu, &es, &eg);
  const int s = T.other(es, u), g = T.other(eg, u);
  SprPrune pr{};
  pr.step_off = (int)plan->steps.size();
  pr.dp = dp;
  pr.move_off = (int)plan->moves.size();
  pr.ds = T.dedge(s, es);
  pr.dg = T.dedge(g, eg);
  // s and g are at depth 1: their other two edges are the NNI regrafts
  const bool down_s = s >= T.n && max_depth >= 1 && down(s, es);
  const bool down_g = g >= T.n && max_depth >= 1 && down(g, eg);
  if (!down_s && !down_g) return;   // no regraft edge wanted beyond s or g
  SprStep st{};
  st.d1 = pr.ds;
  st.d2 = pr.dg;
  st.out1 = st.out2 = -1;
  st.flags = SPR_START | (down_s ? SPR_DOWN1 : 0) | (down_g ? SPR_DOWN2 : 0);
  std::vector<Pending> stack;
  Pending cur{-1, -1, 0};
  bool have = false;
  int max_stack = 0;
  if (down_s && down_g) {
    const bool g_first = pp.tipcnt[pr.dg] < pp.tipcnt[pr.ds];
    if (g_first) st.flags |= SPR_FIRST2;
    // the message into s comes across the merged edge from g's side, and
    // the other way round
    stack.push_back(g_first ? Pending{s, es, 1} : Pending{g, eg, 1});
    cur = g_first ? Pending{g, eg, 1} : Pending{s, es, 1};
  } else {
    cur = down_s ? Pending{s, es, 1} : Pending{g, eg, 1};
  }
  have = true;
  max_stack = (int)stack.size();
  plan->steps.push_back(st);
  while (true) {
    if (!have) {
      if (stack.empty()) break;
      cur = stack.back();
      stack.pop_back();
    }
    const int y = cur.y;
    int e[2], c[2], m = 0;
    for (int j = 0; j < 3; ++j)
      if (T.inc[y][j] != cur.e_in) {
        e[m] = T.inc[y][j];
        c[m++] = T.other(T.inc[y][j], y);
      }
    SprStep v{};
    v.d1 = T.dedge(c[0], e[0]);
    v.d2 = T.dedge(c[1], e[1]);
    v.depth = cur.depth;
    v.out1 = v.out2 = -1;
    for (int h = 0; h < 2; ++h) {
      const int d = h == 0 ? v.d1 : v.d2;
      if (want(y, d)) {
        (h == 0 ? v.out1 : v.out2) = (int)plan->moves.size();
        plan->moves.push_back(SprMove{prune_idx, d, cur.depth, 0});
      }
    }
    const bool deeper = cur.depth + 1 <= max_depth;
    const bool d1 = deeper && c[0] >= T.n && down(c[0], e[0]);
    const bool d2 = deeper && c[1] >= T.n && down(c[1], e[1]);
    v.flags = (d1 ? SPR_DOWN1 : 0) | (d2 ? SPR_DOWN2 : 0);
    const Pending p1{c[0], e[0], cur.depth + 1}, p2{c[1], e[1], cur.depth + 1};
    if (d1 && d2) {
      const bool second_first = pp.tipcnt[v.d2] < pp.tipcnt[v.d1];
      if (second_first) v.flags |= SPR_FIRST2;
      stack.push_back(second_first ? p1 : p2);
      cur = second_first ? p2 : p1;
      have = true;
    } else if (d1 || d2) {
      cur = d1 ? p1 : p2;
      have = true;
    } else {
      have = false;
    }
    max_stack = std::max(max_stack, (int)stack.size());
    plan->steps.push_back(v);
  }
  pr.n_steps = (int)plan->steps.size() - pr.step_off;
  pr.n_moves = (int)plan->moves.size() - pr.move_off;
  if (pr.n_moves == 0) {   // walked but nothing wanted: drop the program
    plan->steps.resize(pr.step_off);
    return;
  }
  plan->merged_len.push_back(T.len[es] + T.len[eg]);
  plan->max_depth = std::max(plan->max_depth, max_stack);
  plan->max_moves_per_prune = std::max(plan->max_moves_per_prune, pr.n_moves);
  plan->prunes.push_back(pr);
}

void plan_reset(SprPlan *out) {
  out->steps.clear();
  out->prunes.clear();
  out->moves.clear();
  out->merged_len.clear();
  out->max_depth = 0;
  out->max_moves_per_prune = 0;
}

}  // namespace

void spr_plan_all(const SprTopo &T, const PoolPlan &pp, SprPlan *out, int join_distance) {
  plan_reset(out);
  const int max_depth = join_distance > 0 ? join_distance : INT_MAX;
  for (int dp = 0; dp < T.n_dedges(); ++dp) {
    if (T.ddst(dp) < T.n) continue;   // u must be internal
    const int idx = (int)out->prunes.size();
    emit_prune(T, pp, idx, dp, out, [](int, int) { return true; }, [](int, int) { return true; },
               max_depth);
  }
}

void tbr_plan(const SprTopo &T, const PoolPlan &pp, int join, int reroot, TbrPlan *out) {
  SprPlan &P = out->emit;
  plan_reset(&P);
  out->cuts.clear();
  out->keep.clear();
  out->n_moves = 0;
  out->n_grid = 0;
  const int J = join > 0 ? join : INT_MAX, Rr = reroot > 0 ? reroot : INT_MAX;
  const int max_depth = std::max(J, Rr);
  const bool filter = J != Rr;
  auto all = [](int, int) { return true; };
  for (int e = 0; e < T.n_edges(); ++e) {
    if (T.ea[e] < T.n || T.eb[e] < T.n) continue;   // both sides rerootable
    const size_t s0 = P.steps.size(), m0 = P.moves.size(), l0 = P.merged_len.size();
    const int p0 = (int)P.prunes.size();
    // directed edge 2e+1 carries b's side away and walks a's (A'), 2e the reverse
    emit_prune(T, pp, p0, 2 * e + 1, &P, all, all, max_depth);
    if ((int)P.prunes.size() == p0) continue;
    emit_prune(T, pp, p0 + 1, 2 * e, &P, all, all, max_depth);
    if ((int)P.prunes.size() == p0 + 1) {   // no attach edge on b's side: drop a's walk too
      P.steps.resize(s0);
      P.moves.resize(m0);
      P.merged_len.resize(l0);
      P.prunes.resize(p0);
      continue;
    }
    TbrCut c{e, p0, p0 + 1, P.prunes[p0].n_moves, P.prunes[p0 + 1].n_moves, out->n_moves,
             out->n_grid};
    if (filter) {
      const SprMove *ma = P.moves.data() + P.prunes[p0].move_off;
      const SprMove *mb = P.moves.data() + P.prunes[p0 + 1].move_off;
      for (int j = 0; j < c.nA; ++j)
        for (int k = 0; k < c.nB; ++k) {
          const int dj = ma[j].depth, dk = mb[k].depth;
          if ((dj <= J && dk <= Rr) || (dj <= Rr && dk <= J))
            out->keep.push_back(c.grid_off + (int64_t)j * c.nB + k);
        }
      out->n_moves = (int64_t)out->keep.size();
    } else {
      out->n_moves += (int64_t)c.nA * c.nB;
    }
    out->n_grid += (int64_t)c.nA * c.nB;
    out->cuts.push_back(c);
  }
}

pgpu_status tbr_apply(pgpu_ctx *ctx, SprTopo *T, int edge, int32_t dj, int32_t dk) {
  if (edge < 0 || edge >= T->n_edges() || T->ea[edge] < T->n || T->eb[edge] < T->n)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tbr: edge %d is not an internal edge", edge);
  // a's side first: spr_apply leaves the cut edge and b's side as they are
  PGPU_TRY(spr_apply(ctx, T, 2 * edge + 1, dj));
  return spr_apply(ctx, T, 2 * edge, dk);
}

pgpu_status spr_plan_selected(pgpu_ctx *ctx, const SprTopo &T, const PoolPlan &pp,
                              const int32_t *dp, const int32_t *dc, int k, SprPlan *out) {
  plan_reset(out);
  const int nd = T.n_dedges(), nn = T.n_nodes();
  std::vector<int> idx(k);
  for (int i = 0; i < k; ++i) {
    if (dp[i] < 0 || dp[i] >= nd || dc[i] < 0 || dc[i] >= nd || T.ddst(dp[i]) < T.n)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: move %d (%d, %d) is not a valid move", i, dp[i],
                          dc[i]);
    idx[i] = i;
  }
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return dp[a] < dp[b]; });
  std::vector<int32_t> par_e(nn), seen(nn);
  std::vector<uint8_t> on_path(nn), wanted_d(nd);
  for (int i0 = 0; i0 < k;) {
    int i1 = i0;
    while (i1 < k && dp[idx[i1]] == dp[idx[i0]]) ++i1;
    const int p_d = dp[idx[i0]], u = T.ddst(p_d), e_pu = p_d >> 1;
    // parent edges of the tree hung from u, without the pruned side
    std::fill(par_e.begin(), par_e.end(), -1);
    std::fill(seen.begin(), seen.end(), 0);
    std::fill(on_path.begin(), on_path.end(), 0);
    std::vector<int> q{u};
    seen[u] = 1;
    for (size_t h = 0; h < q.size(); ++h) {
      const int v = q[h];
      for (int j = 0; j < T.deg(v); ++j) {
        const int e = T.inc[v][j];
        if (v == u && e == e_pu) continue;
        const int w = T.other(e, v);
        if (seen[w]) continue;
        seen[w] = 1;
        par_e[w] = e;
        q.push_back(w);
      }
    }
    int es = -1, eg = -1;
    other_two(T, u, e_pu, &es, &eg);
    for (int i = i0; i < i1; ++i) {
      const int d = dc[idx[i]], y = T.ddst(d), c = T.dsrc(d), e = d >> 1;
      if (!seen[y] || !seen[c] || y == u || c == u || par_e[c] != e)
        return pgpu_set_err(ctx, PGPU_ERR_ARG,
                            "spr: regraft edge of move %d is not an edge beyond u's other "
                            "neighbours, seen from the merged edge",
                            idx[i]);
      wanted_d[d] = 1;
      for (int v = y; v != u && !on_path[v]; v = T.other(par_e[v], v)) on_path[v] = 1;
    }
    const int prune_idx = (int)out->prunes.size();
    emit_prune(
        T, pp, prune_idx, p_d, out, [&](int, int d) { return wanted_d[d] != 0; },
        [&](int w, int) { return on_path[w] != 0; });
    for (int i = i0; i < i1; ++i) wanted_d[dc[idx[i]]] = 0;
    i0 = i1;
  }
  return PGPU_OK;
}

pgpu_status spr_apply(pgpu_ctx *ctx, SprTopo *Tp, int32_t dp, int32_t dc) {
  SprTopo &T = *Tp;
  const int nd = T.n_dedges();
  if (dp < 0 || dp >= nd || dc < 0 || dc >= nd || T.ddst(dp) < T.n)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: (%d, %d) is not a valid move", dp, dc);
  const int u = T.ddst(dp), e_pu = dp >> 1;
  int es = -1, eg = -1;
  other_two(T, u, e_pu, &es, &eg);
  const int s = T.other(es, u), g = T.other(eg, u);
  const int ec = dc >> 1, c = T.dsrc(dc), y = T.ddst(dc);
  if (ec == e_pu || ec == es || ec == eg)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: regraft edge %d is next to the pruned node", ec);
  // the regraft edge must lie on u's side (not inside the pruned subtree)
  {
    std::vector<uint8_t> seen(T.n_nodes(), 0);
    std::vector<int> q{u};
    seen[u] = 1;
    bool found = false;
    for (size_t h = 0; h < q.size() && !found; ++h) {
      const int v = q[h];
      for (int j = 0; j < T.deg(v); ++j) {
        const int e = T.inc[v][j];
        if (v == u && e == e_pu) continue;
        if (e == ec) found = true;
        const int w = T.other(e, v);
        if (!seen[w]) {
          seen[w] = 1;
          q.push_back(w);
        }
      }
    }
    if (!found)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: regraft edge %d is inside the pruned subtree", ec);
  }
  auto replace_inc = [&](int v, int from, int to) {
    for (int j = 0; j < 3; ++j)
      if (T.inc[v][j] == from) {
        T.inc[v][j] = to;
        return;
      }
  };
  // join s and g through edge es; eg becomes free
  T.len[es] += T.len[eg];
  if (T.ea[es] == u) T.ea[es] = g;
  else T.eb[es] = g;
  replace_inc(g, eg, es);
  // split the regraft edge (c, y): ec becomes (c, u), eg becomes (u, y)
  const double half = 0.5 * T.len[ec];
  T.len[ec] = half;
  if (T.ea[ec] == y) T.ea[ec] = u;
  else T.eb[ec] = u;
  T.ea[eg] = u;
  T.eb[eg] = y;
  T.len[eg] = half;
  replace_inc(y, ec, eg);
  T.inc[u] = {e_pu, ec, eg};
  (void)s;
  (void)c;
  return PGPU_OK;
}

// ---------------------------------------------------------------------------
// random-addition parsimony tree: taxa join in a seeded random order, each
// on the edge where it adds the fewest Fitch steps (the first such edge in
// edge order), using the state sets of both sides of every edge
// ---------------------------------------------------------------------------
namespace {

constexpr uint64_t MSB16 = 0x8888888888888888ull;

inline uint64_t empty16(uint64_t v) {
  const uint64_t nz = (((v & ~MSB16) + ~MSB16) | v) & MSB16;
  return nz ^ MSB16;
}
inline uint64_t fitch16(uint64_t a, uint64_t b) {
  const uint64_t x = a & b, e = empty16(x), fill = e | (e - (e >> 3));
  return (x & ~fill) | ((a | b) & fill);
}

struct Splitmix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
};

}  // namespace

extern "C" pgpu_status pgpu_parsimony_stepwise(int32_t n_tips, const uint8_t *tip_codes, size_t ld,
                                               size_t n_pat, const uint8_t *code_mask, int n_codes,
                                               const double *weights, uint64_t seed, double brlen,
                                               int32_t *left, int32_t *right, double *brlen_out,
                                               uint64_t *length) {
  if (n_tips < 3 || !tip_codes || !code_mask || n_codes < 1 || !left || !right || !brlen_out ||
      ld < n_pat || !(brlen >= 0.0))
    return PGPU_ERR_ARG;
  const int n = n_tips;
  const size_t W = (n_pat + 15) / 16;
  // packed 4-bit state sets of the tips and integer weight bit planes
  std::vector<uint64_t> tipset((size_t)n * W, 0);
  for (int t = 0; t < n; ++t)
    for (size_t i = 0; i < n_pat; ++i) {
      const int code = tip_codes[(size_t)t * ld + i];
      const uint64_t m = code < n_codes ? (code_mask[code] & 0xFu) : 0xFu;
      tipset[(size_t)t * W + i / 16] |= m << (4 * (i % 16));
    }
  uint64_t wmax = 1;
  std::vector<uint64_t> wi(n_pat, 1);
  for (size_t i = 0; i < n_pat; ++i) {
    if (weights) {
      if (!(weights[i] >= 0.0) || weights[i] > 1e9) return PGPU_ERR_ARG;
      wi[i] = (uint64_t)llround(weights[i]);
    }
    wmax = std::max(wmax, wi[i]);
  }
  int nb = 1;
  while ((wmax >> nb) != 0) ++nb;
  std::vector<uint64_t> planes((size_t)nb * W, 0);
  for (size_t i = 0; i < n_pat; ++i)
    for (int b = 0; b < nb; ++b)
      if ((wi[i] >> b) & 1u) planes[(size_t)b * W + i / 16] |= 0x8ull << (4 * (i % 16));
  auto wcount = [&](const uint64_t *set_and) {
    uint64_t s = 0;
    for (size_t q = 0; q < W; ++q) {
      const uint64_t e = empty16(set_and[q]);
      if (!e) continue;
      for (int b = 0; b < nb; ++b) s += (uint64_t)__builtin_popcountll(e & planes[(size_t)b * W + q]) << b;
    }
    return s;
  };
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  Splitmix rng{seed};
  for (int i = n - 1; i > 0; --i) std::swap(order[i], order[(int)(rng.next() % (uint64_t)(i + 1))]);
  // adjacency of the growing tree; internal nodes n, n+1, ...
  std::vector<std::array<int, 3>> nb3(2 * n - 2, {-1, -1, -1});
  std::vector<int> deg(2 * n - 2, 0);
  auto link = [&](int a, int b) {
    nb3[a][deg[a]++] = b;
    nb3[b][deg[b]++] = a;
  };
  int next_int = n;
  {
    const int w = next_int++;
    link(order[0], w);
    link(order[1], w);
    link(order[2], w);
  }
  // directed sets keyed by (node, slot of the neighbour): side of node seen from nb3[node][slot]
  std::vector<uint64_t> dset((size_t)(2 * n - 2) * 3 * W);
  std::vector<uint8_t> have((size_t)(2 * n - 2) * 3);
  std::vector<uint64_t> tmp(W);
  auto slot_of = [&](int x, int y) {
    for (int j = 0; j < deg[x]; ++j)
      if (nb3[x][j] == y) return j;
    return -1;
  };
  // F(x | seen from y), computed on demand with an explicit stack
  auto dirset = [&](int x0, int y0) -> const uint64_t * {
    struct Fr {
      int x, y;
    };
    std::vector<Fr> st{{x0, y0}};
    while (!st.empty()) {
      const Fr f = st.back();
      const int sl = slot_of(f.x, f.y);
      const size_t key = (size_t)f.x * 3 + sl;
      if (have[key]) {
        st.pop_back();
        continue;
      }
      uint64_t *out = &dset[key * W];
      if (f.x < n) {
        std::copy(&tipset[(size_t)f.x * W], &tipset[(size_t)f.x * W] + W, out);
        have[key] = 1;
        st.pop_back();
        continue;
      }
      int c[2], m = 0;
      for (int j = 0; j < 3; ++j)
        if (nb3[f.x][j] != f.y) c[m++] = nb3[f.x][j];
      const size_t k1 = (size_t)c[0] * 3 + slot_of(c[0], f.x), k2 = (size_t)c[1] * 3 + slot_of(c[1], f.x);
      if (!have[k1] || !have[k2]) {
        if (!have[k1]) st.push_back({c[0], f.x});
        if (!have[k2]) st.push_back({c[1], f.x});
        continue;
      }
      for (size_t q = 0; q < W; ++q) out[q] = fitch16(dset[k1 * W + q], dset[k2 * W + q]);
      have[key] = 1;
      st.pop_back();
    }
    return &dset[((size_t)x0 * 3 + slot_of(x0, y0)) * W];
  };
  for (int step = 3; step < n; ++step) {
    const int t = order[step];
    std::fill(have.begin(), have.end(), 0);
    uint64_t best = ~0ull;
    int ba = -1, bb = -1;
    for (int a = n; a < next_int; ++a) {
      for (int j = 0; j < 3; ++j) {
        const int b = nb3[a][j];
        if (b >= n && b < a) continue;   // each internal edge once, from its larger end
        const uint64_t *fa = dirset(a, b), *fb = dirset(b, a);
        const uint64_t *ft = &tipset[(size_t)t * W];
        for (size_t q = 0; q < W; ++q) tmp[q] = ft[q] & fitch16(fa[q], fb[q]);
        const uint64_t cost = wcount(tmp.data());
        if (cost < best) {
          best = cost;
          ba = a;
          bb = b;
        }
      }
    }
    const int w = next_int++;
    nb3[ba][slot_of(ba, bb)] = w;
    nb3[bb][slot_of(bb, ba)] = w;
    nb3[w] = {ba, bb, t};
    deg[w] = 3;
    nb3[t][0] = w;
    deg[t] = 1;
  }
  // to the unrooted topology (internal ids n..2n-3 as created), then rooted
  SprTopo T;
  T.n = n;
  T.inc.assign(2 * n - 2, {-1, -1, -1});
  std::vector<int> fill(2 * n - 2, 0);
  for (int a = 0; a < 2 * n - 2; ++a)
    for (int j = 0; j < deg[a]; ++j) {
      const int b = nb3[a][j];
      if (b < a) continue;
      const int e = (int)T.ea.size();
      T.ea.push_back(a);
      T.eb.push_back(b);
      T.len.push_back(brlen);
      T.inc[a][fill[a]++] = e;
      T.inc[b][fill[b]++] = e;
    }
  spr_to_rooted(T, left, right, brlen_out);
  if (length) {
    std::fill(have.begin(), have.end(), 0);
    const int e0a = T.ea[0], e0b = T.eb[0];
    const uint64_t *fa = dirset(e0a, e0b), *fb = dirset(e0b, e0a);
    // total = sum over internal joins; recount with a rooted pass at edge 0
    uint64_t total = 0;
    // every internal node's join seen from the edge-0 rooting
    struct Fr {
      int x, y;
    };
    std::vector<Fr> st{{e0a, e0b}, {e0b, e0a}};
    while (!st.empty()) {
      const Fr f = st.back();
      st.pop_back();
      if (f.x < n) continue;
      int c[2], m = 0;
      for (int j = 0; j < 3; ++j)
        if (nb3[f.x][j] != f.y) c[m++] = nb3[f.x][j];
      const uint64_t *s1 = dirset(c[0], f.x), *s2 = dirset(c[1], f.x);
      for (size_t q = 0; q < W; ++q) tmp[q] = s1[q] & s2[q];
      total += wcount(tmp.data());
      st.push_back({c[0], f.x});
      st.push_back({c[1], f.x});
    }
    for (size_t q = 0; q < W; ++q) tmp[q] = fa[q] & fb[q];
    total += wcount(tmp.data());
    *length = total;
  }
  return PGPU_OK;
}
