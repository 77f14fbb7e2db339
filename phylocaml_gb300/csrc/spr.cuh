// SPR (subtree prune and regraft) engine: host-side topology, traversal
// programs and move lists shared by spr_topo.cpp and spr.cu.
//
// The reference keeps trees as an unrooted topology of handles and edges
// (lib/tree.ml:1-60) and rearranges them with Tree.break / Tree.join
// (lib/tree.ml:299-494); its neighbourhood enumerators are left as TODOs
// (lib/treeNeighborhoods.ml:27-75).  Here an unrooted binary tree of n tips
// has nodes 0..n-1 (tips) and n..2n-3 (internal, degree 3) and 2n-3 edges.
//
// Directed edge d = 2e + s names one side of edge e: s = 0 is the side of
// ea[e] seen from eb[e], s = 1 the side of eb[e] seen from ea[e].  Every
// directed edge owns, per site pattern and rate class, the conditional
// likelihood vector of the subtree on its side (L), that vector carried
// across the whole edge (M = P(t) L) and across half of it (H = P(t/2) L),
// an integer power-of-two scaler, and the Fitch state set of the subtree.
#pragma once
#include <stdint.h>

#include <array>
#include <vector>

#include "pgpu_internal.cuh"

struct SprTopo {
  int n = 0;                 // tips
  std::vector<int32_t> ea, eb;
  std::vector<double> len;
  std::vector<std::array<int32_t, 3>> inc;   // incident edges per node; tips use [0]

  int n_nodes() const { return 2 * n - 2; }
  int n_edges() const { return 2 * n - 3; }
  int n_dedges() const { return 2 * n_edges(); }
  int deg(int v) const { return v < n ? 1 : 3; }
  int other(int e, int v) const { return ea[e] == v ? eb[e] : ea[e]; }
  // directed edge of edge e whose subtree is on `from`'s side
  int dedge(int from, int e) const { return 2 * e + (ea[e] == from ? 0 : 1); }
  int dsrc(int d) const { return (d & 1) ? eb[d >> 1] : ea[d >> 1]; }
  int ddst(int d) const { return (d & 1) ? ea[d >> 1] : eb[d >> 1]; }
};

// One step of a pool pass: L[out] = M[in1] * M[in2]; tips are filled apart.
struct PoolPlan {
  std::vector<int4> ops;        // {out, in1, in2, 0} in dependency order
  std::vector<int4> tips;       // {dedge, tip, edge, 0}
  std::vector<int32_t> tipcnt;  // tips on each directed edge's side
};

// Traversal step of the scan kernels (32 bytes).
//   start step: d1 = s->u, d2 = g->u (the two sides joined by removing u)
//   visit step: node y entered from the merged edge's side; d1 = c1->y and
//               d2 = c2->y are its two other directed edges; out1 / out2 are
//               the move slots of regrafting onto edges (y,c1) and (y,c2)
//               (-1: not wanted)
// flags: SPR_START, SPR_DOWN1 / SPR_DOWN2 (descend into c1 / c2, or into s / g
// for the start step), SPR_FIRST2 (descend into the second one first; the
// other is pushed).  A visit with no pending message pops the stack.
enum : int32_t { SPR_START = 1, SPR_DOWN1 = 2, SPR_DOWN2 = 4, SPR_FIRST2 = 8 };
struct SprStep {
  int32_t d1, d2, out1, out2, flags, depth, pad0, pad1;
};

// One prune: carry the subtree on p's side of edge (p,u) away.
struct SprPrune {
  int32_t step_off, n_steps;   // program range
  int32_t dp;                  // directed edge p->u
  int32_t move_off, n_moves;   // output slots [move_off, move_off + n_moves)
  int32_t ds, dg;              // s->u and g->u
  int32_t pad;
};

struct SprMove {
  int32_t prune;     // index into the prune list
  int32_t dc;        // directed edge c->y: regraft onto edge dc >> 1
  int32_t depth;     // y's distance from the merged edge in nodes (1 for s and g)
  int32_t pad;
};

struct SprPlan {
  std::vector<SprStep> steps;
  std::vector<SprPrune> prunes;
  std::vector<SprMove> moves;
  std::vector<double> merged_len;   // per prune
  int max_depth = 0;                // stack entries needed
  int max_moves_per_prune = 0;
};

// TBR (tree bisection and reconnection) moves that reroot both sides.  Cut
// an edge (a,b) whose ends are both internal; a's side with a dissolved (its
// two other edges joined into one) is A', b's side likewise B'.  A move puts
// a in the middle of an edge j of A' and b in the middle of an edge k of B',
// the cut edge keeping its length between them.  j and k exclude the joined
// edges (putting a back on its joined edge is no reroot: with one side
// rerooted only, the move is an SPR move).  Per cut, an emit plan walks A'
// (the SPR prune carrying b's side away) and B' (carrying a's side away);
// its moves are the attach edges j and k, and pair (j, k) of the cut is
// grid_off + j * nB + k of the grid of all pairs.  With one distance limit
// (or none) every pair of the grid is a move; with a join and a reroot limit
// that differ, the listed moves are the pairs whose one attach edge lies
// within the join limit and whose other lies within the reroot limit (either
// side may be the one moved), in grid order: keep[m] is the grid index of
// move m, and move_off the first listed move of a cut.
struct TbrCut {
  int32_t edge;          // the cut edge
  int32_t pa, pb;        // emit prunes walking A' and B'
  int32_t nA, nB;        // attach edges on each side
  int64_t move_off;      // first listed TBR move of the cut
  int64_t grid_off;      // first pair of the cut in the grid
};

struct TbrPlan {
  SprPlan emit;
  std::vector<TbrCut> cuts;
  int64_t n_moves = 0;   // listed moves
  int64_t n_grid = 0;    // pairs of every cut
  std::vector<int64_t> keep;   // grid index per listed move; empty when every pair is listed
};

// the TBR moves of T: attach edges j (on a's side) and k (on b's side) at
// depths dj and dk nodes from the cut, listed when dj <= join and dk <=
// reroot, or dk <= join and dj <= reroot (0: no limit)
void tbr_plan(const SprTopo &T, const PoolPlan &pp, int join, int reroot, TbrPlan *out);
// apply: cut edge `edge` (a = ea, b = eb), a onto the edge of directed edge
// dj (c->y, y nearer a), b onto that of dk
pgpu_status tbr_apply(pgpu_ctx *ctx, SprTopo *T, int edge, int32_t dj, int32_t dk);

// rooted postorder tree (pgpu_tree layout) -> unrooted topology
pgpu_status spr_from_rooted(pgpu_ctx *ctx, const pgpu_tree *t, SprTopo *out);
// unrooted -> rooted on the edge above tip 0 (half of its length each side);
// ids (optional, 2n-2 entries) receives the rooted id of every node
void spr_to_rooted(const SprTopo &T, int32_t *left, int32_t *right, double *brlen,
                   int32_t *ids = nullptr);
void spr_pool_plan(const SprTopo &T, PoolPlan *out);
// every SPR move of T whose regraft edge lies at most join_distance nodes
// from the merged edge (0: no limit; 1: the NNI moves), or only the listed
// ones (pairs of prune directed edge, regraft directed edge c->y)
void spr_plan_all(const SprTopo &T, const PoolPlan &pp, SprPlan *out, int join_distance = 0);
pgpu_status spr_plan_selected(pgpu_ctx *ctx, const SprTopo &T, const PoolPlan &pp,
                              const int32_t *dp, const int32_t *dc, int k, SprPlan *out);
// apply the move: prune p's side of (p,u), regraft onto the edge of dc
pgpu_status spr_apply(pgpu_ctx *ctx, SprTopo *T, int32_t dp, int32_t dc);
