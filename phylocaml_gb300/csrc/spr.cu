// SPR rearrangement scoring on the GPU.
//
// phylocaml's tree search stops at the interface: Tree.break / Tree.join
// rearrange a topology (lib/tree.ml:299-494), the neighbourhood enumerators
// are TODOs (lib/treeNeighborhoods.ml:27-75) and the likelihood character is
// a stub (lib/likelihood_c.ml).  This file scores every SPR neighbour of a
// tree in one pass, exactly in the chosen arithmetic form, with the branch
// lengths of the move rule in spr_topo.cpp.
//
// Directed-edge pool (spr_pool_kernel, one pass per tree): for every
// directed edge d the conditional likelihood vector L[d] of the subtree on
// its side, M[d] = P(t) L[d] and H[d] = P(t/2) L[d], with per-pattern
// power-of-two scalers, for all patterns and rate classes, in HBM.  A
// thread owns one (pattern, rate class) and walks the pass order, so no
// thread reads a vector another thread wrote.
//
// Scan (spr_scan_kernel, one CTA per prune x pattern-block group): removing
// the subtree on p's side of (p,u) changes only the vectors that look
// toward u.  The CTA walks the remaining tree outward from the joined edge
// (s,g), rebuilding each changed vector from its parent's message and the
// sibling's unchanged M, and at every edge (y,c) it scores the regraft:
//   site = sum_r probs_r sum_i pi_i [P(t_yc/2) L'[y|c]]_i H[c->y]_i M[p->u]_i
// The walk descends into the smaller side first and keeps the other
// message on a stack in shared memory, so the stack holds at most
// log2(n) + 1 entries.  Site log-likelihoods are weighted and summed as
// float pairs per warp, per CTA in warp order, then per move over the CTA
// groups in FP64 (spr_reduce_kernel), which fixes the summation order.
//
// The Fitch part (spr_fitch_*_kernel) runs the same programs on packed
// 4-bit state sets: the parsimony length of every neighbour, exactly.
//
// TBR moves that reroot both sides of a cut edge (a,b): the scan program of
// the prune carrying b's side away walks a's side, and in emit mode stores
// its vector at the middle of every edge it would regraft onto (a's side
// rerooted there); the reverse prune does the same for b's side.
// tbr_pair_kernel then scores every pair of attach edges of the cut as one
// dot product per pattern.
#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstring>

#include "forms.cuh"
#include "pmatrix.cuh"
#include "spr.cuh"

using namespace pgpu_forms;

namespace {

constexpr int SPR_NT = 256;
constexpr int SPR_NW = SPR_NT / 32;
constexpr int SPR_FEATURES = 64;

__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

// ---------------------------------------------------------------------------
// rescaling shared by the pool and scan kernels: exact power of two, agreed
// by the RT lanes (rate classes) of one pattern; all lanes of the warp call
// ---------------------------------------------------------------------------
template <typename Pol, int RT>
__device__ __forceinline__ void rescale(typename Pol::V *acc, int &sc) {
  auto mx = fmax(fmax(Pol::mag(acc[0]), Pol::mag(acc[1])), fmax(Pol::mag(acc[2]), Pol::mag(acc[3])));
  if (__any_sync(0xffffffffu, mx < Pol::thresh && mx > 0)) {
#pragma unroll
    for (int o = 1; o < RT; o <<= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (mx < Pol::thresh && mx > 0) {
      const int ex = frexp_exp(mx);
      sc += ex;
      const int k1 = min(-ex, 120), k2 = -ex - k1;
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[e] = Pol::scale(acc[e], k1);
      if (k2 > 0) {
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] = Pol::scale(acc[e], k2);
      }
    }
  }
}

struct PoolArgs {
  void *L, *M, *H;
  int32_t *sc;
  const void *Dfull, *Dhalf;   // [n_edges][R][16] coefficients
  const int4 *ops;
  const double *pi, *probs, *weights;
  double *site_lnl;
  double2 *partials;
  size_t np;                   // padded patterns
  size_t n_pat;
  int n_ops, R, NP;
};

template <typename Pol, int RT>
__global__ void __launch_bounds__(SPR_NT) spr_pool_kernel(const PoolArgs a) {
  using V = typename Pol::V;
  using Coef = typename Pol::Coef;
  __shared__ double2 red[SPR_NW];
  const int c = threadIdx.x, pl = c / RT, r = c % RT, lane = c & 31;
  const size_t pat = (size_t)blockIdx.x * a.NP + pl;
  const bool on = r < a.R;
  const int R = a.R;
  auto vi = [&](int d) { return ((size_t)d * a.np + pat) * R + r; };
  for (int i = 0; i < a.n_ops; ++i) {
    const int4 op = __ldg(a.ops + i);
    V acc[4];
    int s = a.sc[(size_t)op.y * a.np + pat] + a.sc[(size_t)op.z * a.np + pat];
    if (on) {
      V x[4], y[4];
      Pol::load_tip(a.M, vi(op.y), x);
      Pol::load_tip(a.M, vi(op.z), y);
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[e] = Pol::mul(x[e], y[e]);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[e] = Pol::zero();
    }
    rescale<Pol, RT>(acc, s);
    if (on) {
      const int ed = op.x >> 1;
      V m[4], h[4];
      Pol::rows(static_cast<const Coef *>(a.Dfull) + ((size_t)ed * R + r) * 16, acc, m);
      Pol::rows(static_cast<const Coef *>(a.Dhalf) + ((size_t)ed * R + r) * 16, acc, h);
      Pol::store4(a.L, vi(op.x), acc);
      Pol::store4(a.M, vi(op.x), m);
      Pol::store4(a.H, vi(op.x), h);
    }
    if (r == 0) a.sc[(size_t)op.x * a.np + pat] = s;
  }
  // log-likelihood across edge 0: L[side a] . P(t) L[side b]
  double part = 0.0;
  if (on) {
    V x[4], y[4];
    Pol::load_tip(a.L, vi(0), x);
    Pol::load_tip(a.M, vi(1), y);
    double lr = 0.0;
#pragma unroll
    for (int e = 0; e < 4; ++e) lr += a.pi[e] * Pol::to_d(Pol::mul(x[e], y[e]));
    part = a.probs[r] * lr;
  }
#pragma unroll
  for (int o = 1; o < RT; o <<= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  double sum = 0.0, comp = 0.0;
  if (r == 0 && pat < a.n_pat) {
    const int e2 = a.sc[pat] + a.sc[a.np + pat];
    const double lnl = log(part) + (double)e2 * 0.69314718055994530942;
    if (a.site_lnl) a.site_lnl[pat] = lnl;
    sum = a.weights[pat] * lnl;
  }
  warp_csum(sum, comp);
  if (lane == 0) red[c >> 5] = make_double2(sum, comp);
  __syncthreads();
  if (c < 32) {
    double2 v = lane < SPR_NW ? red[lane] : make_double2(0.0, 0.0);
    double ss = v.x, cc = v.y;
    warp_csum(ss, cc);
    if (lane == 0) a.partials[blockIdx.x] = make_double2(ss, cc);
  }
}

struct TipArgs {
  void *L, *M, *H;
  int32_t *sc;
  const void *tipfull, *tiphalf;   // [n_tips][R][n_codes][4] values of the form
  const double *code_tab;          // [n_codes][4]
  const uint8_t *codes;            // [n_tips][ld]
  const int4 *tips;                // {dedge, tip, edge, 0}
  int *flag;
  size_t np, n_pat, ld;
  int R, n_codes;
};

template <typename Pol>
__global__ void __launch_bounds__(256) spr_tip_kernel(const TipArgs a) {
  using V = typename Pol::V;
  const size_t pat = (size_t)blockIdx.x * 256 + threadIdx.x;
  if (pat >= a.np) return;
  const int4 t = a.tips[blockIdx.y];
  int code = pat < a.n_pat ? a.codes[(size_t)t.y * a.ld + pat] : 0;
  if (code >= a.n_codes) {
    atomicOr(a.flag, PGPU_FLAG_BADCODE);
    code = 0;
  }
  V l[4], m[4], h[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) l[e] = Pol::from_d(a.code_tab[code * 4 + e]);
  for (int r = 0; r < a.R; ++r) {
    const size_t at = ((size_t)t.x * a.np + pat) * a.R + r;
    const size_t tt = ((size_t)t.y * a.R + r) * a.n_codes + code;
    Pol::load_tip(a.tipfull, tt, m);
    Pol::load_tip(a.tiphalf, tt, h);
    Pol::store4(a.L, at, l);
    Pol::store4(a.M, at, m);
    Pol::store4(a.H, at, h);
  }
  a.sc[(size_t)t.x * a.np + pat] = 0;
}

__global__ void __launch_bounds__(1024) spr_pool_finalize_kernel(const double2 *partials, int n,
                                                                double *out) {
  const double v = csum_block<1024>(partials, n);
  if (threadIdx.x == 0) out[0] = v;
}

// ---------------------------------------------------------------------------
// scan
// ---------------------------------------------------------------------------
struct ScanArgs {
  const void *L, *M, *H;
  const int32_t *sc;
  const void *Dhalf, *Dmer;   // [n_edges][R][16], [n_prunes][R][16]
  const SprStep *steps;
  const SprPrune *prunes;
  const double *pi, *probs;
  const float *wts;           // [np], zero beyond n_pat
  const float4 *logtab;       // 64 entries
  double *partials;           // [n_groups][n_moves]
  int *flag;
  size_t np, n_moves;
  int R, NP, G, n_blocks, depth, max_moves;
  // emit mode (TBR): the attach vector of every wanted edge instead of a score
  const void *Dfull;          // [n_edges][R][16]: P(t) of the cut edge (b's side)
  void *xout;                 // [slot][np][R] x 4
  int32_t *xsc;               // [slot][np]
  long long slot_base;        // move index of slot 0
  int prune_base;             // first prune of the launch
};

template <typename Pol>
__host__ __device__ size_t scan_smem(int depth, int max_moves) {
  return 1024 + a16((size_t)SPR_NW * max_moves * sizeof(ff)) +
         (size_t)depth * 4 * SPR_NT * sizeof(typename Pol::V) + (size_t)depth * SPR_NT * sizeof(int);
}

// EMIT: instead of scoring a regraft, store the walked side's vector at the
// middle of the edge, [P(t_yc/2) L'[y|c]] (.) H[c->y], with its scaler: the
// side rerooted there, for TBR.  Emit prunes come in pairs per cut edge
// (a,b): the even one walks a's side and stores X weighted by probs_r pi_i,
// the odd one walks b's side and stores P(t_ab) Y, carried across the cut,
// so that a TBR site likelihood is the plain dot product of the two.
template <typename Pol, int RT, bool EMIT = false>
__global__ void __launch_bounds__(SPR_NT) spr_scan_kernel(const ScanArgs a) {
  using V = typename Pol::V;
  using Coef = typename Pol::Coef;
  constexpr int NT = SPR_NT;
  extern __shared__ __align__(16) unsigned char smem[];
  const SprPrune pr = a.prunes[a.prune_base + blockIdx.x];
  float4 *ltab = reinterpret_cast<float4 *>(smem);
  ff *red = reinterpret_cast<ff *>(smem + 1024);
  V *stk = reinterpret_cast<V *>(smem + 1024 + a16((size_t)SPR_NW * a.max_moves * sizeof(ff)));
  int *stk_sc = reinterpret_cast<int *>(stk + (size_t)a.depth * 4 * NT);
  const int c = threadIdx.x, lane = c & 31, warp = c >> 5, pl = c / RT, r = c % RT;
  const bool on = r < a.R;
  const int R = a.R;
  for (int i = c; i < 64; i += NT) ltab[i] = a.logtab[i];
  for (int i = c; i < SPR_NW * a.max_moves; i += NT) red[i] = ff{0.0f, 0.0f};
  __syncthreads();
  V piv[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) piv[e] = Pol::from_d(a.pi[e]);
  const V prob = Pol::from_d(on ? a.probs[r] : 0.0);
  const bool mine1 = r == 0, mine2 = RT == 1 ? true : r == 1;
  const int lane2 = RT == 1 ? 0 : 1;
  const Coef *Dh = static_cast<const Coef *>(a.Dhalf);
  const Coef *Dm = static_cast<const Coef *>(a.Dmer) + ((size_t)(a.prune_base + blockIdx.x) * R + (on ? r : 0)) * 16;
  bool ok = true;

  for (int g = 0; g < a.G && ok; ++g) {
    const int blk = blockIdx.y * a.G + g;
    if (blk >= a.n_blocks) break;
    const size_t pat = (size_t)blk * a.NP + pl;
    auto vi = [&](int d) { return ((size_t)d * a.np + pat) * R + r; };
    auto scv = [&](int d) { return a.sc[(size_t)d * a.np + pat]; };
    const float w = a.wts[pat];
    V vp[4];
    const int scp = EMIT ? 0 : scv(pr.dp);
    if (on && !EMIT) {
      Pol::load_tip(a.M, vi(pr.dp), vp);
#pragma unroll
      for (int e = 0; e < 4; ++e) vp[e] = Pol::mul(vp[e], piv[e]);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) vp[e] = Pol::zero();
    }
    V in[4];
    int in_sc = 0, sp = 0;
    bool have = false;
    auto push = [&](const V *x, int s) {
      if (sp >= a.depth) {
        ok = false;
        return;
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) stk[((size_t)sp * 4 + e) * NT + c] = x[e];
      stk_sc[sp * NT + c] = s;
      ++sp;
    };
    for (int si = 0; si < pr.n_steps && ok; ++si) {
      const SprStep st = a.steps[pr.step_off + si];
      if (st.flags & SPR_START) {
        V ms[4], mg[4];
        if (on) {
          V ls[4], lg[4];
          Pol::load_tip(a.L, vi(st.d1), ls);
          Pol::load_tip(a.L, vi(st.d2), lg);
          Pol::rows(Dm, lg, ms);   // into s, from g's side across the joined edge
          Pol::rows(Dm, ls, mg);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) ms[e] = mg[e] = Pol::zero();
        }
        const int scs = scv(st.d2), scg = scv(st.d1);
        const bool ds = st.flags & SPR_DOWN1, dg = st.flags & SPR_DOWN2;
        const bool g_first = ds && dg && (st.flags & SPR_FIRST2);
        if (ds && dg) push(g_first ? ms : mg, g_first ? scs : scg);
        const bool take_g = g_first || !ds;
#pragma unroll
        for (int e = 0; e < 4; ++e) in[e] = take_g ? mg[e] : ms[e];
        in_sc = take_g ? scg : scs;
        have = true;
        continue;
      }
      if (!have) {
        if (sp == 0) {
          ok = false;
          break;
        }
        --sp;
#pragma unroll
        for (int e = 0; e < 4; ++e) in[e] = stk[((size_t)sp * 4 + e) * NT + c];
        in_sc = stk_sc[sp * NT + c];
      }
      const int s1 = scv(st.d1), s2 = scv(st.d2);
      V l1[4], l2[4];
      int sc1 = in_sc + s2, sc2 = in_sc + s1;
      if (on) {
        V m1[4], m2[4];
        Pol::load_tip(a.M, vi(st.d1), m1);
        Pol::load_tip(a.M, vi(st.d2), m2);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          l1[e] = Pol::mul(in[e], m2[e]);
          l2[e] = Pol::mul(in[e], m1[e]);
        }
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) l1[e] = l2[e] = Pol::zero();
      }
      rescale<Pol, RT>(l1, sc1);
      rescale<Pol, RT>(l2, sc2);
      const int e1 = st.d1 >> 1, e2 = st.d2 >> 1;
      const Coef *D1 = Dh + ((size_t)e1 * R + (on ? r : 0)) * 16;
      const Coef *D2 = Dh + ((size_t)e2 * R + (on ? r : 0)) * 16;
      V h1[4], h2[4];
      Pol::rows(D1, l1, h1);
      Pol::rows(D2, l2, h2);
      if (EMIT && (st.out1 >= 0 || st.out2 >= 0)) {
        if (on) {
          const bool side_b = ((a.prune_base + blockIdx.x) & 1) != 0;
          V hh[4], x[4], y[4];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int out = h == 0 ? st.out1 : st.out2;
            if (out < 0) continue;
            Pol::load_tip(a.H, vi(h == 0 ? st.d1 : st.d2), hh);
#pragma unroll
            for (int e = 0; e < 4; ++e) x[e] = Pol::mul(h == 0 ? h1[e] : h2[e], hh[e]);
            if (side_b) {
              Pol::rows(static_cast<const Coef *>(a.Dfull) + ((size_t)(pr.dp >> 1) * R + r) * 16, x, y);
            } else {
#pragma unroll
              for (int e = 0; e < 4; ++e) y[e] = Pol::mul(x[e], Pol::from_d(a.probs[r] * a.pi[e]));
            }
            const size_t slot = (size_t)(out - a.slot_base);
            Pol::store4(a.xout, (slot * a.np + pat) * R + r, y);
            if (r == 0) a.xsc[slot * a.np + pat] = h == 0 ? sc1 + s1 : sc2 + s2;
          }
        }
      } else if (st.out1 >= 0 || st.out2 >= 0) {
        V p1 = Pol::zero(), p2 = Pol::zero();
        if (on) {
          V hh[4];
          if (st.out1 >= 0) {
            Pol::load_tip(a.H, vi(st.d1), hh);
#pragma unroll
            for (int e = 0; e < 4; ++e) p1 = Pol::add(p1, Pol::mul(Pol::mul(h1[e], hh[e]), vp[e]));
            p1 = Pol::mul(p1, prob);
          }
          if (st.out2 >= 0) {
            Pol::load_tip(a.H, vi(st.d2), hh);
#pragma unroll
            for (int e = 0; e < 4; ++e) p2 = Pol::add(p2, Pol::mul(Pol::mul(h2[e], hh[e]), vp[e]));
            p2 = Pol::mul(p2, prob);
          }
        }
#pragma unroll
        for (int o = 1; o < RT; o <<= 1) {
          p1 = Pol::add(p1, Pol::shfl_xor(p1, o));
          p2 = Pol::add(p2, Pol::shfl_xor(p2, o));
        }
        ff v1{0.0f, 0.0f}, v2{0.0f, 0.0f};
        if (w != 0.0f) {
          if (mine1 && st.out1 >= 0) {
            if (Pol::positive(p1)) v1 = ff_mul(Pol::site_log(p1, sc1 + s1 + scp, ltab), ff{w, 0.0f});
            else atomicOr(a.flag, PGPU_FLAG_NAN);
          }
          if (mine2 && st.out2 >= 0) {
            if (Pol::positive(p2)) v2 = ff_mul(Pol::site_log(p2, sc2 + s2 + scp, ltab), ff{w, 0.0f});
            else atomicOr(a.flag, PGPU_FLAG_NAN);
          }
        }
#pragma unroll
        for (int o = RT; o < 32; o <<= 1) {
          v1 = ff_add(v1, ff_shfl_xor(v1, o));
          v2 = ff_add(v2, ff_shfl_xor(v2, o));
        }
        if (lane == 0 && st.out1 >= 0) {
          ff &dst = red[warp * a.max_moves + (st.out1 - pr.move_off)];
          dst = ff_add(dst, v1);
        }
        if (lane == lane2 && st.out2 >= 0) {
          ff &dst = red[warp * a.max_moves + (st.out2 - pr.move_off)];
          dst = ff_add(dst, v2);
        }
      }
      const bool dn1 = st.flags & SPR_DOWN1, dn2 = st.flags & SPR_DOWN2;
      if (dn1 || dn2) {
        V n1[4], n2[4];
        if (dn1) Pol::rows(D1, h1, n1);   // P(t/2) P(t/2) L = P(t) L
        if (dn2) Pol::rows(D2, h2, n2);
        const bool second_first = dn1 && dn2 && (st.flags & SPR_FIRST2);
        if (dn1 && dn2) push(second_first ? n1 : n2, second_first ? sc1 : sc2);
        const bool take2 = second_first || !dn1;
#pragma unroll
        for (int e = 0; e < 4; ++e) in[e] = take2 ? n2[e] : n1[e];
        in_sc = take2 ? sc2 : sc1;
        have = true;
      } else {
        have = false;
      }
    }
  }
  if (!ok && c == 0) atomicOr(a.flag, PGPU_FLAG_EIGEN);   // program and stack disagree
  if (EMIT) return;
  __syncthreads();
  for (int j = c; j < pr.n_moves; j += NT) {
    ff s = red[j];
    for (int w = 1; w < SPR_NW; ++w) s = ff_add(s, red[w * a.max_moves + j]);
    a.partials[(size_t)blockIdx.y * a.n_moves + pr.move_off + j] = (double)s.h + (double)s.l;
  }
}

// lnl[m] = sum over CTA groups of the partial sums, in group order
__global__ void spr_reduce_kernel(const double *partials, int n_groups, size_t n_moves, double *lnl) {
  const size_t m = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_moves) return;
  double s = 0.0, c = 0.0;
  for (int g = 0; g < n_groups; ++g) {
    double t, e;
    two_sum(s, partials[(size_t)g * n_moves + m], t, e);
    s = t;
    c += e;
  }
  lnl[m] = s + c;
}

// ---------------------------------------------------------------------------
// TBR pairs.  For a cut edge (a,b) with the attach vectors of both sides
// from the emit walks (a's side weighted, b's side carried across the cut),
//   site(j, k) = sum_r sum_i X_j[r][i] Z_k[r][i]
//              = sum_r probs_r sum_i pi_i X_j[r][i] [P(t_ab) Y_k][r][i],
// with the two scalers added.  A CTA takes 16 x 16 (j, k) pairs, one per
// thread, over a group of pattern blocks; per block of TB_PB patterns the
// X_j and Z_k are staged in shared memory, rows padded by one element so
// that the 16 Z rows a warp reads fall in distinct banks.
// ---------------------------------------------------------------------------
constexpr int TB_T = 16;
constexpr int TB_PB = 16;

struct TbrCutDev {
  int edge, nA, nB, pad;
  long long slotA, slotB;   // first emit slot of each side
  long long move_off;       // first move of the cut within the launch's range
};

struct PairArgs {
  const void *X;            // [slot][np][R] x 4
  const int32_t *xsc;       // [slot][np]
  const int4 *tiles;        // {cut, j0, k0, 0}
  const TbrCutDev *cuts;
  const float *wts;         // [np], zero beyond n_pat
  const float4 *logtab;
  double *partials;         // [n_groups][n_moves]
  int *flag;
  size_t np;
  long long n_moves;
  int R, G, n_pblocks;
};

__host__ __device__ inline int tbr_row(int R) { return TB_PB * R * 4 + 1; }

template <typename Pol>
__host__ __device__ size_t pair_smem(int R) {
  return 1024 + 2 * (size_t)TB_T * tbr_row(R) * sizeof(typename Pol::V) + 2 * TB_T * TB_PB * sizeof(int);
}

// sum_q x_q z_q of one site.  In the float-pair form the terms are
// non-negative, so they are summed as the pruning rows sum: exact products
// (TwoProduct and the two cross terms), the high parts added exactly by a
// Fast2Sum of the larger and the smaller, everything else gathered in one
// float; the pair is normalised once at the end.  About 11 instructions a
// term against 15 for a pair add per term.
template <typename Pol>
__device__ __forceinline__ typename Pol::V pair_dot(const typename Pol::V *x, const typename Pol::V *z, int n) {
  if constexpr (std::is_same<Pol, Ff32>::value) {
    float sh = __fmul_rn(x[0].h, z[0].h);
    float lo = __fmaf_rn(x[0].h, z[0].h, -sh);
    lo = __fmaf_rn(x[0].h, z[0].l, lo);
    lo = __fmaf_rn(x[0].l, z[0].h, lo);
    for (int q = 1; q < n; ++q) {
      const float p = __fmul_rn(x[q].h, z[q].h);
      float e = __fmaf_rn(x[q].h, z[q].h, -p);
      e = __fmaf_rn(x[q].h, z[q].l, e);
      e = __fmaf_rn(x[q].l, z[q].h, e);
      const ff t = fast_two_sum(fmaxf(sh, p), fminf(sh, p));
      sh = t.h;
      lo = __fadd_rn(lo, __fadd_rn(t.l, e));
    }
    return fast_two_sum(sh, lo);
  } else {
    typename Pol::V acc = Pol::zero();
    for (int q = 0; q < n; ++q) acc = Pol::add(acc, Pol::mul(x[q], z[q]));
    return acc;
  }
}

template <typename Pol>
__global__ void __launch_bounds__(256) tbr_pair_kernel(const PairArgs a) {
  using V = typename Pol::V;
  extern __shared__ __align__(16) unsigned char smem[];
  const int R = a.R, RS = tbr_row(R);
  float4 *ltab = reinterpret_cast<float4 *>(smem);
  V *Xs = reinterpret_cast<V *>(smem + 1024);
  V *Zs = Xs + (size_t)TB_T * RS;
  int *xs = reinterpret_cast<int *>(Zs + (size_t)TB_T * RS);
  int *ys = xs + TB_T * TB_PB;
  const int t = threadIdx.x;
  for (int i = t; i < 64; i += 256) ltab[i] = a.logtab[i];
  const int4 tl = a.tiles[blockIdx.x];
  const TbrCutDev cut = a.cuts[tl.x];
  const int jj = t / TB_T, kk = t % TB_T;
  const int j = tl.y + jj, k = tl.z + kk;
  const bool mine = j < cut.nA && k < cut.nB;
  const int per_side = TB_T * TB_PB * R;
  ff sum{0.0f, 0.0f};
  for (int g = 0; g < a.G; ++g) {
    const int blk = blockIdx.y * a.G + g;
    if (blk >= a.n_pblocks) break;
    const size_t pat0 = (size_t)blk * TB_PB;
    __syncthreads();   // the previous block's tiles are consumed
    for (int it = t; it < 2 * per_side; it += 256) {
      const int side = it / per_side, rem = it % per_side;
      const int row = rem / (TB_PB * R), p = (rem / R) % TB_PB, r = rem % R;
      const int idx = (side == 0 ? tl.y : tl.z) + row;
      const size_t pat = pat0 + p;
      V v[4];
      int sc = 0;
      if (idx < (side == 0 ? cut.nA : cut.nB)) {
        const size_t slot = (size_t)((side == 0 ? cut.slotA : cut.slotB) + idx);
        Pol::load_tip(a.X, (slot * a.np + pat) * R + r, v);
        sc = a.xsc[slot * a.np + pat];
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = Pol::zero();
      }
      V *dst = (side == 0 ? Xs : Zs) + (size_t)row * RS + ((size_t)p * R + r) * 4;
#pragma unroll
      for (int e = 0; e < 4; ++e) dst[e] = v[e];
      if (r == 0) (side == 0 ? xs : ys)[row * TB_PB + p] = sc;
    }
    __syncthreads();
    if (!mine) continue;
    for (int p = 0; p < TB_PB; ++p) {
      const float w = a.wts[pat0 + p];
      if (w == 0.0f) continue;
      const V *xr = Xs + (size_t)jj * RS + (size_t)p * R * 4;
      const V *zr = Zs + (size_t)kk * RS + (size_t)p * R * 4;
      const V acc = pair_dot<Pol>(xr, zr, R * 4);
      if (Pol::positive(acc))
        sum = ff_add(sum, ff_mul(Pol::site_log(acc, xs[jj * TB_PB + p] + ys[kk * TB_PB + p], ltab),
                                 ff{w, 0.0f}));
      else
        atomicOr(a.flag, PGPU_FLAG_NAN);
    }
  }
  if (mine)
    a.partials[(size_t)blockIdx.y * a.n_moves + cut.move_off + (long long)j * cut.nB + k] =
        (double)sum.h + (double)sum.l;
}

// ---------------------------------------------------------------------------
// Fitch sets on the directed edges and the parsimony length of every move
// ---------------------------------------------------------------------------
constexpr uint32_t LANE_MSB = 0x88888888u;

__device__ __forceinline__ uint32_t empty_lanes(uint32_t v) {
  const uint32_t nz = (((v & ~LANE_MSB) + ~LANE_MSB) | v) & LANE_MSB;
  return nz ^ LANE_MSB;
}
__device__ __forceinline__ uint32_t fitch_set(uint32_t a, uint32_t b, uint32_t *empty) {
  const uint32_t x = a & b;
  const uint32_t e = empty_lanes(x);
  const uint32_t fill = e | (e - (e >> 3));
  *empty = e;
  return (x & ~fill) | ((a | b) & fill);
}
__device__ __forceinline__ uint4 fitch4(uint4 a, uint4 b, uint4 *e) {
  uint4 o;
  o.x = fitch_set(a.x, b.x, &e->x);
  o.y = fitch_set(a.y, b.y, &e->y);
  o.z = fitch_set(a.z, b.z, &e->z);
  o.w = fitch_set(a.w, b.w, &e->w);
  return o;
}
// weighted count of the lanes flagged in e (lane MSBs), weights as bit planes
__device__ __forceinline__ uint32_t wcount(uint4 e, const uint4 *planes, size_t stride, int n_planes,
                                           size_t at) {
  uint32_t s = 0;
  for (int b = 0; b < n_planes; ++b) {
    const uint4 p = planes[(size_t)b * stride + at];
    s += (uint32_t)(__popc(e.x & p.x) + __popc(e.y & p.y) + __popc(e.z & p.z) + __popc(e.w & p.w)) << b;
  }
  return s;
}

struct FitchTipArgs {
  uint4 *F;
  const uint8_t *codes;
  const uint8_t *code_mask;   // [n_codes] state-set bits
  const int4 *tips;
  size_t W4, n_pat, ld;
  int n_codes;
};

__global__ void __launch_bounds__(256) spr_fitch_tip_kernel(const FitchTipArgs a) {
  const size_t q = (size_t)blockIdx.x * 256 + threadIdx.x;
  if (q >= a.W4) return;
  const int4 t = a.tips[blockIdx.y];
  uint32_t wv[4];
  for (int k = 0; k < 4; ++k) {
    uint32_t word = 0;
    for (int j = 0; j < 8; ++j) {
      const size_t pat = (q * 4 + k) * 8 + j;
      uint32_t m = 0;
      if (pat < a.n_pat) {
        const int code = a.codes[(size_t)t.y * a.ld + pat];
        m = code < a.n_codes ? a.code_mask[code] : 0xFu;
      }
      word |= (m & 0xFu) << (4 * j);
    }
    wv[k] = word;
  }
  a.F[(size_t)t.x * a.W4 + q] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
}

struct FitchPoolArgs {
  uint4 *F;
  const int4 *ops;
  const uint4 *planes;
  unsigned long long *cnt;   // [n_ops + 1]: local cost of each op, then edge 0's join
  size_t W4;
  int n_ops, n_planes;
};

__device__ __forceinline__ void block_add_u64(uint32_t v, unsigned long long *dst) {
  __shared__ unsigned long long acc;
  if (threadIdx.x == 0) acc = 0;
  __syncthreads();
  v = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(&acc, (unsigned long long)v);
  __syncthreads();
  if (threadIdx.x == 0 && acc) atomicAdd(dst, acc);
}

__global__ void __launch_bounds__(256) spr_fitch_pool_kernel(const FitchPoolArgs a) {
  const size_t q = (size_t)blockIdx.x * 256 + threadIdx.x;
  const bool in = q < a.W4;
  for (int i = 0; i < a.n_ops; ++i) {
    const int4 op = __ldg(a.ops + i);
    uint32_t v = 0;
    if (in) {
      uint4 e;
      const uint4 o = fitch4(a.F[(size_t)op.y * a.W4 + q], a.F[(size_t)op.z * a.W4 + q], &e);
      a.F[(size_t)op.x * a.W4 + q] = o;
      v = wcount(e, a.planes, a.W4, a.n_planes, q);
    }
    block_add_u64(v, a.cnt + i);
  }
  uint32_t v = 0;
  if (in) {
    uint4 e;
    (void)fitch4(a.F[q], a.F[a.W4 + q], &e);
    v = wcount(e, a.planes, a.W4, a.n_planes, q);
  }
  block_add_u64(v, a.cnt + a.n_ops);
}

// lenF[d]: parsimony length of the subtree on d's side; lenF[nd] = tree length
__global__ void spr_fitch_len_kernel(const int4 *ops, int n_ops, const unsigned long long *cnt,
                                     unsigned long long *lenF, int nd) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  // tips (and everything) start at 0; ops fill in dependency order
  for (int d = 0; d < nd; ++d) lenF[d] = 0;
  for (int i = 0; i < n_ops; ++i) {
    const int4 op = ops[i];
    lenF[op.x] = lenF[op.y] + lenF[op.z] + cnt[i];
  }
  lenF[nd] = lenF[0] + lenF[1] + cnt[n_ops];
}

struct FitchScanArgs {
  const uint4 *F;
  const uint4 *planes;
  const SprStep *steps;
  const SprPrune *prunes;
  unsigned long long *ins;     // [n_moves] weighted empty joins with the pruned set
  unsigned long long *join;    // [n_prunes] weighted empty joins of s and g
  size_t W4;
  int n_planes, depth, max_moves, *flag;
};

__global__ void __launch_bounds__(256) spr_fitch_scan_kernel(const FitchScanArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SprPrune pr = a.prunes[blockIdx.x];
  unsigned int *red = reinterpret_cast<unsigned int *>(smem);   // [max_moves]
  uint4 *stk = reinterpret_cast<uint4 *>(smem + a16((size_t)a.max_moves * 4));
  __shared__ unsigned int join_acc;
  const int c = threadIdx.x;
  for (int i = c; i < a.max_moves; i += 256) red[i] = 0;
  if (c == 0) join_acc = 0;
  __syncthreads();
  const size_t q = (size_t)blockIdx.y * 256 + c;
  const bool in = q < a.W4;
  const size_t qq = in ? q : 0;
  auto Fd = [&](int d) { return in ? a.F[(size_t)d * a.W4 + qq] : make_uint4(0, 0, 0, 0); };
  const uint4 fp = Fd(pr.dp);
  uint4 cur = make_uint4(0, 0, 0, 0);
  int sp = 0;
  bool have = false, ok = true;
  auto count = [&](uint4 e) { return in ? wcount(e, a.planes, a.W4, a.n_planes, qq) : 0u; };
  auto add = [&](unsigned int *dst, uint32_t v) {
    v = __reduce_add_sync(0xffffffffu, v);
    if ((c & 31) == 0 && v) atomicAdd(dst, v);
  };
  for (int si = 0; si < pr.n_steps && ok; ++si) {
    const SprStep st = a.steps[pr.step_off + si];
    if (st.flags & SPR_START) {
      const uint4 fs = Fd(st.d1), fg = Fd(st.d2);
      uint4 e;
      (void)fitch4(fs, fg, &e);
      add(&join_acc, count(e));
      const bool ds = st.flags & SPR_DOWN1, dg = st.flags & SPR_DOWN2;
      const bool g_first = ds && dg && (st.flags & SPR_FIRST2);
      if (ds && dg) {
        if (sp >= a.depth) { ok = false; break; }
        stk[(size_t)sp * 256 + c] = g_first ? fg : fs;   // set entering s is g's side
        ++sp;
      }
      cur = (g_first || !ds) ? fs : fg;
      have = true;
      continue;
    }
    if (!have) {
      if (sp == 0) { ok = false; break; }
      --sp;
      cur = stk[(size_t)sp * 256 + c];
    }
    const uint4 f1 = Fd(st.d1), f2 = Fd(st.d2);
    uint4 e;
    const uint4 r1 = fitch4(cur, f2, &e);   // y's side seen from c1
    const uint4 r2 = fitch4(cur, f1, &e);
    if (st.out1 >= 0) {
      const uint4 root = fitch4(r1, f1, &e);
      const uint4 x = make_uint4(fp.x & root.x, fp.y & root.y, fp.z & root.z, fp.w & root.w);
      add(&red[st.out1 - pr.move_off],
          count(make_uint4(empty_lanes(x.x), empty_lanes(x.y), empty_lanes(x.z), empty_lanes(x.w))));
    }
    if (st.out2 >= 0) {
      const uint4 root = fitch4(r2, f2, &e);
      const uint4 x = make_uint4(fp.x & root.x, fp.y & root.y, fp.z & root.z, fp.w & root.w);
      add(&red[st.out2 - pr.move_off],
          count(make_uint4(empty_lanes(x.x), empty_lanes(x.y), empty_lanes(x.z), empty_lanes(x.w))));
    }
    const bool dn1 = st.flags & SPR_DOWN1, dn2 = st.flags & SPR_DOWN2;
    if (dn1 || dn2) {
      const bool second_first = dn1 && dn2 && (st.flags & SPR_FIRST2);
      if (dn1 && dn2) {
        if (sp >= a.depth) { ok = false; break; }
        stk[(size_t)sp * 256 + c] = second_first ? r1 : r2;
        ++sp;
      }
      cur = (second_first || !dn1) ? r2 : r1;
      have = true;
    } else {
      have = false;
    }
  }
  if (!ok && c == 0) atomicOr(a.flag, PGPU_FLAG_EIGEN);
  __syncthreads();
  for (int j = c; j < pr.n_moves; j += 256)
    if (red[j]) atomicAdd(a.ins + pr.move_off + j, (unsigned long long)red[j]);
  if (c == 0 && join_acc) atomicAdd(a.join + blockIdx.x, (unsigned long long)join_acc);
}

// ---------------------------------------------------------------------------
// per-directed-edge summaries and per-move features
// ---------------------------------------------------------------------------
struct SummaryArgs {
  const void *L;
  const double *probs, *weights;
  float *out;   // [nd][4]
  size_t np, n_pat;
  int R;
  double inv_w;   // 1 / total weight
};

// weighted mean over patterns of the state profile L_i / sum_j L_j
template <typename Pol>
__global__ void __launch_bounds__(256) spr_summary_kernel(const SummaryArgs a) {
  using V = typename Pol::V;
  __shared__ double red[4][8];
  const int d = blockIdx.x;
  double acc[4] = {0, 0, 0, 0}, wsum = 0.0;
  for (size_t pat = threadIdx.x; pat < a.n_pat; pat += 256) {
    const double w = a.weights[pat];
    for (int r = 0; r < a.R; ++r) {
      V x[4];
      Pol::load_tip(a.L, ((size_t)d * a.np + pat) * a.R + r, x);
      float f[4], s = 0.0f;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        f[e] = (float)Pol::to_d(x[e]);
        s += f[e];
      }
      const double k = s > 0.0f ? w * a.probs[r] / s : 0.0;
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[e] += k * f[e];
    }
    wsum += w;
  }
  (void)wsum;
  for (int e = 0; e < 4; ++e) {
    double v = acc[e];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[e][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0.0;
    for (int w = 0; w < 8; ++w) v += red[threadIdx.x][w];
    a.out[(size_t)d * 4 + threadIdx.x] = (float)(v * a.inv_w);
  }
}

struct FeatArgs {
  const SprMove *moves;
  const SprPrune *prunes;
  const int32_t *tipcnt;
  const double *len;               // [n_edges]
  const float *summ;               // [nd][4], already divided by the total weight
  const unsigned long long *lenF;  // [nd + 1]
  const unsigned long long *ins, *join;
  float *X;                        // [n_moves][64]
  size_t n_moves;
  int n_tips, nd;
  double wtot;
};

__global__ void __launch_bounds__(256) spr_feature_kernel(const FeatArgs a) {
  const size_t m = (size_t)blockIdx.x * 256 + threadIdx.x;
  if (m >= a.n_moves) return;
  const SprMove mv = a.moves[m];
  const SprPrune pr = a.prunes[mv.prune];
  const float ln_n = logf((float)a.n_tips);
  const int dp = pr.dp, dc = mv.dc, dy = dc ^ 1;
  float f[SPR_FEATURES];
#pragma unroll
  for (int i = 0; i < SPR_FEATURES; ++i) f[i] = 0.0f;
  const float P = (float)a.tipcnt[dp];
  f[0] = logf(P) / ln_n;
  f[1] = logf((float)a.n_tips - P) / ln_n;
  f[2] = log1pf((float)mv.depth);
  const double t_pu = a.len[dp >> 1], t_s = a.len[pr.ds >> 1], t_g = a.len[pr.dg >> 1],
               t_c = a.len[dc >> 1];
  f[3] = logf((float)t_pu + 1e-4f);
  f[4] = logf((float)(t_s + t_g) + 1e-4f);
  f[5] = logf((float)t_c + 1e-4f);
  // u's other two neighbours are unordered: only symmetric functions of them
  f[6] = logf((float)fmin(t_s, t_g) + 1e-4f);
  f[7] = logf((float)fmax(t_s, t_g) + 1e-4f);
  // parsimony: length of the rearranged tree minus the current length
  const double lenT = (double)a.lenF[a.nd];
  // remaining tree joined at (s,g) plus the pruned subtree, then the new join
  const double lenR = (double)a.lenF[pr.ds] + (double)a.lenF[pr.dg] + (double)a.join[mv.prune] +
                      (double)a.lenF[dp];
  const double dF = lenR + (double)a.ins[m] - lenT;
  const double sc = 100.0 / a.wtot;
  f[8] = (float)(dF * sc);
  f[9] = dF < 0 ? 1.0f : 0.0f;
  f[10] = dF == 0 ? 1.0f : 0.0f;
  f[11] = dF > 0 ? 1.0f : 0.0f;
  f[12] = asinhf((float)dF);
  f[13] = (float)((lenR - lenT) * sc);
  f[14] = (float)((double)a.ins[m] * sc);
  f[15] = logf((float)a.tipcnt[dc]) / ln_n;
  const float *sp = a.summ + (size_t)dp * 4, *sc_ = a.summ + (size_t)dc * 4,
              *sy = a.summ + (size_t)dy * 4, *ss = a.summ + (size_t)pr.ds * 4,
              *sg = a.summ + (size_t)pr.dg * 4;
  float dot_c = 0.0f, dot_s = 0.0f;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float mean_sg = 0.5f * (ss[e] + sg[e]), diff_sg = fabsf(ss[e] - sg[e]);
    f[16 + e] = sp[e];
    f[20 + e] = sc_[e];
    f[24 + e] = sy[e];
    f[28 + e] = mean_sg;
    f[32 + e] = diff_sg;
    f[36 + e] = sp[e] * sc_[e];
    f[40 + e] = sp[e] * sy[e];
    f[44 + e] = sp[e] * mean_sg;
    f[48 + e] = sp[e] * diff_sg;
    dot_c += sp[e] * sc_[e];
    dot_s += sp[e] * mean_sg;
  }
  f[52] = dot_c;
  f[53] = dot_s;
  f[54] = mv.depth == 1 ? 1.0f : 0.0f;
  float *o = a.X + m * SPR_FEATURES;
#pragma unroll
  for (int i = 0; i < SPR_FEATURES; ++i) o[i] = f[i];
}

}  // namespace

// ---------------------------------------------------------------------------
// branch lengths: Newton steps on every edge at once, from the pool
// ---------------------------------------------------------------------------
namespace {

struct BlArgs {
  const void *L;
  const double *U, *Ui, *lam, *pi, *rates, *probs, *weights;
  float *S;                 // [n_edges][np][R][4]: eigen-basis products
  const double *len_in;
  double *len_out;
  size_t np, n_pat;
  int R, n_edges, iters;
  double tol, tmin, tmax;
};

// S[e][pat][r][k] = (sum_i pi_i L[a|b]_i U_ik) (sum_j Ui_kj L[b|a]_j), so that
// the site likelihood across edge e is sum_r probs_r sum_k S_k exp(lam_k rate_r t)
template <typename Pol>
__global__ void __launch_bounds__(256) bl_sumtab_kernel(const BlArgs a) {
  using V = typename Pol::V;
  const size_t i = (size_t)blockIdx.x * 256 + threadIdx.x;
  if (i >= a.np * a.R) return;
  const int e = blockIdx.y;
  V x[4], y[4];
  Pol::load_tip(a.L, (size_t)(2 * e) * a.np * a.R + i, x);
  Pol::load_tip(a.L, (size_t)(2 * e + 1) * a.np * a.R + i, y);
  float s[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double A = 0.0, B = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      A += a.pi[j] * Pol::to_d(x[j]) * a.U[j * 4 + k];
      B += a.Ui[k * 4 + j] * Pol::to_d(y[j]);
    }
    s[k] = (float)(A * B);
  }
  reinterpret_cast<float4 *>(a.S)[(size_t)e * a.np * a.R + i] = make_float4(s[0], s[1], s[2], s[3]);
}

// One CTA per edge: Newton iterations on t with the derivatives of
// sum_s w_s log f_s(t) summed over all patterns.
__global__ void __launch_bounds__(256) bl_newton_kernel(const BlArgs a) {
  __shared__ double red[2][8];
  __shared__ double t_sh;
  __shared__ int done;
  const int e = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    t_sh = a.len_in[e];
    done = 0;
  }
  __syncthreads();
  for (int it = 0; it < a.iters; ++it) {
    const double t = t_sh;
    float cf[8][4], ex[8][4];
    for (int r = 0; r < a.R; ++r)
      for (int k = 0; k < 4; ++k) {
        cf[r][k] = (float)(a.lam[k] * a.rates[r]);
        ex[r][k] = (float)(exp(a.lam[k] * a.rates[r] * t) * a.probs[r]);
      }
    double g = 0.0, h = 0.0;
    const float4 *S = reinterpret_cast<const float4 *>(a.S) + (size_t)e * a.np * a.R;
    for (size_t pat = tid; pat < a.n_pat; pat += 256) {
      float f = 0.0f, f1 = 0.0f, f2 = 0.0f;
      for (int r = 0; r < a.R; ++r) {
        const float4 s = S[pat * a.R + r];
        const float sv[4] = {s.x, s.y, s.z, s.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float v = sv[k] * ex[r][k];
          f += v;
          f1 = fmaf(v, cf[r][k], f1);
          f2 = fmaf(v * cf[r][k], cf[r][k], f2);
        }
      }
      if (f > 0.0f) {
        const double d1 = (double)(f1 / f);
        const double w = a.weights[pat];
        g += w * d1;
        h += w * ((double)(f2 / f) - d1 * d1);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      g += __shfl_xor_sync(0xffffffffu, g, o);
      h += __shfl_xor_sync(0xffffffffu, h, o);
    }
    if (lane == 0) {
      red[0][warp] = g;
      red[1][warp] = h;
    }
    __syncthreads();
    if (tid == 0) {
      double G = 0.0, Hs = 0.0;
      for (int w = 0; w < 8; ++w) {
        G += red[0][w];
        Hs += red[1][w];
      }
      double tn;
      if (Hs < 0.0) tn = t - G / Hs;
      else tn = G > 0.0 ? t * 2.0 : t * 0.5;
      // keep each step inside a factor of ten of the current length
      tn = fmin(fmax(tn, fmax(a.tmin, 0.1 * t)), fmin(a.tmax, 10.0 * fmax(t, a.tmin)));
      if (fabs(tn - t) <= a.tol * fmax(t, 1e-3)) done = 1;
      t_sh = tn;
    }
    __syncthreads();
    if (done) break;
  }
  if (tid == 0) a.len_out[e] = t_sh;
}

__global__ void spr_fitch_moves_kernel(const SprMove *moves, const SprPrune *prunes, size_t n_moves,
                                       const unsigned long long *lenF, const unsigned long long *ins,
                                       const unsigned long long *join, unsigned long long *out) {
  const size_t m = (size_t)blockIdx.x * 256 + threadIdx.x;
  if (m >= n_moves) return;
  const SprMove mv = moves[m];
  const SprPrune pr = prunes[mv.prune];
  // the rest joined at (s,g), the pruned subtree itself, and its new join
  out[m] = lenF[pr.ds] + lenF[pr.dg] + join[mv.prune] + lenF[pr.dp] + ins[m];
}

}  // namespace

// ---------------------------------------------------------------------------
// the engine object
// ---------------------------------------------------------------------------
struct SprPlanDev {
  SprStep *steps = nullptr;
  SprPrune *prunes = nullptr;
  SprMove *moves = nullptr;
  double *mlen = nullptr;   // merged lengths
  void *Dmer = nullptr;
  size_t cap_steps = 0, cap_prunes = 0, cap_moves = 0;
};

struct pgpu_spr {
  pgpu_ctx *ctx = nullptr;
  int precision = 48, R = 1, n = 0, n_codes = 0, RT = 1, NP = 256, n_planes = 0;
  size_t n_pat = 0, np = 0, ld = 0, W4 = 0, vbytes = 0, cbytes = 0;
  double wtot = 0.0;
  const uint8_t *codes = nullptr;
  // model
  double *Q = nullptr, *pi = nullptr, *rates = nullptr, *probs = nullptr, *ctab = nullptr,
         *U = nullptr, *Ui = nullptr, *lam = nullptr;
  int *status = nullptr;
  uint8_t *cmask = nullptr;
  double *w = nullptr;
  float *wf = nullptr;
  float4 *logtab = nullptr;
  // pool
  void *L = nullptr, *M = nullptr, *H = nullptr;
  int32_t *sc = nullptr;
  void *Dfull = nullptr, *tipfull = nullptr, *tiphalf = nullptr;
  double *elen = nullptr, *tiplen = nullptr, *newlen = nullptr;
  int4 *ops = nullptr, *tips = nullptr;
  double2 *pool_part = nullptr;
  double *tree_lnl = nullptr, *site_lnl = nullptr;
  // fitch
  uint4 *F = nullptr, *planes = nullptr;
  unsigned long long *cntF = nullptr, *lenF = nullptr, *ins = nullptr, *join = nullptr;
  float *summ = nullptr;
  // scratch
  double *partials = nullptr;
  size_t part_cap = 0;
  float *S = nullptr;
  // host state
  SprTopo T;
  PoolPlan pp;
  SprPlan all, sel;
  SprPlanDev all_d, sel_d;
  bool pool_valid = false, plan_valid = false, fitch_valid = false, summ_valid = false;
  int join_distance = 0;   // 0: every SPR move; d: regraft edges at most d nodes from the break
  // TBR: plan, emit walks on the device, attach vectors of a batch of cuts
  TbrPlan tbr;
  SprPlanDev tbr_d;
  bool tbr_valid = false;
  int tbr_join = 0, tbr_reroot = 0;   // attach-edge limits in nodes from the cut (0: none)
  size_t tbr_budget = size_t(2) << 30;   // attach-vector bytes per batch of cuts
  char *tbr_x = nullptr;
  int32_t *tbr_xsc = nullptr;
  TbrCutDev *tbr_cuts = nullptr;
  int4 *tbr_tiles = nullptr;
  size_t tbr_x_cap = 0, tbr_xsc_cap = 0, tbr_cuts_cap = 0, tbr_tiles_cap = 0;
  // with two different limits: every pair's lnL, and the listed pairs' grid indices
  double *tbr_grid = nullptr;
  int64_t *tbr_keep = nullptr;
  size_t tbr_grid_cap = 0, tbr_keep_cap = 0;
  // host copies of a TBR batch's cut and tile lists, owned by the engine so
  // that they outlive the asynchronous copies to the device
  std::vector<TbrCutDev> h_tbr_cuts;
  std::vector<int4> h_tbr_tiles;
  std::vector<void *> owned;
};

namespace {

pgpu_status dalloc(pgpu_spr *s, size_t bytes, void **p) {
  PGPU_CUDA(s->ctx, cudaMalloc(p, std::max<size_t>(bytes, 16)));
  s->owned.push_back(*p);
  return PGPU_OK;
}
template <typename T>
pgpu_status dalloc_t(pgpu_spr *s, size_t n, T **p) {
  void *v;
  PGPU_TRY(dalloc(s, n * sizeof(T), &v));
  *p = static_cast<T *>(v);
  return PGPU_OK;
}
template <typename T>
pgpu_status grow(pgpu_spr *s, T **p, size_t *cap, size_t n) {
  if (*cap >= n) return PGPU_OK;
  if (*p) {
    cudaFree(*p);
    s->owned.erase(std::find(s->owned.begin(), s->owned.end(), (void *)*p));
  }
  *p = nullptr;
  const size_t want = std::max<size_t>(n + n / 4, 64);
  PGPU_TRY(dalloc_t(s, want, p));
  *cap = want;
  return PGPU_OK;
}
template <typename T>
pgpu_status upload(pgpu_spr *s, T *dst, const T *src, size_t n) {
  if (n) PGPU_CUDA(s->ctx, cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s->ctx->stream));
  return PGPU_OK;
}

int p32_mode(int prec) { return prec == 32 ? P32_MINUS_I : prec == 64 ? P32_PLAIN : P32_PAIRS_ROWS4; }
int tip_form(int prec) { return prec == 32 ? 0 : prec == 64 ? 2 : 3; }

pgpu_status compose(pgpu_spr *s, const double *t_dev, int n_br, void *out) {
  return pgpu_launch_compose(s->ctx, s->U, s->lam, s->Ui, 4, t_dev, n_br, s->rates, s->R,
                             s->precision == 64 ? (double *)out : nullptr,
                             s->precision == 64 ? nullptr : (float *)out, false, s->status,
                             p32_mode(s->precision));
}

template <typename Pol, int RT>
pgpu_status launch_pool_rt(pgpu_spr *s) {
  PoolArgs a;
  a.L = s->L;
  a.M = s->M;
  a.H = s->H;
  a.sc = s->sc;
  a.Dfull = s->Dfull;
  a.Dhalf = static_cast<char *>(s->Dfull) + (size_t)s->T.n_edges() * s->cbytes;
  a.ops = s->ops;
  a.pi = s->pi;
  a.probs = s->probs;
  a.weights = s->w;
  a.site_lnl = s->site_lnl;
  a.partials = s->pool_part;
  a.np = s->np;
  a.n_pat = s->n_pat;
  a.n_ops = (int)s->pp.ops.size();
  a.R = s->R;
  a.NP = s->NP;
  spr_pool_kernel<Pol, RT><<<(unsigned)(s->np / s->NP), SPR_NT, 0, s->ctx->stream>>>(a);
  return pgpu_after_launch(s->ctx, "spr_pool_kernel");
}

template <typename Pol>
pgpu_status launch_pool(pgpu_spr *s) {
  TipArgs t;
  t.L = s->L;
  t.M = s->M;
  t.H = s->H;
  t.sc = s->sc;
  t.tipfull = s->tipfull;
  t.tiphalf = s->tiphalf;
  t.code_tab = s->ctab;
  t.codes = s->codes;
  t.tips = s->tips;
  t.flag = s->ctx->d_flag;
  t.np = s->np;
  t.n_pat = s->n_pat;
  t.ld = s->ld;
  t.R = s->R;
  t.n_codes = s->n_codes;
  spr_tip_kernel<Pol><<<dim3((unsigned)((s->np + 255) / 256), (unsigned)s->n), 256, 0, s->ctx->stream>>>(t);
  PGPU_TRY(pgpu_after_launch(s->ctx, "spr_tip_kernel"));
  switch (s->RT) {
    case 1: return launch_pool_rt<Pol, 1>(s);
    case 2: return launch_pool_rt<Pol, 2>(s);
    case 4: return launch_pool_rt<Pol, 4>(s);
    default: return launch_pool_rt<Pol, 8>(s);
  }
}

// Rebuilds everything that depends on the topology and branch lengths.
pgpu_status ensure_pool(pgpu_spr *s) {
  if (s->pool_valid) return PGPU_OK;
  SprTopo &T = s->T;
  spr_pool_plan(T, &s->pp);
  const int ne = T.n_edges();
  std::vector<double> h(2 * ne + 2 * s->n);
  for (int e = 0; e < ne; ++e) {
    h[e] = T.len[e];
    h[ne + e] = 0.5 * T.len[e];
  }
  for (int x = 0; x < s->n; ++x) {
    h[2 * ne + x] = T.len[T.inc[x][0]];
    h[2 * ne + s->n + x] = 0.5 * T.len[T.inc[x][0]];
  }
  PGPU_TRY(upload(s, s->elen, h.data(), h.size()));
  PGPU_TRY(upload(s, s->ops, s->pp.ops.data(), s->pp.ops.size()));
  PGPU_TRY(upload(s, s->tips, s->pp.tips.data(), s->pp.tips.size()));
  PGPU_TRY(compose(s, s->elen, 2 * ne, s->Dfull));
  for (int half = 0; half < 2; ++half)
    PGPU_TRY(pgpu_launch_tip_table(s->ctx, s->U, s->lam, s->Ui, 4, s->elen + 2 * ne + half * s->n, s->n,
                                   s->rates, s->R, s->ctab, s->n_codes,
                                   half ? s->tiphalf : s->tipfull, tip_form(s->precision), s->status));
  if (s->precision == 32) PGPU_TRY(launch_pool<Fp32>(s));
  else if (s->precision == 48) PGPU_TRY(launch_pool<Ff32>(s));
  else PGPU_TRY(launch_pool<Fp64>(s));
  spr_pool_finalize_kernel<<<1, 1024, 0, s->ctx->stream>>>(s->pool_part, (int)(s->np / s->NP), s->tree_lnl);
  PGPU_TRY(pgpu_after_launch(s->ctx, "spr_pool_finalize_kernel"));
  s->pool_valid = true;
  return PGPU_OK;
}

pgpu_status upload_plan(pgpu_spr *s, const SprPlan &p, SprPlanDev *d) {
  PGPU_TRY(grow(s, &d->steps, &d->cap_steps, p.steps.size()));
  size_t cp = d->cap_prunes;
  PGPU_TRY(grow(s, &d->prunes, &d->cap_prunes, p.prunes.size()));
  if (d->cap_prunes != cp || !d->mlen) {
    size_t c2 = 0;
    d->mlen = nullptr;
    PGPU_TRY(grow(s, &d->mlen, &c2, d->cap_prunes));
    void *dm;
    PGPU_TRY(dalloc(s, d->cap_prunes * s->cbytes, &dm));
    d->Dmer = dm;
  }
  PGPU_TRY(grow(s, &d->moves, &d->cap_moves, p.moves.size()));
  PGPU_TRY(upload(s, d->steps, p.steps.data(), p.steps.size()));
  PGPU_TRY(upload(s, d->prunes, p.prunes.data(), p.prunes.size()));
  PGPU_TRY(upload(s, d->moves, p.moves.data(), p.moves.size()));
  PGPU_TRY(upload(s, d->mlen, p.merged_len.data(), p.merged_len.size()));
  if (!p.prunes.empty()) PGPU_TRY(compose(s, d->mlen, (int)p.prunes.size(), d->Dmer));
  return PGPU_OK;
}

pgpu_status ensure_plan(pgpu_spr *s) {
  if (s->plan_valid) return PGPU_OK;
  PGPU_TRY(ensure_pool(s));
  spr_plan_all(s->T, s->pp, &s->all, s->join_distance);
  PGPU_TRY(upload_plan(s, s->all, &s->all_d));
  s->plan_valid = true;
  return PGPU_OK;
}

template <typename Pol, int RT>
pgpu_status launch_scan_rt(pgpu_spr *s, const SprPlan &p, const SprPlanDev &d, int G, int n_groups,
                           int n_blocks) {
  ScanArgs a;
  a.L = s->L;
  a.M = s->M;
  a.H = s->H;
  a.sc = s->sc;
  a.Dhalf = static_cast<char *>(s->Dfull) + (size_t)s->T.n_edges() * s->cbytes;
  a.Dmer = d.Dmer;
  a.steps = d.steps;
  a.prunes = d.prunes;
  a.pi = s->pi;
  a.probs = s->probs;
  a.wts = s->wf;
  a.logtab = s->logtab;
  a.partials = s->partials;
  a.flag = s->ctx->d_flag;
  a.np = s->np;
  a.n_moves = p.moves.size();
  a.R = s->R;
  a.NP = s->NP;
  a.G = G;
  a.n_blocks = n_blocks;
  a.depth = std::max(p.max_depth, 1);
  a.max_moves = std::max(p.max_moves_per_prune, 1);
  a.Dfull = nullptr;
  a.xout = nullptr;
  a.xsc = nullptr;
  a.slot_base = 0;
  a.prune_base = 0;
  const size_t smem = scan_smem<Pol>(a.depth, a.max_moves);
  if (smem > s->ctx->smem_optin)
    return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "spr: scan needs %zu bytes of shared memory", smem);
  PGPU_CUDA(s->ctx, cudaFuncSetAttribute(spr_scan_kernel<Pol, RT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  spr_scan_kernel<Pol, RT><<<dim3((unsigned)p.prunes.size(), (unsigned)n_groups), SPR_NT, smem,
                             s->ctx->stream>>>(a);
  return pgpu_after_launch(s->ctx, "spr_scan_kernel");
}

template <typename Pol>
pgpu_status launch_scan(pgpu_spr *s, const SprPlan &p, const SprPlanDev &d, int G, int n_groups,
                        int n_blocks) {
  switch (s->RT) {
    case 1: return launch_scan_rt<Pol, 1>(s, p, d, G, n_groups, n_blocks);
    case 2: return launch_scan_rt<Pol, 2>(s, p, d, G, n_groups, n_blocks);
    case 4: return launch_scan_rt<Pol, 4>(s, p, d, G, n_groups, n_blocks);
    default: return launch_scan_rt<Pol, 8>(s, p, d, G, n_groups, n_blocks);
  }
}

// lazy log-likelihood of every move of plan p into lnl_dev
pgpu_status run_scan(pgpu_spr *s, const SprPlan &p, const SprPlanDev &d, double *lnl_dev) {
  const size_t nm = p.moves.size();
  if (nm == 0) return PGPU_OK;
  const int n_blocks = (int)(s->np / s->NP);
  // CTA groups of G pattern blocks; partial sums at most 256 MB
  const size_t budget = size_t(256) << 20;
  int G = (int)std::max<size_t>(1, ((size_t)n_blocks * nm * 8 + budget - 1) / budget);
  G = std::min(G, n_blocks);
  const int n_groups = (n_blocks + G - 1) / G;
  if (n_groups > 65535) return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "spr: too many pattern blocks");
  PGPU_TRY(grow(s, &s->partials, &s->part_cap, (size_t)n_groups * nm));
  if (s->precision == 32) PGPU_TRY(launch_scan<Fp32>(s, p, d, G, n_groups, n_blocks));
  else if (s->precision == 48) PGPU_TRY(launch_scan<Ff32>(s, p, d, G, n_groups, n_blocks));
  else PGPU_TRY(launch_scan<Fp64>(s, p, d, G, n_groups, n_blocks));
  spr_reduce_kernel<<<(unsigned)((nm + 255) / 256), 256, 0, s->ctx->stream>>>(s->partials, n_groups, nm,
                                                                              lnl_dev);
  return pgpu_after_launch(s->ctx, "spr_reduce_kernel");
}

// ---------------------------------------------------------------------------
// TBR: per batch of cuts, the emit walks store every attach vector, then the
// pair kernel scores every (j, k) of each cut
// ---------------------------------------------------------------------------
pgpu_status ensure_tbr(pgpu_spr *s) {
  if (s->tbr_valid) return PGPU_OK;
  PGPU_TRY(ensure_pool(s));
  tbr_plan(s->T, s->pp, s->tbr_join, s->tbr_reroot, &s->tbr);
  PGPU_TRY(upload_plan(s, s->tbr.emit, &s->tbr_d));
  if (!s->tbr.keep.empty()) {
    PGPU_TRY(grow(s, &s->tbr_keep, &s->tbr_keep_cap, s->tbr.keep.size()));
    PGPU_TRY(upload(s, s->tbr_keep, s->tbr.keep.data(), s->tbr.keep.size()));
  }
  s->tbr_valid = true;
  return PGPU_OK;
}

template <typename Pol, int RT>
pgpu_status launch_emit_rt(pgpu_spr *s, int prune_base, int n_prunes, long long slot_base) {
  const SprPlan &p = s->tbr.emit;
  ScanArgs a;
  a.L = s->L;
  a.M = s->M;
  a.H = s->H;
  a.sc = s->sc;
  a.Dhalf = static_cast<char *>(s->Dfull) + (size_t)s->T.n_edges() * s->cbytes;
  a.Dmer = s->tbr_d.Dmer;
  a.steps = s->tbr_d.steps;
  a.prunes = s->tbr_d.prunes;
  a.pi = s->pi;
  a.probs = s->probs;
  a.wts = s->wf;
  a.logtab = s->logtab;
  a.partials = nullptr;
  a.flag = s->ctx->d_flag;
  a.np = s->np;
  a.n_moves = p.moves.size();
  a.R = s->R;
  a.NP = s->NP;
  a.G = 1;
  a.n_blocks = (int)(s->np / s->NP);
  a.depth = std::max(p.max_depth, 1);
  a.max_moves = std::max(p.max_moves_per_prune, 1);
  a.Dfull = s->Dfull;
  a.xout = s->tbr_x;
  a.xsc = s->tbr_xsc;
  a.slot_base = slot_base;
  a.prune_base = prune_base;
  if (a.n_blocks > 65535) return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "tbr: too many pattern blocks");
  const size_t smem = scan_smem<Pol>(a.depth, a.max_moves);
  if (smem > s->ctx->smem_optin)
    return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "tbr: walk needs %zu bytes of shared memory", smem);
  PGPU_CUDA(s->ctx, cudaFuncSetAttribute(spr_scan_kernel<Pol, RT, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  spr_scan_kernel<Pol, RT, true><<<dim3((unsigned)n_prunes, (unsigned)a.n_blocks), SPR_NT, smem,
                                   s->ctx->stream>>>(a);
  return pgpu_after_launch(s->ctx, "spr_scan_kernel (emit)");
}

template <typename Pol>
pgpu_status launch_tbr_batch(pgpu_spr *s, size_t c0, size_t c1, double *lnl_dev) {
  const TbrPlan &tp = s->tbr;
  const SprPlan &P = tp.emit;
  const int pb0 = tp.cuts[c0].pa, n_prunes = tp.cuts[c1 - 1].pb + 1 - pb0;
  const long long slot_base = P.prunes[pb0].move_off;
  switch (s->RT) {
    case 1: PGPU_TRY((launch_emit_rt<Pol, 1>(s, pb0, n_prunes, slot_base))); break;
    case 2: PGPU_TRY((launch_emit_rt<Pol, 2>(s, pb0, n_prunes, slot_base))); break;
    case 4: PGPU_TRY((launch_emit_rt<Pol, 4>(s, pb0, n_prunes, slot_base))); break;
    default: PGPU_TRY((launch_emit_rt<Pol, 8>(s, pb0, n_prunes, slot_base))); break;
  }
  // the batch's cuts and tiles, numbered by their pairs in the grid
  const long long move0 = tp.cuts[c0].grid_off;
  const long long nm = tp.cuts[c1 - 1].grid_off + (long long)tp.cuts[c1 - 1].nA * tp.cuts[c1 - 1].nB - move0;
  // the lists live in the engine; a copy from pageable memory returns once
  // its source has been staged, so the next batch may rewrite them
  std::vector<TbrCutDev> &cuts = s->h_tbr_cuts;
  std::vector<int4> &tiles = s->h_tbr_tiles;
  cuts.clear();
  tiles.clear();
  for (size_t c = c0; c < c1; ++c) {
    const TbrCut &x = tp.cuts[c];
    TbrCutDev d{};
    d.edge = x.edge;
    d.nA = x.nA;
    d.nB = x.nB;
    d.slotA = P.prunes[x.pa].move_off - slot_base;
    d.slotB = P.prunes[x.pb].move_off - slot_base;
    d.move_off = x.grid_off - move0;
    cuts.push_back(d);
    for (int j0 = 0; j0 < x.nA; j0 += TB_T)
      for (int k0 = 0; k0 < x.nB; k0 += TB_T) tiles.push_back(make_int4((int)(c - c0), j0, k0, 0));
  }
  if (tiles.size() > 0x7fffffffu) return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "tbr: too many tiles");
  PGPU_TRY(grow(s, &s->tbr_cuts, &s->tbr_cuts_cap, cuts.size()));
  PGPU_TRY(grow(s, &s->tbr_tiles, &s->tbr_tiles_cap, tiles.size()));
  PGPU_CUDA(s->ctx, cudaMemcpyAsync(s->tbr_cuts, cuts.data(), cuts.size() * sizeof(TbrCutDev),
                                    cudaMemcpyHostToDevice, s->ctx->stream));
  PGPU_CUDA(s->ctx, cudaMemcpyAsync(s->tbr_tiles, tiles.data(), tiles.size() * sizeof(int4),
                                    cudaMemcpyHostToDevice, s->ctx->stream));
  // pattern groups: partial sums at most 256 MB
  const int n_pblocks = (int)(s->np / TB_PB);
  const size_t budget = size_t(256) << 20;
  int G = (int)std::max<size_t>(1, ((size_t)n_pblocks * (size_t)nm * 8 + budget - 1) / budget);
  G = std::min(G, n_pblocks);
  const int n_groups = (n_pblocks + G - 1) / G;
  if (n_groups > 65535) return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "tbr: too many pattern groups");
  PGPU_TRY(grow(s, &s->partials, &s->part_cap, (size_t)n_groups * nm));
  PairArgs a;
  a.X = s->tbr_x;
  a.xsc = s->tbr_xsc;
  a.tiles = s->tbr_tiles;
  a.cuts = s->tbr_cuts;
  a.wts = s->wf;
  a.logtab = s->logtab;
  a.partials = s->partials;
  a.flag = s->ctx->d_flag;
  a.np = s->np;
  a.n_moves = nm;
  a.R = s->R;
  a.G = G;
  a.n_pblocks = n_pblocks;
  const size_t smem = pair_smem<Pol>(s->R);
  if (smem > s->ctx->smem_optin)
    return pgpu_set_err(s->ctx, PGPU_ERR_LIMIT, "tbr: pairs need %zu bytes of shared memory", smem);
  PGPU_CUDA(s->ctx, cudaFuncSetAttribute(tbr_pair_kernel<Pol>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max<size_t>(smem, 48 * 1024)));
  tbr_pair_kernel<Pol><<<dim3((unsigned)tiles.size(), (unsigned)n_groups), 256, smem, s->ctx->stream>>>(a);
  PGPU_TRY(pgpu_after_launch(s->ctx, "tbr_pair_kernel"));
  spr_reduce_kernel<<<(unsigned)((nm + 255) / 256), 256, 0, s->ctx->stream>>>(s->partials, n_groups,
                                                                              (size_t)nm, lnl_dev + move0);
  return pgpu_after_launch(s->ctx, "spr_reduce_kernel");
}

// out[m] = grid[keep[m]]: the listed moves' lnL out of every pair's
__global__ void __launch_bounds__(256) tbr_gather_kernel(const double *grid, const int64_t *keep,
                                                        size_t n, double *out) {
  for (size_t m = blockIdx.x * (size_t)blockDim.x + threadIdx.x; m < n;
       m += (size_t)gridDim.x * blockDim.x)
    out[m] = grid[keep[m]];
}

// lnL of every TBR move into lnl_dev, in batches of cuts whose attach
// vectors fit in the budget (at least one cut per batch); with two
// different limits every pair goes into the grid buffer first and the
// listed moves are gathered from it
pgpu_status run_tbr_scan(pgpu_spr *s, double *lnl_dev) {
  PGPU_TRY(ensure_tbr(s));
  const TbrPlan &tp = s->tbr;
  if (tp.n_moves == 0) return PGPU_OK;
  const bool filter = !tp.keep.empty();
  if (filter) PGPU_TRY(grow(s, &s->tbr_grid, &s->tbr_grid_cap, (size_t)tp.n_grid));
  double *out = filter ? s->tbr_grid : lnl_dev;
  const size_t slot_bytes = s->np * s->R * 4 * s->vbytes;
  const size_t max_slots = std::max<size_t>(1, s->tbr_budget / slot_bytes);
  for (size_t c0 = 0; c0 < tp.cuts.size();) {
    size_t c1 = c0, slots = 0;
    while (c1 < tp.cuts.size()) {
      const size_t add = (size_t)tp.cuts[c1].nA + tp.cuts[c1].nB;
      if (c1 > c0 && slots + add > max_slots) break;
      slots += add;
      ++c1;
    }
    PGPU_TRY(grow(s, &s->tbr_x, &s->tbr_x_cap, slots * slot_bytes));
    PGPU_TRY(grow(s, &s->tbr_xsc, &s->tbr_xsc_cap, slots * s->np));
    if (s->precision == 32) PGPU_TRY(launch_tbr_batch<Fp32>(s, c0, c1, out));
    else if (s->precision == 48) PGPU_TRY(launch_tbr_batch<Ff32>(s, c0, c1, out));
    else PGPU_TRY(launch_tbr_batch<Fp64>(s, c0, c1, out));
    c0 = c1;
  }
  if (filter) {
    const size_t n = (size_t)tp.n_moves;
    tbr_gather_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 65535), 256, 0, s->ctx->stream>>>(
        s->tbr_grid, s->tbr_keep, n, lnl_dev);
    PGPU_TRY(pgpu_after_launch(s->ctx, "tbr_gather_kernel"));
  }
  return PGPU_OK;
}

pgpu_status ensure_fitch(pgpu_spr *s) {
  if (s->fitch_valid) return PGPU_OK;
  PGPU_TRY(ensure_pool(s));   // pool plan (ops, tips) must match the topology
  FitchTipArgs t;
  t.F = s->F;
  t.codes = s->codes;
  t.code_mask = s->cmask;
  t.tips = s->tips;
  t.W4 = s->W4;
  t.n_pat = s->n_pat;
  t.ld = s->ld;
  t.n_codes = s->n_codes;
  const unsigned gx = (unsigned)((s->W4 + 255) / 256);
  spr_fitch_tip_kernel<<<dim3(gx, (unsigned)s->n), 256, 0, s->ctx->stream>>>(t);
  PGPU_TRY(pgpu_after_launch(s->ctx, "spr_fitch_tip_kernel"));
  const int n_ops = (int)s->pp.ops.size();
  PGPU_CUDA(s->ctx, cudaMemsetAsync(s->cntF, 0, sizeof(unsigned long long) * (n_ops + 1), s->ctx->stream));
  FitchPoolArgs a;
  a.F = s->F;
  a.ops = s->ops;
  a.planes = s->planes;
  a.cnt = s->cntF;
  a.W4 = s->W4;
  a.n_ops = n_ops;
  a.n_planes = s->n_planes;
  spr_fitch_pool_kernel<<<gx, 256, 0, s->ctx->stream>>>(a);
  PGPU_TRY(pgpu_after_launch(s->ctx, "spr_fitch_pool_kernel"));
  spr_fitch_len_kernel<<<1, 32, 0, s->ctx->stream>>>(s->ops, n_ops, s->cntF, s->lenF, s->T.n_dedges());
  PGPU_TRY(pgpu_after_launch(s->ctx, "spr_fitch_len_kernel"));
  s->fitch_valid = true;
  return PGPU_OK;
}

pgpu_status run_fitch_scan(pgpu_spr *s) {
  PGPU_TRY(ensure_fitch(s));
  PGPU_TRY(ensure_plan(s));
  const SprPlan &p = s->all;
  const size_t nm = p.moves.size();
  PGPU_CUDA(s->ctx, cudaMemsetAsync(s->ins, 0, sizeof(unsigned long long) * std::max<size_t>(nm, 1),
                                    s->ctx->stream));
  PGPU_CUDA(s->ctx, cudaMemsetAsync(s->join, 0,
                                    sizeof(unsigned long long) * std::max<size_t>(p.prunes.size(), 1),
                                    s->ctx->stream));
  if (nm == 0) return PGPU_OK;
  FitchScanArgs a;
  a.F = s->F;
  a.planes = s->planes;
  a.steps = s->all_d.steps;
  a.prunes = s->all_d.prunes;
  a.ins = s->ins;
  a.join = s->join;
  a.W4 = s->W4;
  a.n_planes = s->n_planes;
  a.depth = std::max(p.max_depth, 1);
  a.max_moves = std::max(p.max_moves_per_prune, 1);
  a.flag = s->ctx->d_flag;
  const size_t smem = a16((size_t)a.max_moves * 4) + (size_t)a.depth * 256 * sizeof(uint4);
  PGPU_CUDA(s->ctx, cudaFuncSetAttribute(spr_fitch_scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max<size_t>(smem, 48 * 1024)));
  spr_fitch_scan_kernel<<<dim3((unsigned)p.prunes.size(), (unsigned)((s->W4 + 255) / 256)), 256, smem,
                          s->ctx->stream>>>(a);
  return pgpu_after_launch(s->ctx, "spr_fitch_scan_kernel");
}

pgpu_status sync_check(pgpu_spr *s, const char *what) {
  PGPU_CUDA(s->ctx, cudaStreamSynchronize(s->ctx->stream));
  return pgpu_check_flag(s->ctx, what);
}

void invalidate(pgpu_spr *s) {
  s->pool_valid = s->plan_valid = s->fitch_valid = s->summ_valid = s->tbr_valid = false;
}

}  // namespace

extern "C" {

pgpu_status pgpu_spr_create(pgpu_ctx *ctx, const pgpu_model *m, const pgpu_tip_codes *codes,
                            int32_t n_tips, const uint8_t *tip_codes_dev, size_t ld_pat,
                            const double *weights_dev, size_t n_pat, int precision, pgpu_spr **out) {
  if (!ctx || !out) return PGPU_ERR_ARG;
  *out = nullptr;
  if (!m || !m->Q || !m->pi || !m->rates || !m->probs || !codes || !codes->table || !tip_codes_dev)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: null model, code table or tip codes");
  if (m->n_states != 4)
    return pgpu_set_err(ctx, PGPU_ERR_UNSUPPORTED, "spr: the SPR engine is built for 4 states (DNA)");
  if (m->n_rates < 1 || m->n_rates > 8)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "spr: 1..8 rate classes are supported");
  if (codes->n_codes < 1 || codes->n_codes > 256)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: the code table needs 1..256 rows");
  if (precision != 32 && precision != 48 && precision != 64)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: precision must be 32, 48 or 64");
  if (n_tips < 4) return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: need at least 4 tips");
  if (n_pat < 1 || ld_pat < n_pat) return pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: need n_pat >= 1 and ld_pat >= n_pat");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  pgpu_spr *s = new pgpu_spr();
  s->ctx = ctx;
  s->precision = precision;
  s->R = m->n_rates;
  s->RT = s->R <= 1 ? 1 : s->R <= 2 ? 2 : s->R <= 4 ? 4 : 8;
  s->NP = SPR_NT / s->RT;
  s->n = n_tips;
  s->n_codes = codes->n_codes;
  s->n_pat = n_pat;
  s->np = (n_pat + s->NP - 1) / s->NP * s->NP;
  s->ld = ld_pat;
  s->W4 = (n_pat + 31) / 32;
  s->codes = tip_codes_dev;
  s->vbytes = precision == 32 ? 4 : 8;
  s->cbytes = (size_t)s->R * 16 * (precision == 32 ? 4 : 8);
  auto fail = [&](pgpu_status st) {
    pgpu_spr_destroy(s);
    return st;
  };
#define SPR_TRY(x)                  \
  do {                              \
    pgpu_status st_ = (x);          \
    if (st_ != PGPU_OK) return fail(st_); \
  } while (0)
  const int R = s->R, nc = s->n_codes;
  const int ne = 2 * n_tips - 3, nd = 2 * ne;
  // model block
  double *blk;
  SPR_TRY(dalloc_t(s, 16 + 4 + 2 * 8 + (size_t)nc * 4 + 16 + 16 + 4 + 2, &blk));
  s->Q = blk;
  s->pi = s->Q + 16;
  s->rates = s->pi + 4;
  s->probs = s->rates + 8;
  s->ctab = s->probs + 8;
  s->U = s->ctab + (size_t)nc * 4;
  s->Ui = s->U + 16;
  s->lam = s->Ui + 16;
  s->status = reinterpret_cast<int *>(s->lam + 4);
  std::vector<double> hb(16 + 4 + 16 + (size_t)nc * 4, 0.0);
  std::copy(m->Q, m->Q + 16, hb.begin());
  std::copy(m->pi, m->pi + 4, hb.begin() + 16);
  std::copy(m->rates, m->rates + R, hb.begin() + 20);
  std::copy(m->probs, m->probs + R, hb.begin() + 28);
  std::copy(codes->table, codes->table + (size_t)nc * 4, hb.begin() + 36);
  SPR_TRY(upload(s, blk, hb.data(), hb.size()));
  SPR_TRY(pgpu_launch_eig(ctx, s->Q, s->pi, 4, 1, s->U, s->lam, s->Ui, s->status));
  // state-set masks of the codes
  std::vector<uint8_t> cm(nc);
  for (int c = 0; c < nc; ++c) {
    uint8_t b = 0;
    for (int i = 0; i < 4; ++i)
      if (codes->table[(size_t)c * 4 + i] > 0.0) b |= (uint8_t)(1u << i);
    cm[c] = b;
  }
  SPR_TRY(dalloc_t(s, (size_t)nc, &s->cmask));
  SPR_TRY(upload(s, s->cmask, cm.data(), cm.size()));
  // weights: FP64 and FP32 copies padded with zeros; integer bit planes for Fitch
  std::vector<double> wh(s->np, 0.0);
  if (weights_dev) {
    if (cudaMemcpy(wh.data(), weights_dev, n_pat * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(pgpu_set_err(ctx, PGPU_ERR_CUDA, "spr: weights_dev is not readable device memory"));
    }
  } else {
    std::fill(wh.begin(), wh.begin() + n_pat, 1.0);
  }
  uint64_t wmax = 0;
  for (size_t i = 0; i < n_pat; ++i) {
    if (!(wh[i] >= 0.0) || wh[i] > 1e9) return fail(pgpu_set_err(ctx, PGPU_ERR_ARG, "spr: weight %zu is negative or too large", i));
    s->wtot += wh[i];
    wmax = std::max<uint64_t>(wmax, (uint64_t)llround(wh[i]));
  }
  std::vector<float> wfh(wh.begin(), wh.end());
  SPR_TRY(dalloc_t(s, s->np, &s->w));
  SPR_TRY(dalloc_t(s, s->np, &s->wf));
  SPR_TRY(upload(s, s->w, wh.data(), wh.size()));
  SPR_TRY(upload(s, s->wf, wfh.data(), wfh.size()));
  s->n_planes = 1;
  while ((wmax >> s->n_planes) != 0) ++s->n_planes;
  std::vector<uint32_t> planes((size_t)s->n_planes * s->W4 * 4, 0u);
  for (size_t i = 0; i < n_pat; ++i) {
    const uint64_t wi = (uint64_t)llround(wh[i]);
    for (int b = 0; b < s->n_planes; ++b)
      if ((wi >> b) & 1u) planes[(size_t)b * s->W4 * 4 + i / 8] |= 0x8u << (4 * (i % 8));
  }
  SPR_TRY(dalloc_t(s, (size_t)s->n_planes * s->W4, &s->planes));
  SPR_TRY(upload(s, reinterpret_cast<uint32_t *>(s->planes), planes.data(), planes.size()));
  // logarithm table of the pair form
  std::vector<float4> lt(64);
  ff_log_table(lt.data(), [](double c) { return std::log(c); });
  SPR_TRY(dalloc_t(s, 64, &s->logtab));
  SPR_TRY(upload(s, s->logtab, lt.data(), lt.size()));
  // pool and tables
  const size_t vec = (size_t)nd * s->np * R * 4 * s->vbytes;
  SPR_TRY(dalloc(s, vec, &s->L));
  SPR_TRY(dalloc(s, vec, &s->M));
  SPR_TRY(dalloc(s, vec, &s->H));
  SPR_TRY(dalloc_t(s, (size_t)nd * s->np, &s->sc));
  SPR_TRY(dalloc(s, 2 * (size_t)ne * s->cbytes, &s->Dfull));
  const size_t tt = (size_t)n_tips * R * nc * 4 * s->vbytes;
  SPR_TRY(dalloc(s, tt, &s->tipfull));
  SPR_TRY(dalloc(s, tt, &s->tiphalf));
  SPR_TRY(dalloc_t(s, 2 * (size_t)ne + 2 * (size_t)n_tips, &s->elen));
  SPR_TRY(dalloc_t(s, (size_t)ne, &s->newlen));
  SPR_TRY(dalloc_t(s, (size_t)nd, &s->ops));
  SPR_TRY(dalloc_t(s, (size_t)n_tips, &s->tips));
  SPR_TRY(dalloc_t(s, s->np / s->NP, &s->pool_part));
  SPR_TRY(dalloc_t(s, 1, &s->tree_lnl));
  SPR_TRY(dalloc_t(s, s->np, &s->site_lnl));
  SPR_TRY(dalloc_t(s, (size_t)nd * s->W4, &s->F));
  SPR_TRY(dalloc_t(s, (size_t)nd + 1, &s->cntF));
  SPR_TRY(dalloc_t(s, (size_t)nd + 1, &s->lenF));
  SPR_TRY(dalloc_t(s, (size_t)nd * 4, &s->summ));
  const size_t max_moves = (size_t)nd * 2 * n_tips, max_prunes = (size_t)nd;
  SPR_TRY(dalloc_t(s, max_moves, &s->ins));
  SPR_TRY(dalloc_t(s, max_prunes, &s->join));
  int st = 0;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
      cudaMemcpy(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(pgpu_set_err(ctx, PGPU_ERR_CUDA, "spr: set-up failed on the device"));
  }
  SPR_TRY(pgpu_check_flag(ctx, "spr_create"));
  if (st != 0) return fail(pgpu_set_err(ctx, (pgpu_status)st, "spr: the rate matrix could not be diagonalised"));
#undef SPR_TRY
  *out = s;
  return PGPU_OK;
}

void pgpu_spr_destroy(pgpu_spr *s) {
  if (!s) return;
  if (s->ctx) cudaSetDevice(s->ctx->device);
  for (void *p : s->owned) cudaFree(p);
  delete s;
}

pgpu_status pgpu_spr_set_tree(pgpu_spr *s, const pgpu_tree *tree) {
  if (!s) return PGPU_ERR_ARG;
  if (!tree || tree->n_tips != s->n)
    return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: tree must have %d tips", s->n);
  SprTopo T;
  PGPU_TRY(spr_from_rooted(s->ctx, tree, &T));
  s->T = std::move(T);
  invalidate(s);
  return PGPU_OK;
}

pgpu_status pgpu_spr_get_tree(pgpu_spr *s, int32_t *left, int32_t *right, double *brlen) {
  if (!s || !left || !right || !brlen) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  spr_to_rooted(s->T, left, right, brlen);
  return PGPU_OK;
}

pgpu_status pgpu_spr_lnl(pgpu_spr *s, double *lnl, double *site_lnl) {
  if (!s || !lnl) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(ensure_pool(s));
  double *h = reinterpret_cast<double *>(s->ctx->h_pinned);
  PGPU_CUDA(s->ctx, cudaMemcpyAsync(h, s->tree_lnl, 8, cudaMemcpyDeviceToHost, s->ctx->stream));
  if (site_lnl)
    PGPU_CUDA(s->ctx, cudaMemcpyAsync(site_lnl, s->site_lnl, s->n_pat * 8, cudaMemcpyDeviceToHost, s->ctx->stream));
  PGPU_TRY(sync_check(s, "spr_lnl"));
  *lnl = *h;
  return PGPU_OK;
}

pgpu_status pgpu_spr_n_moves(pgpu_spr *s, size_t *n_moves) {
  if (!s || !n_moves) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(ensure_plan(s));
  *n_moves = s->all.moves.size();
  return PGPU_OK;
}

pgpu_status pgpu_spr_moves(pgpu_spr *s, int32_t *p, int32_t *u, int32_t *c, int32_t *y, size_t cap) {
  if (!s || !p || !u || !c || !y) return PGPU_ERR_ARG;
  size_t nm = 0;
  PGPU_TRY(pgpu_spr_n_moves(s, &nm));
  if (cap < nm) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: %zu moves, room for %zu", nm, cap);
  const int n = s->n;
  std::vector<int32_t> l(n - 1), r(n - 1), ids(2 * n - 2);
  std::vector<double> b(2 * n - 2);
  spr_to_rooted(s->T, l.data(), r.data(), b.data(), ids.data());
  for (size_t i = 0; i < nm; ++i) {
    const SprMove &mv = s->all.moves[i];
    const int dp = s->all.prunes[mv.prune].dp;
    p[i] = ids[s->T.dsrc(dp)];
    u[i] = ids[s->T.ddst(dp)];
    c[i] = ids[s->T.dsrc(mv.dc)];
    y[i] = ids[s->T.ddst(mv.dc)];
  }
  return PGPU_OK;
}

pgpu_status pgpu_spr_scan(pgpu_spr *s, double *lnl_dev) {
  if (!s || !lnl_dev) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(ensure_plan(s));
  PGPU_TRY(run_scan(s, s->all, s->all_d, lnl_dev));
  return sync_check(s, "spr_scan");
}

pgpu_status pgpu_spr_score(pgpu_spr *s, const int64_t *move_idx, size_t k, double *lnl) {
  if (!s || (k && (!move_idx || !lnl))) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(ensure_plan(s));
  if (k == 0) return PGPU_OK;
  const size_t nm = s->all.moves.size();
  std::vector<int32_t> dp(k), dc(k);
  for (size_t i = 0; i < k; ++i) {
    if (move_idx[i] < 0 || (size_t)move_idx[i] >= nm)
      return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: move index %lld out of range", (long long)move_idx[i]);
    const SprMove &mv = s->all.moves[move_idx[i]];
    dp[i] = s->all.prunes[mv.prune].dp;
    dc[i] = mv.dc;
  }
  PGPU_TRY(spr_plan_selected(s->ctx, s->T, s->pp, dp.data(), dc.data(), (int)k, &s->sel));
  PGPU_TRY(upload_plan(s, s->sel, &s->sel_d));
  const size_t ns = s->sel.moves.size();
  double *out_dev;
  PGPU_TRY(pgpu_buf(s->ctx, BUF_OUT, std::max<size_t>(ns, 1) * 8, reinterpret_cast<void **>(&out_dev)));
  PGPU_TRY(run_scan(s, s->sel, s->sel_d, out_dev));
  std::vector<double> got(ns);
  PGPU_CUDA(s->ctx, cudaMemcpyAsync(got.data(), out_dev, ns * 8, cudaMemcpyDeviceToHost, s->ctx->stream));
  PGPU_TRY(sync_check(s, "spr_score"));
  // emitted order -> caller's order (the same move may be asked for twice)
  for (size_t i = 0; i < k; ++i) lnl[i] = NAN;
  for (size_t j = 0; j < ns; ++j) {
    const SprMove &mv = s->sel.moves[j];
    const int pdp = s->sel.prunes[mv.prune].dp;
    for (size_t i = 0; i < k; ++i)
      if (dp[i] == pdp && dc[i] == mv.dc) lnl[i] = got[j];
  }
  return PGPU_OK;
}

pgpu_status pgpu_spr_fitch(pgpu_spr *s, uint64_t *len_dev, uint64_t *tree_len) {
  if (!s || !len_dev) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(run_fitch_scan(s));
  const size_t nm = s->all.moves.size();
  if (nm) {
    spr_fitch_moves_kernel<<<(unsigned)((nm + 255) / 256), 256, 0, s->ctx->stream>>>(
        s->all_d.moves, s->all_d.prunes, nm, s->lenF, s->ins, s->join,
        reinterpret_cast<unsigned long long *>(len_dev));
    PGPU_TRY(pgpu_after_launch(s->ctx, "spr_fitch_moves_kernel"));
  }
  uint64_t *h = reinterpret_cast<uint64_t *>(s->ctx->h_pinned);
  PGPU_CUDA(s->ctx, cudaMemcpyAsync(h, s->lenF + s->T.n_dedges(), 8, cudaMemcpyDeviceToHost, s->ctx->stream));
  PGPU_TRY(sync_check(s, "spr_fitch"));
  if (tree_len) *tree_len = *h;
  return PGPU_OK;
}

pgpu_status pgpu_spr_features(pgpu_spr *s, float *X_dev) {
  if (!s || !X_dev) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(run_fitch_scan(s));
  if (!s->summ_valid) {
    SummaryArgs a;
    a.L = s->L;
    a.probs = s->probs;
    a.weights = s->w;
    a.out = s->summ;
    a.np = s->np;
    a.n_pat = s->n_pat;
    a.R = s->R;
    a.inv_w = s->wtot > 0 ? 1.0 / s->wtot : 0.0;
    const unsigned nd = (unsigned)s->T.n_dedges();
    if (s->precision == 32) spr_summary_kernel<Fp32><<<nd, 256, 0, s->ctx->stream>>>(a);
    else if (s->precision == 48) spr_summary_kernel<Ff32><<<nd, 256, 0, s->ctx->stream>>>(a);
    else spr_summary_kernel<Fp64><<<nd, 256, 0, s->ctx->stream>>>(a);
    PGPU_TRY(pgpu_after_launch(s->ctx, "spr_summary_kernel"));
    s->summ_valid = true;
  }
  const size_t nm = s->all.moves.size();
  if (nm == 0) return sync_check(s, "spr_features");
  // edge lengths as doubles on the device: the first n_edges entries of elen
  FeatArgs f;
  f.moves = s->all_d.moves;
  f.prunes = s->all_d.prunes;
  int32_t *tc;
  PGPU_TRY(pgpu_buf(s->ctx, BUF_A, s->pp.tipcnt.size() * 4, reinterpret_cast<void **>(&tc)));
  PGPU_TRY(upload(s, tc, s->pp.tipcnt.data(), s->pp.tipcnt.size()));
  f.tipcnt = tc;
  f.len = s->elen;
  f.summ = s->summ;
  f.lenF = s->lenF;
  f.ins = s->ins;
  f.join = s->join;
  f.X = X_dev;
  f.n_moves = nm;
  f.n_tips = s->n;
  f.nd = s->T.n_dedges();
  f.wtot = s->wtot > 0 ? s->wtot : 1.0;
  spr_feature_kernel<<<(unsigned)((nm + 255) / 256), 256, 0, s->ctx->stream>>>(f);
  PGPU_TRY(pgpu_after_launch(s->ctx, "spr_feature_kernel"));
  return sync_check(s, "spr_features");
}

pgpu_status pgpu_spr_set_join_distance(pgpu_spr *s, int join_distance) {
  if (!s) return PGPU_ERR_ARG;
  if (join_distance < 0)
    return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: join distance %d < 0", join_distance);
  if (join_distance != s->join_distance) {
    s->join_distance = join_distance;
    s->plan_valid = false;
  }
  return PGPU_OK;
}

pgpu_status pgpu_spr_set_tbr_limits(pgpu_spr *s, int join_distance, int reroot_distance) {
  if (!s) return PGPU_ERR_ARG;
  if (join_distance < 0 || reroot_distance < 0)
    return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "tbr: limits %d, %d must be >= 0", join_distance,
                        reroot_distance);
  if (join_distance != s->tbr_join || reroot_distance != s->tbr_reroot) {
    s->tbr_join = join_distance;
    s->tbr_reroot = reroot_distance;
    s->tbr_valid = false;
  }
  return PGPU_OK;
}

pgpu_status pgpu_spr_set_tbr_distance(pgpu_spr *s, int distance) {
  if (!s) return PGPU_ERR_ARG;
  if (distance < 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "tbr: distance %d < 0", distance);
  return pgpu_spr_set_tbr_limits(s, distance, distance);
}

pgpu_status pgpu_spr_set_tbr_budget(pgpu_spr *s, size_t bytes) {
  if (!s) return PGPU_ERR_ARG;
  s->tbr_budget = bytes ? bytes : size_t(2) << 30;
  return PGPU_OK;
}

pgpu_status pgpu_spr_tbr_n_moves(pgpu_spr *s, size_t *n_moves) {
  if (!s || !n_moves) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(ensure_tbr(s));
  *n_moves = (size_t)s->tbr.n_moves;
  return PGPU_OK;
}

pgpu_status pgpu_spr_tbr_moves(pgpu_spr *s, int32_t *a, int32_t *b, int32_t *jc, int32_t *jy, int32_t *kc,
                               int32_t *ky, size_t cap) {
  if (!s || !a || !b || !jc || !jy || !kc || !ky) return PGPU_ERR_ARG;
  size_t nm = 0;
  PGPU_TRY(pgpu_spr_tbr_n_moves(s, &nm));
  if (cap < nm) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "tbr: %zu moves, room for %zu", nm, cap);
  const int n = s->n;
  std::vector<int32_t> l(n - 1), r(n - 1), ids(2 * n - 2);
  std::vector<double> bl(2 * n - 2);
  spr_to_rooted(s->T, l.data(), r.data(), bl.data(), ids.data());
  const SprPlan &P = s->tbr.emit;
  const std::vector<int64_t> &keep = s->tbr.keep;
  size_t m = 0;   // listed moves, in grid order
  for (const TbrCut &c : s->tbr.cuts) {
    const int ia = ids[s->T.ea[c.edge]], ib = ids[s->T.eb[c.edge]];
    for (int j = 0; j < c.nA; ++j) {
      const int dj = P.moves[P.prunes[c.pa].move_off + j].dc;
      for (int k = 0; k < c.nB; ++k) {
        if (!keep.empty() && (m >= keep.size() || keep[m] != c.grid_off + (int64_t)j * c.nB + k))
          continue;
        const int dk = P.moves[P.prunes[c.pb].move_off + k].dc;
        a[m] = ia;
        b[m] = ib;
        jc[m] = ids[s->T.dsrc(dj)];
        jy[m] = ids[s->T.ddst(dj)];
        kc[m] = ids[s->T.dsrc(dk)];
        ky[m] = ids[s->T.ddst(dk)];
        ++m;
      }
    }
  }
  return PGPU_OK;
}

pgpu_status pgpu_spr_tbr_scan(pgpu_spr *s, double *lnl_dev) {
  if (!s || !lnl_dev) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  PGPU_TRY(run_tbr_scan(s, lnl_dev));
  return sync_check(s, "pgpu_spr_tbr_scan");
}

pgpu_status pgpu_spr_tbr_apply(pgpu_spr *s, int64_t move_idx) {
  if (!s) return PGPU_ERR_ARG;
  size_t nm = 0;
  PGPU_TRY(pgpu_spr_tbr_n_moves(s, &nm));
  if (move_idx < 0 || (size_t)move_idx >= nm)
    return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "tbr: move index %lld out of range", (long long)move_idx);
  const std::vector<TbrCut> &cuts = s->tbr.cuts;
  const int64_t g = s->tbr.keep.empty() ? move_idx : s->tbr.keep[(size_t)move_idx];
  size_t c = std::upper_bound(cuts.begin(), cuts.end(), g,
                              [](int64_t v, const TbrCut &x) { return v < x.grid_off; }) -
             cuts.begin() - 1;
  const TbrCut &x = cuts[c];
  const int64_t rel = g - x.grid_off;
  const SprPlan &P = s->tbr.emit;
  const int dj = P.moves[P.prunes[x.pa].move_off + (int)(rel / x.nB)].dc;
  const int dk = P.moves[P.prunes[x.pb].move_off + (int)(rel % x.nB)].dc;
  PGPU_TRY(tbr_apply(s->ctx, &s->T, x.edge, dj, dk));
  invalidate(s);
  return PGPU_OK;
}

pgpu_status pgpu_spr_apply(pgpu_spr *s, int64_t move_idx) {
  if (!s) return PGPU_ERR_ARG;
  size_t nm = 0;
  PGPU_TRY(pgpu_spr_n_moves(s, &nm));
  if (move_idx < 0 || (size_t)move_idx >= nm)
    return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: move index %lld out of range", (long long)move_idx);
  const SprMove mv = s->all.moves[move_idx];
  PGPU_TRY(spr_apply(s->ctx, &s->T, s->all.prunes[mv.prune].dp, mv.dc));
  invalidate(s);
  return PGPU_OK;
}

pgpu_status pgpu_spr_optimize(pgpu_spr *s, int passes, double tol, double *lnl_out) {
  if (!s) return PGPU_ERR_ARG;
  if (s->T.n == 0) return pgpu_set_err(s->ctx, PGPU_ERR_ARG, "spr: no tree set");
  PGPU_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
  const int ne = s->T.n_edges();
  if (!s->S) PGPU_TRY(dalloc_t(s, (size_t)ne * s->np * s->R * 4, &s->S));
  double cur = 0.0;
  PGPU_TRY(pgpu_spr_lnl(s, &cur, nullptr));
  std::vector<double> old(s->T.len), nl(ne);
  for (int pass = 0; pass < passes; ++pass) {
    BlArgs a;
    a.L = s->L;
    a.U = s->U;
    a.Ui = s->Ui;
    a.lam = s->lam;
    a.pi = s->pi;
    a.rates = s->rates;
    a.probs = s->probs;
    a.weights = s->w;
    a.S = s->S;
    a.len_in = s->elen;
    a.len_out = s->newlen;
    a.np = s->np;
    a.n_pat = s->n_pat;
    a.R = s->R;
    a.n_edges = ne;
    a.iters = 8;
    a.tol = 1e-6;
    a.tmin = 1e-8;
    a.tmax = 10.0;
    const dim3 g((unsigned)((s->np * s->R + 255) / 256), (unsigned)ne);
    if (s->precision == 32) bl_sumtab_kernel<Fp32><<<g, 256, 0, s->ctx->stream>>>(a);
    else if (s->precision == 48) bl_sumtab_kernel<Ff32><<<g, 256, 0, s->ctx->stream>>>(a);
    else bl_sumtab_kernel<Fp64><<<g, 256, 0, s->ctx->stream>>>(a);
    PGPU_TRY(pgpu_after_launch(s->ctx, "bl_sumtab_kernel"));
    bl_newton_kernel<<<(unsigned)ne, 256, 0, s->ctx->stream>>>(a);
    PGPU_TRY(pgpu_after_launch(s->ctx, "bl_newton_kernel"));
    PGPU_CUDA(s->ctx, cudaMemcpyAsync(nl.data(), s->newlen, ne * 8, cudaMemcpyDeviceToHost, s->ctx->stream));
    PGPU_TRY(sync_check(s, "spr_optimize"));
    old = s->T.len;
    // take the joint Newton step; halve it until the likelihood rises
    double alpha = 1.0, got = cur;
    bool accepted = false;
    for (int tries = 0; tries < 10 && !accepted; ++tries, alpha *= 0.5) {
      for (int e = 0; e < ne; ++e) s->T.len[e] = old[e] + alpha * (nl[e] - old[e]);
      invalidate(s);
      PGPU_TRY(pgpu_spr_lnl(s, &got, nullptr));
      accepted = got > cur;
    }
    // the edges' steps interfere: take them a quarter of the edges at a time
    for (int g = 0; g < 4 && !accepted; ++g) {
      s->T.len = old;
      for (int e = g; e < ne; e += 4) s->T.len[e] = nl[e];
      invalidate(s);
      PGPU_TRY(pgpu_spr_lnl(s, &got, nullptr));
      accepted = got > cur;
    }
    if (!accepted) {   // no step improves: converged as far as Newton can see
      s->T.len = old;
      invalidate(s);
      PGPU_TRY(pgpu_spr_lnl(s, &got, nullptr));
      break;
    }
    const double gain = got - cur;
    cur = got;
    if (gain < tol) break;
  }
  if (lnl_out) *lnl_out = cur;
  return PGPU_OK;
}

pgpu_status pgpu_spr_lengths(pgpu_spr *s, double *len, int32_t *ea, int32_t *eb) {
  if (!s || !len) return PGPU_ERR_ARG;
  const int ne = s->T.n_edges();
  std::copy(s->T.len.begin(), s->T.len.end(), len);
  if (ea) std::copy(s->T.ea.begin(), s->T.ea.end(), ea);
  if (eb) std::copy(s->T.eb.begin(), s->T.eb.end(), eb);
  (void)ne;
  return PGPU_OK;
}

}  // extern "C"
