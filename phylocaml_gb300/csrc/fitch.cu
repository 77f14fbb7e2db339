// Fitch parsimony on packed state-set lanes.
//
// Reference semantics: bv_fitch (lib/bitvector/bv.c:148-160) and
// NonAdditive_c.median_2 (lib/nonAdditive_c.ml:19-35): per site
//   m = a & b;  if m == 0 { m = a | b; cost += w }.
//
// Lanes of LB bits (4, 8, 16, 32) are processed a whole 32-bit word at a
// time with no per-site branch.  With H the lane-MSB mask,
//   nz = (((m & ~H) + ~H) | m) & H      MSB set in every non-empty lane
//   e  = nz ^ H                          MSB set in every empty lane
//   fill = e | (e - (e >> (LB-1)))       all bits of every empty lane
//   med  = m | ((a | b) & fill)
// and e >> (LB-1) holds a 1 in the lowest bit of each empty lane, which is
// added to LB-bit lane counters in one integer add (flushed to 32-bit
// per-site counters before a lane counter can wrap).
//
// The tree kernel (fitch_tree_kernel) gives each CTA a tile of W words
// (W*32/LB sites) and walks the whole postorder for it:
//   warp 0, lane 0   producer: streams the tip rows of the tile, in the order
//                    the schedule reads them, into a STAGES-deep shared ring
//                    with 1-D bulk copies (cp.async.bulk) on mbarriers;
//   warps 1..W/32    consumers: one word per thread; children that are
//                    internal nodes come from a per-thread stack in shared
//                    memory, tips from the ring; every median is written
//                    once to its output row with a streaming store.
// HBM traffic is therefore the compulsory minimum: each tip row read once,
// each internal row written once, plus weights and per-site counts.
#include <algorithm>
#include <cstring>

#include "pgpu_internal.cuh"
#include "forms.cuh"

namespace {

template <int LB>
struct Lanes {
  static constexpr uint32_t H =
      LB == 4 ? 0x88888888u : LB == 8 ? 0x80808080u : LB == 16 ? 0x80008000u : 0x80000000u;
  static constexpr int PER = 32 / LB;
  // increments a LB-bit counter can take before it may wrap
  static constexpr uint32_t FLUSH = LB >= 32 ? 0xffffffffu : ((1u << (LB >= 32 ? 0 : LB)) - 1u);
};

// Per LB-bit lane: the intersection, or the union where the intersection is
// empty; e_lsb gets a 1 in the lowest bit of every empty lane.  x has a
// lane's top bit set when the lane's other bits of a & b are not all zero,
// so ~(x | m) & H marks the empty lanes; spreading that mark over the lane
// is a multiply by the lane mask (no carries cross lanes), and
// (a & b) | ((a | b) & fill) is one three-input logic operation.
template <int LB>
__device__ __forceinline__ uint32_t fitch_word(uint32_t a, uint32_t b, uint32_t &e_lsb) {
  constexpr uint32_t H = Lanes<LB>::H;
  constexpr uint32_t LMASK = LB >= 32 ? 0xffffffffu : ((1u << (LB >= 32 ? 0 : LB)) - 1u);
  const uint32_t m = a & b;
  const uint32_t x = (m & ~H) + ~H;
  const uint32_t e = ~(x | m) & H;
  e_lsb = e >> (LB - 1);
  const uint32_t fill = e_lsb * LMASK;
  return (a & b) | ((a | b) & fill);
}

// mask of the valid lanes of word w (all lanes except in the last word)
template <int LB>
__host__ __device__ __forceinline__ uint32_t valid_lanes(size_t w, size_t n_sites) {
  constexpr int PER = Lanes<LB>::PER;
  const size_t first = w * PER;
  if (first + PER <= n_sites) return 0xffffffffu;
  if (first >= n_sites) return 0u;
  const int rem = int(n_sites - first);
  return (1u << (rem * LB)) - 1u;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums v over the block and adds it to *dst (one atomic per block).
__device__ __forceinline__ void block_add_u64(unsigned long long v, unsigned long long *dst,
                                              unsigned long long *red) {
  v = warp_sum_u64(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    unsigned long long s = lane < nw ? red[lane] : 0ull;
    s = warp_sum_u64(s);
    if (lane == 0 && s) atomicAdd(dst, s);
  }
}

// ---------------------------------------------------------------------------
// per-node kernels (fitch_median_2 / distance)
// ---------------------------------------------------------------------------

template <int LB, bool WEIGHTED, bool WRITE>
__global__ void __launch_bounds__(256) fitch_pair_kernel(const uint32_t *__restrict__ a,
                                                         const uint32_t *__restrict__ b,
                                                         const uint32_t *__restrict__ weights,
                                                         uint32_t *__restrict__ out,
                                                         size_t n_words, size_t n_sites,
                                                         unsigned long long *count) {
  __shared__ unsigned long long red[8];
  constexpr int PER = Lanes<LB>::PER;
  unsigned long long acc = 0;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n_words;
       w += (size_t)gridDim.x * blockDim.x) {
    uint32_t e;
    const uint32_t valid = valid_lanes<LB>(w, n_sites);
    const uint32_t med = fitch_word<LB>(__ldg(a + w), __ldg(b + w), e) & valid;
    e &= valid;
    if (WRITE) out[w] = med;
    if (WEIGHTED) {
#pragma unroll
      for (int l = 0; l < PER; ++l)
        if ((e >> (l * LB)) & 1u) acc += __ldg(weights + w * PER + l);
    } else {
      acc += __popc(e);
    }
  }
  block_add_u64(acc, count, red);
}

// 64-bit elements (Bitvector.BV64, lib/bitvector.ml): one character per
// element, two 32-bit words (low word first); the median takes the union
// when the whole element's intersection is empty.
template <bool WEIGHTED, bool WRITE>
__global__ void __launch_bounds__(256) fitch_pair64_kernel(const uint2 *__restrict__ a,
                                                           const uint2 *__restrict__ b,
                                                           const uint32_t *__restrict__ weights,
                                                           uint2 *__restrict__ out, size_t n,
                                                           unsigned long long *count) {
  __shared__ unsigned long long red[8];
  unsigned long long acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint2 x = __ldg(a + i), y = __ldg(b + i);
    uint2 m = make_uint2(x.x & y.x, x.y & y.y);
    const bool empty = (m.x | m.y) == 0u;
    if (empty) m = make_uint2(x.x | y.x, x.y | y.y);
    if (WRITE) out[i] = m;
    if (empty) acc += WEIGHTED ? __ldg(weights + i) : 1u;
  }
  block_add_u64(acc, count, red);
}

// NonAdditive_c.median_2 over the reference's own element types
// (lib/nonAdditive_c.ml:1-5, 19-35): one OCaml int per character -- a state
// set of up to 63 bits, passed sign-extended as int64, so 64-bit AND/OR give
// OCaml's land/lor -- and a float weight per character.  Each term is
// w_i * float(c_i), c_i = 1 where the intersection is empty, as the
// reference forms it; the terms are summed with error-free transformations
// (TwoSum per thread, across the warp and the CTA) into one (sum,
// compensation) pair per CTA, which nonadd_finalize_kernel adds in CTA
// order: deterministic, and within rounding of the exact sum whatever the
// weights.
constexpr int NA_THREADS = 256;

__global__ void __launch_bounds__(NA_THREADS) nonadd_median_kernel(
    const unsigned long long *__restrict__ x, const unsigned long long *__restrict__ y,
    const double *__restrict__ w, unsigned long long *__restrict__ out, size_t n,
    double2 *partials) {
  __shared__ double2 red[NA_THREADS / 32];
  double s = 0.0, c = 0.0;
  for (size_t i = blockIdx.x * (size_t)NA_THREADS + threadIdx.x; i < n;
       i += (size_t)gridDim.x * NA_THREADS) {
    const unsigned long long a = __ldg(x + i), b = __ldg(y + i);
    const unsigned long long m = a & b;
    const bool uni = m == 0ull;
    out[i] = uni ? (a | b) : m;
    const double term = __ldg(w + i) * (uni ? 1.0 : 0.0);
    double t, e;
    pgpu_forms::two_sum(s, term, t, e);
    s = t;
    c += e;
  }
  pgpu_forms::warp_csum(s, c);
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  if (lane == 0) red[wp] = make_double2(s, c);
  __syncthreads();
  if (wp == 0) {
    double2 v = lane < NA_THREADS / 32 ? red[lane] : make_double2(0.0, 0.0);
    double ss = v.x, cc = v.y;
    pgpu_forms::warp_csum(ss, cc);
    if (lane == 0) partials[blockIdx.x] = make_double2(ss, cc);
  }
}

__global__ void __launch_bounds__(1024) nonadd_finalize_kernel(const double2 *partials, int n,
                                                               double *out) {
  const double v = pgpu_forms::csum_block<1024>(partials, n);
  if (threadIdx.x == 0) out[0] = v;
}

// The whole postorder over 64-bit elements: one thread per element walks
// the schedule; the last result stays in registers, a step with two tip
// children sets it aside on a shared-memory stack and a step with two
// internal children takes its first child back.
struct Fitch64Args {
  const uint2 *tips;          // [n_tips][ld / 2]
  const uint32_t *weights;    // [n] or null
  uint2 *node_sets;           // [n_int][ld / 2]
  uint32_t *site_cost;        // [n] or null
  unsigned long long *total;
  const int4 *ops;
  size_t ld2, n;              // row stride in elements, elements
  int32_t n_tips, n_ops, depth;
};

constexpr int F64_THREADS = 128;

__global__ void __launch_bounds__(F64_THREADS) fitch_tree64_kernel(const Fitch64Args p) {
  extern __shared__ uint2 stk64[];   // [depth][F64_THREADS]
  __shared__ unsigned long long red[F64_THREADS / 32];
  const int t = threadIdx.x;
  const size_t i = (size_t)blockIdx.x * F64_THREADS + t;
  const bool on = i < p.n;
  auto tip = [&](int ch) { return on ? __ldg(p.tips + (size_t)ch * p.ld2 + i) : make_uint2(0, 0); };
  uint2 top = make_uint2(0, 0);
  uint32_t cnt = 0;
  int sp = 0;
  bool ok = true;
  for (int k = 0; k < p.n_ops && ok; ++k) {
    const int4 op = __ldg(p.ops + k);
    const int kind = (op.y >= p.n_tips ? 1 : 0) | (op.z >= p.n_tips ? 2 : 0);
    uint2 x, y;
    if (kind == 0) {
      if (k > 0) {
        if (sp < p.depth) stk64[sp++ * F64_THREADS + t] = top;
        else ok = false;
      }
      x = tip(op.y);
      y = tip(op.z);
    } else if (kind == 1) {
      x = top;
      y = tip(op.z);
    } else if (kind == 2) {
      x = tip(op.y);
      y = top;
    } else {
      if (sp > 0) {
        x = stk64[--sp * F64_THREADS + t];
      } else {
        ok = false;
        x = make_uint2(0, 0);
      }
      y = top;
    }
    uint2 m = make_uint2(x.x & y.x, x.y & y.y);
    if ((m.x | m.y) == 0u) {
      m = make_uint2(x.x | y.x, x.y | y.y);
      ++cnt;
    }
    if (on) p.node_sets[(size_t)op.x * p.ld2 + i] = m;
    top = m;
  }
  unsigned long long acc = 0;
  if (on && ok) {
    if (p.site_cost) p.site_cost[i] = cnt;
    acc = (unsigned long long)(p.weights ? __ldg(p.weights + i) : 1u) * cnt;
  }
  block_add_u64(acc, p.total, red);
}

// ---------------------------------------------------------------------------
// tree kernel
// ---------------------------------------------------------------------------

struct FitchTreeArgs {
  const uint32_t *tips;       // [n_tips][ld]
  const uint32_t *weights;    // [n_sites] or null
  uint32_t *node_sets;        // [n_int][ld]
  uint32_t *site_cost;        // [n_sites] or null
  unsigned long long *total;  // accumulated
  const int4 *ops;            // [n_int] SchedOp
  const int32_t *tip_seq;     // [n_tips]
  int *flag;
  size_t ld, n_words, n_sites;
  int32_t n_tips, n_ops;
  int W, depth;               // W words per tile (4 per consumer thread)
};

// Ring depth and tile width of one launch.  Deeper rings keep more tip rows
// in flight per CTA; the depth is the largest of 64/32/16 whose shared
// memory still lets every CTA of the launch be resident at once.
struct FitchPlan {
  size_t W = 128;        // words per tile
  int stages = 16;       // ring depth
  size_t smem = 0;       // dynamic shared memory per CTA
  size_t tiles = 0;
};

inline size_t fitch_smem(int stages, int depth, size_t W) {
  return 16 * (size_t)stages + 4 * (size_t)(stages + depth) * W;
}

// W = 128 * cw words (cw consumer warps of 32 threads x 4 words): the one
// that minimises the words the busiest SM handles, given that every SM takes
// ceil(tiles / SMs) tiles; ties go to the wider tile.
inline FitchPlan fitch_plan(size_t n_words, int depth, int num_sms, size_t smem_optin) {
  FitchPlan pl;
  const size_t sms = (size_t)(num_sms > 0 ? num_sms : 1);
  size_t best = ~size_t(0);
  for (size_t cw = 1; cw <= 4; ++cw) {
    const size_t w = 128 * cw, tiles = (n_words + w - 1) / w;
    const size_t cost = (tiles + sms - 1) / sms * w;
    if (cost <= best) {
      best = cost;
      pl.W = w;
    }
  }
  pl.tiles = (n_words + pl.W - 1) / pl.W;
  const size_t per_sm = std::max<size_t>((pl.tiles + sms - 1) / sms, 1);
  const size_t budget = std::min<size_t>(200 * 1024 / per_sm, smem_optin);
  pl.stages = 16;
  for (int st : {64, 32}) {
    if (fitch_smem(st, depth, pl.W) <= budget) {
      pl.stages = st;
      break;
    }
  }
  pl.smem = fitch_smem(pl.stages, depth, pl.W);
  return pl;
}

template <int LB>
__device__ __forceinline__ uint4 fitch_quad(const uint4 a, const uint4 b, const uint4 valid,
                                            uint4 &e) {
  uint4 m;
  m.x = fitch_word<LB>(a.x, b.x, e.x) & valid.x;
  m.y = fitch_word<LB>(a.y, b.y, e.y) & valid.y;
  m.z = fitch_word<LB>(a.z, b.z, e.z) & valid.z;
  m.w = fitch_word<LB>(a.w, b.w, e.w) & valid.w;
  return m;
}

template <int LB, int ST>
__global__ void __launch_bounds__(160) fitch_tree_kernel(const FitchTreeArgs p) {
  constexpr int PER = Lanes<LB>::PER;
  constexpr uint32_t FLUSH = Lanes<LB>::FLUSH;
  constexpr uint32_t LSB = Lanes<LB>::H >> (LB - 1);
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ unsigned long long red[32];
  const int W = p.W, Q = W / 4;   // Q consumer threads, one uint4 each
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + ST;
  uint4 *ring = reinterpret_cast<uint4 *>(smem + 16 * ST);   // [ST][Q]
  uint4 *stk = ring + (size_t)ST * Q;                         // [depth][Q]
  const size_t tile0 = (size_t)blockIdx.x * W;
  const int tid = threadIdx.x;
  const int n_consumer_warps = Q / 32;

  if (tid == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], n_consumer_warps);
    }
    fence_mbarrier_init();
  }
  __syncthreads();

  if (tid < 32) {
    // ---------------- producer ----------------
    if (tid == 0) {
      const size_t span = min((size_t)W, p.ld - tile0);
      const uint32_t bytes = (uint32_t)(span * sizeof(uint32_t));
      int issued = 0;
      for (int j = 0; j < p.n_tips; ++j) {
        const int slot = j & (ST - 1), round = j / ST;
        if (round > 0 && !mbar_wait_bounded(&empty[slot], (round - 1) & 1, p.flag)) break;
        const int32_t tip = __ldg(p.tip_seq + j);
        mbar_arrive_expect_tx(&full[slot], bytes);
        bulk_g2s(ring + (size_t)slot * Q, p.tips + (size_t)tip * p.ld + tile0, bytes, &full[slot]);
        issued = j + 1;
      }
      // every issued copy must land before this CTA may exit
      for (int j = max(0, issued - ST); j < issued; ++j)
        (void)mbar_wait_bounded(&full[j & (ST - 1)], (j / ST) & 1, p.flag);
    }
    return;
  }

  // ---------------- consumers: words 4c .. 4c+3 of the tile ----------------
  const int c = tid - 32;
  const int lane = tid & 31;
  const size_t word0 = tile0 + 4 * (size_t)c;
  const bool active = word0 < p.ld;           // the quad lies inside the row
  uint4 valid;
  valid.x = valid_lanes<LB>(word0 + 0, p.n_sites);
  valid.y = valid_lanes<LB>(word0 + 1, p.n_sites);
  valid.z = valid_lanes<LB>(word0 + 2, p.n_sites);
  valid.w = valid_lanes<LB>(word0 + 3, p.n_sites);
  uint4 cnt = make_uint4(0, 0, 0, 0);   // LB-bit lane counters
  uint32_t acc[4][PER];                  // per-site counters
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int l = 0; l < PER; ++l) acc[q][l] = 0;
  uint32_t since = 0;
  int sp = 0, taken = 0;
  bool ok = true;

  auto flush = [&]() {
#pragma unroll
    for (int l = 0; l < PER; ++l) {
      acc[0][l] += (cnt.x >> (l * LB)) & FLUSH;
      acc[1][l] += (cnt.y >> (l * LB)) & FLUSH;
      acc[2][l] += (cnt.z >> (l * LB)) & FLUSH;
      acc[3][l] += (cnt.w >> (l * LB)) & FLUSH;
    }
    cnt = make_uint4(0, 0, 0, 0);
  };
  auto take = [&](uint4 &v) {
    const int slot = taken & (ST - 1);
    // every lane waits and the verdict is made warp-uniform before any
    // warp-synchronous step, so a timeout cannot split the warp
    const bool got =
        __all_sync(0xffffffffu, mbar_wait_bounded(&full[slot], (taken / ST) & 1, p.flag));
    if (!got) {
      ok = false;
      return;
    }
    v = ring[(size_t)slot * Q + c];
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[slot]);
    ++taken;
  };

  // the top of the stack stays in registers: most nodes are consumed by the
  // very next step
  uint4 top = make_uint4(0, 0, 0, 0);
  bool top_valid = false;
  auto pop = [&]() -> uint4 {
    if (top_valid) {
      top_valid = false;
      return top;
    }
    return stk[(size_t)(--sp) * Q + c];
  };
  int4 op = p.n_ops > 0 ? __ldg(p.ops) : make_int4(0, 0, 0, 0);
  for (int i = 0; i < p.n_ops && ok; ++i) {
    // the next step's schedule entry is fetched while this one runs
    const int4 next = i + 1 < p.n_ops ? __ldg(p.ops + i + 1) : op;
    uint4 x = make_uint4(0, 0, 0, 0), y = make_uint4(0, 0, 0, 0);
    if (op.z >= p.n_tips) y = pop();
    if (op.y >= p.n_tips) x = pop();
    if (op.y < p.n_tips) take(x);
    if (op.z < p.n_tips && ok) take(y);
    if (!ok) break;
    uint4 e;
    const uint4 med = fitch_quad<LB>(x, y, valid, e);
    if (top_valid) stk[(size_t)(sp++) * Q + c] = top;
    top = med;
    top_valid = true;
    if (active) __stcs(reinterpret_cast<uint4 *>(p.node_sets + (size_t)op.x * p.ld + word0), med);
    op = next;
    cnt.x += e.x & valid.x & LSB;
    cnt.y += e.y & valid.y & LSB;
    cnt.z += e.z & valid.z & LSB;
    cnt.w += e.w & valid.w & LSB;
    if (LB < 32 && ++since == FLUSH) {
      flush();
      since = 0;
    }
  }
  if (LB < 32) {
    flush();
  } else {
    acc[0][0] += cnt.x;
    acc[1][0] += cnt.y;
    acc[2][0] += cnt.z;
    acc[3][0] += cnt.w;
  }

  unsigned long long wsum = 0;
  if (ok) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const size_t s0 = (word0 + q) * PER;
#pragma unroll
      for (int l = 0; l < PER; ++l) {
        const size_t s = s0 + l;
        if (s < p.n_sites) {
          if (p.site_cost) p.site_cost[s] = acc[q][l];
          const uint32_t w = p.weights ? __ldg(p.weights + s) : 1u;
          wsum += (unsigned long long)w * acc[q][l];
        }
      }
    }
  }
  // block reduction over the consumer warps only
  wsum = warp_sum_u64(wsum);
  const int cw = c >> 5;
  if (lane == 0) red[cw] = wsum;
  asm volatile("bar.sync 1, %0;" ::"r"(Q) : "memory");
  if (cw == 0) {
    unsigned long long s = lane < n_consumer_warps ? red[lane] : 0ull;
    s = warp_sum_u64(s);
    if (lane == 0 && s) atomicAdd(p.total, s);
  }
}

// ---------------------------------------------------------------------------
// tree kernel, segmented form.  One CTA of FS_W warps per slice of up to
// 256 words (one or two groups of 4 words per thread, 128 words apart): the
// postorder is cut into up to FS_S disjoint
// subtrees (segments), dealt to the warps longest first; each warp walks its
// segments one after another with its own stack, and each thread keeps its
// next FS_P tip slices in flight with cp.async (LDGSTS) into a per-warp ring.
// A finished segment's result stays at the bottom of its warp's stack; warp
// 0 then finishes the few nodes above the segments.  Splitting the walk
// multiplies the warps per SM by FS_W, which a single postorder walk cannot,
// and dealing more segments than warps keeps the warps' loads even.
// ---------------------------------------------------------------------------
constexpr int FS_W = 4;   // warps per CTA
constexpr int FS_S = 8;   // segments at most
constexpr int FS_P = 4;   // tip slices in flight per thread (a power of two)
static_assert((FS_P & (FS_P - 1)) == 0, "the copy ring is indexed by a mask");

// Shared-memory accesses through 32-bit shared-window addresses.
__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}

__device__ __forceinline__ uint4 lds_v4(uint32_t a) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a)
               : "memory");
  return v;
}
__device__ __forceinline__ void sts_v4(uint32_t a, const uint4 &v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

struct FitchSplitArgs {
  const uint32_t *tips, *weights;
  uint32_t *node_sets, *site_cost;
  unsigned long long *total;
  const int4 *ops, *seg, *top, *wseg;   // wseg[w] = {first segment, count}
  const int32_t *tip_seq;
  size_t ld, n_words, n_sites;
  int32_t n_tips;
  int n_top, rows;                       // rows: ring + stack rows per warp
  int tile_words;                        // words per CTA: 4 per active lane and part
  size_t tile_base;                      // the launch's first tile (host-buffer calls launch by chunk)
  int count16;                           // per-site counts fit 16 bits (< 65,536 internal nodes)
  int tcm_period;                        // TcmOp<true>: steps between flushes of the packed sums
  const uint32_t *table;                 // cost-matrix pair table (TcmOp), else null
  int *flag;                             // error word (TcmOp: a pair without median)
};

// The per-word operation of the segmented tree kernel, with its per-site
// cost bookkeeping.  A lane covers NV parts of 4 words (part j of lane l
// holds words 128 j + 4 l .. + 3 of the CTA's tile, so every part's loads
// and stores are coalesced), PER sites per word; the CTA's per-site counts
// are NV * 4 * PER 32-bit words per lane, [entry][lane]: one per site, or,
// for FitchOp with two 16-bit counts to a word, the first half of them.
//   FitchOp<LB, NV>  the Fitch rule on LB-bit lanes; union events are
//                counted in LB-bit lane counters (one add per word) and
//                flushed into the per-site counts every 2^LB - 1 steps.
//                While a site's count fits 16 bits, one flush add carries
//                two sites' counts (sites 0/4, 2/6, 1/5, 3/7 of a 4-bit
//                word; 0/2, 1/3 of an 8-bit word; 0/1 of a 16-bit word).
//   TcmOp        a cost-matrix character on 4-bit codes (csrc/tcm.cu): one
//                lookup per site in a pair table replicated once per lane in
//                shared memory (entry e of lane l at [e][l], so a warp's
//                lookups never share a bank), the cost summed per site in
//                registers and added to the per-site counts at the end.
// combine<FULL>: FULL is set for CTAs whose words all lie inside the
// alignment, so no lane of theirs needs the valid-lane mask.
template <int LB, int NV_>
struct FitchOp {
  static constexpr int NV = NV_;
  static constexpr int PER = Lanes<LB>::PER;
  // per-site count words of a lane (the packed counts use half of them; a
  // layout that freed the other half let a fifth CTA onto each SM and made
  // the 208-word-tile launch slower, 0.224 against 0.201 ms)
  __host__ __device__ static constexpr int sites(bool) { return NV * 4 * PER; }
  static constexpr uint32_t FLUSH = Lanes<LB>::FLUSH;
  static constexpr int MIN_BLOCKS = NV == 1 ? 8 : 4;
  static constexpr size_t EXTRA_SMEM = 0;
  static constexpr bool FULL_ANY_WIDTH = true;   // idle lanes' counts are never read
  uint32_t cnt[NV][4];
  uint32_t since;
  __device__ __forceinline__ void init(const FitchSplitArgs &, uint32_t *, int) {
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) cnt[j][q] = 0;
    since = 0;
  }
  // the LB-bit lane counters into the shared per-site counts
  __device__ __forceinline__ void flush(const FitchSplitArgs &p, uint32_t *sitecnt, int lane) {
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t c = cnt[j][q];
        uint32_t *s = sitecnt + (size_t)((j * 4 + q) * PER) * 32 + lane;
        if (LB == 32) {
          atomicAdd(s, c);
        } else if (p.count16) {
          if (LB == 4) {
            const uint32_t t = c & 0x0F0F0F0Fu, u = (c >> 4) & 0x0F0F0F0Fu;
            atomicAdd(s, t & 0x00FF00FFu);
            atomicAdd(s + 32, (t >> 8) & 0x00FF00FFu);
            atomicAdd(s + 64, u & 0x00FF00FFu);
            atomicAdd(s + 96, (u >> 8) & 0x00FF00FFu);
          } else if (LB == 8) {
            atomicAdd(s, c & 0x00FF00FFu);
            atomicAdd(s + 32, (c >> 8) & 0x00FF00FFu);
          } else {
            atomicAdd(s, c);
          }
        } else {
#pragma unroll
          for (int l = 0; l < PER; ++l) atomicAdd(s + l * 32, (c >> (l * LB)) & FLUSH);
        }
        cnt[j][q] = 0;
      }
  }
  template <bool FULL>
  __device__ __forceinline__ uint4 combine(const uint4 &x, const uint4 &y, const uint4 &valid, int j) {
    uint32_t e0, e1, e2, e3;
    uint4 m;
    m.x = fitch_word<LB>(x.x, y.x, e0);
    m.y = fitch_word<LB>(x.y, y.y, e1);
    m.z = fitch_word<LB>(x.z, y.z, e2);
    m.w = fitch_word<LB>(x.w, y.w, e3);
    if (!FULL) {
      m.x &= valid.x, m.y &= valid.y, m.z &= valid.z, m.w &= valid.w;
      e0 &= valid.x, e1 &= valid.y, e2 &= valid.z, e3 &= valid.w;
    }
    cnt[j][0] += e0;
    cnt[j][1] += e1;
    cnt[j][2] += e2;
    cnt[j][3] += e3;
    return m;
  }
  // once per step, after its parts
  __device__ __forceinline__ void step(const FitchSplitArgs &p, uint32_t *sitecnt, int lane) {
    if (LB < 32 && ++since == FLUSH) {
      flush(p, sitecnt, lane);
      since = 0;
    }
  }
  __device__ __forceinline__ void finish(const FitchSplitArgs &p, uint32_t *sitecnt, int lane) {
    flush(p, sitecnt, lane);
  }
  __device__ __forceinline__ void check_root(const FitchSplitArgs &, const uint4 (&)[NV],
                                             const bool (&)[NV], const size_t (&)[NV]) const {}
  // the count of site l of word q of part j
  __device__ __forceinline__ uint32_t count(const FitchSplitArgs &p, const uint32_t *sitecnt, int j,
                                            int q, int l, int lane) const {
    const uint32_t *s = sitecnt + (size_t)((j * 4 + q) * PER) * 32 + lane;
    if (LB == 32 || !p.count16) return s[l * 32];
    int e, h;
    if (LB == 4) {
      const int b = l >> 1;
      e = 2 * (l & 1) + (b & 1);
      h = b >> 1;
    } else if (LB == 8) {
      e = l & 1;
      h = l >> 1;
    } else {
      e = 0;
      h = l;
    }
    return (s[e * 32] >> (16 * h)) & 0xFFFFu;
  }
};

// TcmOp<PACKED>: the pair table arrives as cost << 4 | code (bit 31: no
// median).  PACKED re-packs it in shared memory as code << 28 | cost, so one
// add per site sums the cost in the low 28 bits of a register while the
// codes pile up in the top 4 bits and wrap away; the sums go to the per-site
// counts every tcm_period steps, before the cost can reach bit 28.  A pair
// without a median yields code 0, and code 0 has no median with anything,
// so such a pair leaves code 0 at the root: the root's row is checked once
// instead of every entry.
template <bool PACKED>
struct TcmOp {
  static constexpr int NV = 1;
  static constexpr int PER = 8;
  __host__ __device__ static constexpr int sites(bool) { return 32; }
  static constexpr int MIN_BLOCKS = 4;
  static constexpr size_t EXTRA_SMEM = 256 * 32 * 4;
  static constexpr bool FULL_ANY_WIDTH = false;  // an idle lane's code 0 would raise the flag
  static constexpr uint32_t COST = 0x0FFFFFFFu;
  uint32_t tb;   // shared address of this lane's copy of entry 0
  uint32_t acc[32];
  int since;
  // every thread of the CTA takes part in filling the table; the kernel's
  // barrier after init() publishes it
  __device__ __forceinline__ void init(const FitchSplitArgs &p, uint32_t *extra, int tid) {
    for (int i = tid; i < 256 * 32; i += FS_W * 32) {
      uint32_t e = __ldg(p.table + (i >> 5));
      if (PACKED) e = (e >> 31) ? 0u : (e << 28) | ((e >> 4) & COST);
      extra[i] = e;
    }
    tb = static_cast<uint32_t>(__cvta_generic_to_shared(extra + (tid & 31)));
#pragma unroll
    for (int i = 0; i < 32; ++i) acc[i] = 0;
    since = 0;
  }
  template <bool FULL>
  __device__ __forceinline__ uint32_t word(uint32_t xa, uint32_t xb, uint32_t valid, int q) {
    if (!FULL) {
      // lanes past the last site read as code 1, which always has a median
      const uint32_t fill = 0x11111111u & ~valid;
      xa = (xa & valid) | fill;
      xb = (xb & valid) | fill;
    }
    // the table index (a_l << 4) | b_l of every site, as bytes: even sites
    // 2k in byte k of ev, odd sites 2k + 1 in byte k of od
    const uint32_t ev = ((xa << 4) & 0xF0F0F0F0u) | (xb & 0x0F0F0F0Fu);
    const uint32_t od = (xa & 0xF0F0F0F0u) | ((xb >> 4) & 0x0F0F0F0Fu);
    uint32_t e[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      // entry i of this lane's copy lies 128 i bytes after entry 0
      e[2 * k] = lds_u32(tb + (__byte_perm(ev, 0u, 0x4440u + k) << 7));
      e[2 * k + 1] = lds_u32(tb + (__byte_perm(od, 0u, 0x4440u + k) << 7));
    }
#pragma unroll
    for (int l = 0; l < 8; ++l) acc[q * 8 + l] += PACKED ? e[l] : e[l] >> 4;
    uint32_t out;
    if (PACKED) {
      // the median codes are the entries' top nibbles: gather the top bytes
      // of the even and the odd sites' entries, then interleave their nibbles
      const uint32_t ce = __byte_perm(__byte_perm(e[0], e[2], 0x0073u), __byte_perm(e[4], e[6], 0x0073u),
                                      0x5410u);
      const uint32_t co = __byte_perm(__byte_perm(e[1], e[3], 0x0073u), __byte_perm(e[5], e[7], 0x0073u),
                                      0x5410u);
      out = ((ce >> 4) & 0x0F0F0F0Fu) | (co & 0xF0F0F0F0u);
    } else {
      // the median codes are the entries' low nibbles
      const uint32_t ce = __byte_perm(__byte_perm(e[0], e[2], 0x0040u), __byte_perm(e[4], e[6], 0x0040u),
                                      0x5410u);
      const uint32_t co = __byte_perm(__byte_perm(e[1], e[3], 0x0040u), __byte_perm(e[5], e[7], 0x0040u),
                                      0x5410u);
      out = (ce & 0x0F0F0F0Fu) | ((co << 4) & 0xF0F0F0F0u);
    }
    return FULL ? out : out & valid;
  }
  template <bool FULL>
  __device__ __forceinline__ uint4 combine(const uint4 &x, const uint4 &y, const uint4 &valid, int) {
    uint4 m;
    m.x = word<FULL>(x.x, y.x, valid.x, 0);
    m.y = word<FULL>(x.y, y.y, valid.y, 1);
    m.z = word<FULL>(x.z, y.z, valid.z, 2);
    m.w = word<FULL>(x.w, y.w, valid.w, 3);
    return m;
  }
  __device__ __forceinline__ void flush(uint32_t *sitecnt, int lane) {
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const uint32_t v = PACKED ? acc[i] & COST : acc[i];
      if (v) atomicAdd(&sitecnt[i * 32 + lane], v);
      acc[i] = 0;
    }
  }
  __device__ __forceinline__ void step(const FitchSplitArgs &p, uint32_t *sitecnt, int lane) {
    if (PACKED && ++since == p.tcm_period) {
      flush(sitecnt, lane);
      since = 0;
    }
  }
  __device__ __forceinline__ void finish(const FitchSplitArgs &, uint32_t *sitecnt, int lane) {
    flush(sitecnt, lane);
  }
  // warp 0, after the CTA's last barrier: a valid site whose root code is 0
  // met a pair without a median
  __device__ __forceinline__ void check_root(const FitchSplitArgs &p, const uint4 (&valid)[1],
                                             const bool (&act)[1], const size_t (&word)[1]) const {
    if (!act[0]) return;
    const uint4 r = __ldcg(reinterpret_cast<const uint4 *>(p.node_sets + (size_t)(p.n_tips - 2) * p.ld +
                                                           word[0]));
    const uint32_t rw[4] = {r.x, r.y, r.z, r.w}, vw[4] = {valid[0].x, valid[0].y, valid[0].z, valid[0].w};
    uint32_t zero = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t y = rw[q] | ~vw[q];   // lanes past the sites read as 0xF
      zero |= (y - 0x11111111u) & ~y & 0x88888888u;
    }
    if (zero) atomicOr(p.flag, PGPU_FLAG_BADCODE);
  }
  __device__ __forceinline__ uint32_t count(const FitchSplitArgs &, const uint32_t *sitecnt, int,
                                            int q, int l, int lane) const {
    return sitecnt[(q * 8 + l) * 32 + lane];
  }
};

// one warp's region: ring [FS_P] rows then stack [rows - FS_P] rows, a row
// being NV parts x 32 lanes of uint4 (its finished segments' results at the
// bottom of the stack, the walk above them); after the walks the rings hold
// the joining nodes' results, FS_W * FS_P >= FS_S
static_assert(FS_W * FS_P >= FS_S, "joining results overlay the rings");
template <class Op>
__host__ __device__ inline size_t split_smem(int rows, bool count16) {
  return (size_t)FS_W * rows * Op::NV * 32 * 16 + (size_t)Op::sites(count16) * 32 * 4 + Op::EXTRA_SMEM;
}

// Phase 1 of tree_split_kernel: warp w walks its segments.  word[j] is the
// first of part j's 4 words, act[j] whether the lane has them.
template <class Op, bool FULL>
__device__ __forceinline__ void split_walk(const FitchSplitArgs &p, Op &rule, uint4 *ring, uint4 *stk0,
                                           const uint4 (&valid)[Op::NV], const bool (&act)[Op::NV],
                                           const size_t (&word)[Op::NV], uint32_t *sitecnt, int w,
                                           int lane) {
  constexpr int NV = Op::NV;
  // row r of part j: col[j] + r ld (tips) and ncol[j] + r ld (node sets),
  // a 32-bit row stride so that each is one wide multiply-add
  const uint32_t ld32 = (uint32_t)p.ld;
  const uint32_t *col[NV];
  uint32_t *ncol[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    col[j] = p.tips + (act[j] ? word[j] : 0);
    ncol[j] = p.node_sets + word[j];
  }
  // this lane's element of ring row r, part j: ring_s + (r NV + j) 512
  // bytes (and likewise for the stack), as 32-bit shared-window addresses
  const uint32_t ring_s = static_cast<uint32_t>(__cvta_generic_to_shared(ring)) + 16u * lane;
  const int4 ws = p.wseg[w];
  for (int q = 0; q < ws.y; ++q) {
    const int4 sg = p.seg[ws.x + q];   // {op_off, n_ops, tip_off, n_tips}
    uint4 *stk = stk0 + (q + 1) * NV * 32;   // rows below hold earlier results
    const uint32_t stk_s = static_cast<uint32_t>(__cvta_generic_to_shared(stk)) + 16u * lane;
    const int32_t *tseq = p.tip_seq + sg.z;
    // copy counts are unsigned so that the ring slot is a mask, not a
    // signed remainder
    const uint32_t n_seg_tips = (uint32_t)sg.w;
    uint32_t issued = 0, consumed = 0;
    int32_t next_tip = sg.w > 0 ? __ldg(tseq) : 0;
    auto issue = [&]() {
      if (issued < n_seg_tips) {
        const int32_t tip = next_tip;
        if (issued + 1 < n_seg_tips) next_tip = __ldg(tseq + issued + 1);
        const uint64_t roff = (uint64_t)(uint32_t)tip * ld32;
#pragma unroll
        for (int j = 0; j < NV; ++j)
          cp_async16(&ring[((issued & (FS_P - 1)) * NV + j) * 32 + lane], col[j] + roff, act[j]);
      }
      cp_async_commit();   // empty groups keep the count in step
      ++issued;
    };
#pragma unroll
    for (int j = 0; j < FS_P; ++j) issue();
    // The stack discipline is fixed by the postorder: the previous step's
    // result is this step's second child when that is internal, else its
    // first; a step with two tip children sets it aside (push), one with two
    // internal children takes its first child back (pop).  A segment's
    // first step has two tip children and nothing to set aside.
    int sp = 0;
    uint4 top[NV];
    auto from_ring = [&](uint4 (&dst)[NV]) {
#pragma unroll
      for (int j = 0; j < NV; ++j) dst[j] = lds_v4(ring_s + (((consumed & (FS_P - 1)) * NV + j) << 9));
      ++consumed;
    };
    const int4 *ops = p.ops + sg.x;
    int4 op = __ldg(ops);
    for (int i = 0; i < sg.y; ++i) {
      const int4 next = i + 1 < sg.y ? __ldg(ops + i + 1) : op;
      const bool ta = op.y < p.n_tips, tb = op.z < p.n_tips;
      uint4 x[NV], y[NV];
      // a step's tips are the next ones of the sequence: the first needs all
      // copy groups but the FS_P-1 newest, the second all but the FS_P-2 newest
      if (ta && tb) {
        if (i > 0) {
#pragma unroll
          for (int j = 0; j < NV; ++j) sts_v4(stk_s + ((sp * NV + j) << 9), top[j]);
          ++sp;
        }
        cp_async_wait<FS_P - 1>();
        from_ring(x);
        cp_async_wait<FS_P - 2>();
        from_ring(y);
      } else if (ta) {
        cp_async_wait<FS_P - 1>();
        from_ring(x);
#pragma unroll
        for (int j = 0; j < NV; ++j) y[j] = top[j];
      } else if (tb) {
#pragma unroll
        for (int j = 0; j < NV; ++j) x[j] = top[j];
        cp_async_wait<FS_P - 1>();
        from_ring(y);
      } else {
        --sp;
#pragma unroll
        for (int j = 0; j < NV; ++j) {
          x[j] = lds_v4(stk_s + ((sp * NV + j) << 9));
          y[j] = top[j];
        }
      }
      uint4 med[NV];
#pragma unroll
      for (int j = 0; j < NV; ++j) med[j] = rule.template combine<FULL>(x[j], y[j], valid[j], j);
      rule.step(p, sitecnt, lane);
      // slots read this step are refilled only once their values are in use
      while (issued < consumed + FS_P) issue();
      const uint64_t noff = (uint64_t)(uint32_t)op.x * ld32;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        top[j] = med[j];
        if (act[j]) __stcs(reinterpret_cast<uint4 *>(ncol[j] + noff), med[j]);
      }
      op = next;
    }
    cp_async_wait<0>();
#pragma unroll
    for (int j = 0; j < NV; ++j) stk0[(q * NV + j) * 32 + lane] = top[j];   // this segment's result
  }
}

template <class Op>
__global__ void __launch_bounds__(FS_W * 32, Op::MIN_BLOCKS) tree_split_kernel(const FitchSplitArgs p) {
  constexpr int NV = Op::NV;
  constexpr int PER = Op::PER;
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int rows = p.rows;
  uint4 *region = reinterpret_cast<uint4 *>(smem);
  uint4 *ring = region + (size_t)w * rows * NV * 32;
  uint4 *stk0 = ring + FS_P * NV * 32;
  // per-site counts of the CTA's words, shared by its warps (they all work
  // on the same words): [entry][32 lanes]
  uint32_t *sitecnt = reinterpret_cast<uint32_t *>(region + (size_t)FS_W * rows * NV * 32);
  const int n_entries = Op::sites(p.count16 != 0);
  for (int i = tid; i < 32 * n_entries; i += FS_W * 32) sitecnt[i] = 0;
  Op rule;
  rule.init(p, sitecnt + 32 * n_entries, tid);
  __syncthreads();
  // a tile of tile_words words: lanes past it idle (their loads are
  // zero-filled, nothing of theirs is counted or stored)
  const size_t tile0 = ((size_t)blockIdx.x + p.tile_base) * p.tile_words;
  size_t word[NV];
  bool act[NV];
  uint4 valid[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    const bool in_tile = 128 * j + 4 * lane < p.tile_words;
    word[j] = tile0 + 128 * j + 4 * lane;
    act[j] = in_tile && word[j] < p.ld;
    valid[j] = make_uint4(0u, 0u, 0u, 0u);
    if (in_tile) {
      valid[j].x = valid_lanes<32 / PER>(word[j] + 0, p.n_sites);
      valid[j].y = valid_lanes<32 / PER>(word[j] + 1, p.n_sites);
      valid[j].z = valid_lanes<32 / PER>(word[j] + 2, p.n_sites);
      valid[j].w = valid_lanes<32 / PER>(word[j] + 3, p.n_sites);
    }
  }
  const bool full = (tile0 + p.tile_words) * PER <= p.n_sites &&
                    (Op::FULL_ANY_WIDTH || p.tile_words == 128 * NV);

  // ---- phase 1: warp w walks its segments ----
  if (full)
    split_walk<Op, true>(p, rule, ring, stk0, valid, act, word, sitecnt, w, lane);
  else
    split_walk<Op, false>(p, rule, ring, stk0, valid, act, word, sitecnt, w, lane);
  __syncthreads();
  // ---- phase 2: warp 0 joins the segments ----
  // reference of a child: tip id (>= 0), segment result -1 - (warp * 32 +
  // row), joining result -1000 - t (kept in the idle rings, FS_P per warp)
  if (w == 0) {
    for (int i = 0; i < p.n_top; ++i) {
      const int4 op = __ldg(p.top + i);
      uint4 c[2][NV];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int ref = h == 0 ? op.y : op.z;
        size_t at_row = 0;
        if (ref > -1000 && ref < 0) {
          const int at = -1 - ref;
          at_row = (size_t)(at >> 5) * rows + FS_P + (at & 31);
        } else if (ref <= -1000) {
          const int t = -1000 - ref;
          at_row = (size_t)(t / FS_P) * rows + t % FS_P;
        }
#pragma unroll
        for (int j = 0; j < NV; ++j) {
          if (ref >= 0)
            c[h][j] = act[j] ? __ldcs(reinterpret_cast<const uint4 *>(p.tips + (size_t)ref * p.ld + word[j]))
                             : make_uint4(0, 0, 0, 0);
          else
            c[h][j] = region[(at_row * NV + j) * 32 + lane];
        }
      }
      const size_t out_row = (size_t)(i / FS_P) * rows + i % FS_P;
      uint32_t *dst = p.node_sets + (size_t)op.x * p.ld;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const uint4 med = rule.template combine<false>(c[0][j], c[1][j], valid[j], j);
        region[(out_row * NV + j) * 32 + lane] = med;
        if (act[j]) __stcs(reinterpret_cast<uint4 *>(dst + word[j]), med);
      }
      rule.step(p, sitecnt, lane);
    }
  }
  // ---- phase 3: the per-site counts, then the weighted total ----
  rule.finish(p, sitecnt, lane);
  __syncthreads();
  if (w == 0) {
    rule.check_root(p, valid, act, word);
    unsigned long long wsum = 0;
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const size_t s0 = (word[j] + q) * PER;
#pragma unroll
        for (int l = 0; l < PER; ++l) {
          const size_t s = s0 + l;
          if (act[j] && s < p.n_sites) {
            const uint32_t v = rule.count(p, sitecnt, j, q, l, lane);
            if (p.site_cost) p.site_cost[s] = v;
            const uint32_t wt = p.weights ? __ldg(p.weights + s) : 1u;
            wsum += (unsigned long long)wt * v;
          }
        }
      }
    wsum = warp_sum_u64(wsum);
    if (lane == 0 && wsum) atomicAdd(p.total, wsum);
  }
}

template <int LB>
pgpu_status launch_pair(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b, const uint32_t *w,
                        uint32_t *out, size_t n_words, size_t n_sites,
                        unsigned long long *count, int mode) {
  const int threads = 256;
  size_t blocks = (n_words + threads - 1) / threads;
  blocks = std::min<size_t>(std::max<size_t>(blocks, 1), (size_t)ctx->num_sms * 8);
  if (mode == 0)
    fitch_pair_kernel<LB, false, true><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
        a, b, w, out, n_words, n_sites, count);
  else if (mode == 1)
    fitch_pair_kernel<LB, true, true><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
        a, b, w, out, n_words, n_sites, count);
  else
    fitch_pair_kernel<LB, false, false><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
        a, b, w, out, n_words, n_sites, count);
  return pgpu_after_launch(ctx, "fitch_pair_kernel");
}

bool lane_bits_ok(int lb) { return lb == 4 || lb == 8 || lb == 16 || lb == 32; }
bool lane_bits_ok64(int lb) { return lane_bits_ok(lb) || lb == 64; }

size_t words_for(size_t n_sites, int lb) { return (n_sites * (size_t)lb + 31) / 32; }

// mode 0: median + count, 1: median + weighted cost, 2: distance only
pgpu_status pair_host(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b, const uint32_t *w,
                      uint32_t *out, size_t n_sites, int lb, uint64_t *result, int mode) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!lane_bits_ok64(lb))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "lane_bits must be 4, 8, 16, 32 or 64");
  if (!a || !b || !result || (mode != 2 && !out) || (mode == 1 && !w))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch: null buffer");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t n_words = words_for(n_sites, lb);
  // The host buffers hold exactly the sites' bytes, as the reference's
  // vectors do (bv_malloc allocates chars * sizeof(CTYPE), lib/bitvector/
  // bv.c:32-42): a BV8 vector of 5 characters is 5 bytes, not two words.
  // Only those bytes are read and written; the device word they end in is
  // cleared first, so the lanes past the last site are zero.
  const size_t n_bytes = (n_sites * (size_t)lb + 7) / 8;
  void *da, *db, *dout, *dw = nullptr, *dc;
  PGPU_TRY(pgpu_buf(ctx, BUF_A, n_words * 4, &da));
  PGPU_TRY(pgpu_buf(ctx, BUF_B, n_words * 4, &db));
  PGPU_TRY(pgpu_buf(ctx, BUF_OUT, n_words * 4, &dout));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dc));
  if (mode == 1) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n_sites * 4, &dw));
  cudaStream_t s = ctx->stream;
  if (n_bytes < n_words * 4) {
    PGPU_CUDA(ctx, cudaMemsetAsync((uint32_t *)da + (n_words - 1), 0, 4, s));
    PGPU_CUDA(ctx, cudaMemsetAsync((uint32_t *)db + (n_words - 1), 0, 4, s));
  }
  PGPU_CUDA(ctx, cudaMemcpyAsync(da, a, n_bytes, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(db, b, n_bytes, cudaMemcpyHostToDevice, s));
  if (mode == 1) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, w, n_sites * 4, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemsetAsync(dc, 0, 8, s));
  if (n_words) {
    auto *cnt = reinterpret_cast<unsigned long long *>(dc);
    const uint32_t *pa = (const uint32_t *)da, *pb = (const uint32_t *)db,
                   *pw = (const uint32_t *)dw;
    uint32_t *po = (uint32_t *)dout;
    if (lb == 64) {
      const int threads = 256;
      size_t blocks = (n_sites + threads - 1) / threads;
      blocks = std::min<size_t>(std::max<size_t>(blocks, 1), (size_t)ctx->num_sms * 8);
      const uint2 *a2 = (const uint2 *)pa, *b2 = (const uint2 *)pb;
      uint2 *o2 = (uint2 *)po;
      if (mode == 0)
        fitch_pair64_kernel<false, true><<<(unsigned)blocks, threads, 0, s>>>(a2, b2, pw, o2, n_sites, cnt);
      else if (mode == 1)
        fitch_pair64_kernel<true, true><<<(unsigned)blocks, threads, 0, s>>>(a2, b2, pw, o2, n_sites, cnt);
      else
        fitch_pair64_kernel<false, false><<<(unsigned)blocks, threads, 0, s>>>(a2, b2, pw, o2, n_sites, cnt);
      PGPU_TRY(pgpu_after_launch(ctx, "fitch_pair64_kernel"));
    } else switch (lb) {
      case 4: PGPU_TRY(launch_pair<4>(ctx, pa, pb, pw, po, n_words, n_sites, cnt, mode)); break;
      case 8: PGPU_TRY(launch_pair<8>(ctx, pa, pb, pw, po, n_words, n_sites, cnt, mode)); break;
      case 16: PGPU_TRY(launch_pair<16>(ctx, pa, pb, pw, po, n_words, n_sites, cnt, mode)); break;
      default: PGPU_TRY(launch_pair<32>(ctx, pa, pb, pw, po, n_words, n_sites, cnt, mode)); break;
    }
  }
  if (mode != 2) PGPU_CUDA(ctx, cudaMemcpyAsync(out, dout, n_bytes, cudaMemcpyDeviceToHost, s));
  uint64_t *hc = reinterpret_cast<uint64_t *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(hc, dc, 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  *result = *hc;
  return PGPU_OK;
}

template <int LB, int ST>
cudaError_t launch_tree_st(cudaStream_t stream, const FitchTreeArgs &args, const FitchPlan &pl) {
  cudaError_t e = cudaFuncSetAttribute(fitch_tree_kernel<LB, ST>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)std::max<size_t>(pl.smem, 48 * 1024));
  if (e != cudaSuccess) return e;
  fitch_tree_kernel<LB, ST><<<(unsigned)pl.tiles, 32 + (int)pl.W / 4, pl.smem, stream>>>(args);
  return cudaGetLastError();
}

template <int LB>
cudaError_t launch_tree_lb(cudaStream_t stream, const FitchTreeArgs &args, const FitchPlan &pl) {
  switch (pl.stages) {
    case 64: return launch_tree_st<LB, 64>(stream, args, pl);
    case 32: return launch_tree_st<LB, 32>(stream, args, pl);
    default: return launch_tree_st<LB, 16>(stream, args, pl);
  }
}

cudaError_t launch_tree(cudaStream_t stream, int lb, const FitchTreeArgs &args, const FitchPlan &pl) {
  switch (lb) {
    case 4: return launch_tree_lb<4>(stream, args, pl);
    case 8: return launch_tree_lb<8>(stream, args, pl);
    case 16: return launch_tree_lb<16>(stream, args, pl);
    default: return launch_tree_lb<32>(stream, args, pl);
  }
}


// Cuts the postorder into up to FS_S segments: repeatedly split the largest
// remaining subtree at its root (the root joins the top part) while fewer
// than FS_S subtrees remain and the largest has at least two internal nodes.
// Each segment is scheduled like the whole tree (Sethi-Ullman order: the
// child with the larger stack need first).  Segments go to the FS_W warps
// longest first, each to the least loaded warp.
pgpu_status build_split(pgpu_ctx *ctx, const pgpu_tree *tree, SplitSchedule *out) {
  TreeSchedule check;
  PGPU_TRY(pgpu_build_schedule(ctx, tree, &check));   // validates the tree
  const int32_t n = tree->n_tips, n_int = n - 1;
  const int32_t *L = tree->left, *R = tree->right;
  std::vector<int32_t> size(n_int, 1), need(2 * n - 1, 0);
  std::vector<uint8_t> swp(n_int, 0);
  for (int32_t k = 0; k < n_int; ++k) {
    const int32_t a = L[k], b = R[k];
    if (a >= n) size[k] += size[a - n];
    if (b >= n) size[k] += size[b - n];
    const int32_t ha = a >= n, hb = b >= n;
    const int32_t a_first = std::max(need[a], ha + need[b]);
    const int32_t b_first = std::max(need[b], hb + need[a]);
    swp[k] = b_first < a_first;
    need[n + k] = std::max(std::min(a_first, b_first), 1);
  }
  std::vector<int32_t> heap{n_int - 1};
  std::vector<uint8_t> is_top(n_int, 0);
  auto by_size = [&](int32_t x, int32_t y) { return size[x] < size[y]; };
  int n_split = 0;
  while ((int)heap.size() < FS_S && !heap.empty() && n_split < FS_S) {
    std::pop_heap(heap.begin(), heap.end(), by_size);
    const int32_t k = heap.back();
    if (size[k] < 2) {
      std::push_heap(heap.begin(), heap.end(), by_size);
      break;
    }
    heap.pop_back();
    is_top[k] = 1;
    ++n_split;
    for (const int32_t c : {L[k], R[k]})
      if (c >= n) {
        heap.push_back(c - n);
        std::push_heap(heap.begin(), heap.end(), by_size);
      }
  }
  // longest first onto the least loaded warp
  std::sort(heap.begin(), heap.end(), [&](int32_t x, int32_t y) { return size[x] > size[y]; });
  std::vector<std::vector<int32_t>> per_warp(FS_W);
  std::vector<int64_t> load(FS_W, 0);
  for (const int32_t r : heap) {
    const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    per_warp[w].push_back(r);
    load[w] += size[r];
  }
  SplitSchedule sp;
  sp.n_seg = (int)heap.size();
  std::vector<int32_t> ref_of(n_int, 0);   // reference of a segment root
  int max_need = 1;
  for (int w = 0; w < FS_W; ++w) {
    sp.wseg.push_back(make_int4((int)sp.seg.size(), (int)per_warp[w].size(), 0, 0));
    for (int q = 0; q < (int)per_warp[w].size(); ++q) {
      const int32_t root = per_warp[w][q];
      ref_of[root] = -1 - (w * 32 + q);
      const int op_off = (int)sp.ops.size(), tip_off = (int)sp.tips.size();
      struct Fr {
        int32_t v;
        bool done;
      };
      std::vector<Fr> st{{n + root, false}};
      int height = 0, depth = 0;
      while (!st.empty()) {
        const Fr f = st.back();
        st.pop_back();
        const int32_t k = f.v - n;
        const int32_t first = swp[k] ? R[k] : L[k], second = swp[k] ? L[k] : R[k];
        if (!f.done) {
          st.push_back({f.v, true});
          if (second >= n) st.push_back({second, false});
          if (first >= n) st.push_back({first, false});
          continue;
        }
        sp.ops.push_back(make_int4(k, first, second, 0));
        if (first < n) sp.tips.push_back(first);
        if (second < n) sp.tips.push_back(second);
        height += 1 - (first >= n) - (second >= n);
        depth = std::max(depth, height);
      }
      // the walk's stack starts above the q earlier results and this one
      max_need = std::max(max_need, q + 1 + depth);
      sp.seg.push_back(make_int4(op_off, (int)sp.ops.size() - op_off, tip_off,
                                 (int)sp.tips.size() - tip_off));
    }
  }
  if (sp.n_seg > 32) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "fitch_tree: too many segments");
  sp.rows = FS_P + max_need;
  std::vector<int32_t> top_of(n_int, -1);
  int n_top = 0;
  for (int32_t k = 0; k < n_int; ++k) {
    if (!is_top[k]) continue;
    int32_t ref[2];
    for (int h = 0; h < 2; ++h) {
      const int32_t c = h == 0 ? L[k] : R[k];
      ref[h] = c < n ? c : !is_top[c - n] ? ref_of[c - n] : -1000 - top_of[c - n];
    }
    top_of[k] = n_top++;
    sp.top.push_back(make_int4(k, ref[0], ref[1], 0));
  }
  if (n_top > FS_W * FS_P)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "fitch_tree: %d joining nodes (at most %d)", n_top,
                        FS_W * FS_P);
  *out = std::move(sp);
  return PGPU_OK;
}

// the split schedule of `tree`, resident in BUF_SPLIT ({ops, seg, top, tips})
pgpu_status split_device(pgpu_ctx *ctx, const pgpu_tree *tree, const int4 **ops, const int4 **seg,
                         const int4 **top, const int4 **wseg, const int32_t **tips) {
  const int32_t n_int = tree->n_tips - 1;
  const bool hit = ctx->split_valid && (int32_t)ctx->split_left.size() == n_int &&
                   std::memcmp(ctx->split_left.data(), tree->left, n_int * 4) == 0 &&
                   std::memcmp(ctx->split_right.data(), tree->right, n_int * 4) == 0;
  const SplitSchedule &sp = ctx->split;
  if (!hit) {
    ctx->split_valid = false;
    PGPU_TRY(build_split(ctx, tree, &ctx->split));
    const size_t bytes =
        16 * (sp.ops.size() + sp.seg.size() + sp.top.size() + sp.wseg.size()) + 4 * sp.tips.size();
    void *d;
    PGPU_TRY(pgpu_buf(ctx, BUF_SPLIT, std::max<size_t>(bytes, 16), &d));
    std::vector<unsigned char> h(std::max<size_t>(bytes, 16));
    size_t off = 0;
    auto put = [&](const void *src, size_t b) {
      if (b) std::memcpy(h.data() + off, src, b);
      off += b;
    };
    put(sp.ops.data(), 16 * sp.ops.size());
    put(sp.seg.data(), 16 * sp.seg.size());
    put(sp.top.data(), 16 * sp.top.size());
    put(sp.wseg.data(), 16 * sp.wseg.size());
    put(sp.tips.data(), 4 * sp.tips.size());
    PGPU_CUDA(ctx, cudaMemcpyAsync(d, h.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
    PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // h is a temporary
    ctx->split_left.assign(tree->left, tree->left + n_int);
    ctx->split_right.assign(tree->right, tree->right + n_int);
    ctx->split_valid = true;
  }
  const int4 *base = static_cast<const int4 *>(ctx->buf[BUF_SPLIT]);
  *ops = base;
  *seg = base + sp.ops.size();
  *top = *seg + sp.seg.size();
  *wseg = *top + sp.top.size();
  *tips = reinterpret_cast<const int32_t *>(*wseg + sp.wseg.size());
  return PGPU_OK;
}

template <class Op>
cudaError_t launch_split(cudaStream_t stream, const FitchSplitArgs &a, size_t tiles) {
  const size_t smem = split_smem<Op>(a.rows, a.count16 != 0);
  cudaError_t e = cudaFuncSetAttribute(tree_split_kernel<Op>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)std::max<size_t>(smem, 48 * 1024));
  if (e != cudaSuccess) return e;
  tree_split_kernel<Op><<<(unsigned)tiles, FS_W * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

template <int LB>
cudaError_t launch_fitch_split(cudaStream_t stream, const FitchSplitArgs &a, size_t tiles) {
  return a.tile_words > 128 ? launch_split<FitchOp<LB, 2>>(stream, a, tiles)
                            : launch_split<FitchOp<LB, 1>>(stream, a, tiles);
}

// The default tile width of the Fitch tree kernel: of the widths 128..256
// (multiples of 4), the one that gives the busiest SM the fewest words when
// all CTAs are resident at once; ties keep the narrower width.
int default_tile_words(size_t n_words, int n_sm) {
  int best = 128;
  size_t best_cost = SIZE_MAX;
  for (int w = 128; w <= 256; w += 4) {
    const size_t tiles = (n_words + w - 1) / w;
    const size_t cost = ((tiles + n_sm - 1) / n_sm) * (size_t)w;
    if (cost < best_cost) {
      best = w;
      best_cost = cost;
    }
  }
  return best;
}

// 64-bit elements: the element kernel over the plain schedule
pgpu_status tree64_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips, size_t ld,
                       const uint32_t *weights, size_t n_sites, uint32_t *node_sets,
                       uint32_t *site_cost, uint64_t *total) {
  const TreeSchedule *sch;
  const int4 *d_ops;
  const int32_t *d_seq;
  PGPU_TRY(pgpu_schedule_device(ctx, tree, &sch, &d_ops, &d_seq));
  cudaStream_t s = ctx->stream;
  PGPU_CUDA(ctx, cudaMemsetAsync(total, 0, sizeof(uint64_t), s));
  if (n_sites == 0) return PGPU_OK;
  Fitch64Args a;
  a.tips = reinterpret_cast<const uint2 *>(tips);
  a.weights = weights;
  a.node_sets = reinterpret_cast<uint2 *>(node_sets);
  a.site_cost = site_cost;
  a.total = reinterpret_cast<unsigned long long *>(total);
  a.ops = d_ops;
  a.ld2 = ld / 2;
  a.n = n_sites;
  a.n_tips = tree->n_tips;
  a.n_ops = (int)sch->ops.size();
  a.depth = std::max(sch->max_depth, 1);
  const size_t smem = (size_t)a.depth * F64_THREADS * sizeof(uint2);
  if (smem > (size_t)ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "fitch_tree: tree too deep (%d stack entries)", a.depth);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(fitch_tree64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const unsigned grid = (unsigned)((n_sites + F64_THREADS - 1) / F64_THREADS);
  fitch_tree64_kernel<<<grid, F64_THREADS, smem, s>>>(a);
  return pgpu_after_launch(ctx, "fitch_tree64_kernel");
}

// The split kernel's launches over tiles [0, tiles), in up to
// PGPU_COPY_CHUNKS column chunks when the rows are still in host memory
// (io): chunk k's tip columns are copied in on the copy stream, its launch
// waits for them, and its node columns go back on the device-to-host stream
// once the launch is done.  launch(t0, t1) launches tiles [t0, t1).
template <class Launch>
pgpu_status split_chunks(pgpu_ctx *ctx, const FitchSplitArgs &a, size_t tiles, const HostRows *io,
                         Launch launch) {
  const size_t n = (size_t)a.n_tips, tw = (size_t)a.tile_words, ld = a.ld, nw = a.n_words;
  const int K = io ? (int)std::min<size_t>(PGPU_COPY_CHUNKS, tiles) : 1;
  for (int k = 0; k < K; ++k) {
    const size_t t0 = tiles * k / K, t1 = tiles * (k + 1) / K;
    const size_t w0 = t0 * tw, w1 = std::min(t1 * tw, nw);
    if (io) {
      PGPU_CUDA(ctx, cudaMemcpy2DAsync(const_cast<uint32_t *>(a.tips) + w0, ld * 4, io->tips + w0, nw * 4,
                                       (w1 - w0) * 4, n, cudaMemcpyHostToDevice, ctx->copy_stream));
      PGPU_CUDA(ctx, cudaEventRecord(ctx->copy_ev[k], ctx->copy_stream));
      PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[k], 0));
    }
    PGPU_TRY(launch(t0, t1));
    if (io) {
      PGPU_CUDA(ctx, cudaEventRecord(ctx->done_ev[k], ctx->stream));
      PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->d2h_stream, ctx->done_ev[k], 0));
      PGPU_CUDA(ctx, cudaMemcpy2DAsync(io->node_sets + w0, nw * 4, a.node_sets + w0, ld * 4,
                                       (w1 - w0) * 4, n - 1, cudaMemcpyDeviceToHost, ctx->d2h_stream));
    }
  }
  return PGPU_OK;
}

pgpu_status tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips, size_t ld,
                     const uint32_t *weights, size_t n_sites, int lb, uint32_t *node_sets,
                     uint32_t *site_cost, uint64_t *total, const HostRows *io = nullptr) {
  if (!lane_bits_ok64(lb))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "lane_bits must be 4, 8, 16, 32 or 64");
  const size_t n_words = words_for(n_sites, lb);
  if (!tips || !node_sets || !total) return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch_tree: null buffer");
  if (ld % 4 != 0 || ld < n_words)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch_tree: ld_words (%zu) must be a multiple of 4 and >= %zu",
                        ld, n_words);
  if (((uintptr_t)tips | (uintptr_t)node_sets) & 15)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch_tree: tip and node rows must be 16-byte aligned");
  if (!tree || tree->n_tips < 2) return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch_tree: need at least 2 tips");
  if (lb == 64) return tree64_dev(ctx, tree, tips, ld, weights, n_sites, node_sets, site_cost, total);
  FitchSplitArgs a;
  PGPU_TRY(split_device(ctx, tree, &a.ops, &a.seg, &a.top, &a.wseg, &a.tip_seq));
  cudaStream_t s = ctx->stream;
  PGPU_CUDA(ctx, cudaMemsetAsync(total, 0, sizeof(uint64_t), s));
  if (n_words == 0) return PGPU_OK;
  const SplitSchedule &sp = ctx->split;
  a.tips = tips;
  a.weights = weights;
  a.node_sets = node_sets;
  a.site_cost = site_cost;
  a.total = reinterpret_cast<unsigned long long *>(total);
  a.ld = ld;
  a.n_words = n_words;
  a.n_sites = n_sites;
  a.n_tips = tree->n_tips;
  a.n_top = (int)sp.top.size();
  a.rows = sp.rows;
  // LB = 4 has the most per-site counters, so it bounds every width's need
  if (split_smem<FitchOp<4, 1>>(a.rows, false) > ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "fitch_tree: tree needs a stack of %d rows; too deep",
                        a.rows);
  a.tile_words = ctx->fitch_tile_words > 0 ? ctx->fitch_tile_words
                                           : default_tile_words(n_words, ctx->num_sms);
  // two parts per lane only where their stacks fit; the width only shapes
  // the launch, so a narrower one gives the same results
  a.count16 = tree->n_tips - 1 <= 65535;
  if (ld > 0xffffffffull) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "fitch_tree: rows of 2^32 words or more");
  if (a.tile_words > 128 && split_smem<FitchOp<4, 2>>(a.rows, a.count16) > ctx->smem_optin) a.tile_words = 128;
  a.tcm_period = 0;
  a.table = nullptr;
  a.flag = ctx->d_flag;
  const size_t tiles = (n_words + a.tile_words - 1) / a.tile_words;
  if (tiles > 0x7fffffffu) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "fitch_tree: too many tiles");
  return split_chunks(ctx, a, tiles, io, [&](size_t t0, size_t t1) -> pgpu_status {
    a.tile_base = t0;
    cudaError_t e;
    switch (lb) {
      case 4: e = launch_fitch_split<4>(s, a, t1 - t0); break;
      case 8: e = launch_fitch_split<8>(s, a, t1 - t0); break;
      case 16: e = launch_fitch_split<16>(s, a, t1 - t0); break;
      default: e = launch_fitch_split<32>(s, a, t1 - t0); break;
    }
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return pgpu_set_err(ctx, PGPU_ERR_CUDA, "launch of tree_split_kernel failed: %s",
                          cudaGetErrorString(e));
    }
    ctx->launches++;
    return PGPU_OK;
  });
}

}  // namespace

// The cost-matrix postorder (csrc/tcm.cu) on the segmented schedule: 4-bit
// codes, the packed pair table already on the device.  flush_period > 0
// (every cost small enough) selects the re-packed table with one add per
// site.  *launched is false when the tree's stacks and the lane-replicated
// table do not fit one CTA's shared memory; the caller then uses its
// single-walk kernel.
pgpu_status pgpu_tcm_tree_split(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                                size_t ld, const uint32_t *weights, size_t n_sites,
                                const uint32_t *table_dev, int flush_period, uint32_t *node_sets,
                                uint32_t *site_cost, unsigned long long *total, bool *launched,
                                const HostRows *io) {
  *launched = false;
  if (((uintptr_t)tips | (uintptr_t)node_sets) & 15) return PGPU_OK;
  if (ld % 4 != 0 || ld > 0xffffffffull) return PGPU_OK;
  const size_t n_words = (n_sites + 7) / 8;
  FitchSplitArgs a;
  PGPU_TRY(split_device(ctx, tree, &a.ops, &a.seg, &a.top, &a.wseg, &a.tip_seq));
  const SplitSchedule &sp = ctx->split;
  if (split_smem<TcmOp<false>>(sp.rows, false) > ctx->smem_optin) return PGPU_OK;
  a.tips = tips;
  a.weights = weights;
  a.node_sets = node_sets;
  a.site_cost = site_cost;
  a.total = total;
  a.ld = ld;
  a.n_words = n_words;
  a.n_sites = n_sites;
  a.n_tips = tree->n_tips;
  a.n_top = (int)sp.top.size();
  a.rows = sp.rows;
  a.tile_words = 128;
  a.tile_base = 0;
  a.count16 = 0;
  a.tcm_period = flush_period;
  a.table = table_dev;
  a.flag = ctx->d_flag;
  const size_t tiles = (n_words + 127) / 128;
  PGPU_TRY(split_chunks(ctx, a, tiles, io, [&](size_t t0, size_t t1) -> pgpu_status {
    a.tile_base = t0;
    cudaError_t e = flush_period > 0 ? launch_split<TcmOp<true>>(ctx->stream, a, t1 - t0)
                                     : launch_split<TcmOp<false>>(ctx->stream, a, t1 - t0);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return pgpu_set_err(ctx, PGPU_ERR_CUDA, "launch of tree_split_kernel<TcmOp> failed: %s",
                          cudaGetErrorString(e));
    }
    ctx->launches++;
    return PGPU_OK;
  }));
  *launched = true;
  return PGPU_OK;
}

// Launches the tree kernel on device arrays the caller manages (schedule ops,
// tip sequence, error word) on an explicit stream, without a context.  Used
// by the entry point that allocates nothing (noalloc.cu).
pgpu_status pgpu_fitch_tree_launch_raw(cudaStream_t stream, const int4 *ops, const int32_t *tip_seq,
                                       int n_ops, int depth, int *flag, int32_t n_tips,
                                       const uint32_t *tips, size_t ld, const uint32_t *weights,
                                       size_t n_sites, int lb, uint32_t *node_sets,
                                       uint32_t *site_cost, uint64_t *total) {
  if (!lane_bits_ok(lb)) return PGPU_ERR_ARG;
  const size_t n_words = words_for(n_sites, lb);
  if (!tips || !node_sets || !total || ld % 4 != 0 || ld < n_words) return PGPU_ERR_ARG;
  if (((uintptr_t)tips | (uintptr_t)node_sets) & 15) return PGPU_ERR_ARG;
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return PGPU_ERR_CUDA;
  }
  if (cudaMemsetAsync(total, 0, sizeof(uint64_t), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PGPU_ERR_CUDA;
  }
  if (n_words == 0) return PGPU_OK;
  const FitchPlan pl = fitch_plan(n_words, depth, sms, (size_t)optin);
  if (pl.smem > (size_t)optin) return PGPU_ERR_LIMIT;
  FitchTreeArgs a;
  a.tips = tips;
  a.weights = weights;
  a.node_sets = node_sets;
  a.site_cost = site_cost;
  a.total = reinterpret_cast<unsigned long long *>(total);
  a.ops = ops;
  a.tip_seq = tip_seq;
  a.flag = flag;
  a.ld = ld;
  a.n_words = n_words;
  a.n_sites = n_sites;
  a.n_tips = n_tips;
  a.n_ops = n_ops;
  a.W = (int)pl.W;
  a.depth = depth;
  cudaError_t e = launch_tree(stream, lb, a, pl);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return PGPU_ERR_CUDA;
  }
  return PGPU_OK;
}

extern "C" {

pgpu_status pgpu_fitch_median2(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b, uint32_t *out,
                               size_t n_sites, int lane_bits, uint64_t *union_count) {
  return pair_host(ctx, a, b, nullptr, out, n_sites, lane_bits, union_count, 0);
}

pgpu_status pgpu_set_fitch_tile_words(pgpu_ctx *ctx, int words) {
  if (!ctx) return PGPU_ERR_ARG;
  if (words != 0 && (words < 32 || words > 256 || words % 4 != 0))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch tile: 0 or a multiple of 4 in 32..256 words (got %d)",
                        words);
  ctx->fitch_tile_words = words;
  return PGPU_OK;
}

int pgpu_get_fitch_tile_words(const pgpu_ctx *ctx) {
  return ctx ? ctx->fitch_tile_words : 0;
}

pgpu_status pgpu_nonadditive_median2(pgpu_ctx *ctx, const int64_t *x, const int64_t *y,
                                     const double *weights, int64_t *out, size_t n, double *cost) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!cost || (n && (!x || !y || !weights || !out)))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "nonadditive: null buffer");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  if (n == 0) {
    *cost = 0.0;
    return PGPU_OK;
  }
  const int sms = ctx->num_sms > 0 ? ctx->num_sms : 1;
  const size_t blocks =
      std::min<size_t>((n + NA_THREADS - 1) / NA_THREADS, (size_t)sms * 8);
  void *dx, *dy, *dw, *dout, *dpart, *dc;
  PGPU_TRY(pgpu_buf(ctx, BUF_A, n * 8, &dx));
  PGPU_TRY(pgpu_buf(ctx, BUF_B, n * 8, &dy));
  PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n * 8, &dw));
  PGPU_TRY(pgpu_buf(ctx, BUF_OUT, n * 8, &dout));
  PGPU_TRY(pgpu_buf(ctx, BUF_C, blocks * sizeof(double2), &dpart));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dc));
  cudaStream_t s = ctx->stream;
  PGPU_CUDA(ctx, cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dy, y, n * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n * 8, cudaMemcpyHostToDevice, s));
  nonadd_median_kernel<<<(unsigned)blocks, NA_THREADS, 0, s>>>(
      (const unsigned long long *)dx, (const unsigned long long *)dy, (const double *)dw,
      (unsigned long long *)dout, n, (double2 *)dpart);
  PGPU_TRY(pgpu_after_launch(ctx, "nonadd_median_kernel"));
  nonadd_finalize_kernel<<<1, 1024, 0, s>>>((const double2 *)dpart, (int)blocks, (double *)dc);
  PGPU_TRY(pgpu_after_launch(ctx, "nonadd_finalize_kernel"));
  double *hc = reinterpret_cast<double *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(out, dout, n * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(hc, dc, 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  *cost = *hc;
  return PGPU_OK;
}

pgpu_status pgpu_fitch_median2_weighted(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b,
                                        const uint32_t *weights, uint32_t *out, size_t n_sites,
                                        int lane_bits, uint64_t *cost) {
  return pair_host(ctx, a, b, weights, out, n_sites, lane_bits, cost, 1);
}

pgpu_status pgpu_fitch_distance(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b,
                                size_t n_sites, int lane_bits, uint64_t *distance) {
  return pair_host(ctx, a, b, nullptr, nullptr, n_sites, lane_bits, distance, 2);
}

pgpu_status pgpu_fitch_tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips_dev,
                                size_t ld_words, const uint32_t *weights_dev, size_t n_sites,
                                int lane_bits, uint32_t *node_sets_dev, uint32_t *site_cost_dev,
                                uint64_t *total_dev) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  return tree_dev(ctx, tree, tips_dev, ld_words, weights_dev, n_sites, lane_bits, node_sets_dev,
                  site_cost_dev, total_dev);
}

pgpu_status pgpu_fitch_tree(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                            const uint32_t *weights, size_t n_sites, int lane_bits,
                            uint32_t *node_sets, uint32_t *site_cost, uint64_t *total) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!tree || !tips || !node_sets || !total)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "fitch_tree: null argument");
  if (!lane_bits_ok64(lane_bits))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "lane_bits must be 4, 8, 16, 32 or 64");
  if (tree->n_tips < 2) return pgpu_set_err(ctx, PGPU_ERR_ARG, "tree: need at least 2 tips");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t n_words = words_for(n_sites, lane_bits);
  const size_t ld = (n_words + 3) / 4 * 4;
  const size_t n = (size_t)tree->n_tips, n_int = n - 1;
  void *dw = nullptr, *dsc = nullptr, *dtot;
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dtot));
  if (weights) PGPU_TRY(pgpu_buf(ctx, BUF_WEIGHTS, n_sites * 4, &dw));
  if (site_cost) PGPU_TRY(pgpu_buf(ctx, BUF_SITECOST, n_sites * 4, &dsc));
  cudaStream_t s = ctx->stream;
  // Rows in page-locked host memory the device can address, 16-byte aligned
  // and a multiple of 4 words long: the kernel reads the tips and writes the
  // node sets over the CPU-GPU link itself, both directions at once and
  // with no staging buffers.
  const uint32_t *tv = nullptr;
  uint32_t *nv = nullptr;
  if (lane_bits < 64 && n_words > 0 && n_words % 4 == 0) {
    tv = static_cast<const uint32_t *>(pgpu_host_view(tips));
    nv = static_cast<uint32_t *>(pgpu_host_view(node_sets));
    if (((uintptr_t)tv | (uintptr_t)nv) & 15) tv = nullptr;
  }
  if (tv && nv) {
    if (weights) PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_sites * 4, cudaMemcpyHostToDevice, s));
    PGPU_TRY(pgpu_settle_copies(ctx, tree_dev(ctx, tree, tv, n_words, (const uint32_t *)dw, n_sites,
                                               lane_bits, nv, (uint32_t *)dsc, (uint64_t *)dtot)));
    if (site_cost)
      PGPU_CUDA(ctx, cudaMemcpyAsync(site_cost, dsc, n_sites * 4, cudaMemcpyDeviceToHost, s));
    uint64_t *ht = reinterpret_cast<uint64_t *>(ctx->h_pinned);
    PGPU_CUDA(ctx, cudaMemcpyAsync(ht, dtot, 8, cudaMemcpyDeviceToHost, s));
    PGPU_CUDA(ctx, cudaStreamSynchronize(s));
    PGPU_TRY(pgpu_check_flag(ctx, "fitch_tree"));
    *total = *ht;
    return PGPU_OK;
  }
  void *dt, *dn;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, n * ld * 4, &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_OUT, n_int * ld * 4, &dn));
  // below 64-bit lanes the rows go over in column chunks on the copy
  // streams, after everything already queued on the context's stream
  const bool chunked = lane_bits < 64 && n_words > 0;
  if (chunked) {
    PGPU_TRY(pgpu_copy_stream(ctx));
    PGPU_CUDA(ctx, cudaEventRecord(ctx->copy_ev[PGPU_COPY_CHUNKS], s));
    PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[PGPU_COPY_CHUNKS], 0));
    PGPU_CUDA(ctx, cudaStreamWaitEvent(ctx->d2h_stream, ctx->copy_ev[PGPU_COPY_CHUNKS], 0));
  } else if (n_words) {
    PGPU_CUDA(ctx, cudaMemcpy2DAsync(dt, ld * 4, tips, n_words * 4, n_words * 4, n,
                                     cudaMemcpyHostToDevice, s));
  }
  if (n_words && weights)
    PGPU_CUDA(ctx, cudaMemcpyAsync(dw, weights, n_sites * 4, cudaMemcpyHostToDevice, s));
  const HostRows io{tips, node_sets};
  PGPU_TRY(pgpu_settle_copies(ctx, tree_dev(ctx, tree, (const uint32_t *)dt, ld, (const uint32_t *)dw,
                                             n_sites, lane_bits, (uint32_t *)dn, (uint32_t *)dsc,
                                             (uint64_t *)dtot, chunked ? &io : nullptr)));
  if (n_words) {
    if (!chunked)
      PGPU_CUDA(ctx, cudaMemcpy2DAsync(node_sets, n_words * 4, dn, ld * 4, n_words * 4, n_int,
                                       cudaMemcpyDeviceToHost, s));
    if (site_cost)
      PGPU_CUDA(ctx, cudaMemcpyAsync(site_cost, dsc, n_sites * 4, cudaMemcpyDeviceToHost, s));
  }
  uint64_t *ht = reinterpret_cast<uint64_t *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(ht, dtot, 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  if (chunked) PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->d2h_stream));
  PGPU_TRY(pgpu_check_flag(ctx, "fitch_tree"));
  *total = *ht;
  return PGPU_OK;
}

}  // extern "C"
