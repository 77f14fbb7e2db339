// Batched likelihood of many trees, models and pattern sets of uneven size,
// for 20-state (protein) and 61-state (codon) models, on the tensor cores.
//
// Reference: the likelihood character is a stub in phylocaml
// (Likelihood_c.median_2, lib/likelihood_c.ml:15); P matrices follow
// MlModel.compose (lib/mlModel.ml:585-587, P[i][j] = Pr(j | i, t)).  Every
// variant is an independent (tree, model, patterns) problem.
//
// Design (one GB300, one launch for all variants):
//   setup kernels  the FP64 Jacobi eigen systems (pmatrix.cu), then per
//                  variant, internal branch and rate class the FP32 B operand
//                  B[n=i][k=j] = P(t r)[i][j] in the tcgen05 K-major
//                  core-matrix layout, and per tip branch the FP64-formed tip
//                  rows tab[c][i] = sum_j P[i][j] code_tab[c][j];
//   batch_tc_kernel  persistent, one CTA per SM, over work items
//                  (variant, tile of 128 patterns).  A tile's conditional
//                  likelihood vectors live in tensor memory (TMEM lane =
//                  pattern, columns = states) and are the A operand of
//                  tcgen05.mma.kind::tf32 for internal children; D (FP32) is
//                  accumulated in TMEM.  Tip children need no MMA: their rows
//                  come from the staged tip table.  Rate classes are separate
//                  passes with their own power-of-two scalers, joined at the
//                  root with a log-sum-exp in FP64.
//     warp 8       producer and TMEM allocator: per postorder step,
//                  bulk-copies the B blocks of internal children, the
//                  tip-table blocks and tip-code rows of tip children into a
//                  shared ring slot, and publishes the step itself;
//     warp 9       MMA issue (one thread);
//     warps 0-7    epilogue: two warps per TMEM lane group of 32 patterns,
//                  each owning a share of the row (half the states, or a
//                  whole rate class when two share a pass); a thread reads
//                  its D columns (tcgen05.ld) or tip rows, forms the product,
//                  rescales, writes the parent's vector back into TMEM
//                  (tcgen05.st).
//   The MMA (tcgen05.commit -> mma_bar) and the epilogue (an mbarrier,
//   `stored`, after its TMEM stores) alternate per step, so a step's MMA
//   never reads a vector before it is written and no mbarrier phase can be
//   skipped.  With two rate classes per pass the two classes are separate
//   chains, each with its own mma_bar and stored barrier and its own four
//   epilogue warps: the MMAs of one class's next step run while the other
//   class's epilogue runs, and no warp waits for another to agree on a
//   rescaling exponent.
//   Every wait is bounded.  Each work item runs a step loop compiled for its
//   padded state count and rate classes per pass.
//   batch_fp64_kernel  the FP64 comparison form on a sample of patterns.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "forms.cuh"
#include "pgpu_internal.cuh"
#include "pmatrix.cuh"

using namespace pgpu_forms;

namespace {

constexpr int BT_M = 128;          // patterns per tile (TMEM lanes)
constexpr int BT_ST = 4;           // ring slots (power of two)
constexpr int BT_EPI_WARPS = 8;    // epilogue warps, two per TMEM lane group
constexpr int BT_PARTS = BT_EPI_WARPS / 4;   // shares of a row (one per warp of a lane group)
constexpr int BT_EPI = 32 * BT_EPI_WARPS;
constexpr int BT_THREADS = BT_EPI + 64;   // + the producer warp and the MMA warp
constexpr int BT_PRODUCER = BT_EPI_WARPS, BT_MMA = BT_EPI_WARPS + 1;   // their warp indices
constexpr int BT_TMEM_COLS = 512;

struct BVar {
  int n_tips, n_ops, S, R, n_codes;
  int Kp, Np, SpT, NCp;            // padded K (A columns), N (D columns), odd tip-row stride, padded code rows
  int n_slots;                     // TMEM stack slots available
  int RP;                          // rate classes per pass (1 or 2): their MMAs share a step
  int n_tiles;
  long long n_pat;
  long long ld;                    // tip-code row stride in bytes (n_tiles * 128)
  const uint8_t *codes;            // [n_tips][ld] device tip codes of this variant
  const double *weights;           // [n_pat] device weights or null
  long long pat_off;               // first pattern of the variant in the site outputs
  long long tile0;                 // the variant's first partial-sum slot (variant-major)
  long long ops_off;               // int4 entries into the ops array
  long long bmat_off;              // floats into the B array
  long long tip_off;               // floats into the tip-row array
  long long pi_off;                // doubles into the pi array
  long long brlen_off;             // doubles into the branch-length array ([2n-2])
  long long rates_off;             // doubles into the rates array ([R])
  long long ctab_off;              // doubles into the code-table array ([n_codes][S])
  int group, group_idx;            // eigen system: model group_idx of the group of this S
  double probs[4];
  float probsf[4];                 // probs rounded to float (the root's join)
};

// op.x = internal index k, op.y = first child, op.z = second child,
// op.w = slot_a | slot_b << 8 | slot_out << 16 (TMEM stack positions)

__device__ __forceinline__ uint32_t su32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// K-major, no-swizzle shared-memory descriptor: 8-row x 16-byte core
// matrices, K-adjacent ones LBO apart, 8-row groups SBO apart.
__device__ __forceinline__ uint64_t smem_desc(const void *base, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((su32(base) >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// byte offset of element (row n, col k) of a K-major core-matrix tile of
// 32-bit values with Kp columns
__host__ __device__ inline size_t cm_off(int n, int k, int Kp) {
  return (size_t)(n / 8) * (size_t)(Kp / 4) * 128 + (size_t)(k / 4) * 128 + (n % 8) * 16 + (k % 4) * 4;
}

// x rounded to the nearest TF32 value (10-bit mantissa, ties away from
// zero), as bits: the MMA then reads an unbiased operand instead of one
// whose low bits are dropped.  For a finite x >= 0 adding half a TF32 unit
// to the bit pattern and clearing the 13 dropped bits rounds it (a carry
// out of the mantissa raises the exponent), with two integer instructions.
__device__ __forceinline__ uint32_t tf32_bits(float x) {
  return (__float_as_uint(x) + 0x1000u) & 0xffffe000u;
}

// W consecutive TMEM columns of this thread's lane (32x32b shape)
template <int W>
__device__ __forceinline__ void tmem_ld(uint32_t ta, float *v);
template <>
__device__ __forceinline__ void tmem_ld<4>(uint32_t ta, float *v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(ta));
#pragma unroll
  for (int j = 0; j < 4; ++j) v[j] = __uint_as_float(r[j]);
}
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t ta, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(ta));
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}
template <>
__device__ __forceinline__ void tmem_ld<16>(uint32_t ta, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(ta));
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// W consecutive TMEM columns of this thread's lane, each value rounded to
// the nearest TF32 value (32x32b shape)
template <int W>
__device__ __forceinline__ void tmem_st(uint32_t ta, const float *v);
template <>
__device__ __forceinline__ void tmem_st<4>(uint32_t ta, const float *v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(ta), "r"(tf32_bits(v[0])),
               "r"(tf32_bits(v[1])), "r"(tf32_bits(v[2])), "r"(tf32_bits(v[3]))
               : "memory");
}
template <>
__device__ __forceinline__ void tmem_st<8>(uint32_t ta, const float *v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta),
               "r"(tf32_bits(v[0])), "r"(tf32_bits(v[1])), "r"(tf32_bits(v[2])), "r"(tf32_bits(v[3])),
               "r"(tf32_bits(v[4])), "r"(tf32_bits(v[5])), "r"(tf32_bits(v[6])), "r"(tf32_bits(v[7]))
               : "memory");
}
template <>
__device__ __forceinline__ void tmem_st<16>(uint32_t ta, const float *v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          ta),
      "r"(tf32_bits(v[0])), "r"(tf32_bits(v[1])), "r"(tf32_bits(v[2])), "r"(tf32_bits(v[3])), "r"(tf32_bits(v[4])),
      "r"(tf32_bits(v[5])), "r"(tf32_bits(v[6])), "r"(tf32_bits(v[7])), "r"(tf32_bits(v[8])), "r"(tf32_bits(v[9])),
      "r"(tf32_bits(v[10])), "r"(tf32_bits(v[11])), "r"(tf32_bits(v[12])), "r"(tf32_bits(v[13])),
      "r"(tf32_bits(v[14])), "r"(tf32_bits(v[15]))
      : "memory");
}

__device__ __forceinline__ void two_sum_d(double a, double b, double &s, double &e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void warp_csum_d(double &s, double &c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, c, o);
    double t, e;
    two_sum_d(s, s2, t, e);
    s = t;
    c = c + c2 + e;
  }
}

struct BatchArgs {
  const BVar *vars;
  const int2 *work;               // [n_work] (variant, tile)
  long long n_work;
  const int4 *ops;
  const float *bmat;
  const float *tiptab;
  const double *pis;
  const float2 *pis2;             // pis as (hi, lo) float pairs
  const float4 *logtab;           // the float-pair logarithm's table (64 entries)
  double *site_lnl;               // [total patterns] or null
  double2 *partials;              // [n_work]
  int *flag;
  int slot_bytes;                 // ring slot size
};

// ring slot layout: [0,128) codes of child a, [128,256) codes of child b,
// then block a and block b (each the larger of a B block and a tip block)
__device__ __forceinline__ int blk_bytes(const BVar &v) {
  const int b = v.Np * v.Kp * 4, t = v.NCp * v.SpT * 4;
  return ((b > t ? b : t) + 127) & ~127;
}


// What one epilogue step reads.  Shapes that follow from the padded state
// count are template parameters of the step; these are the rest, read from
// the variant once per work item.
struct EpiIn {
  const unsigned char *sl;   // the step's ring slot
  int BB;                    // bytes of one child block in the slot
  int n_tips, n_codes, S;
  uint32_t tmem, lane_base;
  int m;                     // pattern within the tile (TMEM lane)
  int lg;                    // TMEM lane group (its warps of one rate class share a named barrier)
  bool active, last;
  const float2 *pi2;         // the variant's stationary frequencies as float pairs
};

// The share of a row that epilogue warp w owns (PT = w / 4; the warps of a
// TMEM lane group own the BT_PARTS shares).  A rate class of the pass has
// PPR = BT_PARTS / RP shares: share PT is rate class PT / PPR and the
// (PT % PPR)-th range of WD states, WD = Kp / PPR rounded up to a multiple
// of 4, so the last range of a small Kp may be short or empty.  Every range
// starts on a multiple of 4 columns and is a multiple of 4 wide.  With two
// shares per lane group and two rate classes per pass, a warp owns a whole
// rate class's row and needs no exchange with another warp.
template <int KP, int RP, int PT>
struct Share {
  static constexpr int PPR = BT_PARTS / RP;
  static constexpr int WD = ((KP / PPR) + 3) & ~3;
  static constexpr int rate = PT / PPR;
  static constexpr int e0 = (PT % PPR) * WD;
  static constexpr int B = KP - e0 <= 0 ? 0 : (KP - e0 < WD ? KP - e0 : WD);
};

// One postorder step for this warp's share of the row: the product of the
// two children (tip rows from the slot, or the MMA results from TMEM),
// rescaled by a power of two agreed with the other shares of the same rate
// class, written into the node's TMEM stack slot.  KP, RP and the share are
// template parameters so that every state index and TMEM column is a
// compile-time constant and the vectors stay in registers.  TMEM columns: D
// of child h, rate q at (h*RP + q)*NP; stack slot s, rate q at
// 2*RP*NP + (s*RP + q)*KP.
template <int KP, int RP, int PT>
__device__ __forceinline__ void epi_step(const BatchArgs &p, const EpiIn &in, const int4 op, int lane,
                                         int slot, uint64_t *empty, float (*xch)[BT_M], int &escale,
                                         bool &ok, ff &Lp) {
  using SH = Share<KP, RP, PT>;
  constexpr int B = SH::B, e0 = SH::e0, rate = SH::rate;
  constexpr int BA = B > 0 ? B : 1;
  constexpr int NP = (KP + 15) / 16 * 16;
  constexpr int SPT = KP | 1;
  float acc[BA];
#pragma unroll
  for (int e = 0; e < BA; ++e) acc[e] = 1.0f;
  // states S .. KP-1 need no masks: the tip rows and the B blocks are zero
  // there, so every vector's padding is a product of zeros
  if constexpr (B > 0) {
    // TMEM loads of W columns: the widest of 16, 8, 4 that divides both the
    // first column and the width of the share
    constexpr int W = (e0 % 16 == 0 && B % 16 == 0) ? 16 : (e0 % 8 == 0 && B % 8 == 0) ? 8 : 4;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!ok) break;
      const int ch = h == 0 ? op.y : op.z;
      if (ch < in.n_tips) {
        int code = in.sl[h * 128 + in.m];
        if (code >= in.n_codes) {
          if (in.active && PT == 0) atomicOr(p.flag, PGPU_FLAG_BADCODE);
          code = 0;
        }
        const float *row = reinterpret_cast<const float *>(in.sl + 256 + (size_t)(h * RP + rate) * in.BB) +
                           code * SPT + e0;
#pragma unroll
        for (int e = 0; e < B; ++e) acc[e] *= row[e];
      } else {
        float d[B];
#pragma unroll
        for (int c = 0; c < B; c += W)
          tmem_ld<W>(in.tmem + in.lane_base + (uint32_t)((h * RP + rate) * NP + e0 + c), &d[c]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int e = 0; e < B; ++e) acc[e] *= d[e];
      }
    }
  }
  __syncwarp();
  if (lane == 0) mbar_arrive(&empty[slot]);
  // rescale by an exact power of two per rate class; the shares agree
  float mx = 0.0f;
  if constexpr (B > 0) {
    // pairwise maxima: a short dependency chain
    float t[B];
#pragma unroll
    for (int e = 0; e < B; ++e) t[e] = acc[e];
#pragma unroll
    for (int w = 1; w < B; w *= 2)
#pragma unroll
      for (int e = 0; e + w < B; e += 2 * w) t[e] = fmaxf(t[e], t[e + w]);
    mx = t[0];
  }
  constexpr int PPR = SH::PPR;
  float m2 = mx;
  if constexpr (PPR > 1) {
    xch[PT][in.m] = mx;
    // the exchange joins only the warps of this TMEM lane group that share
    // the rate class (named barrier 2 + lg + 4 rate); it also makes the
    // timeout verdict uniform over them, so they leave the step loop
    // together
    uint32_t all_ok;
    asm volatile(
        "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\t"
        "bar.red.and.pred b, %2, %3, a;\n\tselp.u32 %0, 1, 0, b;\n\t}"
        : "=r"(all_ok)
        : "r"((uint32_t)ok), "r"(2 + in.lg + 4 * rate), "n"(PPR * 32)
        : "memory");
    ok = all_ok != 0;
#pragma unroll
    for (int pp = rate * PPR; pp < rate * PPR + PPR; ++pp) m2 = fmaxf(m2, xch[pp][in.m]);
  } else {
    // this warp holds the whole row of its rate class
    ok = __all_sync(0xffffffffu, ok);
  }
  if (m2 < 0x1p-32f && m2 > 0.0f) {
    int ex;
    (void)frexpf(m2, &ex);
    escale += ex;
    const int k1 = min(-ex, 120), k2 = -ex - k1;
    const float f1 = __int_as_float((127 + k1) << 23), f2 = __int_as_float((127 + k2) << 23);
#pragma unroll
    for (int e = 0; e < BA; ++e) acc[e] = acc[e] * f1 * f2;
  }
  if constexpr (B > 0) {
    // into the TMEM stack slot: columns e0 .. e0 + B - 1 of rate class rate
    const int so = (op.w >> 16) & 0xff;
    const uint32_t col = in.tmem + in.lane_base + (uint32_t)(2 * RP * NP + (so * RP + rate) * KP + e0);
    constexpr int WS = (e0 % 16 == 0 && B % 16 == 0) ? 16 : (e0 % 8 == 0 && B % 8 == 0) ? 8 : 4;
#pragma unroll
    for (int c0 = 0; c0 < B; c0 += WS) tmem_st<WS>(col + (uint32_t)c0, &acc[c0]);
    if (in.last) {
      // sum_e pi_e x_e as a float pair: pi as (hi, lo), every product exact
      // with its cross term, the high parts added by an ordered Fast2Sum
      // (the terms are non-negative), all low parts in one float
      float hs = 0.0f, lo = 0.0f;
#pragma unroll
      for (int e = 0; e < B; ++e)
        if (e0 + e < in.S) {
          const float2 pv = in.pi2[e0 + e];
          const float q = __fmul_rn(pv.x, acc[e]);
          float err = __fmaf_rn(pv.x, acc[e], -q);
          err = __fmaf_rn(pv.y, acc[e], err);
          const ff t = fast_two_sum(fmaxf(hs, q), fminf(hs, q));
          hs = t.h;
          lo = __fadd_rn(lo, __fadd_rn(t.l, err));
        }
      Lp = fast_two_sum(hs, lo);
    }
  } else {
    if (in.last) Lp = ff{0.0f, 0.0f};
  }
}

// Shared state of the epilogue warps.
struct EpiShared {
  uint64_t *full, *empty;
  uint64_t *mma_bar;         // [2]: per rate class of the pass (both complete once per step)
  uint64_t *stored;          // [2]: the epilogue warps of the first and second half of the shares
  const int4 *slot_op;       // each ring slot's postorder step, written by the producer
  unsigned char *smem;
  float (*xch)[BT_M];        // [2][BT_PARTS]: per step parity and share, lane: max entry
  ff (*xchd)[BT_M];          // per share, lane: root likelihood (float pair)
  ff (*lnr)[BT_M];           // per rate class, lane: log root likelihood (float pair)
  double2 *red;
  uint32_t tmem;
};

// Every pass and postorder step of one work item (variant, tile) with
// compile-time shapes, for the epilogue warps: each step waits for
// its slot and its MMAs, runs the epilogue, and after its TMEM stores every
// warp arrives on `stored`, which the MMA warp waits for before the next
// step's MMAs.  A pass ends with the epilogue-wide verdict on timeouts, so
// the per-pass barriers below are reached by every warp alike.
template <int KP, int RP>
__device__ __forceinline__ void epi_item(const BatchArgs &p, const EpiShared &sh, const BVar &vg, const int2 wk,
                                         int tid, long long &seq, bool &ok) {
  const int warp = tid >> 5, lane = tid & 31;
  const int lg = warp & 3, pt = warp >> 2;
  const int m = 32 * lg + lane;   // pattern within the tile
  constexpr int PPR = BT_PARTS / RP;
  const int my_rate = pt / PPR;
  // the share that combines its rate class's root likelihood
  const bool lead = pt % PPR == 0;
  // the variant's fields, once per item
  const int n_ops = vg.n_ops, R = vg.R;
  EpiIn in;
  in.BB = blk_bytes(vg);
  in.n_tips = vg.n_tips;
  in.n_codes = vg.n_codes;
  in.S = vg.S;
  in.tmem = sh.tmem;
  in.lane_base = (uint32_t)(32 * lg) << 16;
  in.m = m;
  in.lg = lg;
  const long long pat = (long long)wk.y * BT_M + m;
  in.active = pat < vg.n_pat;
  in.pi2 = p.pis2 + vg.pi_off;
  ff Lp{0.0f, 0.0f};
  for (int r0 = 0; r0 < R && ok; r0 += RP) {
    int escale = 0;
    for (int i = 0; i < n_ops; ++i, ++seq) {
      const int slot = (int)(seq & (BT_ST - 1));
      const uint32_t par = (uint32_t)((seq / BT_ST) & 1);
      in.sl = sh.smem + (size_t)slot * p.slot_bytes;
      bool got = mbar_wait_bounded_for(&sh.full[slot], par, p.flag);
      got = got && mbar_wait_bounded_for(&sh.mma_bar[my_rate], (uint32_t)(seq & 1), p.flag);
      got = __all_sync(0xffffffffu, got);
      if (!got) {
        ok = false;
        atomicOr(p.flag, PGPU_FLAG_TIMEOUT);
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int4 op = sh.slot_op[slot];
      in.last = i == n_ops - 1;
      // the max exchange is double-buffered by step parity: a group's next
      // write cannot meet a read of the previous step's values
      float(*xch)[BT_M] = sh.xch + (seq & 1) * BT_PARTS;
      // pt is warp-uniform
      switch (pt) {
        case 0: epi_step<KP, RP, 0>(p, in, op, lane, slot, sh.empty, xch, escale, ok, Lp); break;
        case 1: epi_step<KP, RP, 1>(p, in, op, lane, slot, sh.empty, xch, escale, ok, Lp); break;
        case 2: epi_step<KP, RP, 2>(p, in, op, lane, slot, sh.empty, xch, escale, ok, Lp); break;
        default: epi_step<KP, RP, 3>(p, in, op, lane, slot, sh.empty, xch, escale, ok, Lp); break;
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      // this warp's vectors of the step are in TMEM and its D columns read
      __syncwarp();
      if (lane == 0) mbar_arrive(&sh.stored[pt / (BT_PARTS / 2)]);
      if (!ok) break;
    }
    // one verdict for every epilogue warp before the barriers below
    {
      uint32_t all_ok;
      asm volatile(
          "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\t"
          "bar.red.and.pred b, 1, %2, a;\n\tselp.u32 %0, 1, 0, b;\n\t}"
          : "=r"(all_ok)
          : "r"((uint32_t)ok), "n"(BT_EPI)
          : "memory");
      ok = all_ok != 0;
    }
    if (!ok) break;
    // roots of this pass's rate classes: the shares of each meet
    sh.xchd[pt][m] = Lp;
    asm volatile("bar.sync 1, %0;" ::"n"(BT_EPI) : "memory");
    if (lead) {
      ff L{0.0f, 0.0f};
#pragma unroll
      for (int pp = my_rate * PPR; pp < my_rate * PPR + PPR; ++pp) L = ff_add(L, sh.xchd[pp][m]);
      // log(L 2^escale) in float pairs (no FP64 instruction: the FP64 pipe
      // of this GPU retires a warp's instruction in tens of cycles)
      sh.lnr[r0 + my_rate][m] = L.h > 0.0f ? ff_log(L, escale, p.logtab) : ff{-INFINITY, 0.0f};
    }
    asm volatile("bar.sync 1, %0;" ::"n"(BT_EPI) : "memory");
  }
  // join the rate classes: log sum_r probs[r] exp(lnr[r]), the largest
  // class's logarithm as a float pair plus the float logarithm of a sum in
  // [probs_min, 1]
  ff s{0.0f, 0.0f};
  if (ok && in.active && pt == 0) {
    ff mx = sh.lnr[0][m];
    for (int r = 1; r < R; ++r)
      if (sh.lnr[r][m].h > mx.h) mx = sh.lnr[r][m];
    ff lnl = mx;
    if (mx.h != -INFINITY) {
      float sum = 0.0f;
      for (int r = 0; r < R; ++r) {
        const ff v = sh.lnr[r][m];
        sum += vg.probsf[r] * expf((v.h - mx.h) + (v.l - mx.l));
      }
      lnl = ff_add(mx, ff{logf(sum), 0.0f});
    }
    if (p.site_lnl) p.site_lnl[vg.pat_off + pat] = (double)lnl.h + (double)lnl.l;
    if (vg.weights) {
      const double w = vg.weights[pat];
      const float wh = (float)w;
      s = ff_mul(lnl, ff{wh, (float)(w - (double)wh)});
    } else {
      s = lnl;
    }
  }
  if (pt == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = ff_add(s, ff_shfl_xor(s, o));
    if (lane == 0) sh.red[lg] = make_double2((double)s.h, (double)s.l);
  }
  asm volatile("bar.sync 1, %0;" ::"n"(BT_EPI) : "memory");
  if (tid == 0) {
    double ss = 0.0, cc = 0.0;
    for (int k = 0; k < 4; ++k) {
      double t, e;
      two_sum_d(ss, sh.red[k].x, t, e);
      ss = t;
      cc += e + sh.red[k].y;
    }
    // by (variant, tile), whatever order the work list runs in
    p.partials[vg.tile0 + wk.y] = make_double2(ss, cc);
  }
  asm volatile("bar.sync 1, %0;" ::"n"(BT_EPI) : "memory");
}

// The MMA warp's side of one work item: per step, once the slot is loaded,
// one thread issues the step's tcgen05.mma for the internal children, rate
// class by rate class.  A class's MMAs wait until its epilogue warps have
// stored the previous step's vectors (and read its D columns), and are
// committed to that class's mma_bar; the last commit also goes to the
// slot's empty barrier.  With one rate class per pass the MMAs wait for
// both halves of the epilogue and are committed to both mma_bar barriers,
// so each barrier completes once per step either way.
template <int KP, int RP>
__device__ __forceinline__ void mma_item(const BatchArgs &p, const EpiShared &sh, const BVar &vg,
                                         long long &seq, bool &ok) {
  constexpr int NP = (KP + 15) / 16 * 16;
  constexpr uint32_t LBO = 128, SBO = (uint32_t)(KP / 4) * 128;
  constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NP >> 3) << 17) |
                             ((uint32_t)(BT_M >> 4) << 24);
  const int n_ops = vg.n_ops, R = vg.R, n_tips = vg.n_tips, BB = blk_bytes(vg);
  auto commit = [&](uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     su32(bar))
                 : "memory");
  };
  for (int r0 = 0; r0 < R && ok; r0 += RP) {
    for (int i = 0; i < n_ops; ++i, ++seq) {
      const int slot = (int)(seq & (BT_ST - 1));
      const uint32_t par = (uint32_t)((seq / BT_ST) & 1);
      if (!mbar_wait_bounded_for(&sh.full[slot], par, p.flag)) {
        ok = false;
        atomicOr(p.flag, PGPU_FLAG_TIMEOUT);
        return;
      }
      const int4 op = sh.slot_op[slot];
      const unsigned char *sl = sh.smem + (size_t)slot * p.slot_bytes;
      const bool any = op.y >= n_tips || op.z >= n_tips;
#pragma unroll
      for (int q = 0; q < RP; ++q) {
        // this class's epilogue warps are done with the previous step (with
        // one class per pass, all of them)
        bool got = true;
        if (seq > 0) {
          const uint32_t prev = (uint32_t)((seq - 1) & 1);
          got = mbar_wait_bounded_for(&sh.stored[q], prev, p.flag);
          if (RP == 1) got = got && mbar_wait_bounded_for(&sh.stored[1], prev, p.flag);
        }
        if (!got) {
          ok = false;
          atomicOr(p.flag, PGPU_FLAG_TIMEOUT);
          return;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int ch = h == 0 ? op.y : op.z;
          if (ch < n_tips) continue;
          const int sa = (op.w >> (8 * h)) & 0xff;
          const uint32_t d_col = (uint32_t)((h * RP + q) * NP);
          const uint32_t a_col = (uint32_t)(2 * RP * NP + (sa * RP + q) * KP);
          const unsigned char *blk = sl + 256 + (size_t)(h * RP + q) * BB;
#pragma unroll
          for (int ks = 0; ks < KP / 8; ++ks) {
            const uint64_t bd = smem_desc(blk + (size_t)ks * 2 * LBO, LBO, SBO);
            const uint32_t accf = ks > 0 ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, q;\n\t}" ::"r"(sh.tmem + d_col),
                "r"(sh.tmem + a_col + (uint32_t)(ks * 8)), "l"(bd), "r"(IDESC), "r"(accf)
                : "memory");
          }
        }
        if (any)
          commit(&sh.mma_bar[q]);
        else
          mbar_arrive(&sh.mma_bar[q]);
      }
      if (any) {
        if (RP == 1) commit(&sh.mma_bar[1]);
        commit(&sh.empty[slot]);
      } else {
        if (RP == 1) mbar_arrive(&sh.mma_bar[1]);
        mbar_arrive(&sh.empty[slot]);
      }
    }
  }
}

template <int KP>
__device__ __forceinline__ void mma_item_rp(const BatchArgs &p, const EpiShared &sh, const BVar &vg,
                                            long long &seq, bool &ok) {
  if constexpr (KP <= 32) {
    if (vg.RP == 2) {
      mma_item<KP, 2>(p, sh, vg, seq, ok);
      return;
    }
  }
  mma_item<KP, 1>(p, sh, vg, seq, ok);
}

template <int KP>
__device__ __forceinline__ void epi_item_rp(const BatchArgs &p, const EpiShared &sh, const BVar &vg,
                                            const int2 wk, int tid, long long &seq, bool &ok) {
  if constexpr (KP <= 32) {
    if (vg.RP == 2) {
      epi_item<KP, 2>(p, sh, vg, wk, tid, seq, ok);
      return;
    }
  }
  epi_item<KP, 1>(p, sh, vg, wk, tid, seq, ok);
}

__global__ void __launch_bounds__(BT_THREADS, 1) batch_tc_kernel(const BatchArgs p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t full[BT_ST], empty[BT_ST], mma_bar[2], stored[2];
  __shared__ int4 slot_op[BT_ST];
  __shared__ uint32_t tmem_base;
  __shared__ float xch[2 * BT_PARTS][BT_M];   // per step parity and share, lane: max entry
  __shared__ ff xchd[BT_PARTS][BT_M];   // per share, lane: root likelihood
  __shared__ ff lnr[4][BT_M];           // per rate class, lane: log root likelihood
  __shared__ double2 red[4];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == BT_EPI_WARPS) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     su32(&tmem_base)),
                 "r"(BT_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < BT_ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1 + BT_EPI_WARPS);   // the MMA commit + the epilogue warps
    }
    for (int q = 0; q < 2; ++q) {
      mbar_init(&mma_bar[q], 1);
      mbar_init(&stored[q], BT_EPI_WARPS / 2);   // half the epilogue warps, after a step's TMEM stores
    }
    fence_mbarrier_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  const EpiShared sh{full, empty, mma_bar, stored, slot_op, smem, xch, xchd, lnr, red, tmem};
  if (warp == BT_PRODUCER) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      long long seq = 0;
      bool ok = true;
      for (long long w = blockIdx.x; w < p.n_work && ok; w += gridDim.x) {
        const int2 wk = __ldg(p.work + w);
        const BVar &v = p.vars[wk.x];
        const int BB = blk_bytes(v);
        const uint32_t bmat_bytes = (uint32_t)(v.Np * v.Kp * 4);
        const uint32_t tip_bytes = (uint32_t)(v.NCp * v.SpT * 4);
        const int RP = v.RP, R = v.R, n_ops = v.n_ops, n_tips = v.n_tips;
        const long long ops_off = v.ops_off, ld = v.ld, tip_off = v.tip_off, bmat_off = v.bmat_off;
        const uint8_t *codes = v.codes;
        const long long bstride = (long long)v.Np * v.Kp, tstride = (long long)v.NCp * v.SpT;
        for (int r0 = 0; r0 < R && ok; r0 += RP) {
          for (int i = 0; i < n_ops; ++i, ++seq) {
            const int slot = (int)(seq & (BT_ST - 1));
            const long long round = seq / BT_ST;
            const int4 op = __ldg(p.ops + ops_off + i);
            if (round > 0 && !mbar_wait_bounded_for(&empty[slot], (uint32_t)((round - 1) & 1), p.flag)) {
              ok = false;
              break;
            }
            unsigned char *sl = smem + (size_t)slot * p.slot_bytes;
            uint32_t tx = 0;
            for (int h = 0; h < 2; ++h) {
              const int ch = h == 0 ? op.y : op.z;
              tx += ch < n_tips ? 128u + RP * tip_bytes : RP * bmat_bytes;
            }
            // the step itself, published by the arrive below (release)
            slot_op[slot] = op;
            mbar_arrive_expect_tx(&full[slot], tx);
            for (int h = 0; h < 2; ++h) {
              const int ch = h == 0 ? op.y : op.z;
              if (ch < n_tips)
                bulk_g2s(sl + h * 128, codes + (long long)ch * ld + (long long)wk.y * 128, 128u, &full[slot]);
              for (int q = 0; q < RP; ++q) {
                unsigned char *blk = sl + 256 + (size_t)(h * RP + q) * BB;
                if (ch < n_tips)
                  bulk_g2s(blk, p.tiptab + tip_off + ((long long)ch * R + r0 + q) * tstride, tip_bytes,
                           &full[slot]);
                else
                  bulk_g2s(blk, p.bmat + bmat_off + ((long long)(ch - n_tips) * R + r0 + q) * bstride,
                           bmat_bytes, &full[slot]);
              }
            }
          }
        }
      }
      for (long long s = seq - BT_ST; s < seq; ++s)
        if (s >= 0) (void)mbar_wait_bounded_for(&full[s & (BT_ST - 1)], (uint32_t)((s / BT_ST) & 1), p.flag);
    }
  } else if (warp == BT_MMA) {
    // ------------------------------------------------------------ MMA issue
    if (lane == 0) {
      long long seq = 0;
      bool ok = true;
      for (long long w = blockIdx.x; w < p.n_work && ok; w += gridDim.x) {
        const int2 wk = __ldg(p.work + w);
        const BVar &v = p.vars[wk.x];
        switch (v.Kp) {
          case 8: mma_item_rp<8>(p, sh, v, seq, ok); break;
          case 16: mma_item_rp<16>(p, sh, v, seq, ok); break;
          case 24: mma_item_rp<24>(p, sh, v, seq, ok); break;
          case 32: mma_item_rp<32>(p, sh, v, seq, ok); break;
          case 40: mma_item_rp<40>(p, sh, v, seq, ok); break;
          case 48: mma_item_rp<48>(p, sh, v, seq, ok); break;
          case 56: mma_item_rp<56>(p, sh, v, seq, ok); break;
          default: mma_item_rp<64>(p, sh, v, seq, ok); break;
        }
      }
      // the last MMAs finish before TMEM is released
      if (seq > 0) (void)mbar_wait_bounded_for(&mma_bar[1], (uint32_t)((seq - 1) & 1), p.flag);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // warp w: TMEM lanes 32 (w % 4) .. 32 (w % 4) + 31, share w / 4 of the
    // row.
    long long seq = 0;
    bool ok = true;
    for (long long w = blockIdx.x; w < p.n_work && ok; w += gridDim.x) {
      const int2 wk = __ldg(p.work + w);
      const BVar &v = p.vars[wk.x];
      switch (v.Kp) {
        case 8: epi_item_rp<8>(p, sh, v, wk, tid, seq, ok); break;
        case 16: epi_item_rp<16>(p, sh, v, wk, tid, seq, ok); break;
        case 24: epi_item_rp<24>(p, sh, v, wk, tid, seq, ok); break;
        case 32: epi_item_rp<32>(p, sh, v, wk, tid, seq, ok); break;
        case 40: epi_item_rp<40>(p, sh, v, wk, tid, seq, ok); break;
        case 48: epi_item_rp<48>(p, sh, v, wk, tid, seq, ok); break;
        case 56: epi_item_rp<56>(p, sh, v, wk, tid, seq, ok); break;
        default: epi_item_rp<64>(p, sh, v, wk, tid, seq, ok); break;
      }
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == BT_EPI_WARPS)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BT_TMEM_COLS));
}

// Per variant: sum its tiles' (sum, compensation) pairs in tile order.
__global__ void __launch_bounds__(256) batch_finalize_kernel(const double2 *partials,
                                                            const long long *tile_base,
                                                            const int *n_tiles, int n_var, double *out) {
  const int v = blockIdx.x;
  if (v >= n_var) return;
  const double sum = pgpu_forms::csum_block<256>(partials + tile_base[v], n_tiles[v]);
  if (threadIdx.x == 0) out[v] = sum;
}

// Setup: for every branch of every variant of one state count S and every
// rate class, P = U diag(exp(lambda r t)) Ui in FP64 (shared memory), then
//   tip branch      tip rows tab[c][i] = sum_j P[i][j] code_tab[c][j]  (float)
//   internal branch B block B[n=i][k=j] = P[i][j] in the core-matrix layout
struct SetupArgs {
  const BVar *vars;
  const int *members;             // variants of this group
  const double *U, *lam, *Ui;     // group eigen systems [g][S][S], [g][S], [g][S][S]
  const int *status;              // [g]
  const double *brlen, *rates, *ctab;
  float *bmat, *tiptab;
  int *flag;
  int S;
};

__global__ void __launch_bounds__(256) batch_setup_kernel(const SetupArgs a) {
  extern __shared__ __align__(16) double P[];   // [S][S] then e[S]
  const int S = a.S, SS = S * S;
  const int vi = a.members[blockIdx.z];
  const BVar &v = a.vars[vi];
  const int c = blockIdx.x, r = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int n_br = 2 * v.n_tips - 2;
  if (c >= n_br || r >= v.R) return;
  const int g = v.group_idx;
  if (a.status[g]) {
    if (c == 0 && r == 0 && tid == 0) atomicOr(a.flag, pgpu_model_flag(a.status[g]));
    return;
  }
  const double *U = a.U + (size_t)g * SS, *Ui = a.Ui + (size_t)g * SS, *lam = a.lam + (size_t)g * S;
  double *e = P + SS;
  const double t = a.brlen[v.brlen_off + c], rate = a.rates[v.rates_off + r];
  const bool ident = !(t * rate >= 1e-10);   // effective time: a rate-0 class gets I exactly
  for (int k = tid; k < S; k += nt) e[k] = exp(lam[k] * rate * t);
  __syncthreads();
  for (int o = tid; o < SS; o += nt) {
    const int i = o / S, j = o % S;
    double x = 0.0;
    if (ident) {
      x = i == j ? 1.0 : 0.0;
    } else {
      for (int k = 0; k < S; ++k) x = fma(U[i * S + k] * e[k], Ui[k * S + j], x);
    }
    P[o] = fmax(x, 0.0);   // transition probabilities: clamp eigen-product noise below 0
  }
  __syncthreads();
  if (c < v.n_tips) {
    float *out = a.tiptab + v.tip_off + ((size_t)c * v.R + r) * v.NCp * v.SpT;
    const double *ct = a.ctab + v.ctab_off;
    for (int o = tid; o < v.NCp * v.SpT; o += nt) {
      const int code = o / v.SpT, i = o % v.SpT;
      double y = 0.0;
      if (i < S && code < v.n_codes)
        for (int j = 0; j < S; ++j) y = fma(P[i * S + j], ct[code * S + j], y);
      out[o] = (float)y;
    }
  } else {
    unsigned char *out = reinterpret_cast<unsigned char *>(
        a.bmat + v.bmat_off + ((size_t)(c - v.n_tips) * v.R + r) * (size_t)v.Np * v.Kp);
    for (int o = tid; o < v.Np * v.Kp; o += nt) {
      const int n = o / v.Kp, k = o % v.Kp;
      const float x = (n < S && k < S) ? (float)P[n * S + k] : 0.0f;   // P >= 0 after clamping
      *reinterpret_cast<uint32_t *>(out + cm_off(n, k, v.Kp)) = tf32_bits(x);
    }
  }
}

// The FP64 comparison form over the first `sample` patterns of every
// variant: one CTA per (variant, block of 32 patterns), thread = pattern,
// all rate classes and states in FP64; the stack of vectors in shared
// memory, each branch's P rebuilt in shared memory from the eigen system.
struct F64Args {
  const BVar *vars;
  const int4 *ops;
  const double *U, *lam, *Ui;     // per group, indexed through vars[].group / group_idx
  long long gU[8], gL[8];         // group bases (doubles) into U/Ui and lam
  const double *brlen, *rates, *ctab, *pis;
  double2 *partials;              // [n_var][blocks]
  int blocks;                     // blocks per variant
  long long sample;
  int max_depth;
};

constexpr int F64_NP = 32;

__global__ void __launch_bounds__(F64_NP) batch_fp64_kernel(const F64Args a) {
  extern __shared__ __align__(16) double sm[];
  const int vi = blockIdx.y, blk = blockIdx.x, tid = threadIdx.x;
  const BVar &v = a.vars[vi];
  const int S = v.S, SS = S * S, R = v.R;
  double *P = sm;                                   // [S][S]
  double *e = P + SS;                               // [S]
  double *stk = e + 64;                             // [depth][S][32]
  const long long n_use = min(a.sample, v.n_pat);
  const long long pat = (long long)blk * F64_NP + tid;
  const bool active = pat < n_use;
  const double *U = a.U + a.gU[v.group] + (size_t)v.group_idx * SS;
  const double *Ui = a.Ui + a.gU[v.group] + (size_t)v.group_idx * SS;
  const double *lam = a.lam + a.gL[v.group] + (size_t)v.group_idx * S;
  const double *ct = a.ctab + v.ctab_off;
  double lnr[4];
  double x[2][64];
  for (int r = 0; r < R; ++r) {
    int sp = 0;
    long long esc = 0;
    for (int i = 0; i < v.n_ops; ++i) {
      const int4 op = a.ops[v.ops_off + i];
      // pop the internal children (b above a)
      for (int h = 1; h >= 0; --h) {
        const int ch = h == 0 ? op.y : op.z;
        if (ch >= v.n_tips) {
          --sp;
          for (int j = 0; j < S; ++j) x[h][j] = stk[((size_t)sp * S + j) * F64_NP + tid];
        }
      }
      double out[64];
      for (int j = 0; j < S; ++j) out[j] = 1.0;
      for (int h = 0; h < 2; ++h) {
        const int ch = h == 0 ? op.y : op.z;
        __syncthreads();
        const double t = a.brlen[v.brlen_off + ch], rate = a.rates[v.rates_off + r];
        const bool ident = !(t * rate >= 1e-10);
        for (int k = tid; k < S; k += F64_NP) e[k] = exp(lam[k] * rate * t);
        __syncthreads();
        for (int o = tid; o < SS; o += F64_NP) {
          const int ii = o / S, jj = o % S;
          double y = 0.0;
          if (ident) y = ii == jj ? 1.0 : 0.0;
          else
            for (int k = 0; k < S; ++k) y = fma(U[ii * S + k] * e[k], Ui[k * S + jj], y);
          P[o] = fmax(y, 0.0);
        }
        __syncthreads();
        if (ch < v.n_tips) {
          int code = active ? v.codes[(long long)ch * v.ld + pat] : 0;
          if (code >= v.n_codes) code = 0;
          for (int j = 0; j < S; ++j) x[h][j] = ct[code * S + j];
        }
        for (int ii = 0; ii < S; ++ii) {
          double y = 0.0;
          for (int jj = 0; jj < S; ++jj) y = fma(P[ii * S + jj], x[h][jj], y);
          out[ii] *= y;
        }
      }
      double mx = 0.0;
      for (int j = 0; j < S; ++j) mx = fmax(mx, out[j]);
      if (mx > 0.0 && mx < 0x1p-256) {
        int ex;
        (void)frexp(mx, &ex);
        esc += ex;
        for (int j = 0; j < S; ++j) out[j] = ldexp(out[j], -ex);
      }
      if (i + 1 < v.n_ops) {
        for (int j = 0; j < S; ++j) stk[((size_t)sp * S + j) * F64_NP + tid] = out[j];
        ++sp;
      } else {
        double L = 0.0;
        for (int j = 0; j < S; ++j) L += a.pis[v.pi_off + j] * out[j];
        lnr[r] = log(L) + (double)esc * 0.69314718055994530942;
      }
    }
  }
  double s = 0.0, c = 0.0;
  if (active) {
    double mxl = -INFINITY;
    for (int r = 0; r < R; ++r) mxl = fmax(mxl, lnr[r]);
    double sum = 0.0;
    for (int r = 0; r < R; ++r) sum += v.probs[r] * exp(lnr[r] - mxl);
    const double lnl = mxl + log(sum);
    s = v.weights ? v.weights[pat] * lnl : lnl;
  }
  warp_csum_d(s, c);
  if (tid == 0) a.partials[(size_t)vi * a.blocks + blk] = make_double2(s, c);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct pgpu_batch {
  int n_var = 0;
  int max_depth = 0;
  long long n_work = 0, total_pat = 0;
  std::vector<BVar> hvars;
  std::vector<int> group_S;                     // state count of each group
  std::vector<std::vector<int>> group_members;  // variant ids per group
  // device
  BVar *vars = nullptr;
  int2 *work = nullptr;
  int4 *ops = nullptr;
  float *bmat = nullptr, *tiptab = nullptr;
  double *pis = nullptr, *brlen = nullptr, *rates = nullptr, *ctab = nullptr;
  float2 *pis2 = nullptr;
  float4 *logtab = nullptr;
  double *Q = nullptr, *U = nullptr, *Ui = nullptr, *lam = nullptr;
  int *status = nullptr, *members = nullptr;
  long long *tile_base = nullptr;
  int *n_tiles = nullptr;
  double2 *partials = nullptr;
  std::vector<long long> gQ, gL, gM;            // group bases (doubles, doubles, ints)
  int slot_bytes = 0;
};

namespace {

template <typename T>
pgpu_status upload(pgpu_ctx *ctx, T **dst, const std::vector<T> &src) {
  const size_t bytes = std::max<size_t>(src.size() * sizeof(T), 16);
  PGPU_CUDA(ctx, cudaMalloc(reinterpret_cast<void **>(dst), bytes));
  if (!src.empty())
    PGPU_CUDA(ctx, cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return PGPU_OK;
}

void free_batch(pgpu_batch *b) {
  void *ptrs[] = {b->vars, b->work,   b->ops, b->bmat,   b->tiptab,  b->pis,      b->brlen,
                  b->rates, b->ctab,  b->Q,   b->U,      b->Ui,      b->lam,      b->status,
                  b->members, b->tile_base, b->n_tiles, b->partials, b->pis2, b->logtab};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete b;
}

}  // namespace

extern "C" {

pgpu_status pgpu_batch_create(pgpu_ctx *ctx, const pgpu_variant *vs, int n_var, pgpu_batch **out) {
  return pgpu_batch_create_opts(ctx, vs, n_var, nullptr, out);
}

pgpu_status pgpu_batch_create_opts(pgpu_ctx *ctx, const pgpu_variant *vs, int n_var,
                                   const pgpu_batch_options *opts, pgpu_batch **out) {
  if (!ctx || !out) return PGPU_ERR_ARG;
  *out = nullptr;
  const int rate_pairs = opts ? opts->rate_pairs : 1;
  const int order = opts ? opts->order : PGPU_BATCH_ORDER_VARIANT;
  if (order != PGPU_BATCH_ORDER_VARIANT && order != PGPU_BATCH_ORDER_COST)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "batch: unknown work order %d", order);
  if (!vs || n_var < 1) return pgpu_set_err(ctx, PGPU_ERR_ARG, "batch: no variants");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  pgpu_batch *b = new pgpu_batch();
  b->n_var = n_var;
  std::vector<int4> ops;
  std::vector<int2> work;
  std::vector<double> pis, brl, rts, ctab, Qg;
  std::vector<long long> tile_base;
  std::vector<int> ntiles, members;
  long long bm_off = 0, tt_off = 0, pat_off = 0;
  size_t max_blk = 0;
  auto fail = [&](pgpu_status st, const char *msg, int v) {
    free_batch(b);
    return pgpu_set_err(ctx, st, "batch: variant %d: %s", v, msg);
  };
  for (int vi = 0; vi < n_var; ++vi) {
    const pgpu_variant &x = vs[vi];
    const pgpu_model &m = x.model;
    if (!x.tree.brlen || !m.Q || !m.pi || !m.rates || !m.probs || !x.codes.table || !x.tip_codes)
      return fail(PGPU_ERR_ARG, "null field", vi);
    if (m.n_states < 2 || m.n_states > 64) return fail(PGPU_ERR_LIMIT, "2..64 states", vi);
    if (m.n_rates < 1 || m.n_rates > 4) return fail(PGPU_ERR_LIMIT, "1..4 rate classes", vi);
    if (x.codes.n_codes < 1 || x.codes.n_codes > 255) return fail(PGPU_ERR_ARG, "1..255 codes", vi);
    if (x.tree.n_tips < 2 || x.tree.n_tips > 255) return fail(PGPU_ERR_LIMIT, "2..255 tips", vi);
    const long long nt = (long long)((x.n_pat + BT_M - 1) / BT_M);
    if (x.ld_pat % 128 != 0 || (long long)x.ld_pat < nt * BT_M || ((uintptr_t)x.tip_codes & 15))
      return fail(PGPU_ERR_ARG, "ld_pat must be a multiple of 128 covering the padded tiles", vi);
    TreeSchedule sch;
    pgpu_status st = pgpu_build_schedule(ctx, &x.tree, &sch);
    if (st != PGPU_OK) {
      free_batch(b);
      return st;
    }
    const int n = x.tree.n_tips, S = m.n_states, R = m.n_rates;
    BVar v{};
    v.n_tips = n;
    v.n_ops = n - 1;
    v.S = S;
    v.R = R;
    v.n_codes = x.codes.n_codes;
    v.Kp = (S + 7) / 8 * 8;
    v.Np = (S + 15) / 16 * 16;
    v.SpT = v.Kp | 1;                     // odd row stride (distinct codes, distinct banks), entries S.. zero
    v.NCp = (x.codes.n_codes + 3) / 4 * 4; // rows padded so a block is a multiple of 16 bytes
    v.n_slots = (BT_TMEM_COLS - 2 * v.Np) / v.Kp;
    v.n_tiles = (int)nt;
    v.n_pat = (long long)x.n_pat;
    v.ld = (long long)x.ld_pat;
    v.codes = x.tip_codes;
    v.weights = x.weights;
    v.pat_off = pat_off;
    v.ops_off = (long long)ops.size();
    v.bmat_off = bm_off;
    v.tip_off = tt_off;
    v.pi_off = (long long)pis.size();
    v.brlen_off = (long long)brl.size();
    v.rates_off = (long long)rts.size();
    v.ctab_off = (long long)ctab.size();
    for (int r = 0; r < 4; ++r) {
      v.probs[r] = r < R ? m.probs[r] : 0.0;
      v.probsf[r] = (float)v.probs[r];
    }
    if (sch.max_depth > v.n_slots) return fail(PGPU_ERR_LIMIT, "tree too deep for the TMEM stack", vi);
    // two rate classes per pass when their D columns and stacks fit in TMEM
    v.RP = 1;
    if (rate_pairs && R % 2 == 0 && v.Kp <= 32 &&
        (BT_TMEM_COLS - 4 * v.Np) / (2 * v.Kp) >= sch.max_depth)
      v.RP = 2;
    b->max_depth = std::max(b->max_depth, sch.max_depth);
    // TMEM stack positions from the stack simulation
    int sp = 0;
    for (const SchedOp &o : sch.ops) {
      int sa = 0, sb = 0;
      if (o.b >= n) sb = --sp;
      if (o.a >= n) sa = --sp;
      const int so = sp++;
      ops.push_back(make_int4(o.k, o.a, o.b, sa | (sb << 8) | (so << 16)));
    }
    v.tile0 = (long long)work.size();
    for (long long t = 0; t < nt; ++t) work.push_back(make_int2(vi, (int)t));
    tile_base.push_back((long long)work.size() - nt);
    ntiles.push_back((int)nt);
    pis.insert(pis.end(), m.pi, m.pi + S);
    brl.insert(brl.end(), x.tree.brlen, x.tree.brlen + 2 * n - 2);
    rts.insert(rts.end(), m.rates, m.rates + R);
    ctab.insert(ctab.end(), x.codes.table, x.codes.table + (size_t)v.n_codes * S);
    bm_off += (long long)(n - 2) * R * v.Np * v.Kp;
    tt_off += (long long)n * R * v.NCp * v.SpT;
    bm_off = (bm_off + 3) / 4 * 4;
    tt_off = (tt_off + 3) / 4 * 4;
    pat_off += v.n_pat;
    const size_t blk = std::max<size_t>((size_t)v.Np * v.Kp * 4, (size_t)v.NCp * v.SpT * 4);
    max_blk = std::max(max_blk, (size_t)v.RP * ((blk + 127) & ~size_t(127)));
    // eigen group by state count
    int g = -1;
    for (size_t k = 0; k < b->group_S.size(); ++k)
      if (b->group_S[k] == S) g = (int)k;
    if (g < 0) {
      g = (int)b->group_S.size();
      b->group_S.push_back(S);
      b->group_members.emplace_back();
    }
    v.group = g;
    v.group_idx = (int)b->group_members[g].size();
    b->group_members[g].push_back(vi);
    b->hvars.push_back(v);
  }
  if (b->group_S.size() > 8) return fail(PGPU_ERR_LIMIT, "at most 8 distinct state counts", 0);
  // group layout of Q / pi / eigen arrays
  std::vector<double> Qall, PIall;
  long long q_acc = 0, l_acc = 0;
  for (size_t g = 0; g < b->group_S.size(); ++g) {
    const int S = b->group_S[g];
    b->gQ.push_back(q_acc);
    b->gL.push_back(l_acc);
    b->gM.push_back((long long)members.size());
    for (int vi : b->group_members[g]) {
      Qall.insert(Qall.end(), vs[vi].model.Q, vs[vi].model.Q + (size_t)S * S);
      PIall.insert(PIall.end(), vs[vi].model.pi, vs[vi].model.pi + S);
      members.push_back(vi);
    }
    q_acc += (long long)b->group_members[g].size() * S * S;
    l_acc += (long long)b->group_members[g].size() * S;
  }
  if (order == PGPU_BATCH_ORDER_COST && !work.empty()) {
    // Largest items first, dealt back and forth over the persistent CTAs
    // (CTA c runs items c, c + G, c + 2G, ...), so every CTA's total is close
    // to the mean.  An item's cost is its postorder steps times the state
    // columns each step handles.
    const long long G = std::min<long long>(ctx->num_sms, (long long)work.size());
    std::vector<double> cost(work.size());
    for (size_t i = 0; i < work.size(); ++i) {
      const BVar &v = b->hvars[work[i].x];
      cost[i] = (double)(v.R / v.RP) * v.n_ops * (v.RP * v.Kp + 16.0);
    }
    std::vector<size_t> idx(work.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t c) { return cost[a] > cost[c]; });
    std::vector<std::vector<int2>> per(G);
    for (size_t r = 0; r < idx.size(); ++r) {
      const long long round = (long long)r / G, pos = (long long)r % G;
      per[round % 2 == 0 ? pos : G - 1 - pos].push_back(work[idx[r]]);
    }
    // CTA c's k-th item goes to position k G + c; the last, partial round
    // is packed to the front of its row
    std::vector<int2> compact;
    compact.reserve(work.size());
    const size_t rounds = (work.size() + G - 1) / G;
    for (size_t k = 0; k < rounds; ++k)
      for (long long c = 0; c < G; ++c)
        if (k < per[c].size()) compact.push_back(per[c][k]);
    work.swap(compact);
  }
  b->n_work = (long long)work.size();
  b->total_pat = pat_off;
  b->slot_bytes = (int)(256 + 2 * max_blk);
  pgpu_status st = PGPU_OK;
  if (st == PGPU_OK) st = upload(ctx, &b->vars, b->hvars);
  if (st == PGPU_OK) st = upload(ctx, &b->work, work);
  if (st == PGPU_OK) st = upload(ctx, &b->ops, ops);
  if (st == PGPU_OK) st = upload(ctx, &b->pis, pis);
  std::vector<float2> pis2(pis.size());
  for (size_t i = 0; i < pis.size(); ++i) {
    const float h = (float)pis[i];
    pis2[i] = make_float2(h, (float)(pis[i] - (double)h));
  }
  std::vector<float4> lt(64);
  ff_log_table(lt.data(), [](double c) { return std::log(c); });
  if (st == PGPU_OK) st = upload(ctx, &b->pis2, pis2);
  if (st == PGPU_OK) st = upload(ctx, &b->logtab, lt);
  if (st == PGPU_OK) st = upload(ctx, &b->brlen, brl);
  if (st == PGPU_OK) st = upload(ctx, &b->rates, rts);
  if (st == PGPU_OK) st = upload(ctx, &b->ctab, ctab);
  if (st == PGPU_OK) st = upload(ctx, &b->Q, Qall);
  if (st == PGPU_OK) st = upload(ctx, &b->tile_base, tile_base);
  if (st == PGPU_OK) st = upload(ctx, &b->n_tiles, ntiles);
  if (st == PGPU_OK) st = upload(ctx, &b->members, members);
  std::vector<double> pig(PIall);
  double *dpig = nullptr;
  if (st == PGPU_OK) st = upload(ctx, &dpig, pig);
  auto alloc = [&](void **p, size_t bytes) -> pgpu_status {
    PGPU_CUDA(ctx, cudaMalloc(p, std::max<size_t>(bytes, 16)));
    return PGPU_OK;
  };
  if (st == PGPU_OK) st = alloc((void **)&b->bmat, (size_t)bm_off * 4);
  if (st == PGPU_OK) st = alloc((void **)&b->tiptab, (size_t)tt_off * 4);
  if (st == PGPU_OK) st = alloc((void **)&b->U, (size_t)q_acc * 8);
  if (st == PGPU_OK) st = alloc((void **)&b->Ui, (size_t)q_acc * 8);
  if (st == PGPU_OK) st = alloc((void **)&b->lam, (size_t)l_acc * 8);
  if (st == PGPU_OK) st = alloc((void **)&b->status, (size_t)n_var * 4);
  if (st == PGPU_OK) st = alloc((void **)&b->partials, (size_t)std::max<long long>(b->n_work, 1) * 16);
  // the eigen systems depend on the models only: solved once here
  if (st == PGPU_OK) {
    for (size_t g = 0; g < b->group_S.size() && st == PGPU_OK; ++g) {
      const int S = b->group_S[g];
      st = pgpu_launch_eig(ctx, b->Q + b->gQ[g], dpig + b->gL[g], S,
                           (int)b->group_members[g].size(), b->U + b->gQ[g], b->lam + b->gL[g],
                           b->Ui + b->gQ[g], b->status + b->gM[g]);
    }
  }
  if (st == PGPU_OK) {
    std::vector<int> hst(n_var, 0);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy(hst.data(), b->status, (size_t)n_var * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) st = pgpu_set_err(ctx, PGPU_ERR_CUDA, "batch: %s", cudaGetErrorString(e));
    for (int k = 0; k < n_var && st == PGPU_OK; ++k)
      if (hst[k]) st = pgpu_set_err(ctx, hst[k], "batch: model %d failed its eigendecomposition (%d)", k, hst[k]);
  }
  if (dpig) cudaFree(dpig);
  if (st != PGPU_OK) {
    free_batch(b);
    return st;
  }
  *out = b;
  return PGPU_OK;
}

void pgpu_batch_destroy(pgpu_batch *b) {
  if (b) free_batch(b);
}

pgpu_status pgpu_batch_run(pgpu_ctx *ctx, pgpu_batch *b, double *lnl_dev, double *site_lnl_dev) {
  if (!ctx || !b || !lnl_dev) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  // B blocks and tip rows for every branch (FP64 P from the eigen systems)
  for (size_t g = 0; g < b->group_S.size(); ++g) {
    const int S = b->group_S[g];
    SetupArgs a;
    a.vars = b->vars;
    a.members = b->members + b->gM[g];
    a.U = b->U + b->gQ[g];
    a.lam = b->lam + b->gL[g];
    a.Ui = b->Ui + b->gQ[g];
    a.status = b->status + b->gM[g];
    a.brlen = b->brlen;
    a.rates = b->rates;
    a.ctab = b->ctab;
    a.bmat = b->bmat;
    a.tiptab = b->tiptab;
    a.flag = ctx->d_flag;
    a.S = S;
    int max_tips = 0, max_R = 0;
    for (int vi : b->group_members[g]) {
      max_tips = std::max(max_tips, b->hvars[vi].n_tips);
      max_R = std::max(max_R, b->hvars[vi].R);
    }
    const size_t smem = sizeof(double) * ((size_t)S * S + S);
    PGPU_CUDA(ctx, cudaFuncSetAttribute(batch_setup_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)std::max<size_t>(smem, 1024)));
    batch_setup_kernel<<<dim3(2 * max_tips - 2, max_R, (unsigned)b->group_members[g].size()), 256, smem,
                         ctx->stream>>>(a);
    PGPU_TRY(pgpu_after_launch(ctx, "batch_setup_kernel"));
  }
  BatchArgs a;
  a.vars = b->vars;
  a.work = b->work;
  a.n_work = b->n_work;
  a.ops = b->ops;
  a.bmat = b->bmat;
  a.tiptab = b->tiptab;
  a.pis = b->pis;
  a.pis2 = b->pis2;
  a.logtab = b->logtab;
  a.site_lnl = site_lnl_dev;
  a.partials = b->partials;
  a.flag = ctx->d_flag;
  a.slot_bytes = b->slot_bytes;
  // at least 120 KB, so that one CTA (which holds all 512 TMEM columns)
  // occupies each SM
  const size_t smem = std::max<size_t>((size_t)BT_ST * b->slot_bytes, 120 * 1024);
  if (smem > ctx->smem_optin)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "batch: %zu bytes of shared memory needed", smem);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(batch_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
  const long long grid = std::min<long long>(ctx->num_sms, b->n_work);
  batch_tc_kernel<<<(unsigned)std::max<long long>(grid, 1), BT_THREADS, smem, ctx->stream>>>(a);
  PGPU_TRY(pgpu_after_launch(ctx, "batch_tc_kernel"));
  batch_finalize_kernel<<<b->n_var, 256, 0, ctx->stream>>>(b->partials, b->tile_base,
                                                                        b->n_tiles, b->n_var, lnl_dev);
  return pgpu_after_launch(ctx, "batch_finalize_kernel");
}

pgpu_status pgpu_batch_run_fp64(pgpu_ctx *ctx, pgpu_batch *b, size_t sample, double *lnl_dev) {
  if (!ctx || !b || !lnl_dev || sample == 0) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  F64Args a;
  a.vars = b->vars;
  a.ops = b->ops;
  a.U = b->U;
  a.Ui = b->Ui;
  a.lam = b->lam;
  for (size_t g = 0; g < 8; ++g) {
    a.gU[g] = g < b->gQ.size() ? b->gQ[g] : 0;
    a.gL[g] = g < b->gL.size() ? b->gL[g] : 0;
  }
  a.brlen = b->brlen;
  a.rates = b->rates;
  a.ctab = b->ctab;
  a.pis = b->pis;
  long long max_pat = 0;
  int max_S = 0;
  for (const BVar &v : b->hvars) {
    max_pat = std::max(max_pat, std::min<long long>(v.n_pat, (long long)sample));
    max_S = std::max(max_S, v.S);
  }
  a.blocks = (int)((max_pat + F64_NP - 1) / F64_NP);
  a.sample = (long long)sample;
  a.max_depth = b->max_depth;
  double2 *dpart = nullptr;
  PGPU_TRY(pgpu_buf(ctx, BUF_D, (size_t)a.blocks * b->n_var * sizeof(double2), (void **)&dpart));
  a.partials = dpart;
  const size_t smem = sizeof(double) * ((size_t)max_S * max_S + 64 + (size_t)b->max_depth * max_S * F64_NP);
  if (smem > ctx->smem_optin) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "batch fp64: tree too deep");
  PGPU_CUDA(ctx, cudaFuncSetAttribute(batch_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
  batch_fp64_kernel<<<dim3(a.blocks, b->n_var), F64_NP, smem, ctx->stream>>>(a);
  PGPU_TRY(pgpu_after_launch(ctx, "batch_fp64_kernel"));
  // per variant: blocks * F64_NP patterns, partials at [v * blocks]
  std::vector<long long> base(b->n_var);
  std::vector<int> cnt(b->n_var, a.blocks);
  for (int v = 0; v < b->n_var; ++v) base[v] = (long long)v * a.blocks;
  long long *dbase = nullptr;
  int *dcnt = nullptr;
  PGPU_TRY(pgpu_buf(ctx, BUF_E, base.size() * 8, (void **)&dbase));
  PGPU_TRY(pgpu_buf(ctx, BUF_F, cnt.size() * 4, (void **)&dcnt));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dbase, base.data(), base.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dcnt, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  batch_finalize_kernel<<<b->n_var, 256, 0, ctx->stream>>>(dpart, dbase, dcnt,
                                                                        b->n_var, lnl_dev);
  return pgpu_after_launch(ctx, "batch_finalize_kernel");
}

long long pgpu_batch_work_items(const pgpu_batch *b) { return b ? b->n_work : 0; }
long long pgpu_batch_patterns(const pgpu_batch *b) { return b ? b->total_pat : 0; }

}  // extern "C"
