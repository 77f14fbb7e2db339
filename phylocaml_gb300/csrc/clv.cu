// Likelihood_c one node at a time: the NodeData.S operator
// (lib/nodeData.ml:20-30) whose slot lib/likelihood_c.ml:14-21 leaves as
// `failwith "TODO"`.
//
//   m  (pgpu_lk)   the substitution model's eigen system (FP64, on the GPU),
//                  its rate classes, the tip-code table and the character
//                  block's pattern count and weights;
//   t  (pgpu_clv)  one node's conditional likelihoods on the device,
//                  [n_pat][R][S] in the storage type (float or double), a
//                  power-of-two exponent per pattern, the length of the
//                  branch above the node and that branch's P matrices.
//
// median_1/2/3 combine one, two or three neighbours: y = prod_k P(t_k) x_k
// per pattern and rate class.  Every result is normalised so that each
// pattern's largest entry lies in [1/2, 1): stored = true * 2^-E with an
// exact power of two e_p applied at the node and E summed over the subtree.
// The node's cost is what its own normalisation moved out of the
// likelihood, -ln 2 sum_p w_p e_p, and root_cost is
// -sum_p w_p log(sum_r probs_r sum_i pi_i stored).  The costs of all
// internal nodes plus the root's root_cost are then -lnL, which is how
// Node.Make1D sums node costs (lib/node.ml:191).
//
// One thread per (pattern, rate class): RL = the power of two >= R lanes
// per pattern, so a pattern's maximum is a shuffle over its lanes.  Loads
// of a child's vector are contiguous per thread and contiguous across the
// warp, so the kernel streams at HBM speed; P blocks are read through the
// read-only cache.  Each CTA writes a compensated partial of its cost, and
// the last CTA to finish adds the partials in CTA order, so costs are
// deterministic.
//
// Handles are allocated stream-ordered (cudaMallocAsync) on the context's
// stream; passing the node's previous value (the reference's `t option`)
// reuses its memory instead.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pgpu_internal.cuh"
#include "forms.cuh"
#include "pmatrix.cuh"

using namespace pgpu_forms;

struct pgpu_lk {
  pgpu_ctx *ctx = nullptr;
  int S = 0, R = 0, RL = 1, n_codes = 0, precision = 64;
  size_t n_pat = 0;
  double *block = nullptr;   // U, Ui, lam, pi, rates, probs, code table, weights
  double *U = nullptr, *Ui = nullptr, *lam = nullptr, *pi = nullptr, *rates = nullptr,
         *probs = nullptr, *tab = nullptr, *weights = nullptr;
  int *status = nullptr;     // eigendecomposition status
  double2 *part = nullptr;   // per-CTA partial sums
  // integer weights (pattern counts): the node costs are summed exactly as
  // sum_p w_p e_p in int64 on the integer units, the FP64 units being slow
  bool int_w = false;
  int32_t *wint = nullptr;   // [n_pat] or null (all 1)
  long long *ipart = nullptr;   // per-CTA integer partial sums
  unsigned *counter = nullptr;
  size_t n_cta = 0;
  long long live = 0;        // handles not yet destroyed
};

struct pgpu_clv {
  pgpu_lk *lk = nullptr;
  char *mem = nullptr;       // one stream-ordered allocation
  void *x = nullptr;         // [n_pat][R][S]
  int32_t *ex = nullptr;     // [n_pat]
  void *P = nullptr;         // [R][S][S] of the branch above
  double *scal = nullptr;    // [0] cost, [1] branch length, [2] root cost
  double brlen = 0.0;
  bool has_P = false;
  bool leaf = false;
};

namespace {

constexpr int CLV_THREADS = 256;

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

size_t vbytes(const pgpu_lk *lk) { return lk->precision == 32 ? 4 : 8; }

template <typename V> __device__ __forceinline__ V scale2(V v, int e);
template <> __device__ __forceinline__ float scale2<float>(float v, int e) {
  // v * 2^e, exact; e beyond a float exponent's range (a denormal maximum)
  // takes two steps
  if (e > 126) {
    v *= pow2f(126);
    e -= 126;
  } else if (e < -126) {
    v *= pow2f(-126);
    e += 126;
  }
  return v * pow2f(e);
}
template <> __device__ __forceinline__ double scale2<double>(double v, int e) { return ldexp(v, e); }

// Compensated sum of (s, c) over the CTA into part[blockIdx.x]; the last
// CTA adds all partials in order into *out (times `sign`) and resets the
// counter.
template <int NT>
__device__ __forceinline__ void cta_partial_and_finish(double s, double c, double2 *part,
                                                       unsigned *counter, double *out,
                                                       double sign) {
  __shared__ double2 red[NT / 32];
  __shared__ bool last;
  warp_csum(s, c);
  const int t = threadIdx.x, lane = t & 31;
  if (lane == 0) red[t >> 5] = make_double2(s, c);
  __syncthreads();
  if (t < 32) {
    double2 v = lane < NT / 32 ? red[lane] : make_double2(0.0, 0.0);
    double ss = v.x, cc = v.y;
    warp_csum(ss, cc);
    if (lane == 0) {
      part[blockIdx.x] = make_double2(ss, cc);
      __threadfence();
      last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const double tot = csum_block<NT>(part, gridDim.x);
  if (t == 0) {
    *out = sign * tot;
    *counter = 0u;
  }
}

// The same for an exact integer sum v: the last CTA adds the per-CTA
// partials in int64 and writes scale * total.
template <int NT>
__device__ __forceinline__ void cta_i64_and_finish(long long v, long long *part, unsigned *counter,
                                                   double *out, double scale) {
  __shared__ long long red[NT / 32];
  __shared__ bool last;
  const int t = threadIdx.x, lane = t & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    long long x = lane < NT / 32 ? red[lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) {
      part[blockIdx.x] = x;
      __threadfence();
      last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  long long sum = 0;
  for (unsigned i = t; i < gridDim.x; i += NT) sum += __ldcg(part + i);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  __syncthreads();
  if (lane == 0) red[t >> 5] = sum;
  __syncthreads();
  if (t == 0) {
    long long tot = 0;
    for (int k = 0; k < NT / 32; ++k) tot += red[k];
    *out = scale * (double)tot;
    *counter = 0u;
  }
}

// Leaf vectors: x[p][r][i] = code_tab[code_p][i] for every rate class.
template <typename V>
__global__ void __launch_bounds__(CLV_THREADS) clv_leaf_kernel(const uint8_t *codes,
                                                               const double *tab, int n_codes,
                                                               size_t n_pat, int S, int R,
                                                               V *x, int32_t *ex, int *flag) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t row = (size_t)R * S;
  if (g >= n_pat * row) return;
  const size_t p = g / row;
  const int i = (int)(g % row) % S;
  int c = codes[p];
  if (c >= n_codes) {
    atomicOr(flag, PGPU_FLAG_BADCODE);
    c = 0;
  }
  x[g] = (V)tab[c * S + i];
  if (g % row == 0) ex[p] = 0;
}

struct MedArgs {
  const void *x[3];
  const int32_t *ex[3];
  const void *P[3];
  void *y;
  int32_t *ey;
  const double *weights;
  double2 *part;
  unsigned *counter;
  double *cost;
  size_t n_pat;
  int n_ch, S, R, RL;
  int int_w;                 // integer weights: exact int64 cost sums
  const int32_t *wint;
  long long *ipart;
};

// 16-byte vector access to one (pattern, rate class) row of 4 states
template <typename V> struct Row4;
template <> struct Row4<float> {
  __device__ __forceinline__ static void load(const float *p, float *v) {
    const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
  }
  __device__ __forceinline__ static void store(float *p, const float *v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <> struct Row4<double> {
  __device__ __forceinline__ static void load(const double *p, double *v) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
  __device__ __forceinline__ static void store(double *p, const double *v) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
  }
};

// y = prod_k P_k x_k, normalised per pattern.  SC: the state count at
// compile time (4), or 0 for any S up to 64 read at run time.  A grid of a
// few CTAs per SM strides over the (pattern, rate class) items, a warp at a
// time (the stride is a multiple of 32, so a pattern's RL lanes stay in one
// warp and one iteration); each thread keeps one compensated cost sum and
// the CTA reduces it once at the end.
template <typename V, int SC>
__global__ void __launch_bounds__(CLV_THREADS) clv_median_kernel(const MedArgs a) {
  const int S = SC ? SC : a.S, R = a.R, RL = a.RL;
  const int lane = threadIdx.x & 31;
  const size_t n_items = a.n_pat * (size_t)RL;
  const size_t stride = (size_t)gridDim.x * CLV_THREADS;
  V *y = static_cast<V *>(a.y);
  double s = 0.0, c = 0.0;
  long long iacc = 0;
  for (size_t base = (size_t)blockIdx.x * CLV_THREADS + (threadIdx.x & ~31); base < n_items;
       base += stride) {
    const size_t g = base + lane;
    const size_t p = g / RL;
    const int r = (int)(g % RL);
    const bool act = g < n_items && r < R;
    const size_t off = (p * R + r) * (size_t)S;
    // the pattern's first lane reads the children's exponents and its
    // weight up front, so their latency overlaps the rows' (loaded after the
    // vector stores below, they would wait on a second round trip)
    const bool lead = act && r == 0;
    int ex_sum = 0;
    long long wi = 0;
    double wd = 0.0;
    if (lead) {
      for (int k = 0; k < a.n_ch; ++k) ex_sum += __ldg(a.ex[k] + p);
      if (a.int_w) wi = a.wint ? (long long)__ldg(a.wint + p) : 1;
      else wd = a.weights ? __ldg(a.weights + p) : 1.0;
    }
    V m = (V)0;
    int e;
    if (SC == 4) {
      V acc[4] = {(V)1, (V)1, (V)1, (V)1};
      if (act) {
        for (int k = 0; k < a.n_ch; ++k) {
          V xv[4], Pr[16];
          Row4<V>::load(static_cast<const V *>(a.x[k]) + off, xv);
          const V *P = static_cast<const V *>(a.P[k]) + (size_t)r * 16;
#pragma unroll
          for (int i = 0; i < 4; ++i) Row4<V>::load(P + 4 * i, Pr + 4 * i);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            V t = (V)0;
#pragma unroll
            for (int j = 0; j < 4; ++j) t = fma(Pr[4 * i + j], xv[j], t);
            acc[i] *= t;
          }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) m = acc[i] > m ? acc[i] : m;
      }
      V mm = m;
      for (int o = 1; o < RL; o <<= 1) {
        const V q = __shfl_xor_sync(0xffffffffu, mm, o);
        mm = q > mm ? q : mm;
      }
      e = frexp_exp(mm);
      if (act) {
        V out[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) out[i] = scale2<V>(acc[i], -e);
        Row4<V>::store(y + off, out);
      }
    } else {
      if (act) {
        for (int i = 0; i < S; ++i) {
          V v = (V)1;
          for (int k = 0; k < a.n_ch; ++k) {
            const V *xs = static_cast<const V *>(a.x[k]) + off;
            const V *P = static_cast<const V *>(a.P[k]) + ((size_t)r * S + i) * S;
            V t = (V)0;
            for (int j = 0; j < S; ++j) t = fma(__ldg(P + j), xs[j], t);
            v *= t;
          }
          y[off + i] = v;
          m = v > m ? v : m;
        }
      }
      V mm = m;
      for (int o = 1; o < RL; o <<= 1) {
        const V q = __shfl_xor_sync(0xffffffffu, mm, o);
        mm = q > mm ? q : mm;
      }
      e = frexp_exp(mm);
      if (act)
        for (int i = 0; i < S; ++i) y[off + i] = scale2<V>(y[off + i], -e);
    }
    // exponent bookkeeping and this node's cost, by the pattern's first lane
    if (lead) {
      a.ey[p] = e + ex_sum;
      if (a.int_w) {
        iacc += wi * e;
      } else {
        double t, err;
        two_sum(s, wd * (double)e, t, err);
        s = t;
        c += err;
      }
    }
  }
  // cost = -ln 2 * sum_p w_p e_p
  if (a.int_w)
    cta_i64_and_finish<CLV_THREADS>(iacc, a.ipart, a.counter, a.cost, -0.69314718055994530942);
  else
    cta_partial_and_finish<CLV_THREADS>(s, c, a.part, a.counter, a.cost, -0.69314718055994530942);
}

// root_cost: -sum_p w_p log(sum_r probs_r sum_i pi_i x[p][r][i]); the
// node costs carry every normalisation, so the root's own exponent E is
// left out (costs + root_cost = -lnL).  Grid-stride as the median kernel.
template <typename V>
__global__ void __launch_bounds__(CLV_THREADS) clv_root_kernel(
    const V *x, const int32_t *ex, const double *pi, const double *probs, const double *weights,
    size_t n_pat, int S, int R, int RL, double *site_lnl, double2 *part, unsigned *counter,
    double *out) {
  const int lane = threadIdx.x & 31;
  const size_t n_items = n_pat * (size_t)RL;
  const size_t stride = (size_t)gridDim.x * CLV_THREADS;
  double s = 0.0, c = 0.0;
  for (size_t base = (size_t)blockIdx.x * CLV_THREADS + (threadIdx.x & ~31); base < n_items;
       base += stride) {
    const size_t g = base + lane;
    const size_t p = g / RL;
    const int r = (int)(g % RL);
    const bool act = g < n_items && r < R;
    double v = 0.0;
    if (act) {
      const V *xs = x + (p * R + r) * (size_t)S;
      for (int i = 0; i < S; ++i) v = fma(pi[i], (double)xs[i], v);
      v *= probs[r];
    }
    for (int o = 1; o < RL; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (act && r == 0) {
      const double site = log(v);
      if (site_lnl) site_lnl[p] = site + (double)ex[p] * 0.69314718055994530942;
      double t, err;
      two_sum(s, weights ? weights[p] * site : site, t, err);
      s = t;
      c += err;
    }
  }
  cta_partial_and_finish<CLV_THREADS>(s, c, part, counter, out, -1.0);
}

// costs of many nodes: out[i] = *src[i]
__global__ void __launch_bounds__(256) clv_gather_kernel(const double *const *src, size_t n,
                                                        double *out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = *src[i];
}

pgpu_status lk_err(pgpu_lk *lk, pgpu_status st, const char *msg) {
  return pgpu_set_err(lk->ctx, st, "%s", msg);
}

// allocation of a handle for lk (or reuse of `reuse`'s memory)
pgpu_status clv_alloc(pgpu_lk *lk, pgpu_clv *reuse, pgpu_clv **out) {
  pgpu_ctx *ctx = lk->ctx;
  if (reuse) {
    if (reuse->lk != lk)
      return lk_err(lk, PGPU_ERR_ARG, "likelihood: the reused node belongs to another model");
    *out = reuse;
    reuse->has_P = false;
    reuse->leaf = false;
    reuse->brlen = 0.0;
    return PGPU_OK;
  }
  const size_t vb = vbytes(lk);
  const size_t xb = al256(lk->n_pat * lk->R * lk->S * vb), eb = al256(lk->n_pat * 4),
               pb = al256((size_t)lk->R * lk->S * lk->S * vb), sb = 256;
  pgpu_clv *t = new (std::nothrow) pgpu_clv();
  if (!t) return lk_err(lk, PGPU_ERR_OOM, "likelihood: host allocation failed");
  void *mem = nullptr;
  cudaError_t e = cudaMallocAsync(&mem, xb + eb + pb + sb, ctx->stream);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    delete t;
    return pgpu_set_err(ctx, e == cudaErrorMemoryAllocation ? PGPU_ERR_OOM : PGPU_ERR_CUDA,
                        "likelihood: node allocation of %zu bytes failed: %s", xb + eb + pb + sb,
                        cudaGetErrorString(e));
  }
  t->lk = lk;
  t->mem = static_cast<char *>(mem);
  t->x = t->mem;
  t->ex = reinterpret_cast<int32_t *>(t->mem + xb);
  t->P = t->mem + xb + eb;
  t->scal = reinterpret_cast<double *>(t->mem + xb + eb + pb);
  lk->live++;
  *out = t;
  return PGPU_OK;
}

pgpu_status check_cta(pgpu_lk *lk) {
  // grid of every per-pattern kernel: n_pat * RL threads
  const size_t n_cta = std::max<size_t>((lk->n_pat * lk->RL + CLV_THREADS - 1) / CLV_THREADS, 1);
  if (n_cta > 0x7fffffffu) return lk_err(lk, PGPU_ERR_LIMIT, "likelihood: too many patterns");
  return PGPU_OK;
}

pgpu_status median(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *const *ch, int n_ch,
                   pgpu_clv **out) {
  if (!lk || !out) return PGPU_ERR_ARG;
  pgpu_ctx *ctx = lk->ctx;
  for (int k = 0; k < n_ch; ++k) {
    if (!ch[k]) return lk_err(lk, PGPU_ERR_ARG, "likelihood: null neighbour");
    if (ch[k]->lk != lk) return lk_err(lk, PGPU_ERR_ARG, "likelihood: neighbour of another model");
    if (!ch[k]->has_P)
      return lk_err(lk, PGPU_ERR_ARG,
                    "likelihood: a neighbour has no branch length (pgpu_clv_set_brlen)");
    if (ch[k] == reuse)
      return lk_err(lk, PGPU_ERR_ARG, "likelihood: the reused node is also a neighbour");
  }
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  pgpu_clv *t = nullptr;
  PGPU_TRY(clv_alloc(lk, reuse, &t));
  MedArgs a{};
  for (int k = 0; k < n_ch; ++k) {
    a.x[k] = ch[k]->x;
    a.ex[k] = ch[k]->ex;
    a.P[k] = ch[k]->P;
  }
  a.y = t->x;
  a.ey = t->ex;
  a.weights = lk->weights;
  a.int_w = lk->int_w ? 1 : 0;
  a.wint = lk->wint;
  a.ipart = lk->ipart;
  a.part = lk->part;
  a.counter = lk->counter;
  a.cost = t->scal;
  a.n_pat = lk->n_pat;
  a.n_ch = n_ch;
  a.S = lk->S;
  a.R = lk->R;
  a.RL = lk->RL;
  const unsigned grid = (unsigned)lk->n_cta;
  if (lk->precision == 32) {
    if (lk->S == 4) clv_median_kernel<float, 4><<<grid, CLV_THREADS, 0, ctx->stream>>>(a);
    else clv_median_kernel<float, 0><<<grid, CLV_THREADS, 0, ctx->stream>>>(a);
  } else {
    if (lk->S == 4) clv_median_kernel<double, 4><<<grid, CLV_THREADS, 0, ctx->stream>>>(a);
    else clv_median_kernel<double, 0><<<grid, CLV_THREADS, 0, ctx->stream>>>(a);
  }
  PGPU_TRY(pgpu_after_launch(ctx, "clv_median_kernel"));
  *out = t;
  return PGPU_OK;
}

}  // namespace

extern "C" {

pgpu_status pgpu_lk_create(pgpu_ctx *ctx, const pgpu_model *m, const pgpu_tip_codes *codes,
                           size_t n_pat, const double *weights, int precision, pgpu_lk **out) {
  if (!ctx || !out) return PGPU_ERR_ARG;
  *out = nullptr;
  if (!m || !m->Q || !m->pi || !m->rates || !m->probs)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "likelihood: null model field");
  if (m->n_states < 2 || m->n_states > 64)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "likelihood: 2..64 states are supported");
  if (m->n_rates < 1 || m->n_rates > 8)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "likelihood: 1..8 rate classes are supported");
  if (!codes || !codes->table || codes->n_codes < 1 || codes->n_codes > 256)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "likelihood: tip code table must have 1..256 rows");
  if (precision != 32 && precision != 64)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "likelihood: precision must be 32 or 64");
  if (n_pat == 0) return pgpu_set_err(ctx, PGPU_ERR_ARG, "likelihood: no patterns");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  pgpu_lk *lk = new (std::nothrow) pgpu_lk();
  if (!lk) return pgpu_set_err(ctx, PGPU_ERR_OOM, "likelihood: host allocation failed");
  lk->ctx = ctx;
  lk->S = m->n_states;
  lk->R = m->n_rates;
  lk->RL = lk->R <= 1 ? 1 : lk->R <= 2 ? 2 : lk->R <= 4 ? 4 : 8;
  lk->n_codes = codes->n_codes;
  lk->precision = precision;
  lk->n_pat = n_pat;
  if (check_cta(lk) != PGPU_OK) {
    delete lk;
    return PGPU_ERR_LIMIT;
  }
  // the per-pattern kernels stride over the patterns with a few CTAs per SM
  const size_t want = (n_pat * lk->RL + CLV_THREADS - 1) / CLV_THREADS;
  lk->n_cta = std::max<size_t>(std::min<size_t>(want, (size_t)std::max(ctx->num_sms, 1) * 8), 1);
  const int S = lk->S, R = lk->R;
  const size_t SS = (size_t)S * S;
  // one block, every part on a 256-byte boundary (the partials are double2
  // and must be 16-byte aligned whatever the pattern count)
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += al256(bytes);
    return o;
  };
  const size_t oU = take(SS * 8), oUi = take(SS * 8), olam = take(S * 8), opi = take(S * 8),
               orates = take(R * 8), oprobs = take(R * 8),
               otab = take((size_t)codes->n_codes * S * 8), ow = take(n_pat * 8), oq = take(SS * 8),
               ost = take(64), opart = take(lk->n_cta * sizeof(double2)),
               owi = take(n_pat * 4), oipart = take(lk->n_cta * sizeof(long long));
  const size_t bytes = off;
  void *blk = nullptr;
  cudaError_t e = cudaMalloc(&blk, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    delete lk;
    return pgpu_set_err(ctx, PGPU_ERR_OOM, "likelihood: model allocation failed");
  }
  char *base = static_cast<char *>(blk);
  lk->block = reinterpret_cast<double *>(base);
  lk->U = reinterpret_cast<double *>(base + oU);
  lk->Ui = reinterpret_cast<double *>(base + oUi);
  lk->lam = reinterpret_cast<double *>(base + olam);
  lk->pi = reinterpret_cast<double *>(base + opi);
  lk->rates = reinterpret_cast<double *>(base + orates);
  lk->probs = reinterpret_cast<double *>(base + oprobs);
  lk->tab = reinterpret_cast<double *>(base + otab);
  double *w = reinterpret_cast<double *>(base + ow);
  double *q = reinterpret_cast<double *>(base + oq);
  lk->weights = weights ? w : nullptr;
  lk->status = reinterpret_cast<int *>(base + ost);
  lk->counter = reinterpret_cast<unsigned *>(lk->status + 4);
  lk->part = reinterpret_cast<double2 *>(base + opart);
  lk->ipart = reinterpret_cast<long long *>(base + oipart);
  // integer weights, small enough that sum_p w_p e_p fits int64 (|e_p| <= 1074)
  std::vector<int32_t> wi;
  lk->int_w = true;
  if (weights) {
    wi.resize(n_pat);
    double wmax = 0.0;
    for (size_t i = 0; i < n_pat && lk->int_w; ++i) {
      const double v = weights[i];
      if (!(v >= 0.0) || v >= 2147483647.0 || v != std::floor(v)) lk->int_w = false;
      else wi[i] = (int32_t)v, wmax = std::max(wmax, v);
    }
    if (lk->int_w && (double)n_pat * std::max(wmax, 1.0) * 1100.0 >= 4.0e18) lk->int_w = false;
  }
  lk->wint = lk->int_w && weights ? reinterpret_cast<int32_t *>(base + owi) : nullptr;
  cudaStream_t s = ctx->stream;
  auto fail = [&](pgpu_status st) {
    cudaFree(blk);
    delete lk;
    return st;
  };
#define LK_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      (void)cudaGetLastError();                                                         \
      return fail(pgpu_set_err(ctx, PGPU_ERR_CUDA, "%s failed: %s", #call,              \
                               cudaGetErrorString(e_)));                                \
    }                                                                                   \
  } while (0)
  LK_CUDA(cudaMemcpyAsync(q, m->Q, SS * 8, cudaMemcpyHostToDevice, s));
  LK_CUDA(cudaMemcpyAsync(lk->pi, m->pi, S * 8, cudaMemcpyHostToDevice, s));
  LK_CUDA(cudaMemcpyAsync(lk->rates, m->rates, R * 8, cudaMemcpyHostToDevice, s));
  LK_CUDA(cudaMemcpyAsync(lk->probs, m->probs, R * 8, cudaMemcpyHostToDevice, s));
  LK_CUDA(cudaMemcpyAsync(lk->tab, codes->table, (size_t)codes->n_codes * S * 8,
                          cudaMemcpyHostToDevice, s));
  if (weights) LK_CUDA(cudaMemcpyAsync(w, weights, n_pat * 8, cudaMemcpyHostToDevice, s));
  if (lk->wint) LK_CUDA(cudaMemcpyAsync(lk->wint, wi.data(), n_pat * 4, cudaMemcpyHostToDevice, s));
  LK_CUDA(cudaMemsetAsync(lk->status, 0, 64, s));
  pgpu_status st = pgpu_launch_eig(ctx, q, lk->pi, S, 1, lk->U, lk->lam, lk->Ui, lk->status);
  if (st != PGPU_OK) return fail(st);
  int *hst = reinterpret_cast<int *>(ctx->h_pinned);
  LK_CUDA(cudaMemcpyAsync(hst, lk->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  LK_CUDA(cudaStreamSynchronize(s));
#undef LK_CUDA
  if (*hst) {
    const int code = *hst;
    return fail(pgpu_set_err(ctx, code,
                             code == PGPU_ERR_NAN ? "likelihood: NaN or Inf in Q or pi"
                             : code == PGPU_ERR_NONREVERSIBLE
                                 ? "likelihood: Q is not reversible with respect to pi"
                                 : "likelihood: eigendecomposition did not converge"));
  }
  *out = lk;
  return PGPU_OK;
}

void pgpu_lk_destroy(pgpu_lk *lk) {
  if (!lk) return;
  cudaSetDevice(lk->ctx->device);
  cudaStreamSynchronize(lk->ctx->stream);
  cudaFree(lk->block);
  delete lk;
}

pgpu_status pgpu_clv_leaf(pgpu_lk *lk, pgpu_clv *reuse, const uint8_t *codes, pgpu_clv **out) {
  if (!lk || !codes || !out) return lk ? lk_err(lk, PGPU_ERR_ARG, "likelihood: null argument")
                                       : PGPU_ERR_ARG;
  pgpu_ctx *ctx = lk->ctx;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  pgpu_clv *t = nullptr;
  PGPU_TRY(clv_alloc(lk, reuse, &t));
  // the codes are copied into the context's tip buffer; later calls on the
  // stream are ordered after this leaf's kernel
  void *dc;
  PGPU_TRY(pgpu_buf(ctx, BUF_TIPS, std::max<size_t>(lk->n_pat, 16), &dc));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dc, codes, lk->n_pat, cudaMemcpyHostToDevice, ctx->stream));
  const size_t n = lk->n_pat * lk->R * lk->S;
  const unsigned grid = (unsigned)((n + CLV_THREADS - 1) / CLV_THREADS);
  if (lk->precision == 32)
    clv_leaf_kernel<float><<<grid, CLV_THREADS, 0, ctx->stream>>>(
        (const uint8_t *)dc, lk->tab, lk->n_codes, lk->n_pat, lk->S, lk->R, (float *)t->x, t->ex,
        ctx->d_flag);
  else
    clv_leaf_kernel<double><<<grid, CLV_THREADS, 0, ctx->stream>>>(
        (const uint8_t *)dc, lk->tab, lk->n_codes, lk->n_pat, lk->S, lk->R, (double *)t->x, t->ex,
        ctx->d_flag);
  PGPU_TRY(pgpu_after_launch(ctx, "clv_leaf_kernel"));
  PGPU_CUDA(ctx, cudaMemsetAsync(t->scal, 0, sizeof(double), ctx->stream));
  t->leaf = true;
  *out = t;
  return PGPU_OK;
}

pgpu_status pgpu_clv_set_brlen(pgpu_clv *t, double brlen) {
  if (!t) return PGPU_ERR_ARG;
  pgpu_lk *lk = t->lk;
  pgpu_ctx *ctx = lk->ctx;
  if (!(brlen >= 0.0) || !std::isfinite(brlen))
    return lk_err(lk, PGPU_ERR_ARG, "likelihood: branch length must be finite and >= 0");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  void *h, *d;
  PGPU_TRY(pgpu_stage(ctx, sizeof(double), &h, &d));
  *static_cast<double *>(h) = brlen;
  PGPU_TRY(pgpu_stage_commit(ctx, sizeof(double)));
  PGPU_CUDA(ctx, cudaMemcpyAsync(t->scal + 1, d, sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  PGPU_TRY(pgpu_launch_compose(ctx, lk->U, lk->lam, lk->Ui, lk->S, t->scal + 1, 1, lk->rates, lk->R,
                               lk->precision == 64 ? (double *)t->P : nullptr,
                               lk->precision == 64 ? nullptr : (float *)t->P, false, lk->status,
                               P32_PLAIN));
  t->brlen = brlen;
  t->has_P = true;
  return PGPU_OK;
}

pgpu_status pgpu_clv_get_brlen(const pgpu_clv *t, double *brlen) {
  if (!t || !brlen) return PGPU_ERR_ARG;
  *brlen = t->brlen;
  return PGPU_OK;
}

pgpu_status pgpu_clv_median1(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *a, pgpu_clv **out) {
  const pgpu_clv *ch[1] = {a};
  return median(lk, reuse, ch, 1, out);
}

pgpu_status pgpu_clv_median2(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *a, const pgpu_clv *b,
                             pgpu_clv **out) {
  const pgpu_clv *ch[2] = {a, b};
  return median(lk, reuse, ch, 2, out);
}

pgpu_status pgpu_clv_median3(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *a, const pgpu_clv *b,
                             const pgpu_clv *c, pgpu_clv **out) {
  const pgpu_clv *ch[3] = {a, b, c};
  return median(lk, reuse, ch, 3, out);
}

pgpu_status pgpu_clv_cost(pgpu_clv *t, double *cost) {
  if (!t || !cost) return PGPU_ERR_ARG;
  pgpu_ctx *ctx = t->lk->ctx;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  double *h = reinterpret_cast<double *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(h, t->scal, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  PGPU_TRY(pgpu_check_flag(ctx, "likelihood"));
  *cost = *h;
  return PGPU_OK;
}

pgpu_status pgpu_clv_costs(pgpu_lk *lk, const pgpu_clv *const *nodes, size_t n, double *costs) {
  if (!lk || (n && (!nodes || !costs))) return PGPU_ERR_ARG;
  if (n == 0) return PGPU_OK;
  pgpu_ctx *ctx = lk->ctx;
  for (size_t i = 0; i < n; ++i)
    if (!nodes[i] || nodes[i]->lk != lk)
      return lk_err(lk, PGPU_ERR_ARG, "likelihood: a node is null or belongs to another model");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  void *h, *d, *dout;
  PGPU_TRY(pgpu_stage(ctx, n * sizeof(double *), &h, &d));
  const double **src = static_cast<const double **>(h);
  for (size_t i = 0; i < n; ++i) src[i] = nodes[i]->scal;
  PGPU_TRY(pgpu_stage_commit(ctx, n * sizeof(double *)));
  PGPU_TRY(pgpu_buf(ctx, BUF_F, n * sizeof(double), &dout));
  const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 1024);
  clv_gather_kernel<<<grid, 256, 0, ctx->stream>>>(static_cast<const double *const *>(d), n,
                                                   static_cast<double *>(dout));
  PGPU_TRY(pgpu_after_launch(ctx, "clv_gather_kernel"));
  PGPU_CUDA(ctx, cudaMemcpyAsync(costs, dout, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return pgpu_check_flag(ctx, "likelihood");
}

pgpu_status pgpu_clv_root_cost(pgpu_clv *t, double *cost, double *site_lnl) {
  if (!t || !cost) return PGPU_ERR_ARG;
  pgpu_lk *lk = t->lk;
  pgpu_ctx *ctx = lk->ctx;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  void *dsl = nullptr;
  if (site_lnl) PGPU_TRY(pgpu_buf(ctx, BUF_SITECOST, lk->n_pat * 8, &dsl));
  const unsigned grid = (unsigned)lk->n_cta;
  if (lk->precision == 32)
    clv_root_kernel<float><<<grid, CLV_THREADS, 0, ctx->stream>>>(
        (const float *)t->x, t->ex, lk->pi, lk->probs, lk->weights, lk->n_pat, lk->S, lk->R,
        lk->RL, (double *)dsl, lk->part, lk->counter, t->scal + 2);
  else
    clv_root_kernel<double><<<grid, CLV_THREADS, 0, ctx->stream>>>(
        (const double *)t->x, t->ex, lk->pi, lk->probs, lk->weights, lk->n_pat, lk->S, lk->R,
        lk->RL, (double *)dsl, lk->part, lk->counter, t->scal + 2);
  PGPU_TRY(pgpu_after_launch(ctx, "clv_root_kernel"));
  double *h = reinterpret_cast<double *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(h, t->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (site_lnl)
    PGPU_CUDA(ctx, cudaMemcpyAsync(site_lnl, dsl, lk->n_pat * 8, cudaMemcpyDeviceToHost, ctx->stream));
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  PGPU_TRY(pgpu_check_flag(ctx, "likelihood"));
  *cost = *h;
  return PGPU_OK;
}

void pgpu_clv_destroy(pgpu_clv *t) {
  if (!t) return;
  pgpu_ctx *ctx = t->lk->ctx;
  cudaSetDevice(ctx->device);
  cudaFreeAsync(t->mem, ctx->stream);
  t->lk->live--;
  delete t;
}

}  // extern "C"
