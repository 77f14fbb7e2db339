// Arithmetic forms of the conditional-likelihood kernels (pruning, SPR).
//
// Each form is a policy struct: the value type V of a likelihood entry, the
// coefficient type Coef of the transition-matrix blocks it reads, and the
// operations the kernels need (products, exact power-of-two rescaling,
// matrix-vector rows).  The P blocks are built in FP64 on the GPU
// (pmatrix.cu) and rounded once into the form's coefficient type.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pgpu_forms {

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// compensated sum of (s, c) pairs over the 32 lanes of a warp
__device__ __forceinline__ void warp_csum(double &s, double &c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, c, o);
    double t, e;
    two_sum(s, s2, t, e);
    s = t;
    c = c + c2 + e;
  }
}

// Compensated sum of n (sum, compensation) pairs by one CTA of NT threads
// (a multiple of 32, at most 1024): thread t adds a contiguous chunk in
// order, then the chunks are combined by a fixed butterfly, so the result
// does not depend on scheduling.  Every thread returns the total.
template <int NT>
__device__ __forceinline__ double csum_block(const double2 *p, long long n) {
  __shared__ double2 red[NT / 32];
  const int t = threadIdx.x;
  const long long per = (n + NT - 1) / NT, lo = (long long)t * per;
  const long long hi = lo + per < n ? lo + per : n;
  double s = 0.0, c = 0.0;
  for (long long i = lo; i < hi; ++i) {
    const double2 v = p[i];
    double u, e;
    two_sum(s, v.x, u, e);
    s = u;
    c += e + v.y;
  }
  warp_csum(s, c);
  if ((t & 31) == 0) red[t >> 5] = make_double2(s, c);
  __syncthreads();
  const int lane = t & 31;
  double2 v = lane < NT / 32 ? red[lane] : make_double2(0.0, 0.0);
  double ss = v.x, cc = v.y;
  warp_csum(ss, cc);
  __syncthreads();
  return ss + cc;
}


// ---- the three arithmetic forms -------------------------------------------
// Fp32  values float;  P buffer holds fl32(P - I);  y_i = x_i + sum_j D_ij x_j
// Fp64  values double; P buffer holds P;            y_i = sum_j P_ij x_j
// Ff32  values are unevaluated float pairs (hi + lo, about 48 significant
//       bits); P buffer holds (hi, lo) pairs of P; every sum and product is
//       an error-free float transformation, so the only roundings are of the
//       order of 2^-48.  Sites that share subtree patterns share their
//       rounding errors, which then add up linearly over the patterns; the
//       pair form keeps that sum far below 1e-3 where plain FP32 cannot.

struct ff {
  float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}

// 2^k as a float for 0 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// frexp's exponent E of a finite v >= 0 (v = f 2^E, f in [0.5, 1); 0 for
// v = 0, as frexp gives), read from the bits so the float forms issue no
// FP64 instruction
__device__ __forceinline__ int frexp_exp(float v) {
  const int b = __float_as_int(v) & 0x7fffffff;
  const int e = b >> 23;
  return e ? e - 126 : b ? -126 - __clz(b << 9) : 0;
}
__device__ __forceinline__ int frexp_exp(double v) {
  int e;
  (void)frexp(v, &e);
  return e;
}


__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ ff ff_from_d(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ ff ff_shfl_xor(ff v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}

// ln 2 split so that k * LN2_HI is exact for |k| < 2^12
constexpr float LN2_HI = 0.693145751953125f;
constexpr float LN2_LO = 1.42860682030941723212e-6f;

// an integer |E| < 2^22 as a float, through the bits of 2^23 + 2^22 + E
// instead of a conversion instruction
__device__ __forceinline__ float small_int_to_float(int E) {
  return __int_as_float(0x4B400000 + E) - 12582912.0f;
}

// E * ln 2 as a float pair (exact high part for |E| < 4096)
__device__ __forceinline__ ff ff_exp2_log(int E) {
  if (E > -4096 && E < 4096) {
    const float e = small_int_to_float(E);
    return fast_two_sum(e * LN2_HI, e * LN2_LO);
  }
  return ff_from_d((double)E * 0.69314718055994530942);
}

// The table ff_log reads: tab[k] = {log c hi, log c lo, 1/c hi, 1/c lo},
// c = 1 + (2k + 1) / 128, formed in FP64 (host code; std::log).
template <class Log>
inline void ff_log_table(float4 *tab, Log log_fn) {
  for (int k = 0; k < 64; ++k) {
    const double c = 1.0 + (2.0 * k + 1.0) / 128.0, l = log_fn(c), inv = 1.0 / c;
    const float lh = (float)l, ih = (float)inv;
    tab[k] = make_float4(lh, (float)(l - (double)lh), ih, (float)(inv - (double)ih));
  }
}

// Natural logarithm of x = h + l (x > 0, h normal) times 2^e2, as a float
// pair.  Table-driven reduction (Tang's method): m = h 2^-ex in [1, 2),
// c = 1 + (2k + 1) / 128 the centre of m's 1/64-wide cell, r = (m - c) / c
// with |r| < 2^-7, and log m = log c + log1p(r), the series carried to r^7.
// tab[k] = {log c hi, log c lo, 1/c hi, 1/c lo}, built in FP64 on the host.
// Absolute error about 1e-12 plus the rounding of x itself.
__device__ __forceinline__ ff ff_log(ff x, int e2, const float4 *tab) {
  if (x.h < 0x1p-120f) {
    x.h *= 0x1p64f;
    x.l *= 0x1p64f;
    e2 -= 64;
  }
  const int bits = __float_as_int(x.h);
  const int ex = ((bits >> 23) & 0xff) - 127;
  const float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);
  // x.l 2^-ex by two exact power-of-two factors (each exponent within
  // [-64, 64]), so no library scaling routine is called
  const int k1 = -ex / 2, k2 = -ex - k1;
  const float ml = x.l * __int_as_float((127 + k1) << 23) * __int_as_float((127 + k2) << 23);
  const int k = (bits >> 17) & 63;
  const float4 t = tab[k];
  // c = 1 + (2k + 1) / 128, written into the mantissa bits directly
  const float c = __int_as_float(0x3f800000 | ((2 * k + 1) << 16));
  const ff d = two_sum(__fsub_rn(m, c), ml);          // m - c is exact
  const ff r = ff_mul(d, ff{t.z, t.w});
  const ff r2 = ff_mul(r, r);
  const float rh = r.h;
  const float tail =
      rh * rh * rh *
      (0.333333333333f - rh * (0.25f - rh * (0.2f - rh * (0.166666666667f - rh * 0.142857142857f))));
  ff acc = ff_add(ff{t.x, t.y}, r);
  acc = ff_add(acc, ff{-0.5f * r2.h, -0.5f * r2.l});
  acc = ff_add(acc, ff{tail, 0.0f});
  return ff_add(ff_exp2_log(ex + e2), acc);
}

struct Fp32 {
  using V = float;
  using Coef = float;
  static constexpr float thresh = 0x1p-32f;
  __device__ static V from_d(double x) { return (float)x; }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V shfl_xor(V v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
  __device__ static bool positive(V v) { return v > 0.0f; }
  __device__ static void store4(void *tab, size_t at, const V *y) {
    reinterpret_cast<float4 *>(tab)[at] = make_float4(y[0], y[1], y[2], y[3]);
  }
  // ln(v 2^e2): logf of the mantissa (about 1 ulp) plus the exponent term
  __device__ static ff site_log(V v, int e2, const float4 *) {
    if (v < 0x1p-120f) {
      v *= 0x1p64f;
      e2 -= 64;
    }
    const int bits = __float_as_int(v);
    const int ex = ((bits >> 23) & 0xff) - 127;
    const float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);
    return ff_add(ff_exp2_log(ex + e2), ff{logf(m), 0.0f});
  }
  __device__ static V zero() { return 0.0f; }
  __device__ static float mag(V v) { return v; }
  __device__ static double to_d(V v) { return (double)v; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static void mul4(const V *a, const V *b, V *y) {
#pragma unroll
    for (int e = 0; e < 4; ++e) y[e] = a[e] * b[e];
  }
  __device__ static V scale(V v, int k) { return v * pow2f(k); }
  __device__ static void load_tip(const void *tab, size_t at, V *y) {
    const float4 v = reinterpret_cast<const float4 *>(tab)[at];
    y[0] = v.x;
    y[1] = v.y;
    y[2] = v.z;
    y[3] = v.w;
  }
  // y[i] = x[i] + sum_j D[i][j] x[j]
  __device__ static void rows(const Coef *D, const V *x, V *y) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 d = reinterpret_cast<const float4 *>(D)[i];
      float s = d.x * x[0];
      s = fmaf(d.y, x[1], s);
      s = fmaf(d.z, x[2], s);
      s = fmaf(d.w, x[3], s);
      y[i] = x[i] + s;
    }
  }
};

struct Fp64 {
  using V = double;
  using Coef = double;
  static constexpr double thresh = 0x1p-256;
  __device__ static V from_d(double x) { return x; }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V shfl_xor(V v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
  __device__ static bool positive(V v) { return v > 0.0; }
  __device__ static void store4(void *tab, size_t at, const V *y) {
    reinterpret_cast<double2 *>(tab)[2 * at] = make_double2(y[0], y[1]);
    reinterpret_cast<double2 *>(tab)[2 * at + 1] = make_double2(y[2], y[3]);
  }
  __device__ static ff site_log(V v, int e2, const float4 *) {
    return ff_from_d(log(v) + (double)e2 * 0.69314718055994530942);
  }
  __device__ static V zero() { return 0.0; }
  __device__ static double mag(V v) { return v; }
  __device__ static double to_d(V v) { return v; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static void mul4(const V *a, const V *b, V *y) {
#pragma unroll
    for (int e = 0; e < 4; ++e) y[e] = a[e] * b[e];
  }
  __device__ static V scale(V v, int k) { return v * __longlong_as_double((long long)(1023 + k) << 52); }
  __device__ static void load_tip(const void *tab, size_t at, V *y) {
    const double2 a = reinterpret_cast<const double2 *>(tab)[2 * at];
    const double2 b = reinterpret_cast<const double2 *>(tab)[2 * at + 1];
    y[0] = a.x;
    y[1] = a.y;
    y[2] = b.x;
    y[3] = b.y;
  }
  __device__ static void rows(const Coef *P, const V *x, V *y) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const double2 a = reinterpret_cast<const double2 *>(P)[2 * i];
      const double2 b = reinterpret_cast<const double2 *>(P)[2 * i + 1];
      double s = a.x * x[0];
      s = fma(a.y, x[1], s);
      s = fma(b.x, x[2], s);
      s = fma(b.y, x[3], s);
      y[i] = s;
    }
  }
};

struct Ff32 {
  using V = ff;
  using Coef = float2;
  static constexpr float thresh = 0x1p-32f;
  __device__ static V from_d(double x) { return ff_from_d(x); }
  __device__ static V add(V a, V b) { return ff_add(a, b); }
  __device__ static V shfl_xor(V v, int o) { return ff_shfl_xor(v, o); }
  __device__ static bool positive(V v) { return v.h > 0.0f; }
  // four pairs stored element pairs first: {h0, h1, l0, l1}, {h2, h3, l2, l3},
  // so that a 16-byte load gives packed float2 operands
  __device__ static void store4(void *tab, size_t at, const V *y) {
    reinterpret_cast<float4 *>(tab)[2 * at] = make_float4(y[0].h, y[1].h, y[0].l, y[1].l);
    reinterpret_cast<float4 *>(tab)[2 * at + 1] = make_float4(y[2].h, y[3].h, y[2].l, y[3].l);
  }
  __device__ static ff site_log(V v, int e2, const float4 *tab) { return ff_log(v, e2, tab); }
  __device__ static V zero() { return {0.0f, 0.0f}; }
  __device__ static float mag(V v) { return v.h; }
  __device__ static double to_d(V v) { return (double)v.h + (double)v.l; }
  // exact product left unnormalised: the low word stays within a few ulps
  // of the high word, which every consumer of the pair tolerates
  __device__ static V mul(V a, V b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return {p, e};
  }
  __device__ static V scale(V v, int k) {
    const float f = pow2f(k);
    return {v.h * f, v.l * f};
  }
  __device__ static void load_tip(const void *tab, size_t at, V *y) {
    const float4 a = reinterpret_cast<const float4 *>(tab)[2 * at];
    const float4 b = reinterpret_cast<const float4 *>(tab)[2 * at + 1];
    y[0] = {a.x, a.z};
    y[1] = {a.y, a.w};
    y[2] = {b.x, b.z};
    y[3] = {b.y, b.w};
  }
  // y[e] = a[e] b[e] for four elements, two per packed float2 instruction:
  // each product exact and left unnormalised, as mul
  __device__ static void mul4(const V *a, const V *b, V *y) {
    const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const float2 ah = make_float2(a[2 * k].h, a[2 * k + 1].h), al = make_float2(a[2 * k].l, a[2 * k + 1].l);
      const float2 bh = make_float2(b[2 * k].h, b[2 * k + 1].h), bl = make_float2(b[2 * k].l, b[2 * k + 1].l);
      const float2 p = __fmul2_rn(ah, bh);
      float2 e = __ffma2_rn(ah, bh, __fmul2_rn(p, m1));
      e = __ffma2_rn(ah, bl, e);
      e = __ffma2_rn(al, bh, e);
      y[2 * k] = {p.x, e.x};
      y[2 * k + 1] = {p.y, e.y};
    }
  }
  // y_i = sum_j P_ij x_j with P as (hi, lo) pairs: every product exact
  // (TwoProduct), the hi products summed exactly (ordered Fast2Sum), the small cross
  // terms (P_hi x_lo, P_lo x_hi) and all rounding errors gathered in one
  // float.  The pair keeps about 48 bits and is left unnormalised.  Rows go
  // two at a time through packed float2 arithmetic (FFMA2, FADD2, FMUL2:
  // two rows per instruction, each lane rounded as the scalar instruction
  // would be), reading P in the P32_PAIRS_ROWS4 layout: float4 4 (i / 2) + j
  // = {hi P[i][j], hi P[i+1][j], lo P[i][j], lo P[i+1][j]}.
  __device__ static void rows(const Coef *P, const V *x, V *y) {
    const float4 *Q = reinterpret_cast<const float4 *>(P);
    const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
    for (int ip = 0; ip < 2; ++ip) {
      float2 sh = make_float2(0.0f, 0.0f), lo = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float4 q = Q[ip * 4 + j];
        const float2 ph = make_float2(q.x, q.y), pl = make_float2(q.z, q.w);
        const float2 xh = make_float2(x[j].h, x[j].h), xl = make_float2(x[j].l, x[j].l);
        const float2 p = __fmul2_rn(ph, xh);
        float2 e = __ffma2_rn(ph, xh, __fmul2_rn(p, m1));   // ph xh - p, exact
        e = __ffma2_rn(ph, xl, e);
        e = __ffma2_rn(pl, xh, e);
        if (j == 0) {
          sh = p;
          lo = e;
        } else {
          // Fast2Sum of the larger and the smaller term (all terms are
          // non-negative): the ordering on the ALU pipe, the three adds
          // packed on the FMA pipe
          const float2 a = make_float2(fmaxf(sh.x, p.x), fmaxf(sh.y, p.y));
          const float2 b = make_float2(fminf(sh.x, p.x), fminf(sh.y, p.y));
          const float2 s = __fadd2_rn(a, b);
          const float2 err = __ffma2_rn(__ffma2_rn(a, m1, s), m1, b);   // b - (s - a)
          sh = s;
          lo = __fadd2_rn(lo, __fadd2_rn(err, e));
        }
      }
      y[2 * ip] = {sh.x, lo.x};
      y[2 * ip + 1] = {sh.y, lo.y};
    }
  }
};

}  // namespace pgpu_forms
