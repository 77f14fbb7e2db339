// FP64 transition matrices on the GPU: eigendecomposition of a reversible
// rate matrix and P(t) = U exp(D t) U^-1.
//
// Reference: MlModel.diagonalize (lib/mlModel.ml:554-583) calls LAPACK
// dsyev/dgeev + dgetrf/dgetri through lib/mlmodel.c:163-262, and
// MlModel.compose (lib/mlModel.ml:585-587) builds P with two dgemm calls
// (compose_gtr, lib/mlmodel.c:325-342): P = exp(Q t) read row-major,
// P[i][j] = Pr(j | i, t); t == -1 returns Q itself and t < 1e-10 the
// identity (EPSILON, lib/mlmodel.h:17).
//
// Here a reversible Q (pi_i Q_ij = pi_j Q_ji) is symmetrised,
// B = Pi^1/2 Q Pi^-1/2, and B = V diag(lambda) V^T is found with the cyclic
// two-sided Jacobi method in round-robin order (all n/2 disjoint rotations of
// a step applied at once), one CTA per matrix, everything in FP64 shared
// memory.  Then U = Pi^-1/2 V and U^-1 = V^T Pi^1/2, so Q = U diag(lambda) U^-1
// and P(t) = U diag(exp(lambda t)) U^-1.  Jacobi needs no LAPACK and gives
// orthogonal V to working precision.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pgpu_internal.cuh"
#include "pmatrix.cuh"

namespace {

constexpr int MAXS = 64;
constexpr int LDA = MAXS + 1;   // padded rows against bank conflicts

// pi == null selects the symmetric mode of diagonalize_sym
// (lib/mlmodel.c:163-197): B is Q's lower triangle mirrored (the upper
// triangle dsyev('U') reads in column-major order), U receives the
// eigenvectors as rows (the row-major view of dsyev's column-major V), in
// ascending order of their eigenvalues as dsyev returns them, and Ui is not
// written.
struct EigArgs {
  const double *Q;    // [n_models][S][S]
  const double *pi;   // [n_models][S], or null: symmetric mode
  double *U;          // [n_models][S][S]
  double *lam;        // [n_models][S]
  double *Ui;         // [n_models][S][S] (unused in the symmetric mode)
  int *status;        // [n_models]: 0 ok, PGPU_ERR_* otherwise
  int S;
  int max_sweeps;
};

__global__ void __launch_bounds__(256) jacobi_eig_kernel(const EigArgs p) {
  extern __shared__ __align__(16) double sm[];
  const int S = p.S, N = S + (S & 1);
  double *A = sm;                     // [N][LDA]
  double *V = A + (size_t)N * LDA;    // [N][LDA]
  double *cs = V + (size_t)N * LDA;   // [N/2][2]
  int *pr = reinterpret_cast<int *>(cs + N);  // [N/2][2]
  int *order = pr + N;                        // [N]
  __shared__ double red[8];
  __shared__ int bad;
  const int m = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const double *Q = p.Q + (size_t)m * S * S;
  const bool sym = p.pi == nullptr;
  const double *pi = sym ? nullptr : p.pi + (size_t)m * S;
  if (tid == 0) bad = 0;
  __syncthreads();

  // B = Pi^1/2 Q Pi^-1/2, checked for NaN/Inf and for reversibility; in the
  // symmetric mode B is Q's lower triangle, mirrored
  for (int e = tid; e < N * N; e += nt) {
    const int i = e / N, j = e % N;
    double v = 0.0, vt = 0.0;
    if (sym) {
      if (i < S && j < S) {
        v = vt = Q[(i > j ? i : j) * S + (i > j ? j : i)];
        if (!isfinite(v)) atomicOr(&bad, 1);
      }
    } else if (i < S && j < S) {
      const double qi = Q[i * S + j], qt = Q[j * S + i];
      const double pi_i = pi[i], pi_j = pi[j];
      if (!isfinite(qi) || !isfinite(pi_i) || !(pi_i > 0.0)) atomicOr(&bad, 1);
      v = sqrt(pi_i) * qi / sqrt(pi_j);
      vt = sqrt(pi_j) * qt / sqrt(pi_i);
      if (fabs(v - vt) > 1e-10 * (fabs(v) + fabs(vt)) + 1e-300 && fabs(v - vt) > 1e-12)
        atomicOr(&bad, 2);
    }
    A[i * LDA + j] = 0.5 * (v + vt);
    V[i * LDA + j] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  if (bad) {
    if (tid == 0) p.status[m] = (bad & 1) ? PGPU_ERR_NAN : PGPU_ERR_NONREVERSIBLE;
    return;
  }
  if (tid < N) order[tid] = tid;
  __syncthreads();

  int sweep = 0;
  bool converged = false;
  for (; sweep < p.max_sweeps; ++sweep) {
    // off-diagonal and total squared norms
    double off = 0.0, fro = 0.0;
    for (int e = tid; e < N * N; e += nt) {
      const int i = e / N, j = e % N;
      const double a = A[i * LDA + j];
      fro += a * a;
      if (i != j) off += a * a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      fro += __shfl_xor_sync(0xffffffffu, fro, o);
    }
    if ((tid & 31) == 0) red[tid >> 5] = off;
    __syncthreads();
    double off_t = 0.0;
    for (int w = 0; w < (nt >> 5); ++w) off_t += red[w];
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = fro;
    __syncthreads();
    double fro_t = 0.0;
    for (int w = 0; w < (nt >> 5); ++w) fro_t += red[w];
    __syncthreads();
    if (off_t <= 1e-34 * fro_t) {
      converged = true;
      break;
    }
    for (int step = 0; step < N - 1; ++step) {
      // rotation parameters of the N/2 disjoint pairs of this step
      if (tid < N / 2) {
        int a = order[tid], b = order[N - 1 - tid];
        if (a > b) {
          const int t = a;
          a = b;
          b = t;
        }
        const double apq = A[a * LDA + b];
        double c = 1.0, s = 0.0;
        if (fabs(apq) > 1e-300) {
          const double th = (A[b * LDA + b] - A[a * LDA + a]) / (2.0 * apq);
          double t;
          if (th == 0.0) t = 1.0;
          else if (fabs(th) > 1e150) t = 0.5 / th;
          else t = copysign(1.0, th) / (fabs(th) + sqrt(th * th + 1.0));
          c = 1.0 / sqrt(t * t + 1.0);
          s = t * c;
        }
        pr[2 * tid] = a;
        pr[2 * tid + 1] = b;
        cs[2 * tid] = c;
        cs[2 * tid + 1] = s;
      }
      __syncthreads();
      // rows p, q of every pair
      for (int e = tid; e < (N / 2) * N; e += nt) {
        const int k = e / N, j = e % N;
        const int a = pr[2 * k], b = pr[2 * k + 1];
        const double c = cs[2 * k], s = cs[2 * k + 1];
        const double xa = A[a * LDA + j], xb = A[b * LDA + j];
        A[a * LDA + j] = c * xa - s * xb;
        A[b * LDA + j] = s * xa + c * xb;
      }
      __syncthreads();
      // columns p, q of every pair, and of V
      for (int e = tid; e < (N / 2) * N; e += nt) {
        const int k = e / N, i = e % N;
        const int a = pr[2 * k], b = pr[2 * k + 1];
        const double c = cs[2 * k], s = cs[2 * k + 1];
        const double xa = A[i * LDA + a], xb = A[i * LDA + b];
        A[i * LDA + a] = c * xa - s * xb;
        A[i * LDA + b] = s * xa + c * xb;
        const double va = V[i * LDA + a], vb = V[i * LDA + b];
        V[i * LDA + a] = c * va - s * vb;
        V[i * LDA + b] = s * va + c * vb;
      }
      __syncthreads();
      if (tid < N / 2) {
        const int a = pr[2 * tid], b = pr[2 * tid + 1];
        A[a * LDA + b] = 0.0;
        A[b * LDA + a] = 0.0;
      }
      // next round-robin arrangement: position 0 fixed, the rest rotate
      if (tid == 0) {
        const int last = order[N - 1];
        for (int i = N - 1; i > 1; --i) order[i] = order[i - 1];
        order[1] = last;
      }
      __syncthreads();
    }
  }
  if (sym) {
    // eigenpairs in ascending order (ties by index): order[k] is the
    // column of V with the k-th smallest eigenvalue
    __syncthreads();
    for (int i = tid; i < S; i += nt) {
      const double li = A[i * LDA + i];
      int rank = 0;
      for (int j = 0; j < S; ++j) {
        const double lj = A[j * LDA + j];
        rank += (lj < li) || (lj == li && j < i);
      }
      order[rank] = i;
    }
    __syncthreads();
    for (int e = tid; e < S * S; e += nt) {
      const int k = e / S, i = e % S;
      p.U[(size_t)m * S * S + e] = V[i * LDA + order[k]];
    }
    for (int k = tid; k < S; k += nt) p.lam[(size_t)m * S + k] = A[order[k] * LDA + order[k]];
    if (tid == 0) p.status[m] = converged ? 0 : PGPU_ERR_EIGEN;
    return;
  }
  // outputs: lambda, U = Pi^-1/2 V, Ui = V^T Pi^1/2
  for (int e = tid; e < S * S; e += nt) {
    const int i = e / S, j = e % S;
    p.U[(size_t)m * S * S + e] = V[i * LDA + j] / sqrt(pi[i]);
    p.Ui[(size_t)m * S * S + e] = V[j * LDA + i] * sqrt(pi[j]);
  }
  for (int i = tid; i < S; i += nt) p.lam[(size_t)m * S + i] = A[i * LDA + i];
  if (tid == 0) p.status[m] = converged ? 0 : PGPU_ERR_EIGEN;
}

// Stationary distribution of one rate matrix: pi Q = 0 with sum(pi) = 1,
// i.e. Q^T pi = 0 with its last equation replaced by the sum, solved by
// Gaussian elimination with partial pivoting in FP64 shared memory, one CTA.
// The reference's diagonalize_gtr (lib/mlmodel.c:208-262) takes Q alone;
// the Jacobi solver above needs pi to symmetrise Q, so it is recovered here.
// status: 0, PGPU_ERR_NAN (a NaN or Inf in Q), or PGPU_ERR_NONREVERSIBLE (no
// stationary vector with every entry above 1e-15 of the total: a singular
// system or a reducible Q).
__global__ void __launch_bounds__(256) stationary_kernel(const double *Q, int S, double *pi,
                                                         int *status) {
  extern __shared__ __align__(16) double sm[];
  const int L = S + 1;   // S coefficients and the right-hand side per row
  double *M = sm;        // [S][L]
  __shared__ int piv, bad;
  __shared__ double pval;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int e = tid; e < S * S; e += nt) {
    const int i = e / S, j = e % S;
    const double q = Q[j * S + i];   // row i of Q^T
    if (!isfinite(q)) atomicOr(&bad, 1);
    M[i * L + j] = (i == S - 1) ? 1.0 : q;
  }
  for (int i = tid; i < S; i += nt) M[i * L + S] = (i == S - 1) ? 1.0 : 0.0;
  __syncthreads();
  if (bad) {
    if (tid == 0) *status = PGPU_ERR_NAN;
    return;
  }
  for (int k = 0; k < S; ++k) {
    if (tid < 32) {
      double best = -1.0;
      int row = k;
      for (int r = k + lane; r < S; r += 32) {
        const double v = fabs(M[r * L + k]);
        if (v > best) {
          best = v;
          row = r;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int orow = __shfl_xor_sync(0xffffffffu, row, o);
        if (ob > best || (ob == best && orow < row)) {
          best = ob;
          row = orow;
        }
      }
      if (lane == 0) {
        piv = row;
        pval = best;
      }
    }
    __syncthreads();
    if (!(pval > 0.0) || !isfinite(pval)) {
      if (tid == 0) *status = PGPU_ERR_NONREVERSIBLE;
      return;
    }
    if (piv != k) {
      for (int c = k + tid; c <= S; c += nt) {
        const double t = M[k * L + c];
        M[k * L + c] = M[piv * L + c];
        M[piv * L + c] = t;
      }
      __syncthreads();
    }
    const int rows = S - 1 - k, cols = S - k;   // rows below k; columns k+1..S
    for (int e = tid; e < rows * cols; e += nt) {
      const int r = k + 1 + e / cols, c = k + 1 + e % cols;
      M[r * L + c] -= (M[r * L + k] / M[k * L + k]) * M[k * L + c];
    }
    __syncthreads();
  }
  if (tid == 0) {
    double sum = 0.0;
    int ok = 1;
    for (int i = S - 1; i >= 0; --i) {
      double x = M[i * L + S];
      for (int j = i + 1; j < S; ++j) x -= M[i * L + j] * M[j * L + S];
      x /= M[i * L + i];
      M[i * L + S] = x;
      sum += x;
      ok &= (x > 0.0) && isfinite(x);
    }
    // a frequency below 1e-15 of the total is a state the chain never
    // reaches (rounding leaves it near zero rather than at zero)
    for (int i = 0; ok && i < S; ++i) ok &= M[i * L + S] > 1e-15 * sum;
    if (ok)
      for (int i = 0; i < S; ++i) pi[i] = M[i * L + S] / sum;
    *status = ok ? 0 : PGPU_ERR_NONREVERSIBLE;
  }
}

// P[b][r] = U diag(exp(lambda * rate_r * t_b)) Ui for every branch b and
// rate r of a model.  One CTA per branch and model (blockIdx.y).  Writes
// FP64 and, if P32 is given, an FP32 copy.  t == -1 (compose only) gives Q;
// t < 1e-10 gives I.
struct ComposeArgs {
  const double *U, *lam, *Ui;   // model 0; model m at m*S*S, m*S, m*S*S
  const double *t;              // [n_br]
  const double *rates;          // [R] or null (rate 1); model m at m*R
  double *P;                    // [n_br][R][S][S] or null
  float *P32;                   // [n_br][R][S][S] or null
  int S, R;
  int n_br;
  int allow_q;                  // t == -1 returns Q (the reference's compose)
  const int *status;            // eigendecomposition status or null; model m at m
  int *flag;
  int p32_mode;                 // P32Mode
  size_t model_bytes;           // byte stride of P and P32 between models
};

__global__ void __launch_bounds__(256) compose_kernel(const ComposeArgs p) {
  extern __shared__ __align__(16) double sm[];
  const int S = p.S, R = p.R, SS = S * S;
  double *U = sm, *Ui = U + SS, *e = Ui + SS;   // e: [R][S]
  const int b = blockIdx.x, m = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int *status = p.status ? p.status + m : nullptr;
  if (status && *status) {
    if (b == 0 && tid == 0) atomicOr(p.flag, pgpu_model_flag(*status));
    return;
  }
  const double *gU = p.U + (size_t)m * SS, *gUi = p.Ui + (size_t)m * SS;
  const double *lam = p.lam + (size_t)m * S;
  const double *rates = p.rates ? p.rates + (size_t)m * R : nullptr;
  double *P = p.P ? (double *)((char *)p.P + m * p.model_bytes) : nullptr;
  float *P32 = p.P32 ? (float *)((char *)p.P32 + m * p.model_bytes) : nullptr;
  for (int i = tid; i < SS; i += nt) {
    U[i] = gU[i];
    Ui[i] = gUi[i];
  }
  const double t = p.t[b];
  const bool q_mode = p.allow_q && t == -1.0;
  for (int i = tid; i < R * S; i += nt) {
    const int r = i / S, k = i % S;
    const double rate = rates ? rates[r] : 1.0;
    e[i] = q_mode ? lam[k] * rate : exp(lam[k] * rate * t);
  }
  __syncthreads();
  for (int o = tid; o < R * SS; o += nt) {
    const int r = o / SS, i = (o % SS) / S, j = o % S;
    // the identity below an effective time of 1e-10 (rate times length):
    // a rate-0 class (invariant sites) gets I exactly, not U Ui to rounding
    const bool ident = !q_mode && !(t * (rates ? rates[r] : 1.0) >= 1e-10);
    double v;
    if (ident) {
      v = (i == j) ? 1.0 : 0.0;
    } else {
      v = 0.0;
      for (int k = 0; k < S; ++k) v = fma(U[i * S + k] * e[r * S + k], Ui[k * S + j], v);
    }
    const size_t off = ((size_t)b * R + r) * SS + (size_t)i * S + j;
    if (P) P[off] = v;
    if (P32) {
      const double d = (p.p32_mode == P32_MINUS_I && i == j) ? v - 1.0 : v;
      if (p.p32_mode == P32_PAIRS_ROWS4) {
        // S == 4 (checked by the launcher): 32 floats per (branch, rate)
        const size_t at = ((size_t)b * R + r) * 32 + 4 * ((i >> 1) * 4 + j) + (i & 1);
        const float hi = (float)d;
        P32[at] = hi;
        P32[at + 2] = (float)(d - (double)hi);
      } else {
        P32[off] = (float)d;
      }
    }
  }
}

// Tip rows: tab[t][r][c][i] = sum_j P(t, r)[i][j] * code_tab[c][j] for every
// tip t (the branch above it), rate r and tip code c, formed in FP64 from the
// eigen system and stored as float, float pair (hi, lo) or double.  A tip
// child then costs the pruning kernel one table read instead of a
// matrix-vector product.
struct TipTabArgs {
  const double *U, *lam, *Ui;   // model 0; model m at m*S*S, m*S, m*S*S
  const double *t;          // [n_tips] branch lengths above the tips
  const double *rates;      // [R]; model m at m*R
  const double *code_tab;   // [n_codes][S]
  void *out;
  int S, R, n_codes, form;  // form: 0 float, 1 float pair, 2 double, 3 float pairs element pairs first (S = 4)
  const int *status;        // model m at m
  size_t model_bytes;       // byte stride of out between models
};

// One CTA per tip, rate (blockIdx.y) and model (blockIdx.z).
__global__ void __launch_bounds__(128) tip_table_kernel(const TipTabArgs p) {
  extern __shared__ __align__(16) double sm[];
  const int S = p.S, SS = S * S;
  double *P = sm;   // [S][S]
  const int tip = blockIdx.x, r = blockIdx.y, m = blockIdx.z, tid = threadIdx.x, nt = blockDim.x;
  if (p.status && p.status[m]) return;
  const double *U = p.U + (size_t)m * SS, *Ui = p.Ui + (size_t)m * SS;
  const double *lam = p.lam + (size_t)m * S;
  char *out = static_cast<char *>(p.out) + m * p.model_bytes;
  const double tt = p.t[tip], rate = p.rates ? p.rates[(size_t)m * p.R + r] : 1.0;
  const bool ident = !(tt * rate >= 1e-10);   // effective time, as in compose_kernel
  for (int o = tid; o < SS; o += nt) {
    const int i = o / S, j = o % S;
    double v = 0.0;
    if (ident) {
      v = i == j ? 1.0 : 0.0;
    } else {
      for (int k = 0; k < S; ++k) v = fma(U[i * S + k] * exp(lam[k] * rate * tt), Ui[k * S + j], v);
    }
    P[o] = v;
  }
  __syncthreads();
  const size_t base = ((size_t)tip * p.R + r) * p.n_codes * S;
  for (int o = tid; o < p.n_codes * S; o += nt) {
    const int c = o / S, i = o % S;
    double v = 0.0;
    for (int j = 0; j < S; ++j) v = fma(P[i * S + j], p.code_tab[c * S + j], v);
    const size_t at = base + o;
    if (p.form == 3) {
      // float pairs of S = 4 entries, element pairs first: {h0, h1, l0, l1}, {h2, h3, l2, l3}
      float *q = reinterpret_cast<float *>(out) + 2 * (base + (size_t)c * 4) + (i >> 1) * 4 + (i & 1);
      const float hi = (float)v;
      q[0] = hi;
      q[2] = (float)(v - (double)hi);
    } else if (p.form == 0) {
      reinterpret_cast<float *>(out)[at] = (float)v;
    } else if (p.form == 1) {
      const float hi = (float)v;
      reinterpret_cast<float *>(out)[2 * at] = hi;
      reinterpret_cast<float *>(out)[2 * at + 1] = (float)(v - (double)hi);
    } else {
      reinterpret_cast<double *>(out)[at] = v;
    }
  }
}

size_t eig_smem(int S) {
  const int N = S + (S & 1);
  return sizeof(double) * (2 * (size_t)N * LDA + N) + sizeof(int) * 2 * (size_t)N;
}

}  // namespace

pgpu_status pgpu_launch_eig(pgpu_ctx *ctx, const double *Q_dev, const double *pi_dev, int S,
                            int n_models, double *U_dev, double *lam_dev, double *Ui_dev,
                            int *status_dev) {
  if (S < 1 || S > MAXS)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "model: %d states; at most %d are supported", S, MAXS);
  EigArgs a{Q_dev, pi_dev, U_dev, lam_dev, Ui_dev, status_dev, S, 40};
  const size_t smem = eig_smem(S);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(jacobi_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  jacobi_eig_kernel<<<n_models, S <= 8 ? 64 : 256, smem, ctx->stream>>>(a);
  return pgpu_after_launch(ctx, "jacobi_eig_kernel");
}

pgpu_status pgpu_launch_compose(pgpu_ctx *ctx, const double *U_dev, const double *lam_dev,
                                const double *Ui_dev, int S, const double *t_dev, int n_br,
                                const double *rates_dev, int R, double *P_dev, float *P32_dev,
                                bool allow_q, const int *status_dev, int p32_mode, int n_models,
                                size_t model_bytes) {
  if (n_br <= 0 || n_models <= 0) return PGPU_OK;
  if (p32_mode == P32_PAIRS_ROWS4 && S != 4)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "compose: the row-pair layout is for 4 states (got %d)", S);
  if (n_models > 65535)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "compose: %d models in one launch; at most 65535",
                        n_models);
  ComposeArgs a{U_dev, lam_dev, Ui_dev, t_dev,       rates_dev,  P_dev,       P32_dev,
                S,     R,       n_br,   allow_q ? 1 : 0, status_dev, ctx->d_flag,
                p32_mode, model_bytes};
  const size_t smem = sizeof(double) * (2 * (size_t)S * S + (size_t)R * S);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(compose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 1024)));
  const int threads = R * S * S <= 64 ? 64 : (R * S * S <= 128 ? 128 : 256);
  compose_kernel<<<dim3(n_br, n_models), threads, smem, ctx->stream>>>(a);
  return pgpu_after_launch(ctx, "compose_kernel");
}

pgpu_status pgpu_launch_tip_table(pgpu_ctx *ctx, const double *U_dev, const double *lam_dev,
                                  const double *Ui_dev, int S, const double *t_dev, int n_tips,
                                  const double *rates_dev, int R, const double *code_tab_dev,
                                  int n_codes, void *out_dev, int form, const int *status_dev,
                                  int n_models, size_t model_bytes) {
  if (n_tips <= 0 || n_models <= 0) return PGPU_OK;
  if (form == 3 && S != 4)
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "tip table: the element-pair layout is for 4 states (got %d)", S);
  if (n_models > 65535)
    return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "tip table: %d models in one launch; at most 65535",
                        n_models);
  TipTabArgs a{U_dev, lam_dev, Ui_dev, t_dev, rates_dev, code_tab_dev, out_dev, S, R, n_codes, form,
               status_dev, model_bytes};
  const size_t smem = sizeof(double) * (size_t)S * S;
  PGPU_CUDA(ctx, cudaFuncSetAttribute(tip_table_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 1024)));
  tip_table_kernel<<<dim3(n_tips, R, n_models), 128, smem, ctx->stream>>>(a);
  return pgpu_after_launch(ctx, "tip_table_kernel");
}

// ---------------------------------------------------------------------------
// C ABI (host buffers)
// ---------------------------------------------------------------------------

static pgpu_status status_to_err(pgpu_ctx *ctx, int st) {
  switch (st) {
    case 0: return PGPU_OK;
    case PGPU_ERR_NAN: return pgpu_set_err(ctx, st, "model: NaN or Inf in Q or pi (or pi <= 0)");
    case PGPU_ERR_NONREVERSIBLE:
      return pgpu_set_err(ctx, st, "model: Q is not reversible with respect to pi");
    case PGPU_ERR_EIGEN:
      return pgpu_set_err(ctx, st, "model: Jacobi eigendecomposition did not converge");
    default: return pgpu_set_err(ctx, PGPU_ERR_CUDA, "model: status %d", st);
  }
}

extern "C" {

pgpu_status pgpu_model_diagonalize(pgpu_ctx *ctx, const double *Q, const double *pi, int S,
                                   double *U, double *lambda, double *Ui) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!Q || !pi || !U || !lambda || !Ui) return pgpu_set_err(ctx, PGPU_ERR_ARG, "model: null buffer");
  if (S < 1 || S > MAXS) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "model: 1..%d states", MAXS);
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t SS = (size_t)S * S;
  void *dq, *dpi, *du, *dl, *dui, *dst;
  PGPU_TRY(pgpu_buf(ctx, BUF_A, SS * 8, &dq));
  PGPU_TRY(pgpu_buf(ctx, BUF_B, S * 8, &dpi));
  PGPU_TRY(pgpu_buf(ctx, BUF_C, SS * 8, &du));
  PGPU_TRY(pgpu_buf(ctx, BUF_D, S * 8, &dl));
  PGPU_TRY(pgpu_buf(ctx, BUF_E, SS * 8, &dui));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dst));
  cudaStream_t s = ctx->stream;
  PGPU_CUDA(ctx, cudaMemcpyAsync(dq, Q, SS * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dpi, pi, S * 8, cudaMemcpyHostToDevice, s));
  PGPU_TRY(pgpu_launch_eig(ctx, (double *)dq, (double *)dpi, S, 1, (double *)du, (double *)dl,
                           (double *)dui, (int *)dst));
  int *hst = reinterpret_cast<int *>(ctx->h_pinned);
  PGPU_CUDA(ctx, cudaMemcpyAsync(hst, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(U, du, SS * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(lambda, dl, S * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(Ui, dui, SS * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  return status_to_err(ctx, *hst);
}

pgpu_status pgpu_model_compose(pgpu_ctx *ctx, const double *U, const double *lambda,
                               const double *Ui, int S, const double *t, size_t n_t,
                               double *P_out) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!U || !lambda || !Ui || !P_out || (n_t && !t))
    return pgpu_set_err(ctx, PGPU_ERR_ARG, "compose: null buffer");
  if (S < 1 || S > MAXS) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "compose: 1..%d states", MAXS);
  if (n_t == 0) return PGPU_OK;
  if (n_t > 0x7fffffff) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "compose: too many branch lengths");
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t SS = (size_t)S * S;
  void *du, *dl, *dui, *dt, *dp;
  PGPU_TRY(pgpu_buf(ctx, BUF_C, SS * 8, &du));
  PGPU_TRY(pgpu_buf(ctx, BUF_D, S * 8, &dl));
  PGPU_TRY(pgpu_buf(ctx, BUF_E, SS * 8, &dui));
  PGPU_TRY(pgpu_buf(ctx, BUF_F, n_t * 8, &dt));
  PGPU_TRY(pgpu_buf(ctx, BUF_G, n_t * SS * 8, &dp));
  cudaStream_t s = ctx->stream;
  PGPU_CUDA(ctx, cudaMemcpyAsync(du, U, SS * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dl, lambda, S * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dui, Ui, SS * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(dt, t, n_t * 8, cudaMemcpyHostToDevice, s));
  PGPU_TRY(pgpu_launch_compose(ctx, (double *)du, (double *)dl, (double *)dui, S, (double *)dt,
                               (int)n_t, nullptr, 1, (double *)dp, nullptr, true));
  PGPU_CUDA(ctx, cudaMemcpyAsync(P_out, dp, n_t * SS * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  return PGPU_OK;
}

// ---- the reference's four externals, at their own arity -------------------
// likelihood_CAML_diagonalize_gtr / _sym and likelihood_CAML_compose_gtr /
// _sym (lib/mlmodel.c:200-205, 265-271, 304-323, 344-365; declared at
// lib/mlModel.ml:73-90).  Matrices are row-major n x n FP64, as the OCaml
// Bigarrays are; D is a diagonal matrix.

pgpu_status pgpu_diagonalize_gtr(pgpu_ctx *ctx, double *U, double *D, double *Ui, int n) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!U || !D || !Ui) return pgpu_set_err(ctx, PGPU_ERR_ARG, "diagonalize_gtr: null buffer");
  if (n < 1 || n > MAXS) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "diagonalize_gtr: 1..%d states", MAXS);
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t SS = (size_t)n * n;
  void *dq, *dpi, *du, *dl, *dui, *dst;
  PGPU_TRY(pgpu_buf(ctx, BUF_A, SS * 8, &dq));
  PGPU_TRY(pgpu_buf(ctx, BUF_B, n * 8, &dpi));
  PGPU_TRY(pgpu_buf(ctx, BUF_C, SS * 8, &du));
  PGPU_TRY(pgpu_buf(ctx, BUF_D, n * 8, &dl));
  PGPU_TRY(pgpu_buf(ctx, BUF_E, SS * 8, &dui));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dst));
  cudaStream_t s = ctx->stream;
  int *st = static_cast<int *>(dst);
  PGPU_CUDA(ctx, cudaMemcpyAsync(dq, U, SS * 8, cudaMemcpyHostToDevice, s));
  PGPU_CUDA(ctx, cudaMemsetAsync(dpi, 0, n * 8, s));
  PGPU_CUDA(ctx, cudaMemsetAsync(dst, 0, 2 * sizeof(int), s));
  const size_t smem = sizeof(double) * (size_t)n * (n + 1);
  PGPU_CUDA(ctx, cudaFuncSetAttribute(stationary_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 1024)));
  stationary_kernel<<<1, 256, smem, s>>>((const double *)dq, n, (double *)dpi, st + 1);
  PGPU_TRY(pgpu_after_launch(ctx, "stationary_kernel"));
  PGPU_TRY(pgpu_launch_eig(ctx, (double *)dq, (double *)dpi, n, 1, (double *)du, (double *)dl,
                           (double *)dui, st));
  int *hst = reinterpret_cast<int *>(ctx->h_pinned);
  std::vector<double> lam(n);
  PGPU_CUDA(ctx, cudaMemcpyAsync(hst, dst, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(lam.data(), dl, n * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  if (hst[1] == PGPU_ERR_NAN) return status_to_err(ctx, PGPU_ERR_NAN);
  if (hst[1])
    return pgpu_set_err(ctx, PGPU_ERR_NONREVERSIBLE,
                        "diagonalize_gtr: Q has no stationary distribution with every state above 0");
  PGPU_TRY(status_to_err(ctx, hst[0]));
  PGPU_CUDA(ctx, cudaMemcpyAsync(U, du, SS * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(Ui, dui, SS * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  for (size_t i = 0; i < SS; ++i) D[i] = 0.0;
  for (int i = 0; i < n; ++i) D[(size_t)i * n + i] = lam[i];
  return PGPU_OK;
}

pgpu_status pgpu_diagonalize_sym(pgpu_ctx *ctx, double *U, double *D, int n) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!U || !D) return pgpu_set_err(ctx, PGPU_ERR_ARG, "diagonalize_sym: null buffer");
  if (n < 1 || n > MAXS) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "diagonalize_sym: 1..%d states", MAXS);
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t SS = (size_t)n * n;
  void *dq, *du, *dl, *dst;
  PGPU_TRY(pgpu_buf(ctx, BUF_A, SS * 8, &dq));
  PGPU_TRY(pgpu_buf(ctx, BUF_C, SS * 8, &du));
  PGPU_TRY(pgpu_buf(ctx, BUF_D, n * 8, &dl));
  PGPU_TRY(pgpu_buf(ctx, BUF_SCALAR, 64, &dst));
  cudaStream_t s = ctx->stream;
  PGPU_CUDA(ctx, cudaMemcpyAsync(dq, U, SS * 8, cudaMemcpyHostToDevice, s));
  PGPU_TRY(pgpu_launch_eig(ctx, (double *)dq, nullptr, n, 1, (double *)du, (double *)dl, nullptr,
                           (int *)dst));
  int *hst = reinterpret_cast<int *>(ctx->h_pinned);
  std::vector<double> lam(n);
  PGPU_CUDA(ctx, cudaMemcpyAsync(hst, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaMemcpyAsync(lam.data(), dl, n * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  if (*hst == PGPU_ERR_NAN) return pgpu_set_err(ctx, PGPU_ERR_NAN, "diagonalize_sym: NaN or Inf in Q");
  PGPU_TRY(status_to_err(ctx, *hst));
  PGPU_CUDA(ctx, cudaMemcpyAsync(U, du, SS * 8, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(ctx, cudaStreamSynchronize(s));
  for (size_t i = 0; i < SS; ++i) D[i] = 0.0;
  for (int i = 0; i < n; ++i) D[(size_t)i * n + i] = lam[i];
  return PGPU_OK;
}

pgpu_status pgpu_compose_gtr(pgpu_ctx *ctx, const double *U, const double *D, const double *Ui,
                             int n, double t, double *P) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!U || !D || !Ui || !P) return pgpu_set_err(ctx, PGPU_ERR_ARG, "compose_gtr: null buffer");
  if (n < 1 || n > MAXS) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "compose_gtr: 1..%d states", MAXS);
  std::vector<double> lam(n);
  for (int i = 0; i < n; ++i) lam[i] = D[(size_t)i * n + i];
  return pgpu_model_compose(ctx, U, lam.data(), Ui, n, &t, 1, P);
}

pgpu_status pgpu_compose_sym(pgpu_ctx *ctx, const double *U, const double *D, int n, double t,
                             double *P) {
  if (!ctx) return PGPU_ERR_ARG;
  if (!U || !D || !P) return pgpu_set_err(ctx, PGPU_ERR_ARG, "compose_sym: null buffer");
  if (n < 1 || n > MAXS) return pgpu_set_err(ctx, PGPU_ERR_LIMIT, "compose_sym: 1..%d states", MAXS);
  // the reference takes t as a float here (`const float t`, lib/mlmodel.c:280)
  const double t32 = (double)(float)t;
  // U holds the eigenvectors as rows, so P = U^T exp(D t) U: compose with
  // U^T in the left factor's place and U in the right one's
  const size_t SS = (size_t)n * n;
  std::vector<double> lam(n), ut(SS);
  for (int i = 0; i < n; ++i) lam[i] = D[(size_t)i * n + i];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) ut[(size_t)i * n + j] = U[(size_t)j * n + i];
  return pgpu_model_compose(ctx, ut.data(), lam.data(), U, n, &t32, 1, P);
}

}  // extern "C"
