/* Test infrastructure (oracle) -- not part of the product.
 *
 * FP64 Felsenstein pruning, the checker for the GPU likelihood kernels and
 * the timed CPU baseline for them.  phylocaml has no pruning code to follow
 * (Likelihood_c.median_2 is `failwith "TODO"`, lib/likelihood_c.ml:15); this
 * is the standard recursion over the transition matrices that the
 * reference's compose_gtr builds (lib/mlmodel.c:325-342, row-major
 * P[i][j] = Pr(j | i, t)), checked in the tests against brute-force
 * enumeration of ancestral states on small trees.
 *
 *   CLV_v[r][i] = (sum_j P_{l,r}[i][j] CLV_l[r][j]) * (sum_j P_{r,r}[i][j] CLV_r[r][j])
 *   L_site      = sum_r probs[r] sum_i pi[i] CLV_root[r][i]
 *   lnL         = sum_s w_s (log L_site + e_s ln 2)       (Neumaier-compensated)
 *
 * where e_s collects the exact power-of-two rescalings applied whenever a
 * node's largest entry drops below 2^-128.  Tips read their partial vector
 * from code_table[tip_code] (one row of S entries per code).  P holds one
 * [R][S][S] block per node id (the branch above that node; the root has
 * none, so P has 2*n_tips-2 blocks). */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>

typedef struct {
  double sum, comp;
} neum_t;

static void neum_add(neum_t *a, double x)
{
  double t = a->sum + x;
  if (fabs(a->sum) >= fabs(x)) a->comp += (a->sum - t) + x;
  else a->comp += (x - t) + a->sum;
  a->sum = t;
}

typedef struct {
  int32_t n_tips; const int32_t *left, *right; const double *P;
  int S, R; const double *pi, *probs;
  const uint8_t *tip_codes; int n_codes; const double *code_table;
  const double *weights; uint64_t n_pat, lo, hi;
  double *site_lnl; neum_t acc; int err;
} prune_job;

static void prune_range(prune_job *j)
{
  const int S = j->S, R = j->R, RS = R * S;
  const int32_t n_tips = j->n_tips, n_int = n_tips - 1;
  double *clv = (double *)malloc((size_t)n_int * (size_t)RS * sizeof(double));
  double *tipbuf = (double *)malloc(2 * (size_t)RS * sizeof(double));
  uint64_t s;
  neum_t acc = {0.0, 0.0};
  for (s = j->lo; s < j->hi; ++s) {
    int64_t escale = 0;
    int32_t k;
    double L = 0.0, lnl;
    for (k = 0; k < n_int; ++k) {
      const double *cv[2];
      int32_t ch[2];
      int c, r, i, jj;
      double *out = clv + (size_t)k * RS, mx = 0.0;
      ch[0] = j->left[k]; ch[1] = j->right[k];
      for (c = 0; c < 2; ++c) {
        if (ch[c] < n_tips) {
          uint8_t code = j->tip_codes[(uint64_t)ch[c] * j->n_pat + s];
          if (code >= j->n_codes) { j->err = 1; code = 0; }
          for (r = 0; r < R; ++r)
            memcpy(tipbuf + (size_t)c * RS + (size_t)r * S,
                   j->code_table + (size_t)code * S, (size_t)S * sizeof(double));
          cv[c] = tipbuf + (size_t)c * RS;
        } else {
          cv[c] = clv + (size_t)(ch[c] - n_tips) * RS;
        }
      }
      for (r = 0; r < R; ++r) {
        const double *Pl = j->P + ((size_t)ch[0] * R + r) * S * S;
        const double *Pr = j->P + ((size_t)ch[1] * R + r) * S * S;
        const double *xl = cv[0] + (size_t)r * S, *xr = cv[1] + (size_t)r * S;
        for (i = 0; i < S; ++i) {
          double sl = 0.0, sr = 0.0;
          for (jj = 0; jj < S; ++jj) {
            sl += Pl[i * S + jj] * xl[jj];
            sr += Pr[i * S + jj] * xr[jj];
          }
          out[r * S + i] = sl * sr;
          if (sl * sr > mx) mx = sl * sr;
        }
      }
      if (mx > 0.0 && mx < 0x1p-128) {
        int e;
        (void)frexp(mx, &e);
        for (i = 0; i < RS; ++i) out[i] = ldexp(out[i], -e);
        escale += e;
      }
    }
    {
      const double *root = clv + (size_t)(n_int - 1) * RS;
      int r, i;
      for (r = 0; r < R; ++r) {
        double sr = 0.0;
        for (i = 0; i < S; ++i) sr += j->pi[i] * root[r * S + i];
        L += j->probs[r] * sr;
      }
    }
    lnl = log(L) + (double)escale * 0.69314718055994530942;
    if (j->site_lnl) j->site_lnl[s] = lnl;
    neum_add(&acc, j->weights ? j->weights[s] * lnl : lnl);
  }
  j->acc = acc;
  free(clv);
  free(tipbuf);
}

static void *prune_thread(void *p)
{
  prune_range((prune_job *)p);
  return NULL;
}

/* Returns 0 on success, -1 on bad arguments, -2 if a tip code is out of
 * range.  n_threads > 1 splits the patterns into contiguous blocks; the
 * per-block compensated sums are combined in block order. */
int orc_prune_lnl(int32_t n_tips, const int32_t *left, const int32_t *right,
                  const double *P, int S, int R, const double *pi,
                  const double *probs, const uint8_t *tip_codes, int n_codes,
                  const double *code_table, const double *weights,
                  uint64_t n_pat, double *site_lnl, double *lnl_out, int n_threads)
{
  int t, err = 0;
  uint64_t per;
  pthread_t *th;
  prune_job *jobs;
  neum_t tot = {0.0, 0.0};
  if (n_tips < 2 || S < 1 || R < 1 || n_codes < 1) return -1;
  if (n_threads < 1) n_threads = 1;
  th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
  jobs = (prune_job *)calloc((size_t)n_threads, sizeof(prune_job));
  per = (n_pat + (uint64_t)n_threads - 1) / (uint64_t)n_threads;
  for (t = 0; t < n_threads; ++t) {
    prune_job *j = &jobs[t];
    j->n_tips = n_tips; j->left = left; j->right = right; j->P = P;
    j->S = S; j->R = R; j->pi = pi; j->probs = probs;
    j->tip_codes = tip_codes; j->n_codes = n_codes; j->code_table = code_table;
    j->weights = weights; j->n_pat = n_pat; j->site_lnl = site_lnl;
    j->lo = per * (uint64_t)t; j->hi = j->lo + per;
    if (j->lo > n_pat) j->lo = n_pat;
    if (j->hi > n_pat) j->hi = n_pat;
    if (n_threads == 1) prune_range(j);
    else pthread_create(&th[t], NULL, prune_thread, j);
  }
  for (t = 0; t < n_threads; ++t) {
    if (n_threads > 1) pthread_join(th[t], NULL);
    neum_add(&tot, jobs[t].acc.sum);
    neum_add(&tot, jobs[t].acc.comp);
    err |= jobs[t].err;
  }
  *lnl_out = tot.sum + tot.comp;
  free(th);
  free(jobs);
  return err ? -2 : 0;
}
