/* Test infrastructure (oracle) -- not part of the product.
 *
 * CPU restatements of phylocaml's Fitch parsimony, used (1) as the checker
 * the GPU kernels are compared against and (2) as the timed CPU baseline on
 * machines where the reference's own bv.c cannot be compiled.
 *
 *   orc_bv8_*          restate bv_fitch / bv_copy (lib/bitvector/bv.c:148-178)
 *                      for the one-character-per-byte layout (WIDTH=8,
 *                      lib/bitvector/bv.h:29-34): same loop, same per-node
 *                      result allocation as bv_CAML_fitch_median2 (bv.c:463-480).
 *   orc_nonadditive_median2
 *                      restates NonAdditive_c.median_2 (lib/nonAdditive_c.ml:19-35).
 *   orc_fitch_tree_packed
 *                      the same rule over packed lanes of 4/8/16/32 bits in
 *                      uint32 words (or 64-bit elements as word pairs, low
 *                      word first), lane by lane, with per-site union counts
 *                      and the weighted total.
 *
 * Tree convention: tips are ids 0..n_tips-1; internal node k has id n_tips+k
 * and children left[k], right[k] with smaller ids. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

/* ---- bv_fitch restated for 8-bit elements ------------------------------ */

uint64_t orc_bv8_fitch(uint8_t *c, const uint8_t *a, const uint8_t *b, uint64_t chars)
{
  uint64_t i, res;
  for (i = 0, res = 0; i < chars; ++i) {
    c[i] = a[i] & b[i];
    if (0 == c[i]) {
      c[i] = a[i] | b[i];
      ++res;
    }
  }
  return res;
}

uint64_t orc_bv8_distance(const uint8_t *a, const uint8_t *b, uint64_t chars)
{
  uint64_t i, res = 0;
  for (i = 0; i < chars; ++i)
    if (0 == (a[i] & b[i])) res++;
  return res;
}

/* postorder with one freshly allocated result per node, like an OCaml
 * caller of fitch_median_2 (bv_copy + bv_fitch) */
static uint64_t bv8_tree_alloc(int32_t n_tips, const int32_t *left,
                               const int32_t *right, const uint8_t *tips,
                               uint64_t ld, uint64_t off, uint64_t chars,
                               uint8_t *internal)
{
  int32_t k, n_int = n_tips - 1;
  uint64_t total = 0;
  const uint8_t **row = (const uint8_t **)calloc((size_t)n_tips + (size_t)n_int,
                                                 sizeof(uint8_t *));
  for (k = 0; k < n_tips; ++k) row[k] = tips + (uint64_t)k * ld + off;
  for (k = 0; k < n_int; ++k) {
    uint8_t *c = (uint8_t *)malloc(chars ? chars : 1);
    total += orc_bv8_fitch(c, row[left[k]], row[right[k]], chars);
    row[n_tips + k] = c;
  }
  for (k = 0; k < n_int; ++k) {
    if (internal) memcpy(internal + (uint64_t)k * ld + off, row[n_tips + k], chars);
    free((void *)row[n_tips + k]);
  }
  free(row);
  return total;
}

uint64_t orc_bv8_fitch_tree_alloc(int32_t n_tips, const int32_t *left,
                                  const int32_t *right, const uint8_t *tips,
                                  uint64_t chars, uint8_t *internal)
{
  return bv8_tree_alloc(n_tips, left, right, tips, chars, 0, chars, internal);
}

struct bv8_job {
  int32_t n_tips; const int32_t *left, *right; const uint8_t *tips;
  uint64_t ld, off, chars; uint8_t *internal; uint64_t total;
};

static void *bv8_run(void *p)
{
  struct bv8_job *j = (struct bv8_job *)p;
  j->total = bv8_tree_alloc(j->n_tips, j->left, j->right, j->tips, j->ld,
                            j->off, j->chars, j->internal);
  return NULL;
}

uint64_t orc_bv8_fitch_tree_alloc_mt(int32_t n_tips, const int32_t *left,
                                     const int32_t *right, const uint8_t *tips,
                                     uint64_t chars, uint8_t *internal, int n_threads)
{
  int t;
  uint64_t total = 0, per;
  pthread_t *th;
  struct bv8_job *jobs;
  if (n_threads < 1) n_threads = 1;
  th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
  jobs = (struct bv8_job *)calloc((size_t)n_threads, sizeof(struct bv8_job));
  per = (chars + (uint64_t)n_threads - 1) / (uint64_t)n_threads;
  for (t = 0; t < n_threads; ++t) {
    uint64_t lo = per * (uint64_t)t, hi = lo + per;
    if (hi > chars) hi = chars;
    if (lo > chars) lo = chars;
    jobs[t].n_tips = n_tips; jobs[t].left = left; jobs[t].right = right;
    jobs[t].tips = tips; jobs[t].ld = chars; jobs[t].off = lo;
    jobs[t].chars = hi - lo; jobs[t].internal = internal;
    pthread_create(&th[t], NULL, bv8_run, &jobs[t]);
  }
  for (t = 0; t < n_threads; ++t) {
    pthread_join(th[t], NULL);
    total += jobs[t].total;
  }
  free(th);
  free(jobs);
  return total;
}

/* ---- NonAdditive_c.median_2 -------------------------------------------- */

/* states are OCaml ints; the cost accumulates x.weights.(i) *. float c in
 * site order, weighting by the left operand's weights (nonAdditive_c.ml:31) */
double orc_nonadditive_median2(const int64_t *xs, const int64_t *ys,
                               const double *weights, uint64_t n, int64_t *out)
{
  uint64_t i;
  double cost = 0.0;
  for (i = 0; i < n; ++i) {
    int64_t m = xs[i] & ys[i];
    int c = 0;
    if (0 == m) { m = xs[i] | ys[i]; c = 1; }
    out[i] = m;
    cost = cost + weights[i] * (double)c;
  }
  return cost;
}

/* ---- packed lanes ------------------------------------------------------- */

/* 64-bit lanes (BV64): site s is words 2s (low) and 2s+1 (high) */
static uint64_t lane_get64(const uint32_t *row, uint64_t site)
{
  return (uint64_t)row[2 * site] | ((uint64_t)row[2 * site + 1] << 32);
}

static void lane_set64(uint32_t *row, uint64_t site, uint64_t v)
{
  row[2 * site] = (uint32_t)v;
  row[2 * site + 1] = (uint32_t)(v >> 32);
}

static uint32_t lane_get(const uint32_t *row, uint64_t site, int lb)
{
  uint64_t per = 32u / (unsigned)lb;
  uint32_t w = row[site / per];
  uint32_t mask = lb == 32 ? 0xffffffffu : ((1u << lb) - 1u);
  return (w >> ((site % per) * (unsigned)lb)) & mask;
}

static void lane_set(uint32_t *row, uint64_t site, int lb, uint32_t v)
{
  uint64_t per = 32u / (unsigned)lb;
  uint32_t sh = (uint32_t)((site % per) * (unsigned)lb);
  uint32_t mask = lb == 32 ? 0xffffffffu : ((1u << lb) - 1u);
  row[site / per] = (row[site / per] & ~(mask << sh)) | ((v & mask) << sh);
}

/* Fitch postorder over packed lanes.  tip_words: [n_tips][ld_words];
 * node_sets: [n_tips-1][ld_words] (lanes past n_sites are left 0);
 * weights: [n_sites] or NULL for unit weights; site_cost: [n_sites] union
 * counts per site or NULL; node_counts: [n_tips-1] unweighted union count
 * per node (bv_fitch's return) or NULL; *total = sum_s w_s * site count.
 * Returns 0, or -1 on bad arguments. */
int orc_fitch_tree_packed(int32_t n_tips, const int32_t *left, const int32_t *right,
                          const uint32_t *tip_words, uint64_t ld_words,
                          uint64_t n_sites, int lane_bits, const uint32_t *weights,
                          uint32_t *node_sets, uint32_t *site_cost,
                          uint64_t *total, uint64_t *node_counts)
{
  int32_t k, n_int = n_tips - 1;
  uint64_t s, tot = 0;
  uint32_t *cnt;
  if (lane_bits != 4 && lane_bits != 8 && lane_bits != 16 && lane_bits != 32 && lane_bits != 64)
    return -1;
  if (n_tips < 2) return -1;
  if (lane_bits == 64 ? ld_words < 2 * n_sites : ld_words * (32u / (unsigned)lane_bits) < n_sites)
    return -1;
  cnt = (uint32_t *)calloc(n_sites ? n_sites : 1, sizeof(uint32_t));
  memset(node_sets, 0, (size_t)n_int * ld_words * sizeof(uint32_t));
  for (k = 0; k < n_int; ++k) {
    int32_t l = left[k], r = right[k];
    const uint32_t *ra = l < n_tips ? tip_words + (uint64_t)l * ld_words
                                    : node_sets + (uint64_t)(l - n_tips) * ld_words;
    const uint32_t *rb = r < n_tips ? tip_words + (uint64_t)r * ld_words
                                    : node_sets + (uint64_t)(r - n_tips) * ld_words;
    uint32_t *rc = node_sets + (uint64_t)k * ld_words;
    uint64_t nc = 0;
    if (l >= n_tips + k || r >= n_tips + k || l < 0 || r < 0) { free(cnt); return -1; }
    for (s = 0; s < n_sites; ++s) {
      if (lane_bits == 64) {
        uint64_t a = lane_get64(ra, s), b = lane_get64(rb, s), m = a & b;
        if (m == 0) { m = a | b; cnt[s]++; nc++; }
        lane_set64(rc, s, m);
        continue;
      }
      uint32_t a = lane_get(ra, s, lane_bits), b = lane_get(rb, s, lane_bits);
      uint32_t m = a & b;
      if (m == 0) { m = a | b; cnt[s]++; nc++; }
      lane_set(rc, s, lane_bits, m);
    }
    if (node_counts) node_counts[k] = nc;
  }
  for (s = 0; s < n_sites; ++s) {
    tot += (uint64_t)(weights ? weights[s] : 1u) * (uint64_t)cnt[s];
    if (site_cost) site_cost[s] = cnt[s];
  }
  *total = tot;
  free(cnt);
  return 0;
}
