/* Test infrastructure (oracle) -- not part of the product.
 *
 * Drives phylocaml's own Fitch kernel, bv_fitch (lib/bitvector/bv.c:148-160),
 * compiled unmodified from the reference tree with -DWIDTH=8/16/32/64 against
 * the shim headers in oracle/shim.  One character per CTYPE element, exactly
 * the reference layout (lib/bitvector/bv.h:57-63).
 *
 * Tree convention shared by every oracle and by the product: tips have ids
 * 0..n_tips-1; internal node k (0 <= k < n_tips-1) has id n_tips+k and its
 * children left[k], right[k] have smaller ids (postorder). */
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include "bv.h"

/* pure-C routines of lib/bitvector/bv.c that bv.h does not declare */
unsigned long bv_fitch(vect *c, const vect *a, const vect *b);
unsigned long bv_distance(const vect *a, const vect *b);
void bv_union(vect *c, vect *a, vect *b);
void bv_inter(vect *c, vect *a, vect *b);
vect *bv_copy(const vect *a, const int fill);

static void wrap(vect *v, const CTYPE *data, unsigned long chars)
{
  v->length = chars;
  v->chars = chars;
  v->code = 0;
  v->msize = WIDTH;
  v->data = (CTYPE *)data;
}

int bvref_width(void) { return WIDTH; }

/* Bitvector.BVn.fitch_median_2 minus the OCaml boxing (bv.c:463-480). */
uint64_t bvref_fitch_median2(const CTYPE *a, const CTYPE *b, CTYPE *out, uint64_t chars)
{
  vect va, vb, vc;
  wrap(&va, a, chars); wrap(&vb, b, chars); wrap(&vc, out, chars);
  return bv_fitch(&vc, &va, &vb);
}

/* Bitvector.BVn.distance (bv.c:46-55, :455-461). */
uint64_t bvref_distance(const CTYPE *a, const CTYPE *b, uint64_t chars)
{
  vect va, vb;
  wrap(&va, a, chars); wrap(&vb, b, chars);
  return bv_distance(&va, &vb);
}

void bvref_union(const CTYPE *a, const CTYPE *b, CTYPE *out, uint64_t chars)
{
  vect va, vb, vc;
  wrap(&va, a, chars); wrap(&vb, b, chars); wrap(&vc, out, chars);
  bv_union(&vc, &va, &vb);
}

void bvref_inter(const CTYPE *a, const CTYPE *b, CTYPE *out, uint64_t chars)
{
  vect va, vb, vc;
  wrap(&va, a, chars); wrap(&vb, b, chars); wrap(&vc, out, chars);
  bv_inter(&vc, &va, &vb);
}

static const CTYPE *row_of(int32_t id, int32_t n_tips, const CTYPE *tips,
                           const CTYPE *internal, uint64_t chars)
{
  return id < n_tips ? tips + (uint64_t)id * chars
                     : internal + (uint64_t)(id - n_tips) * chars;
}

/* Postorder over the tree with bv_fitch writing into caller rows. */
int bvref_fitch_tree(int32_t n_tips, const int32_t *left, const int32_t *right,
                     const CTYPE *tips, uint64_t chars, CTYPE *internal,
                     uint64_t *node_counts)
{
  int32_t k;
  for (k = 0; k < n_tips - 1; ++k) {
    vect va, vb, vc;
    wrap(&va, row_of(left[k], n_tips, tips, internal, chars), chars);
    wrap(&vb, row_of(right[k], n_tips, tips, internal, chars), chars);
    wrap(&vc, internal + (uint64_t)k * chars, chars);
    node_counts[k] = bv_fitch(&vc, &va, &vb);
  }
  return 0;
}

/* The postorder the way an OCaml caller of fitch_median_2 runs it: each
 * median allocates its result with bv_copy (bv.c:472) before bv_fitch.
 * Results are copied to `internal` (if non-NULL) and freed.  Returns the
 * summed union count. */
static uint64_t fitch_tree_alloc(int32_t n_tips, const int32_t *left,
                                 const int32_t *right, const CTYPE *tips,
                                 uint64_t ld, uint64_t off, uint64_t chars,
                                 CTYPE *internal)
{
  int32_t k, n_int = n_tips - 1;
  uint64_t total = 0;
  vect **node = (vect **)calloc((size_t)n_tips + (size_t)n_int, sizeof(vect *));
  vect *tipv = (vect *)calloc((size_t)n_tips, sizeof(vect));
  for (k = 0; k < n_tips; ++k) {
    wrap(&tipv[k], tips + (uint64_t)k * ld + off, chars);
    node[k] = &tipv[k];
  }
  for (k = 0; k < n_int; ++k) {
    const vect *a = node[left[k]], *b = node[right[k]];
    vect *c = bv_copy(a, 0);
    total += bv_fitch(c, a, b);
    node[n_tips + k] = c;
  }
  for (k = 0; k < n_int; ++k) {
    vect *c = node[n_tips + k];
    if (internal)
      memcpy(internal + (uint64_t)k * ld + off, c->data, chars * sizeof(CTYPE));
    free(c->data);
    free(c);
  }
  free(tipv);
  free(node);
  return total;
}

uint64_t bvref_fitch_tree_alloc(int32_t n_tips, const int32_t *left,
                                const int32_t *right, const CTYPE *tips,
                                uint64_t chars, CTYPE *internal)
{
  return fitch_tree_alloc(n_tips, left, right, tips, chars, 0, chars, internal);
}

struct mt_job {
  int32_t n_tips; const int32_t *left, *right; const CTYPE *tips;
  uint64_t ld, off, chars; CTYPE *internal; uint64_t total;
};

static void *mt_run(void *p)
{
  struct mt_job *j = (struct mt_job *)p;
  j->total = fitch_tree_alloc(j->n_tips, j->left, j->right, j->tips, j->ld,
                              j->off, j->chars, j->internal);
  return NULL;
}

/* The same allocation path over contiguous character blocks, one block per
 * thread (the reference itself is single-threaded; this spreads its own
 * routine over the host cores). */
uint64_t bvref_fitch_tree_alloc_mt(int32_t n_tips, const int32_t *left,
                                   const int32_t *right, const CTYPE *tips,
                                   uint64_t chars, CTYPE *internal, int n_threads)
{
  int t;
  uint64_t total = 0, per;
  pthread_t *th;
  struct mt_job *jobs;
  if (n_threads < 1) n_threads = 1;
  th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
  jobs = (struct mt_job *)calloc((size_t)n_threads, sizeof(struct mt_job));
  per = (chars + (uint64_t)n_threads - 1) / (uint64_t)n_threads;
  for (t = 0; t < n_threads; ++t) {
    uint64_t lo = per * (uint64_t)t, hi = lo + per;
    if (hi > chars) hi = chars;
    if (lo > chars) lo = chars;
    jobs[t].n_tips = n_tips; jobs[t].left = left; jobs[t].right = right;
    jobs[t].tips = tips; jobs[t].ld = chars; jobs[t].off = lo;
    jobs[t].chars = hi - lo; jobs[t].internal = internal;
    pthread_create(&th[t], NULL, mt_run, &jobs[t]);
  }
  for (t = 0; t < n_threads; ++t) {
    pthread_join(th[t], NULL);
    total += jobs[t].total;
  }
  free(th);
  free(jobs);
  return total;
}
