/* phylo_gpu.h -- C ABI of the GB300 (sm_103a) tree-scoring library.
 *
 * This is the boundary that phylocaml's OCaml externals would bind in place
 * of its CPU stubs: plain pointers and sizes, status codes, no OCaml or
 * torch types.  Each entry point names the reference interface it replaces
 * (paths inside the phylocaml tree).
 *
 * Conventions
 *   - Every call returns pgpu_status; PGPU_OK is 0.  On failure the context
 *     keeps a message readable with pgpu_last_error().  An OCaml stub turns
 *     a non-zero status into `failwith msg`, as lib/mlmodel.c does for LAPACK
 *     failures (lib/mlmodel.c:110-120).
 *   - "Host" entry points take caller-owned host buffers, copy them to the
 *     device, run, copy results back and return when the results are in the
 *     caller's buffers (synchronous, like the reference's externals).
 *   - "_dev" entry points take device pointers and are asynchronous on the
 *     context's stream (pgpu_set_stream); call pgpu_synchronize() before
 *     reading results.
 *   - A context owns its device memory and stream.  Calls on different
 *     contexts may run concurrently from different threads; calls on one
 *     context must not overlap.
 *
 * Tree layout (pgpu_tree)
 *   A rooted binary tree with n_tips leaves.  Tips have ids 0..n_tips-1.
 *   Internal node k (0 <= k < n_tips-1) has id n_tips+k; its children
 *   left[k] and right[k] must have ids smaller than n_tips+k (a postorder,
 *   as produced by Tree.post_order_edges, lib/tree.ml:171-187).  The root is
 *   id 2*n_tips-2.  brlen[id] is the length of the branch above node id
 *   (2*n_tips-2 entries; the root has none); Fitch ignores it.
 */
#ifndef PHYLO_GPU_H
#define PHYLO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int pgpu_status;

enum {
  PGPU_OK = 0,
  PGPU_ERR_ARG = 1,            /* bad size, pointer, layout or tree        */
  PGPU_ERR_CUDA = 2,           /* CUDA runtime error                        */
  PGPU_ERR_OOM = 3,            /* device allocation failed                  */
  PGPU_ERR_NAN = 4,            /* NaN/Inf in a model matrix (mlModel.ml:557-568) */
  PGPU_ERR_NONREVERSIBLE = 5,  /* Q is not reversible w.r.t. pi             */
  PGPU_ERR_EIGEN = 6,          /* eigendecomposition did not converge       */
  PGPU_ERR_OVERFLOW = 7,       /* a count does not fit its output type      */
  PGPU_ERR_TIMEOUT = 8,        /* a bounded device wait gave up             */
  PGPU_ERR_UNSUPPORTED = 9,    /* device or configuration not supported     */
  PGPU_ERR_LIMIT = 10          /* size above a documented maximum           */
};

typedef struct pgpu_ctx pgpu_ctx;

typedef struct {
  int32_t n_tips;
  const int32_t *left;   /* [n_tips-1] */
  const int32_t *right;  /* [n_tips-1] */
  const double *brlen;   /* [2*n_tips-2] or NULL */
} pgpu_tree;

/* ---- context ------------------------------------------------------------
 * No reference counterpart: phylocaml's externals run on the caller's
 * thread with no device state.  The context carries what a custom block's
 * finalizer would own (lib/bitvector/bv.c:183-189). */
pgpu_status pgpu_create(pgpu_ctx **out, int device);
void pgpu_destroy(pgpu_ctx *ctx);
const char *pgpu_last_error(const pgpu_ctx *ctx);
/* Runs the context's work on cuda_stream (a cudaStream_t).  NULL gives the
 * context its own non-blocking stream back; the legacy default stream
 * (handle 0) therefore cannot be selected -- pass an explicit stream. */
pgpu_status pgpu_set_stream(pgpu_ctx *ctx, void *cuda_stream);
pgpu_status pgpu_synchronize(pgpu_ctx *ctx);
/* The cudaStream_t the context's work runs on (its own stream unless
 * pgpu_set_stream chose another), for callers that order their own work
 * against it with events. */
void *pgpu_get_stream(const pgpu_ctx *ctx);
/* Number of kernels this library launched on ctx since creation. */
uint64_t pgpu_kernel_launches(const pgpu_ctx *ctx);
/* Library version as 10000*major + 100*minor + patch. */
int pgpu_version(void);

/* Host-only: the stack-machine evaluation order the kernels use for `tree`
 * (no device work, ctx may be NULL).  ops_out receives 3*(n_tips-1) ints,
 * (internal index k, first child id, second child id) per step in
 * evaluation order; *max_depth the largest number of intermediate node
 * results alive at once.  No reference counterpart: phylocaml recurses
 * (lib/tree.ml:171-187). */
pgpu_status pgpu_tree_schedule(pgpu_ctx *ctx, const pgpu_tree *tree, int32_t *ops_out,
                               int32_t *max_depth);

/* ---- Fitch parsimony -----------------------------------------------------
 * State sets are packed lanes of lane_bits bits (4, 8, 16 or 32) in uint32
 * words, site s in lane s % (32/lane_bits) of word s / (32/lane_bits),
 * lowest lane in the lowest bits.  lane_bits 8 with one state bit per
 * alphabet code is the reference's BV8 layout (lib/bitvector/bv.h:29-34);
 * lane_bits 4 packs the four nucleotides (A=1, C=2, G=4, T=8,
 * lib/alphabet.ml:301-307) eight sites to a word.  lane_bits 64 is BV64:
 * site s is the 64-bit element in words 2s (low half) and 2s + 1, the
 * little-endian layout of a uint64_t array.  Lanes past the last site are
 * ignored on input and written as zero.  pgpu_fitch_tree_noalloc takes
 * lane_bits 4..32 only. */

/* Bitvector.BVn.fitch_median_2 (lib/bitvector.mli:94; bv_CAML_fitch_median2,
 * lib/bitvector/bv.c:463-480, and bv_fitch, bv.c:148-160).  out[i] = a&b,
 * or a|b where a&b is empty; *union_count = number of such sites.
 * The three pair entry points below read and write exactly
 * ceil(n_sites * lane_bits / 8) bytes of a, b and out -- the size of the
 * reference's vectors (bv_malloc, bv.c:32-42) -- so the buffers need no
 * padding to whole words and need no particular alignment. */
pgpu_status pgpu_fitch_median2(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b,
                               uint32_t *out, size_t n_sites, int lane_bits,
                               uint64_t *union_count);

/* NonAdditive_c.median_2 (lib/nonAdditive_c.ml:19-35): the same median with
 * the cost sum_i weights[i] * [a_i & b_i == 0], weights taken per site (the
 * left operand's weights in the reference).  Integer weights make the
 * float sum of the reference exact. */
pgpu_status pgpu_fitch_median2_weighted(pgpu_ctx *ctx, const uint32_t *a,
                                        const uint32_t *b, const uint32_t *weights,
                                        uint32_t *out, size_t n_sites, int lane_bits,
                                        uint64_t *cost);

/* NonAdditive_c.median_2 (lib/nonAdditive_c.ml:19-35) over the reference's
 * own record fields: x.states and y.states as OCaml ints (state sets of up
 * to 63 bits, sign-extended to int64 by Long_val, so land / lor are 64-bit
 * AND / OR), x.weights as doubles (any value: fractional weights are
 * legal).  out[i] = x_i & y_i, or x_i | y_i where that is 0;
 * *cost = sum_i weights[i] * float([x_i & y_i == 0]), each term formed as
 * the reference forms it and summed with error-free transformations in a
 * fixed order, so the result is deterministic and within rounding of the
 * exact sum (the reference's left-to-right sum may differ from it by its
 * own rounding). */
pgpu_status pgpu_nonadditive_median2(pgpu_ctx *ctx, const int64_t *x, const int64_t *y,
                                     const double *weights, int64_t *out, size_t n, double *cost);

/* Bitvector.BVn.distance (lib/bitvector.mli:90; bv_distance, bv.c:46-55). */
pgpu_status pgpu_fitch_distance(pgpu_ctx *ctx, const uint32_t *a, const uint32_t *b,
                                size_t n_sites, int lane_bits, uint64_t *distance);

/* The whole Fitch postorder: Node.Make1D.median_2 (lib/node.ml:183-198)
 * applied at every internal node of Tree.post_order_edges
 * (lib/tree.ml:171-187), node cost summed as in lib/node.ml:191.
 *   tips       [n_tips][n_words] packed state sets, n_words = ceil(n_sites*lane_bits/32)
 *   weights    [n_sites] per-site weights, or NULL for 1
 *   node_sets  [n_tips-1][n_words] out: state set of internal node k in row k
 *   site_cost  [n_sites] out (or NULL): number of internal nodes at which
 *              site s took the union
 *   total      out: sum_s weights[s] * site_cost[s] (a per-site count is at
 *              most n_tips-1, so it always fits uint32; the total is exact
 *              while it stays below 2^64)
 * Below 64-bit lanes, when tips and node_sets both lie in page-locked host
 * memory the device can address (cudaMallocHost, cudaHostAlloc,
 * cudaHostRegister), start on 16-byte boundaries and n_words is a multiple
 * of 4, the kernel reads the tips and writes the node sets in host memory
 * itself over the CPU-GPU link, both directions at once.  Otherwise the
 * rows are copied in column chunks on two further streams of the context,
 * so the copies in and out overlap each other and the kernels (pinned host
 * memory lets them run asynchronously).  The call returns once every
 * output is written. */
pgpu_status pgpu_fitch_tree(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                            const uint32_t *weights, size_t n_sites, int lane_bits,
                            uint32_t *node_sets, uint32_t *site_cost, uint64_t *total);

/* Launch shape of the Fitch tree kernel on this context: the words of a
 * state-set row each CTA covers (a multiple of 4 in 32..256; above 128 each
 * lane carries two groups of 4 words).  0, the default, picks the width per
 * launch: of 128..256, the one that gives the busiest SM the fewest words.
 * A width whose stacks do not fit shared memory falls back to 128.  Results
 * do not depend on it; the time does, through how evenly the CTAs fall on
 * the SMs and how many words each step covers, so an autotuner picks it by
 * timing (fitch.autotune_tile).  pgpu_get_fitch_tile_words returns the width
 * set, 0 for the default.  No reference counterpart. */
pgpu_status pgpu_set_fitch_tile_words(pgpu_ctx *ctx, int words);
int pgpu_get_fitch_tile_words(const pgpu_ctx *ctx);

/* Device-pointer form of pgpu_fitch_tree, asynchronous on the context's
 * stream.  Rows are ld_words apart (ld_words % 4 == 0, every pointer 16-byte
 * aligned); tree arrays are host pointers.  *total_dev is overwritten. */
pgpu_status pgpu_fitch_tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree,
                                const uint32_t *tips_dev, size_t ld_words,
                                const uint32_t *weights_dev, size_t n_sites,
                                int lane_bits, uint32_t *node_sets_dev,
                                uint32_t *site_cost_dev, uint64_t *total_dev);

/* No counterpart in the reference (phylocaml allocates a result per call,
 * lib/bitvector/bv.c:163-178).  pgpu_fitch_tree_dev for callers that may not
 * allocate device memory: a program that keeps the GPU's memory in its own
 * pool, or a service that forbids cudaMalloc once it is serving (an
 * allocation can synchronise the device).  It takes no context and
 * allocates nothing: its scratch (the tree's schedule and an error word)
 * lives in one fixed device array in the library, about 320 KB, held on
 * every GPU that loads the library until the process exits.
 *   - trees of at most 16,384 tips; larger ones return PGPU_ERR_LIMIT;
 *   - runs on cuda_stream (a cudaStream_t, or NULL for the legacy stream) of
 *     the current device and returns after that stream has finished;
 *     PGPU_ERR_TIMEOUT if a bounded device wait gave up;
 *   - all calls share the array: calls whose GPU work overlaps (other
 *     streams or host threads on the same device) race and must be
 *     serialised by the caller;
 *   - the first call in each device's context looks the array up with
 *     cudaGetSymbolAddress; make it before any stream capture starts.  A
 *     device reset between calls is not supported.
 * Arguments as for pgpu_fitch_tree_dev. */
pgpu_status pgpu_fitch_tree_noalloc(const pgpu_tree *tree, const uint32_t *tips_dev,
                                    size_t ld_words, const uint32_t *weights_dev,
                                    size_t n_sites, int lane_bits, uint32_t *node_sets_dev,
                                    uint32_t *site_cost_dev, uint64_t *total_dev,
                                    void *cuda_stream);

/* ---- cost-matrix (TCM) medians of state sets ----
 * The median rule a transformation cost matrix declares
 * (lib/costMatrix.ml:145-149): find_median_general (:68-86), _metric
 * (:104-122, medians drawn from the union of the two sets) or _equal
 * (:89-101, intersection or union at the matrix's equal / unequal cost). */
enum { PGPU_TCM_GENERAL = 0, PGPU_TCM_METRIC = 1, PGPU_TCM_EQUAL = 2 };

/* Host-only (ctx may be NULL): CostMatrix.Make.create (lib/costMatrix.ml:
 * 168-183, fill_cm :141-166) for a bit-flag alphabet of n_states (1..4)
 * atomic states.  tcm is the row-major n_states x n_states cost of atomic
 * state i to j, each in [0, 2^25].  For every pair of codes a, b in 0..15:
 *   table[a*16 + b]   packed for the kernels: cost << 4 | median code, or
 *                     0x80000000 where the pair has no median (a code 0 or
 *                     a code with bits at or above n_states);
 *   cost, assign      (optional) the same as plain integers, INT64_MAX / 0
 *                     where there is no median (the reference's inf, 0).
 * symmetric != 0 fills a <= b and mirrors it, as the reference does for a
 * matrix declared symmetric. */
pgpu_status pgpu_tcm_tables(pgpu_ctx *ctx, const int32_t *tcm, int n_states, int mode,
                            int symmetric, uint32_t *table, int64_t *cost, int32_t *assign);

/* A tree's postorder under a cost-matrix character (Node.Make1D.median_2,
 * lib/node.ml:183-198, with CostMatrix.Make.median, lib/costMatrix.ml:194):
 * internal node k takes table's median code of its children's codes and
 * adds table's cost.  Sites are 4-bit codes, eight to a word, as for
 * pgpu_fitch_tree with lane_bits 4; node_sets, site_cost and total as
 * there, site_cost[s] the sum of the costs over the internal nodes (the
 * call fails with PGPU_ERR_OVERFLOW if that could exceed 2^32 - 1).  A code
 * without a median in a site returns PGPU_ERR_ARG.  The rows are read and
 * written in page-locked host memory, or copied, as for pgpu_fitch_tree. */
pgpu_status pgpu_tcm_tree(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                          const uint32_t *weights, size_t n_sites, const uint32_t *table,
                          uint32_t *node_sets, uint32_t *site_cost, uint64_t *total);

/* Device-pointer form of pgpu_tcm_tree, asynchronous on the context's
 * stream; rows ld_words apart, table a host array of 256 entries (staged).
 * *total_dev is overwritten. */
pgpu_status pgpu_tcm_tree_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips_dev,
                              size_t ld_words, const uint32_t *weights_dev, size_t n_sites,
                              const uint32_t *table, uint32_t *node_sets_dev,
                              uint32_t *site_cost_dev, uint64_t *total_dev);

/* Cost-matrix medians for alphabets of up to 32 atomic states (the
 * reference's fill_cm takes any BitFlag alphabet, lib/costMatrix.ml:141-166,
 * e.g. Alphabet.aminoacids' 22 states, lib/alphabet.ml:328-343).  A table
 * over every pair of codes no longer fits, so each node forms its medians
 * from the TCM itself with the same rule (mode as for pgpu_tcm_tables;
 * symmetric != 0 orders each pair's codes first, as the reference's table
 * for a symmetric TCM is filled for i <= j and mirrored).  Sites are codes
 * of lane_bits (8, 16 or 32) bits, one site per lane as for pgpu_fitch_tree,
 * n_states <= lane_bits; tcm is the row-major n_states x n_states cost of
 * atomic state i to j, each in [0, 2^25].  node_sets, site_cost and total as
 * for pgpu_tcm_tree; a code of 0 or with bits at or above n_states returns
 * PGPU_ERR_ARG, and a tree whose per-site cost could exceed 2^32 - 1
 * PGPU_ERR_OVERFLOW. */
pgpu_status pgpu_tcm_tree_wide(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                               const uint32_t *weights, size_t n_sites, int lane_bits,
                               const int32_t *tcm, int n_states, int mode, int symmetric,
                               uint32_t *node_sets, uint32_t *site_cost, uint64_t *total);
/* Host-only (no context): the median cost and code of one pair of codes
 * under the rule, as CostMatrix.Make's cost / assign accessors read them
 * (lib/costMatrix.ml:192-194) for an alphabet of up to 32 states; a code of
 * 0 or with bits at or above n_states gives INT64_MAX and 0 (the
 * reference's inf, 0). */
pgpu_status pgpu_tcm_median(const int32_t *tcm, int n_states, int mode, int symmetric, uint32_t i,
                            uint32_t j, int64_t *cost, uint32_t *code);
/* Device-pointer form, asynchronous on the context's stream (rows ld_words
 * apart; tcm is a host array, staged). */
pgpu_status pgpu_tcm_tree_wide_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips_dev,
                                   size_t ld_words, const uint32_t *weights_dev, size_t n_sites,
                                   int lane_bits, const int32_t *tcm, int n_states, int mode,
                                   int symmetric, uint32_t *node_sets_dev, uint32_t *site_cost_dev,
                                   uint64_t *total_dev);

/* ---- substitution models and transition matrices (FP64 on the GPU) ----
 * Q is row-major, rows sum to zero, and reversible with respect to pi
 * (pi_i Q_ij = pi_j Q_ji) -- the models MlModel.create builds
 * (lib/mlModel.ml:664-746: JC69 ... GTR).  Non-reversible matrices are
 * rejected with PGPU_ERR_NONREVERSIBLE. */
typedef struct {
  int32_t n_states;      /* S */
  int32_t n_rates;       /* R, rate classes (DiscreteGamma/Custom, mlModel.mli:11-19) */
  const double *Q;       /* [S][S] */
  const double *pi;      /* [S] stationary frequencies (priors) */
  const double *rates;   /* [R] rate multipliers */
  const double *probs;   /* [R] class probabilities */
} pgpu_model;

/* Partial likelihood of each tip code: row c is the vector a tip with code
 * c contributes (1 for every state the code allows; all ones for a gap
 * treated as missing). */
typedef struct {
  int32_t n_codes;       /* 1..256 */
  const double *table;   /* [n_codes][S] */
} pgpu_tip_codes;

/* MlModel.diagonalize (lib/mlModel.ml:554-583; likelihood_CAML_diagonalize_gtr
 * and _sym, lib/mlmodel.c:200-271): Q = U diag(lambda) Ui, row-major, on
 * the GPU in FP64 (Jacobi on Pi^1/2 Q Pi^-1/2).  S <= 64. */
pgpu_status pgpu_model_diagonalize(pgpu_ctx *ctx, const double *Q, const double *pi, int S,
                                   double *U, double *lambda, double *Ui);

/* MlModel.compose for n_t branch lengths (lib/mlModel.ml:585-587;
 * compose_gtr, lib/mlmodel.c:325-342): P_out[k] = U diag(exp(lambda t[k])) Ui,
 * row-major, P[i][j] = Pr(j | i, t).  t == -1 returns Q, t < 1e-10 the
 * identity, as the reference does. */
pgpu_status pgpu_model_compose(pgpu_ctx *ctx, const double *U, const double *lambda,
                               const double *Ui, int S, const double *t, size_t n_t,
                               double *P_out);

/* The reference's own four externals, at their arity (declared at
 * lib/mlModel.ml:73-90 and called by MlModel.diagonalize / compose,
 * lib/mlModel.ml:554-587), so an OCaml stub binds them without changing
 * mlModel.ml.  Matrices are row-major n x n FP64 (C-layout Bigarrays), 1 <= n
 * <= 64; the work runs on the GPU in FP64.
 *
 * likelihood_CAML_diagonalize_gtr (lib/mlmodel.c:208-262, 265-271): U holds
 * Q on entry and receives the eigenvectors; D (filled with zeros by the
 * caller in the reference) receives the eigenvalues on its diagonal and
 * zeros elsewhere; Ui receives U's inverse; Q = U D Ui.  Q must be
 * reversible: its stationary distribution is found on the GPU (no pi
 * argument is needed) and used to symmetrise Q for the Jacobi solver.  A Q
 * without a stationary distribution above zero, or not reversible, returns
 * PGPU_ERR_NONREVERSIBLE; NaN or Inf returns PGPU_ERR_NAN. */
pgpu_status pgpu_diagonalize_gtr(pgpu_ctx *ctx, double *U, double *D, double *Ui, int n);

/* likelihood_CAML_diagonalize_sym (lib/mlmodel.c:163-197, 200-205): U holds
 * a symmetric Q on entry (only its lower triangle is read, the triangle
 * dsyev('U') reads in column-major order) and receives the orthonormal
 * eigenvectors as ROWS, in ascending order of eigenvalue; D the eigenvalues
 * on its diagonal.  Q = U^T D U. */
pgpu_status pgpu_diagonalize_sym(pgpu_ctx *ctx, double *U, double *D, int n);

/* likelihood_CAML_compose_gtr (lib/mlmodel.c:325-342, 344-365):
 * P = U exp(D t) Ui (only D's diagonal is read); t == -1 gives Q = U D Ui,
 * t < 1e-10 the identity. */
pgpu_status pgpu_compose_gtr(pgpu_ctx *ctx, const double *U, const double *D, const double *Ui,
                             int n, double t, double *P);

/* likelihood_CAML_compose_sym (lib/mlmodel.c:280-302, 304-323):
 * P = U^T exp(D t) U for U from pgpu_diagonalize_sym.  t is rounded to
 * float first, as the reference's `const float t` parameter does; then -1
 * gives Q and anything below 1e-10 the identity. */
pgpu_status pgpu_compose_sym(pgpu_ctx *ctx, const double *U, const double *D, int n, double t,
                             double *P);

/* ---- Felsenstein pruning -------------------------------------------------
 * The tree log-likelihood that Likelihood_c.median_2 / root_cost would
 * compute (lib/likelihood_c.ml:15-21, stubs in the reference) for
 * n_pat weighted site patterns:
 *   tip_codes  [n_tips][n_pat] codes into codes->table
 *   weights    [n_pat] pattern weights, or NULL for 1
 *   precision  32: FP32 conditional likelihoods (P - I rounded once to FP32);
 *              48: FP32 pairs -- every value an unevaluated sum of two
 *              floats, every sum and product error-free, about 48
 *              significant bits, on the FP32 units;
 *              64: the FP64 form.  P matrices are always built in FP64 on
 *              the GPU; the log-likelihood is always summed in FP64 with
 *              compensation.
 *   lnl        out: sum_s weights[s] * site_lnl[s]
 *   site_lnl   [n_pat] out (or NULL)
 * tree->brlen is required.  This entry point takes S = 4 (DNA); 20- and
 * 61-state models go through the batched tensor-core path.  The tip codes
 * are copied in column chunks on a second stream of the context, so the
 * copy overlaps the scoring (pinned host memory lets the copies run
 * asynchronously): the first chunk is one wave of the scoring kernel's
 * CTAs, each next a fixed factor larger.  The call returns once lnl is
 * written. */
pgpu_status pgpu_prune_lnl(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *model,
                           const pgpu_tip_codes *codes, const uint8_t *tip_codes,
                           const double *weights, size_t n_pat, int precision, double *lnl,
                           double *site_lnl);

/* Device-pointer form, asynchronous on the context's stream: tip rows
 * ld_pat bytes apart (ld_pat % 16 == 0, 16-byte aligned), *lnl_dev a
 * device double.  tree, model and codes stay host structures. */
pgpu_status pgpu_prune_lnl_dev(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *model,
                               const pgpu_tip_codes *codes, const uint8_t *tip_codes_dev,
                               size_t ld_pat, const double *weights_dev, size_t n_pat,
                               int precision, double *lnl_dev, double *site_lnl_dev);

/* Many models over one tree and one set of patterns in one pruning launch
 * (lnl[v] for models[v]; every model of S = 4 states and the same number of
 * rate classes): the 2k + 1 perturbed models of a central-difference
 * gradient of MlModel's parameters (the hooks gen_subst_opt_func /
 * gen_rates_opt_func / gen_prior_opt_func are a TODO in the reference,
 * lib/mlModel.ml:822-829), or any set of candidate models.  The host form
 * copies tip_codes and weights as pgpu_prune_lnl does and fills the host
 * array lnl[n_models]; the device form writes lnl_dev[n_models]
 * asynchronously. */
pgpu_status pgpu_prune_lnl_models(pgpu_ctx *ctx, const pgpu_tree *tree, const pgpu_model *models,
                                  int n_models, const pgpu_tip_codes *codes,
                                  const uint8_t *tip_codes, const double *weights, size_t n_pat,
                                  int precision, double *lnl);
pgpu_status pgpu_prune_lnl_models_dev(pgpu_ctx *ctx, const pgpu_tree *tree,
                                      const pgpu_model *models, int n_models,
                                      const pgpu_tip_codes *codes, const uint8_t *tip_codes_dev,
                                      size_t ld_pat, const double *weights_dev, size_t n_pat,
                                      int precision, double *lnl_dev);

/* ---- Likelihood_c one node at a time (NodeData.S) ------------------------
 * The operator Node.Make1D applies per node (median_2 : m -> t option -> t
 * -> t -> t, median_1, median_3, cost, root_cost; lib/nodeData.ml:20-30),
 * whose Likelihood_c slot is `failwith "TODO"` in the reference
 * (lib/likelihood_c.ml:14-21).  pgpu_prune_lnl scores a whole tree in one
 * launch and is the fast path; these calls let a caller fold the postorder
 * itself, node by node, with the vectors staying on the GPU.
 *   pgpu_lk   the m: model eigen system (FP64, on the GPU), rate classes,
 *             tip-code table, and the character block's n_pat patterns and
 *             weights (host arrays, copied; weights NULL for 1);
 *   pgpu_clv  a t: one node's conditional likelihoods [n_pat][R][S] on the
 *             device, stored in float (precision 32) or double (64), each
 *             pattern normalised by an exact power of two so that its
 *             largest entry lies in [1/2, 1), plus the length of the branch
 *             above the node (pgpu_clv_set_brlen) and its P matrices.
 * The costs: pgpu_clv_cost of an internal node is what its normalisation
 * moved out of the likelihood, -ln 2 sum_p w_p e_p; pgpu_clv_root_cost is
 * -sum_p w_p log(sum_r probs_r sum_i pi_i x[p][r][i]).  The costs of all
 * internal nodes plus the root's root_cost equal -lnL, the sum of node
 * costs that lib/node.ml:191 forms.  Leaves cost 0.
 * median calls are asynchronous on the context's stream; cost and
 * root_cost synchronise.  `reuse` is the reference's `t option`: the node's
 * previous value, whose device memory the result takes over (the result is
 * then that same handle); NULL allocates a new handle (stream-ordered).
 * Destroy every handle of a pgpu_lk before the pgpu_lk itself.  2..64
 * states, 1..8 rate classes. */
typedef struct pgpu_lk pgpu_lk;
typedef struct pgpu_clv pgpu_clv;

pgpu_status pgpu_lk_create(pgpu_ctx *ctx, const pgpu_model *model, const pgpu_tip_codes *codes,
                           size_t n_pat, const double *weights, int precision, pgpu_lk **out);
void pgpu_lk_destroy(pgpu_lk *lk);
/* A leaf: codes is a host array [n_pat] of rows of the tip-code table.
 * Its branch length is 0 until set. */
pgpu_status pgpu_clv_leaf(pgpu_lk *lk, pgpu_clv *reuse, const uint8_t *codes, pgpu_clv **out);
/* Length of the branch above the node (>= 0); builds that branch's P
 * matrices in FP64 on the GPU.  A node must have one before it is used as
 * a neighbour. */
pgpu_status pgpu_clv_set_brlen(pgpu_clv *t, double brlen);
pgpu_status pgpu_clv_get_brlen(const pgpu_clv *t, double *brlen);
/* median_1: P(t_a) a.  median_2: (P(t_a) a) * (P(t_b) b).  median_3: the
 * same over three neighbours (an unrooted tree's node). */
pgpu_status pgpu_clv_median1(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *a, pgpu_clv **out);
pgpu_status pgpu_clv_median2(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *a, const pgpu_clv *b,
                             pgpu_clv **out);
pgpu_status pgpu_clv_median3(pgpu_lk *lk, pgpu_clv *reuse, const pgpu_clv *a, const pgpu_clv *b,
                             const pgpu_clv *c, pgpu_clv **out);
pgpu_status pgpu_clv_cost(pgpu_clv *t, double *cost);
/* The costs of n nodes of one pgpu_lk at once (costs[i] of nodes[i]), with
 * one synchronisation: what Node.Make1D's sum over a tree's nodes needs
 * (lib/node.ml:191). */
pgpu_status pgpu_clv_costs(pgpu_lk *lk, const pgpu_clv *const *nodes, size_t n, double *costs);
/* site_lnl (host [n_pat], or NULL) receives each pattern's lnL at this
 * root. */
pgpu_status pgpu_clv_root_cost(pgpu_clv *t, double *cost, double *site_lnl);
void pgpu_clv_destroy(pgpu_clv *t);

/* ---- batched scoring of many trees and models --------------------------
 * One variant = one tree, one model and its own site patterns; the batch
 * holds any mix, e.g. 20-state protein models with 4 rate classes and
 * 61-state codon models, with uneven pattern counts.  No reference
 * counterpart beyond Likelihood_c's slot (lib/likelihood_c.ml:1-33): the
 * reference scores one tree at a time. */
typedef struct {
  pgpu_tree tree;            /* brlen required; 2..255 tips */
  pgpu_model model;          /* 2..64 states, 1..4 rate classes */
  pgpu_tip_codes codes;      /* 1..255 codes */
  const uint8_t *tip_codes;  /* DEVICE [n_tips][ld_pat] codes (pad with any valid code) */
  const double *weights;     /* DEVICE [n_pat] or NULL */
  size_t n_pat;
  size_t ld_pat;             /* row stride in bytes: multiple of 128, >= n_pat rounded up to 128 */
} pgpu_variant;

typedef struct pgpu_batch pgpu_batch;

/* Validates the variants, builds their schedules, and solves the models'
 * eigen systems (FP64, on the GPU).  The device buffers the variants point
 * to must outlive the batch. */
pgpu_status pgpu_batch_create(pgpu_ctx *ctx, const pgpu_variant *variants, int n_variants,
                              pgpu_batch **out);

/* Launch-shape options of a batch, for an autotuner to choose between
 * (results are the same to rounding, since each variant's sum runs in tile
 * order whatever the work order):
 *   rate_pairs  non-zero: two rate classes share a pass where their vectors
 *               fit in tensor memory together (the default); zero: one
 *               rate class per pass;
 *   order       PGPU_BATCH_ORDER_VARIANT: (variant, tile) items in variant
 *               order, the persistent CTAs striding over them (the default);
 *               PGPU_BATCH_ORDER_COST: items by estimated cost, largest
 *               first, dealt back and forth over the CTAs. */
enum { PGPU_BATCH_ORDER_VARIANT = 0, PGPU_BATCH_ORDER_COST = 1 };
typedef struct {
  int rate_pairs;
  int order;
} pgpu_batch_options;
pgpu_status pgpu_batch_create_opts(pgpu_ctx *ctx, const pgpu_variant *variants, int n_variants,
                                   const pgpu_batch_options *options, pgpu_batch **out);
void pgpu_batch_destroy(pgpu_batch *batch);

/* Scores every variant, asynchronously on the context's stream and without
 * host synchronisation or allocation, so the call can be captured in a CUDA
 * graph: FP64 P matrices, then one persistent tensor-core launch
 * (tcgen05.mma kind::tf32, FP32 accumulate, FP32 vectors, per-pattern power-
 * of-two scalers), then the per-variant compensated sums into
 * lnl_dev[n_variants]; site_lnl_dev (or NULL) receives every pattern's lnL,
 * variants one after another. */
pgpu_status pgpu_batch_run(pgpu_ctx *ctx, pgpu_batch *batch, double *lnl_dev,
                           double *site_lnl_dev);

/* The FP64 comparison form over the first `sample` patterns of every variant
 * (lnl_dev[v] = weighted FP64 lnL of those patterns). */
pgpu_status pgpu_batch_run_fp64(pgpu_ctx *ctx, pgpu_batch *batch, size_t sample, double *lnl_dev);

long long pgpu_batch_work_items(const pgpu_batch *batch);
long long pgpu_batch_patterns(const pgpu_batch *batch);

/* ---------------------------------------------------------------------------
 * SPR rearrangements (Tree.break / Tree.join, lib/tree.ml:299-494; the
 * neighbourhood enumerators lib/treeNeighborhoods.ml:27-75 are TODOs there)
 *
 * An engine holds one unrooted tree over fixed DNA data (4 states, 1..8 rate
 * classes) and, on the GPU, the conditional likelihood vectors of both sides
 * of every edge.  A move (p, u, c, y) cuts edge (p,u), carries p's side away,
 * joins u's two other neighbours into one edge (lengths added) and puts u in
 * the middle of edge (c,y) (half its length on each side); the pruned branch
 * keeps its length.  Moves are listed in a fixed order per tree; indices refer
 * to the current tree's list.  `precision` is 32, 48 (float pairs) or 64, as
 * for pgpu_prune_lnl.
 * ------------------------------------------------------------------------- */
typedef struct pgpu_spr pgpu_spr;

/* tip_codes_dev: DEVICE [n_tips][ld_pat]; weights_dev: DEVICE [n_pat] or NULL
 * (all 1); both must outlive the engine. */
pgpu_status pgpu_spr_create(pgpu_ctx *ctx, const pgpu_model *model, const pgpu_tip_codes *codes,
                            int32_t n_tips, const uint8_t *tip_codes_dev, size_t ld_pat,
                            const double *weights_dev, size_t n_pat, int precision,
                            pgpu_spr **out);
void pgpu_spr_destroy(pgpu_spr *spr);
/* The tree as a rooted postorder (root ignored: its two branches become one
 * edge); brlen required. */
pgpu_status pgpu_spr_set_tree(pgpu_spr *spr, const pgpu_tree *tree);
/* The current tree, rooted on the edge above tip 0 (half of it each side):
 * left/right [n_tips-1], brlen [2 n_tips - 2]. */
pgpu_status pgpu_spr_get_tree(pgpu_spr *spr, int32_t *left, int32_t *right, double *brlen);
/* lnL of the current tree (host scalar) and optionally every pattern's. */
pgpu_status pgpu_spr_lnl(pgpu_spr *spr, double *lnl, double *site_lnl);
/* Limits the neighbourhood to regraft edges at most join_distance nodes from
 * the break (0, the default: every SPR move; 1: the NNI moves, each NNI tree
 * four times).  It mirrors TreeNeighborhoods.generate_spr ?join_distance and
 * generate_nni (lib/treeNeighborhoods.ml:71-75) and holds until changed. */
pgpu_status pgpu_spr_set_join_distance(pgpu_spr *spr, int join_distance);
pgpu_status pgpu_spr_n_moves(pgpu_spr *spr, size_t *n_moves);
/* Node ids of every move, in the numbering of pgpu_spr_get_tree. */
pgpu_status pgpu_spr_moves(pgpu_spr *spr, int32_t *p, int32_t *u, int32_t *c, int32_t *y, size_t cap);
/* lnL of the tree after each move (no branch-length optimisation), into
 * DEVICE lnl_dev[n_moves]. */
pgpu_status pgpu_spr_scan(pgpu_spr *spr, double *lnl_dev);
/* The same for k chosen moves only; lnl is a host array [k]. */
pgpu_status pgpu_spr_score(pgpu_spr *spr, const int64_t *move_idx, size_t k, double *lnl);
/* Fitch (parsimony) length of the tree after each move into DEVICE
 * len_dev[n_moves]; tree_len receives the current tree's. */
pgpu_status pgpu_spr_fitch(pgpu_spr *spr, uint64_t *len_dev, uint64_t *tree_len);
/* 64 FP32 features per move into DEVICE X_dev[n_moves][64]: subtree sizes,
 * the branch lengths at the prune and regraft points, the Fitch length
 * change, and pattern-averaged state profiles of the sides involved. */
pgpu_status pgpu_spr_features(pgpu_spr *spr, float *X_dev);
pgpu_status pgpu_spr_apply(pgpu_spr *spr, int64_t move_idx);

/* TBR (tree bisection and reconnection), the moves that reroot both sides:
 * cut an edge (a,b) whose ends are both internal, dissolve a and b (each
 * one's two other edges become one, lengths added), put a in the middle of
 * an edge (jc,jy) of its side and b in the middle of an edge (kc,ky) of its
 * side, and keep the cut edge's length between them.  Rerooting one side
 * only gives the SPR moves above, so the two lists together are the TBR
 * neighbourhood.  The reference's TreeNeighborhoods.generate_tbr
 * ?join_distance ?reroot_distance is a TODO (lib/treeNeighborhoods.ml:27-69);
 * `distance` limits both attach edges to that many nodes from the cut (0:
 * no limit).  Moves are listed per cut edge, a's attach edge major. */
pgpu_status pgpu_spr_set_tbr_distance(pgpu_spr *spr, int distance);
/* The two limits of generate_tbr ?join_distance ?reroot_distance
 * (lib/treeNeighborhoods.ml:27-75): a cut leaves two sides, either of which
 * may be the one moved, so a move is listed when one side's attach edge lies
 * within join_distance of the cut and the other's within reroot_distance (0:
 * no limit).  pgpu_spr_set_tbr_distance(d) is (d, d).  Moves stay in the same
 * order, those outside the limits left out. */
pgpu_status pgpu_spr_set_tbr_limits(pgpu_spr *spr, int join_distance, int reroot_distance);
/* Device bytes for the attach vectors of one batch of cut edges (0: 2 GB);
 * a scan runs as many batches as it needs, at least one cut each.  A cut
 * needs (attach edges on both sides) x n_pat x n_rates x 4 values of the
 * form (4 bytes for precision 32, 8 otherwise), plus 4 bytes of scaler per
 * attach edge and pattern, whatever the budget: about 3 GB for the middle
 * cut of a 256-taxon tree at 45,675 patterns in the float-pair form.  A cut
 * that does not fit on the device fails with the allocation's error. */
pgpu_status pgpu_spr_set_tbr_budget(pgpu_spr *spr, size_t bytes);
pgpu_status pgpu_spr_tbr_n_moves(pgpu_spr *spr, size_t *n_moves);
/* Node ids of every TBR move (arrays [n_moves]), numbered as by
 * pgpu_spr_get_tree. */
pgpu_status pgpu_spr_tbr_moves(pgpu_spr *spr, int32_t *a, int32_t *b, int32_t *jc, int32_t *jy,
                               int32_t *kc, int32_t *ky, size_t cap);
/* lnL of the tree after each TBR move into DEVICE lnl_dev[n_moves]. */
pgpu_status pgpu_spr_tbr_scan(pgpu_spr *spr, double *lnl_dev);
pgpu_status pgpu_spr_tbr_apply(pgpu_spr *spr, int64_t move_idx);
/* Newton steps on all branch lengths at once, up to `passes` rounds or until
 * a round gains less than tol; lnl (or NULL) receives the final lnL. */
pgpu_status pgpu_spr_optimize(pgpu_spr *spr, int passes, double tol, double *lnl);
/* Edge lengths and endpoints of the engine's unrooted tree [2 n_tips - 3]. */
pgpu_status pgpu_spr_lengths(pgpu_spr *spr, double *len, int32_t *ea, int32_t *eb);

/* ---------------------------------------------------------------------------
 * Learned SPR ranking: BF16 MLP 64 -> 256 -> 256 -> 256 -> 1 (GELU), FP32
 * accumulation on the tensor cores (tcgen05.mma kind::f16), FP32 master
 * weights, AdamW.  Inputs are the 64 move features of pgpu_spr_features,
 * normalised per column with statistics set by pgpu_mlp_fit_norm.  The flat
 * parameter vector is W1[256][64], b1[256], W2[256][256], b2, W3[256][256],
 * b3, w4[256], b4.
 * ------------------------------------------------------------------------- */
typedef struct pgpu_mlp pgpu_mlp;

long long pgpu_mlp_n_params(void);
/* He-uniform weights from `seed`; training batches of up to max_batch rows. */
pgpu_status pgpu_mlp_create(pgpu_ctx *ctx, uint64_t seed, int max_batch, pgpu_mlp **out);
void pgpu_mlp_destroy(pgpu_mlp *mlp);
pgpu_status pgpu_mlp_get_params(pgpu_mlp *mlp, float *host);
pgpu_status pgpu_mlp_set_params(pgpu_mlp *mlp, const float *host);
pgpu_status pgpu_mlp_get_norm(pgpu_mlp *mlp, float *mu, float *inv_sd);
/* column means and inverse standard deviations of DEVICE X_dev[n][64] */
pgpu_status pgpu_mlp_fit_norm(pgpu_mlp *mlp, const float *X_dev, size_t n);
/* y_dev[n] = network(X_dev[n][64]) (device arrays, asynchronous) */
pgpu_status pgpu_mlp_forward(pgpu_mlp *mlp, const float *X_dev, size_t n, float *y_dev);
/* Gradients of sum_i sw_i (y_i - t_i)^2 / sum_i sw_i (sw_dev NULL: all 1)
 * into the host vector grad[n_params]; loss (or NULL) gets the loss. */
pgpu_status pgpu_mlp_grads(pgpu_mlp *mlp, const float *X_dev, const float *t_dev, const float *sw_dev,
                           size_t n, float *grad, float *loss);
/* One AdamW step (beta 0.9 / 0.999, eps 1e-8, decoupled weight decay on the
 * weight matrices) on that loss; loss (or NULL: no synchronisation). */
pgpu_status pgpu_mlp_train_step(pgpu_mlp *mlp, const float *X_dev, const float *t_dev,
                                const float *sw_dev, size_t n, float lr, float weight_decay,
                                float *loss);

/* Random-addition parsimony tree (host only): taxa join in a seeded random
 * order, each where it adds the fewest Fitch steps.  tip_codes is HOST
 * [n_tips][ld]; code_mask[c] holds the state bits of code c; every branch
 * gets length brlen.  length (or NULL) receives the tree's Fitch length. */
pgpu_status pgpu_parsimony_stepwise(int32_t n_tips, const uint8_t *tip_codes, size_t ld,
                                    size_t n_pat, const uint8_t *code_mask, int n_codes,
                                    const double *weights, uint64_t seed, double brlen,
                                    int32_t *left, int32_t *right, double *brlen_out,
                                    uint64_t *length);

#ifdef __cplusplus
}
#endif
#endif /* PHYLO_GPU_H */
