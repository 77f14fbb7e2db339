// Launchers shared by the likelihood translation units (pmatrix.cu).
#pragma once
#include "pgpu_internal.cuh"

// Eigendecomposition of n_models reversible S x S rate matrices (device
// buffers).  status_dev[m] receives 0 or a PGPU_ERR_* code per model.
pgpu_status pgpu_launch_eig(pgpu_ctx *ctx, const double *Q_dev, const double *pi_dev, int S,
                            int n_models, double *U_dev, double *lam_dev, double *Ui_dev,
                            int *status_dev);

// P[b][r] = U diag(exp(lambda * rates[r] * t[b])) Ui for n_br branch lengths
// of one model; FP64 into P_dev and/or FP32 into P32_dev (either may be
// null).  With allow_q, t == -1 yields Q (MlModel.compose's special case).
// If status_dev is given and non-zero the matrices are not built and the
// context's error word records the model failure.  p32_mode selects the FP32
// copy: P, P - I (formed in FP64 before rounding, which keeps the small
// entries of short branches at full relative precision), or P as (hi, lo)
// float pairs in the pair form's row-pair layout.  n_models > 1 composes that many models in one
// launch: model m reads U, Ui at m*S*S, lam at m*S, rates at m*R and
// status_dev[m], and writes its matrices model_bytes further on than model
// m - 1's (the same byte stride for P_dev and P32_dev).
enum P32Mode {
  P32_PLAIN = 0,          // fl32(P)
  P32_MINUS_I = 1,        // fl32(P - I)
  // (hi, lo) float pairs of a 4 x 4 P, rows taken two at a time for packed
  // float2 arithmetic: float4 k = 4 (i / 2) + j of a block holds
  // {hi P[i][j], hi P[i+1][j], lo P[i][j], lo P[i+1][j]} for even i
  P32_PAIRS_ROWS4 = 4
};
pgpu_status pgpu_launch_compose(pgpu_ctx *ctx, const double *U_dev, const double *lam_dev,
                                const double *Ui_dev, int S, const double *t_dev, int n_br,
                                const double *rates_dev, int R, double *P_dev, float *P32_dev,
                                bool allow_q, const int *status_dev = nullptr,
                                int p32_mode = P32_PLAIN, int n_models = 1,
                                size_t model_bytes = 0);

// Tip rows tab[t][r][c][i] = (P(t, r) code_tab[c])[i] for the n_tips branches
// above the tips (t_dev holds their lengths), in FP64, stored as float
// (form 0), (hi, lo) float pairs (form 1), double (form 2), or for S = 4
// float pairs with the elements two at a time, {h0, h1, l0, l1}, {h2, h3,
// l2, l3} per code (form 3, the pair form's packed layout).  n_models and
// model_bytes batch models as in pgpu_launch_compose.
pgpu_status pgpu_launch_tip_table(pgpu_ctx *ctx, const double *U_dev, const double *lam_dev,
                                  const double *Ui_dev, int S, const double *t_dev, int n_tips,
                                  const double *rates_dev, int R, const double *code_tab_dev,
                                  int n_codes, void *out_dev, int form, const int *status_dev,
                                  int n_models = 1, size_t model_bytes = 0);
