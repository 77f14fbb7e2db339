"""MlModel for the GPU (lib/mlModel.ml, lib/mlModel.mli).

The specification types and ``create`` follow the reference: the rate matrix
Q of each substitution model is assembled on the host in FP64 exactly as
lib/mlModel.ml does (off-diagonal rates times the target frequency, diagonal
the negative row sum, then mean rate normalised to 1, m_meanrate
lib/mlModel.ml:204-213), and the eigendecomposition (``diagonalize``) and
``compose`` run on the GPU in FP64 through the C ABI.

Supported: JC69, F81, K2P, F84, HKY85, TN93, GTR and Const (a given matrix,
m_file lib/mlModel.ml:473-488) with gaps as missing data; site variation
Constant, DiscreteGamma(k, alpha) and DiscreteCustom.  DiscreteGamma uses the
means of k equal-probability categories (Yang 1994), which is what
lib/mlModel.mli:12-13 documents and test/mlModelTest.ml:44-60 checks (mean
rate 1); the reference's own gamma_rates (lib/mlModel.ml:93-99) takes
quantiles at i/k instead and gives a first rate of 0 -- ``gamma_rates_quantile``
reproduces that for comparison.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native

MINIMUM = 1e-13          # lib/mlModel.ml:8
EPSILON_FLOAT = 2.220446049250313e-16


class Error(ValueError):
    """MlModel.Error (lib/mlModel.ml:3)."""


@dataclass
class Spec:
    """MlModel.s (lib/mlModel.ml:38-44) for a gap-as-missing alphabet."""
    substitution: tuple                 # ("JC69",) ("F81",) ("K2P", b) ("F84", k) ("HKY85", k)
                                        # ("TN93", (a, b)) ("GTR", co) ("Const", matrix)
    site_variation: tuple = ("Constant",)   # ("DiscreteGamma", k, alpha) | ("DiscreteCustom", [(r, p)])
                                            # | ("DiscreteTheta", k, alpha, pinvar)
    base_priors: object = "Equal"           # "Equal" | ("Empirical", freqs)
    alphabet_size: int = 4


@dataclass
class Model:
    """MlModel.t (lib/mlModel.ml:53-63) with the eigen system from the GPU."""
    spec: Spec
    priors: np.ndarray
    rates: np.ndarray
    probs: np.ndarray
    q: np.ndarray
    u: np.ndarray
    lam: np.ndarray
    ui: np.ndarray
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_states(self) -> int:
        return self.q.shape[0]

    def to_pgpu(self):
        """(pgpu_model struct, keepalive list)."""
        q = np.ascontiguousarray(self.q, np.float64)
        pi = np.ascontiguousarray(self.priors, np.float64)
        r = np.ascontiguousarray(self.rates, np.float64)
        p = np.ascontiguousarray(self.probs, np.float64)
        m = _native.PgpuModel()
        m.n_states = q.shape[0]
        m.n_rates = len(r)
        dp = C.POINTER(C.c_double)
        m.Q, m.pi, m.rates, m.probs = (a.ctypes.data_as(dp) for a in (q, pi, r, p))
        return m, [q, pi, r, p]


# ---- rate matrices (host FP64, as lib/mlModel.ml assembles them) ----------

def m_meanrate(srm: np.ndarray, pi: np.ndarray) -> np.ndarray:
    mr = float(np.sum(-np.diag(srm) * pi))
    return srm / mr


def _fill_diag(srm: np.ndarray) -> np.ndarray:
    np.fill_diagonal(srm, 0.0)
    np.fill_diagonal(srm, -srm.sum(axis=1))
    return srm


def m_jc69(a: int) -> np.ndarray:
    srm = np.ones((a, a))
    np.fill_diagonal(srm, -(a - 1.0))
    return m_meanrate(srm, np.full(a, 1.0 / a))


def m_k2p(beta: float, a: int) -> np.ndarray:
    if a != 4:
        raise Error("Alphabet does not support this model")
    beta = max(beta, MINIMUM)
    srm = np.full((a, a), beta)
    srm[1, 3] = srm[3, 1] = srm[2, 0] = srm[0, 2] = 1.0
    np.fill_diagonal(srm, -1.0 - 2.0 * beta)
    return m_meanrate(srm, np.full(a, 1.0 / a))


def m_tn93(pi: np.ndarray, alpha: float, beta: float, a: int) -> np.ndarray:
    if a != 4:
        raise Error("Alphabet size does not support this model")
    srm = np.ones((a, a))
    srm[0, 2] = srm[2, 0] = alpha
    srm[1, 3] = srm[3, 1] = beta
    srm = srm * pi[None, :]
    return m_meanrate(_fill_diag(srm), pi)


def m_f81(pi: np.ndarray, a: int) -> np.ndarray:
    srm = np.tile(pi, (a, 1)).astype(np.float64)
    return m_meanrate(_fill_diag(srm), pi)


def m_hky85(pi: np.ndarray, kappa: float, a: int) -> np.ndarray:
    return m_tn93(pi, kappa, kappa, a)


def m_f84(pi: np.ndarray, kappa: float, a: int) -> np.ndarray:
    y = pi[1] + pi[3]
    r = pi[0] + pi[2]
    return m_tn93(pi, 1.0 + kappa / r, 1.0 + kappa / y, a)


def m_gtr(pi: np.ndarray, co, a: int) -> np.ndarray:
    co = np.asarray(co, np.float64)
    want = ((a + 1) * (a - 2)) // 2
    if len(co) != want:
        raise Error(f"Length of GTR parameters (I) is incorrect for the alphabet. "
                    f"They should be {want}, but are {len(co)}.")
    full = np.append(co, 1.0)            # the last exchangeability is fixed to 1
    iu = np.triu_indices(a, 1)
    srm = np.zeros((a, a))
    srm[iu] = full * pi[iu[1]]
    srm[(iu[1], iu[0])] = full * pi[iu[0]]
    return m_meanrate(_fill_diag(srm), pi)


def m_file(pi: np.ndarray, f_rr, a: int) -> np.ndarray:
    f = np.asarray(f_rr, np.float64)
    if f.shape != (a, a):
        raise Error("Const matrix does not match the alphabet")
    return m_meanrate(_fill_diag(f.copy()), pi)


# ---- site rate classes ------------------------------------------------------

def gamma_rates(alpha: float, k: int) -> np.ndarray:
    """Mean rate of each of k equal-probability categories of Gamma(alpha,
    rate alpha) (Yang 1994); the rates average to 1."""
    from scipy.special import gammainc, gammaincinv
    if k == 1:
        return np.ones(1)
    cuts = np.append(gammaincinv(alpha, np.arange(1, k) / k) / alpha, np.inf)
    upper = np.append(gammainc(alpha + 1.0, alpha * cuts[:-1]), 1.0)
    lower = np.concatenate([[0.0], upper[:-1]])
    return k * (upper - lower)


def gamma_rates_quantile(alpha: float, k: int) -> np.ndarray:
    """The reference's gamma_rates (lib/mlModel.ml:93-99): the quantile at
    p = i/k of Gamma(shape alpha, scale alpha); rate 0 first."""
    from scipy.special import gammaincinv
    p = np.arange(k) / k
    return gammaincinv(alpha, p) * alpha


def _priors(spec: Spec) -> np.ndarray:
    a = spec.alphabet_size
    if spec.base_priors == "Equal":
        return np.full(a, 1.0 / a)
    kind, p = spec.base_priors
    p = np.maximum(np.asarray(p, np.float64), MINIMUM)
    s = p.sum()
    if abs(s - 1.0) >= EPSILON_FLOAT:       # `=.` (lib/internal.ml:12)
        p = p / s
    if len(p) != a:
        raise Error(f"Priors (length {len(p)}) don't match alphabet (length {a})")
    return p


def _site_classes(spec: Spec):
    sv = spec.site_variation
    if sv[0] == "Constant":
        return np.ones(1), np.ones(1)
    if sv[0] == "DiscreteGamma":
        k, alpha = sv[1], sv[2]
        return gamma_rates(alpha, k), np.full(k, 1.0 / k)
    if sv[0] == "DiscreteCustom":
        arr = np.asarray(sv[1], np.float64)
        return arr[:, 0].copy(), arr[:, 1].copy()
    if sv[0] == "DiscreteTheta":
        # (GAMMA_SITES, ALPHA, PERCENT_INVAR), lib/mlModel.ml:684-694: w Gamma
        # classes (one rate-1 class when w = 1) and the proportion of invariant
        # sites.  The reference's likelihood is a stub, so how that proportion
        # enters is not fixed there; here it is the usual mixture, an extra
        # class of rate 0 (P = I) with probability pinvar and the Gamma classes
        # sharing 1 - pinvar.
        w, alpha, pinv = int(sv[1]), float(sv[2]), float(sv[3])
        if w < 1:
            raise Error("Number of rate categories must be >= 1 (if invar w/out gamma)")
        if not 0.0 <= pinv < 1.0:
            raise Error("proportion of invariant sites must lie in [0, 1)")
        g = np.ones(1) if w == 1 else gamma_rates(alpha, w)
        return (np.concatenate([[0.0], g]),
                np.concatenate([[pinv], np.full(w, (1.0 - pinv) / w)]))
    raise Error(f"site variation {sv[0]} is not supported")


def substitution_matrix(spec: Spec, priors: np.ndarray) -> tuple[np.ndarray, bool]:
    """(Q, sym) as MlModel.create chooses them (lib/mlModel.ml:723-741)."""
    a = spec.alphabet_size
    s = spec.substitution
    name = s[0]
    if name == "JC69":
        return m_jc69(a), True
    if name == "K2P":
        return m_k2p(s[1], a), True
    if name == "F81":
        return m_f81(priors, a), False
    if name == "F84":
        return m_f84(priors, s[1], a), False
    if name == "HKY85":
        return m_hky85(priors, s[1], a), False
    if name == "TN93":
        return m_tn93(priors, s[1][0], s[1][1], a), False
    if name == "GTR":
        co = s[1] if len(s) > 1 and len(s[1]) else np.ones(((a - 2) * (a + 1)) // 2)
        return m_gtr(priors, co, a), False
    if name == "Const":
        return m_file(priors, s[1], a), False
    raise Error(f"substitution model {name} is not supported")


def diagonalize(q: np.ndarray, pi: np.ndarray, ctx: _native.Context | None = None):
    """GPU FP64 eigen system: (U, lambda, Ui) with Q = U diag(lambda) Ui."""
    if np.isnan(q).any():
        # MlModel.diagonalize asserts the matrix holds no NaN (lib/mlModel.ml:557-568)
        raise Error("rate matrix contains NaN")
    ctx = ctx or _native.default_context()
    S = q.shape[0]
    q = np.ascontiguousarray(q, np.float64)
    pi = np.ascontiguousarray(pi, np.float64)
    U = np.empty((S, S))
    lam = np.empty(S)
    Ui = np.empty((S, S))
    ctx.call("pgpu_model_diagonalize", q.ctypes.data, pi.ctypes.data, S, U.ctypes.data,
             lam.ctypes.data, Ui.ctypes.data)
    return U, lam, Ui


# ---- the reference's externals at their own arity (lib/mlModel.ml:73-90) ---
# Matrices are C-contiguous float64 [n, n] arrays, changed in place as the
# reference's Bigarrays are.

def _mat(a: np.ndarray, name: str) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.ndim == 2
            and a.shape[0] == a.shape[1] and a.flags.c_contiguous):
        raise Error(f"{name} must be a C-contiguous float64 square matrix")
    return a


def diagonalize_gtr(u: np.ndarray, d: np.ndarray, ui: np.ndarray,
                    ctx: _native.Context | None = None) -> None:
    """likelihood_CAML_diagonalize_gtr: ``u`` holds Q and becomes U, ``d``
    the diagonal matrix of eigenvalues, ``ui`` U's inverse (Q = U D Ui)."""
    n = _mat(u, "U").shape[0]
    if _mat(d, "D").shape[0] != n or _mat(ui, "Ui").shape[0] != n:
        raise Error("U, D and Ui must have the same size")
    ctx = ctx or _native.default_context()
    ctx.call("pgpu_diagonalize_gtr", u.ctypes.data, d.ctypes.data, ui.ctypes.data, n)


def diagonalize_sym(u: np.ndarray, d: np.ndarray, ctx: _native.Context | None = None) -> None:
    """likelihood_CAML_diagonalize_sym: ``u`` holds a symmetric Q and becomes
    the eigenvectors as rows (ascending eigenvalues), ``d`` the diagonal
    matrix of eigenvalues (Q = U^T D U)."""
    n = _mat(u, "U").shape[0]
    if _mat(d, "D").shape[0] != n:
        raise Error("U and D must have the same size")
    ctx = ctx or _native.default_context()
    ctx.call("pgpu_diagonalize_sym", u.ctypes.data, d.ctypes.data, n)


def compose_gtr(u: np.ndarray, d: np.ndarray, ui: np.ndarray, t: float,
                ctx: _native.Context | None = None) -> np.ndarray:
    """likelihood_CAML_compose_gtr: P = U exp(D t) Ui (Q for t == -1)."""
    n = _mat(u, "U").shape[0]
    _mat(d, "D"), _mat(ui, "Ui")
    ctx = ctx or _native.default_context()
    out = np.empty((n, n))
    ctx.call("pgpu_compose_gtr", u.ctypes.data, d.ctypes.data, ui.ctypes.data, n, float(t),
             out.ctypes.data)
    return out


def compose_sym(u: np.ndarray, d: np.ndarray, t: float,
                ctx: _native.Context | None = None) -> np.ndarray:
    """likelihood_CAML_compose_sym: P = U^T exp(D t) U, t rounded to float."""
    n = _mat(u, "U").shape[0]
    _mat(d, "D")
    ctx = ctx or _native.default_context()
    out = np.empty((n, n))
    ctx.call("pgpu_compose_sym", u.ctypes.data, d.ctypes.data, n, float(t), out.ctypes.data)
    return out


def diagonalize_matrix(sym: bool, mat: np.ndarray, ctx: _native.Context | None = None):
    """MlModel.diagonalize (lib/mlModel.ml:554-583) over the externals above:
    (U, D, Ui or None)."""
    if np.isnan(mat).any():
        raise Error("rate matrix contains NaN")
    n = mat.shape[0]
    u = np.ascontiguousarray(mat, np.float64).copy()
    d = np.zeros((n, n))
    if sym:
        diagonalize_sym(u, d, ctx)
        return u, d, None
    ui = np.zeros((n, n))
    diagonalize_gtr(u, d, ui, ctx)
    return u, d, ui


def compose_decomposed(decomp, t: float, ctx: _native.Context | None = None) -> np.ndarray:
    """MlModel.compose (lib/mlModel.ml:585-587) on diagonalize_matrix's
    result: compose_gtr when Ui is present, else compose_sym."""
    u, d, ui = decomp
    return compose_sym(u, d, t, ctx) if ui is None else compose_gtr(u, d, ui, t, ctx)


def create(spec: Spec, ctx: _native.Context | None = None, eigen: bool = True) -> Model:
    """MlModel.create (lib/mlModel.ml:664-746).  ``eigen=False`` leaves the
    eigen system to be solved when ``compose`` first needs it (the pruning
    entry points solve their own on the GPU)."""
    priors = _priors(spec)
    rates, probs = _site_classes(spec)
    q, sym = substitution_matrix(spec, priors)
    m = Model(spec, priors, rates, probs, q, None, None, None)
    if eigen:
        _solve(m, ctx)
    return m


def _solve(m: Model, ctx) -> None:
    # JC69 and K2P are symmetric (the reference diagonalises them with dsyev,
    # lib/mlmodel.c:163-197): their stationary distribution is uniform
    # whatever the priors field holds
    sym = m.spec is not None and m.spec.substitution[0] in ("JC69", "K2P")
    eq = np.full(m.n_states, 1.0 / m.n_states) if sym else m.priors
    m.u, m.lam, m.ui = diagonalize(m.q, eq, ctx)


def compose(model: Model, t, ctx: _native.Context | None = None) -> np.ndarray:
    """MlModel.compose (lib/mlModel.ml:585-587): P = exp(Q t), or Q for
    t == -1, I for t < 1e-10.  ``t`` may be a scalar or an array of lengths
    (then [n, S, S] is returned)."""
    ctx = ctx or _native.default_context()
    ts = np.atleast_1d(np.asarray(t, np.float64))
    S = model.n_states
    out = np.empty((len(ts), S, S))
    if model.u is None:
        _solve(model, ctx)
    ctx.call("pgpu_model_compose", model.u.ctypes.data, model.lam.ctypes.data,
             model.ui.ctypes.data, S, ts.ctypes.data, len(ts), out.ctypes.data)
    return out[0] if np.ndim(t) == 0 else out


# ---- model-parameter optimisation hooks ------------------------------------
# MlModel.gen_subst_opt_func / gen_rates_opt_func / gen_prior_opt_func
# (lib/mlModel.ml:822-829, "todo" in the reference): each returns the model's
# current free parameters as a vector and a function that builds the model
# for another vector.  Vectors are unconstrained, so any optimiser can move
# them: positive parameters (exchangeabilities, kappa, the Gamma shape) as
# logs, base frequencies as logs relative to the last state.

def _with(model: Model, ctx, **changes) -> Model:
    from dataclasses import replace
    return create(replace(model.spec, **changes), ctx, eigen=False)


def gen_subst_opt_func(model: Model, ctx: _native.Context | None = None):
    """Substitution parameters: GTR's free exchangeabilities (the last is fixed
    at 1, lib/mlModel.ml:396-400), kappa of K2P/F84/HKY85, (alpha, beta) of
    TN93; JC69, F81 and a given matrix have none."""
    s = model.spec.substitution
    a = model.spec.alphabet_size
    name = s[0]
    if name == "GTR":
        co = np.asarray(s[1] if len(s) > 1 and len(s[1]) else np.ones(((a - 2) * (a + 1)) // 2),
                        np.float64)
        return np.log(co), lambda x: _with(model, ctx, substitution=("GTR", list(np.exp(x))))
    if name in ("K2P", "F84", "HKY85"):
        return np.log([float(s[1])]), lambda x: _with(model, ctx, substitution=(name, float(np.exp(x[0]))))
    if name == "TN93":
        return (np.log([float(s[1][0]), float(s[1][1])]),
                lambda x: _with(model, ctx, substitution=(name, (float(np.exp(x[0])), float(np.exp(x[1]))))))
    return np.zeros(0), lambda x: model


def gen_rates_opt_func(model: Model, ctx: _native.Context | None = None):
    """Site-rate parameters: the shape of DiscreteGamma; the shape (when more
    than one class) and the invariant proportion (as a logit) of
    DiscreteTheta; Constant and a custom rate list have none."""
    sv = model.spec.site_variation
    if sv[0] == "DiscreteTheta":
        w, alpha, pinv = int(sv[1]), float(sv[2]), float(sv[3])
        if w > 1:
            return (np.array([np.log(alpha), np.log(pinv / (1.0 - pinv))]),
                    lambda x: _with(model, ctx, site_variation=(
                        "DiscreteTheta", w, float(np.exp(x[0])), float(1.0 / (1.0 + np.exp(-x[1]))))))
        return (np.array([np.log(pinv / (1.0 - pinv))]),
                lambda x: _with(model, ctx, site_variation=(
                    "DiscreteTheta", w, alpha, float(1.0 / (1.0 + np.exp(-x[0]))))))
    if sv[0] == "DiscreteGamma":
        k = sv[1]
        return np.log([float(sv[2])]), lambda x: _with(model, ctx,
                                                       site_variation=("DiscreteGamma", k, float(np.exp(x[0]))))
    return np.zeros(0), lambda x: model


def gen_prior_opt_func(model: Model, ctx: _native.Context | None = None):
    """Base frequencies: a - 1 log-ratios against the last state.  JC69 and
    K2P have uniform stationary frequencies whatever the priors field holds,
    so they have none."""
    if model.spec.substitution[0] in ("JC69", "K2P"):
        return np.zeros(0), lambda x: model
    pi = np.asarray(model.priors, np.float64)

    def build(x):
        e = np.exp(np.append(np.asarray(x, np.float64), 0.0))
        return _with(model, ctx, base_priors=("Empirical", list(e / e.sum())))

    return np.log(pi[:-1] / pi[-1]), build


HOOKS = {"subst": gen_subst_opt_func, "rates": gen_rates_opt_func, "prior": gen_prior_opt_func}


def lnl_and_gradient(x: np.ndarray, build, lnl_many, h: float = 1e-4, central: bool = True):
    """lnL at a hook's parameter vector x and its finite-difference gradient,
    from one batched evaluation (lnl_many: list of models -> array of lnL,
    e.g. likelihood.tree_lnl_models, which scores them all in one pruning
    launch): central differences from the 2k + 1 models build(x),
    build(x +- h e_i), or forward differences from the k + 1 models build(x),
    build(x + h e_i)."""
    x = np.asarray(x, np.float64)
    k = len(x)
    pts = [x] + [x + h * e for e in np.eye(k)]
    if central:
        pts += [x - h * e for e in np.eye(k)]
    vals = np.asarray(lnl_many([build(p) for p in pts]), np.float64)
    if central:
        grad = (vals[1:k + 1] - vals[k + 1:]) / (2.0 * h)
    else:
        grad = (vals[1:k + 1] - vals[0]) / h
    return float(vals[0]), grad


def optimize_model(model: Model, lnl_of=None, hooks=("subst", "rates", "prior"), rounds: int = 8,
                   tol: float = 1e-4, ctx: _native.Context | None = None, lnl_many=None,
                   central: bool = True):
    """Maximise the tree's lnL over the hooks' parameters, one hook at a time,
    until a round gains less than tol.  Returns (model, lnl, evaluations).

    With ``lnl_many`` (list of models -> array of lnL) every L-BFGS step takes
    the lnL and its gradient from one batched evaluation
    (``lnl_and_gradient``: 2k + 1 models for central differences, k + 1 with
    ``central=False``); otherwise ``lnl_of`` (model -> lnL) is called once
    per point, L-BFGS forming forward differences itself.  ``evaluations``
    counts models scored."""
    from scipy.optimize import minimize
    if lnl_of is None and lnl_many is None:
        raise ValueError("optimize_model needs lnl_of or lnl_many")
    calls = 0
    one = lnl_of if lnl_of is not None else (lambda m: float(lnl_many([m])[0]))
    best = one(model)
    calls += 1
    for _ in range(rounds):
        start = best
        for hname in hooks:
            x0, build = HOOKS[hname](model, ctx)
            if len(x0) == 0:
                continue
            if lnl_many is not None:
                def fg(x):
                    nonlocal calls
                    calls += (2 if central else 1) * len(x) + 1
                    f, g = lnl_and_gradient(x, build, lnl_many, central=central)
                    return -f, -g

                res = minimize(fg, x0, jac=True, method="L-BFGS-B", options={"maxiter": 60})
            else:
                cache = {}

                def neg(x):
                    nonlocal calls
                    key = tuple(np.round(x, 12))
                    if key not in cache:
                        calls += 1
                        cache[key] = -lnl_of(build(x))
                    return cache[key]

                res = minimize(neg, x0, method="L-BFGS-B", options={"eps": 1e-5, "maxiter": 60})
            if -res.fun > best:
                model, best = build(res.x), -res.fun
        if best - start < tol:
            break
    return model, best, calls
