"""GPU: the four MlModel externals at the reference's own arity.

likelihood_CAML_diagonalize_gtr : U D Ui, likelihood_CAML_diagonalize_sym :
U D, likelihood_CAML_compose_gtr : U D Ui t and likelihood_CAML_compose_sym :
U D t (lib/mlModel.ml:73-90, lib/mlmodel.c:200-365) go through the C ABI
with the reference's buffers and are checked against the LAPACK oracle,
which restates the reference's calls (dgeev / dsyev, dgetrf / dgetri, the
column-major conventions and compose_sym's float truncation of t).
Eigenvectors are not unique, so the composed matrices and the
reconstructions are what must agree.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlmodel_oracle as O
from phylocaml_gb300 import _native, mlmodel as M

pytestmark = pytest.mark.gpu

# mlModelTest.ml:5-7 lengths, -1 (Q itself), below and above EPSILON, and a
# length float32 rounds (0.1)
TS = [np.finfo(float).tiny, 0.0, 1e-11, 2e-10, 0.05, 0.1, 1.0, 100.0, -1.0]


def reversible_q(rng, S):
    pi = rng.dirichlet(np.ones(S))
    ex = rng.lognormal(size=(S, S))
    ex = (ex + ex.T) / 2
    q = ex * pi[None, :]
    np.fill_diagonal(q, 0.0)
    np.fill_diagonal(q, -q.sum(axis=1))
    return q / -(np.diag(q) * pi).sum(), pi


@pytest.mark.parametrize("name,q", [("JC69", O.m_jc69(4)), ("K2P", O.m_k2p(0.3, 4)),
                                    ("JC69-20", O.m_jc69(20))])
def test_sym_externals_match_oracle(ctx, name, q):
    u = np.ascontiguousarray(q).copy()
    d = np.zeros_like(u)
    M.diagonalize_sym(u, d, ctx)
    n = q.shape[0]
    # D diagonal, ascending (dsyev's order), U orthonormal rows, Q = U^T D U
    assert np.all(d[~np.eye(n, dtype=bool)] == 0.0)
    lam = np.diag(d)
    assert np.all(np.diff(lam) >= 0)
    assert np.abs(u @ u.T - np.eye(n)).max() < 1e-13
    assert np.abs(u.T @ d @ u - q).max() < 1e-13
    ou, od = O.diagonalize_sym(q)
    assert np.abs(np.diag(od) - lam).max() < 1e-13
    for t in TS:
        got = M.compose_sym(u, d, t, ctx)
        exp = O.compose_sym(ou, od, t)
        assert np.abs(got - exp).max() < 1e-12, (name, t)


def test_compose_sym_rounds_t_to_float(ctx):
    q = O.m_k2p(0.3, 4)
    u = q.copy()
    d = np.zeros_like(u)
    M.diagonalize_sym(u, d, ctx)
    t = 0.1
    t32 = float(np.float32(t))
    assert t32 != t
    # bit-identical: the same float length goes in either way
    assert np.array_equal(M.compose_sym(u, d, t, ctx), M.compose_sym(u, d, t32, ctx))
    # and that is the float length's matrix, not the double one's
    from scipy.linalg import expm
    assert np.abs(M.compose_sym(u, d, t, ctx) - expm(q * t32)).max() < 1e-13
    assert np.abs(expm(q * t32) - expm(q * t)).max() > 1e-10


@pytest.mark.parametrize("S,seed", [(4, 1), (4, 2), (20, 3), (61, 4), (64, 5)])
def test_gtr_externals_match_oracle(ctx, S, seed):
    rng = np.random.default_rng(seed)
    q, pi = reversible_q(rng, S)
    u = q.copy()
    d = np.full((S, S), 7.0)     # overwritten entirely
    ui = np.zeros((S, S))
    M.diagonalize_gtr(u, d, ui, ctx)
    assert np.all(d[~np.eye(S, dtype=bool)] == 0.0)
    assert np.abs(u @ d @ ui - q).max() < 1e-12
    assert np.abs(u @ ui - np.eye(S)).max() < 1e-12
    ou, od, oui = O.diagonalize_gtr(q)
    assert np.allclose(np.sort(np.diag(d)), np.sort(np.diag(od)), atol=1e-12)
    for t in TS:
        got = M.compose_gtr(u, d, ui, t, ctx)
        exp = O.compose_gtr(ou, od, oui, t)
        assert np.abs(got - exp).max() < 1e-12, (S, t)


@pytest.mark.parametrize("name", ["F81", "HKY85", "TN93", "GTR"])
def test_mlmodel_diagonalize_and_compose_over_externals(ctx, name):
    """MlModel.diagonalize false / compose over the externals equal the model
    that MlModel.create builds (which passes pi explicitly)."""
    pri = ("Empirical", [0.1, 0.2, 0.3, 0.4])
    specs = {"F81": M.Spec(("F81",), base_priors=pri), "HKY85": M.Spec(("HKY85", 2.0), base_priors=pri),
             "TN93": M.Spec(("TN93", (2.0, 3.0)), base_priors=pri),
             "GTR": M.Spec(("GTR", [1.1, 0.7, 1.9, 0.6, 1.4]), ("DiscreteGamma", 4, 0.5),
                           ("Empirical", [0.3, 0.2, 0.25, 0.25]))}
    m = M.create(specs[name], ctx)
    dec = M.diagonalize_matrix(False, m.q, ctx)
    for t in (0.0, 0.03, 0.7, -1.0):
        assert np.abs(M.compose_decomposed(dec, t, ctx) - M.compose(m, t, ctx)).max() < 1e-13


def test_externals_reject_bad_matrices(ctx):
    q = O.m_jc69(4)
    bad = q.copy()
    bad[1, 2] = np.nan
    with pytest.raises(_native.NativeError) as e:
        M.diagonalize_gtr(bad.copy(), np.zeros((4, 4)), np.zeros((4, 4)), ctx)
    assert e.value.status == 4
    # the symmetric external reads only the lower triangle (dsyev('U') on the
    # column-major view), so a NaN above the diagonal goes unseen, as there
    lower = q.copy()
    lower[2, 1] = np.nan
    with pytest.raises(_native.NativeError) as e:
        M.diagonalize_sym(lower, np.zeros((4, 4)), ctx)
    assert e.value.status == 4
    u = bad.copy()
    M.diagonalize_sym(u, np.zeros((4, 4)), ctx)
    assert np.isfinite(u).all()
    # not reversible: a cyclic flow 0 -> 1 -> 2 -> 3 -> 0 on top of JC69
    nr = q.copy()
    for i in range(4):
        nr[i, (i + 1) % 4] += 0.5
        nr[i, i] -= 0.5
    with pytest.raises(_native.NativeError) as e:
        M.diagonalize_gtr(nr, np.zeros((4, 4)), np.zeros((4, 4)), ctx)
    assert e.value.status == 5
    # reducible: state 3 never reached
    red = np.array([[-1.0, 0.5, 0.5, 0.0], [0.5, -1.0, 0.5, 0.0], [0.5, 0.5, -1.0, 0.0],
                    [0.3, 0.3, 0.4, -1.0]])
    with pytest.raises(_native.NativeError) as e:
        M.diagonalize_gtr(red, np.zeros((4, 4)), np.zeros((4, 4)), ctx)
    assert e.value.status == 5
