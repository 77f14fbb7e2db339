"""Test infrastructure (oracle) -- not part of the product.

MlModel restated in numpy with the LAPACK routines phylocaml's mlmodel.c
calls (dsyev, dgeev, dgetrf, dgetri), reached through scipy.linalg.lapack,
and the same column-major conventions:

  rate matrices      lib/mlModel.ml:204-213 (m_meanrate), :216-244 (jc69),
                     :247-289 (k2p), :292-326 (tn93), :329-352 (f81),
                     :355-365 (hky85, f84), :390-421 (gtr), :473-488 (file)
  diagonalize_sym    lib/mlmodel.c:163-197   dsyev('V','U') in place
  diagonalize_gtr    lib/mlmodel.c:208-262   dgeev, |Im lambda| > 1e-10 fails,
                                             U := inverse(VR) (dgetrf+dgetri)
  compose_sym        lib/mlmodel.c:280-302   t truncated to float
  compose_gtr        lib/mlmodel.c:325-342

The C code hands row-major buffers to column-major LAPACK, so dgeev factors
Q^T and the composed column-major product exp(Q^T t) reads row-major as
exp(Q t); the functions below keep the buffers in that convention.  LAPACK
and GSL are unpinned dependencies of the reference (linked as -llapack
-lblas, myocamlbuild.ml:7); scipy 1.18's LAPACK stands in for them.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import lapack

EPSILON = 1e-10
MINIMUM = 1e-13


def m_meanrate(srm, pi):
    a = srm.shape[0]
    mr = 0.0
    for i in range(a):
        mr = mr + (-srm[i, i]) * pi[i]
    out = srm.copy()
    for i in range(a):
        for j in range(a):
            out[i, j] = srm[i, j] / mr
    return out


def _diag_rowsum(srm):
    a = srm.shape[0]
    for i in range(a):
        d = 0.0
        for j in range(a):
            if i != j:
                d = d + srm[i, j]
        srm[i, i] = -d
    return srm


def m_jc69(a):
    srm = np.ones((a, a))
    for i in range(a):
        srm[i, i] = -1.0 * (a - 1)
    return m_meanrate(srm, np.full(a, 1.0 / a))


def m_k2p(beta, a):
    assert a == 4
    beta = max(beta, MINIMUM)
    srm = np.full((a, a), beta)
    srm[1, 3] = srm[3, 1] = srm[2, 0] = srm[0, 2] = 1.0
    for i in range(a):
        srm[i, i] = -1.0 - beta - beta
    return m_meanrate(srm, np.full(a, 1.0 / a))


def m_tn93(pi, alpha, beta, a):
    assert a == 4
    srm = np.ones((a, a))
    srm[0, 2] = alpha
    srm[1, 3] = beta
    srm[2, 0] = alpha
    srm[3, 1] = beta
    for i in range(a):
        for j in range(a):
            srm[i, j] = srm[i, j] * pi[j]
    return m_meanrate(_diag_rowsum(srm), pi)


def m_f81(pi, a):
    srm = np.zeros((a, a))
    for i in range(a):
        for j in range(a):
            if i != j:
                srm[i, j] = pi[j] * 1.0
    return m_meanrate(_diag_rowsum(srm), pi)


def m_hky85(pi, kappa, a):
    return m_tn93(pi, kappa, kappa, a)


def m_f84(pi, kappa, a):
    y = pi[1] + pi[3]
    r = pi[0] + pi[2]
    return m_tn93(pi, 1.0 + kappa / r, 1.0 + kappa / y, a)


def m_gtr_independent(pi, co, a):
    assert ((a + 1) * (a - 2)) // 2 == len(co)
    size = ((a - 1) * a) // 2
    co = [1.0 if i == size - 1 else co[i] for i in range(size)]
    srm = np.zeros((a, a))
    n = 0
    for i in range(a):
        for j in range(i + 1, a):
            srm[i, j] = co[n] * pi[j]
            srm[j, i] = co[n] * pi[i]
            n += 1
    return m_meanrate(_diag_rowsum(srm), pi)


def m_file(pi, f_rr, a):
    srm = np.zeros((a, a))
    for r in range(a):
        d = 0.0
        for c in range(a):
            if c != r:
                d = d + f_rr[r][c]
                srm[r, c] = f_rr[r][c]
        srm[r, r] = -d
    return m_meanrate(srm, pi)


def diagonalize_sym(q):
    """(U, D) buffers of likelihood_CAML_diagonalize_sym (row-major view)."""
    n = q.shape[0]
    a_cm = np.array(q, dtype=np.float64, order="C").reshape(n, n).T.copy(order="F")
    w, v, info = lapack.dsyev(a_cm, compute_v=1, lower=0)
    if info != 0:
        raise ValueError("dsyev_ failed")
    u_buf = np.asarray(v, order="F").ravel(order="F").reshape(n, n)   # row-major read of column-major V
    d = np.diag(w)
    return u_buf, d


def diagonalize_gtr(q):
    """(U, D, Ui) buffers of likelihood_CAML_diagonalize_gtr (row-major view)."""
    n = q.shape[0]
    a_cm = np.asarray(q, dtype=np.float64).T.copy(order="F")          # column-major view = Q^T
    wr, wi, vl, vr, info = lapack.dgeev(a_cm, compute_vl=1, compute_vr=1)
    if np.any(np.abs(wi) > EPSILON):
        raise ValueError("Imaginary eigenvalues")
    if info != 0:
        raise ValueError("dgeev_ failed")
    vr = np.asarray(vr, order="F")
    lu, piv, info = lapack.dgetrf(vr)
    if info != 0:
        raise ValueError("dgetrf_ failed")
    inv, info = lapack.dgetri(lu, piv)
    if info != 0:
        raise ValueError("dgetri_ singular")
    ui_buf = vr.ravel(order="F").reshape(n, n)
    u_buf = np.asarray(inv, order="F").ravel(order="F").reshape(n, n)
    return u_buf, np.diag(wr), ui_buf


def _cm(buf):
    """column-major matrix held in a row-major buffer"""
    n = buf.shape[0]
    return np.asarray(buf).ravel().reshape(n, n, order="F")


def compose_gtr(u_buf, d, ui_buf, t):
    n = u_buf.shape[0]
    if t == -1.0:
        core = d.copy()
    elif t >= EPSILON:
        core = d.copy()
        for i in range(n):
            core[i, i] = np.exp(d[i, i] * t)
    else:
        return np.eye(n)
    p_cm = _cm(ui_buf) @ _cm(core) @ _cm(u_buf)
    return p_cm.ravel(order="F").reshape(n, n)


def compose_sym(u_buf, d, t):
    n = u_buf.shape[0]
    t = float(np.float32(t))        # `const float t` (lib/mlmodel.c:280)
    if t == -1.0:
        core = d.copy()
    elif t >= EPSILON:
        core = d.copy()
        for i in range(n):
            core[i, i] = np.exp(d[i, i] * t)
    else:
        return np.eye(n)
    U = _cm(u_buf)
    p_cm = U @ _cm(core) @ U.T
    return p_cm.ravel(order="F").reshape(n, n)


def gamma_rates_mean(alpha, k):
    """Yang (1994) category means, written independently of the product."""
    from scipy import integrate, stats
    g = stats.gamma(a=alpha, scale=1.0 / alpha)
    edges = [0.0] + [g.ppf(i / k) for i in range(1, k)] + [np.inf]
    return np.array([k * integrate.quad(lambda x: x * g.pdf(x), edges[i], edges[i + 1])[0]
                     for i in range(k)])


def pmatrices(q, pi, rates, brlen):
    """P[b][r] = exp(Q rate_r t_b) through diagonalize_gtr/compose_gtr."""
    u, d, ui = diagonalize_gtr(q)
    S, R = q.shape[0], len(rates)
    out = np.empty((len(brlen), R, S, S))
    for b, t in enumerate(brlen):
        for r, rate in enumerate(rates):
            out[b, r] = compose_gtr(u, d, ui, float(t * rate))
    return out
