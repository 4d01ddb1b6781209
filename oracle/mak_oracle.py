"""numpy/scipy restatement of the reference's CPU algorithms (test infrastructure).

Every public function cites the reference file:line it restates.  LAPACK is
reached through ``scipy.linalg.lapack`` -- the same ``?geqrt``/``?gemqrt``/
``?gesdd``/``?gesvd`` routines the reference calls through libblastrampoline
(OpenBLAS) in src/yalapack.jl.  Nothing here runs on a GPU.
"""

from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack

__all__ = [
    "defaulttol", "sign_safe", "default_qr_blocksize",
    "qr_compact", "qr_r", "qr_full", "qr_null", "project_hermitian", "svd_compact",
    "left_polar_svd", "left_polar_newton", "qr_rank", "qr_pullback",
    "remove_qr_gauge_dependence", "left_polar_pullback", "sylvester",
    "gaussian", "haar", "polar_test_matrix", "rank_deficient", "batched_blocks",
    "qr_residual", "orth_error", "rel_err", "qr_flops", "polar_flops",
    "is_complex", "real_dtype", "eps",
    "lq_via_qr", "lq_compact", "lq_full", "lq_householder_native", "right_polar_newton",
    "right_polar_svd", "right_polar_pullback", "left_polar_pushforward",
    "right_polar_pushforward", "qr_null_pullback", "remove_qr_null_gauge_dependence",
    "lq_pullback", "remove_lq_gauge_dependence", "lq_null_pullback",
    "remove_lq_null_gauge_dependence", "lq_null",
]


# ---------------------------------------------------------------- scalars ---

def is_complex(dtype) -> bool:
    return np.issubdtype(np.dtype(dtype), np.complexfloating)


def real_dtype(dtype):
    return np.finfo(np.dtype(dtype)).dtype


def eps(dtype) -> float:
    return float(np.finfo(real_dtype(dtype)).eps)


def defaulttol(dtype) -> float:
    """``defaulttol(x) = eps(real(eltype(x)))^(2/3)`` (src/common/defaults.jl:10)."""
    return eps(dtype) ** (2.0 / 3.0)


def _eps_of(x: float, dtype) -> float:
    """Julia ``eps(x)``: the spacing of floating-point numbers at ``x``."""
    rd = real_dtype(dtype)
    x = rd.type(abs(x))
    if x == 0:
        return float(np.finfo(rd).smallest_subnormal)
    return float(np.spacing(x))


def sign_safe(s):
    """``sign_safe`` (src/common/safemethods.jl:10-11): real ``s<0 ? -1 : +1``;
    complex ``s/|s|`` with 0 -> 1."""
    s = np.asarray(s)
    if is_complex(s.dtype):
        a = np.abs(s)
        out = np.ones_like(s)
        nz = a != 0
        out[nz] = s[nz] / a[nz]
        return out
    return np.where(s < 0, -np.ones_like(s), np.ones_like(s))


def default_qr_blocksize(m: int, n: int) -> int:
    """``default_qr_blocksize(A) = min(size(A)..., 36)`` (src/yalapack.jl:88-89)."""
    return min(m, n, 36)


def _pfx(dtype) -> str:
    return {np.dtype(np.float64): "d", np.dtype(np.float32): "s",
            np.dtype(np.complex128): "z", np.dtype(np.complex64): "c"}[np.dtype(dtype)]


def _lp(name: str, dtype):
    return getattr(lapack, _pfx(dtype) + name)


# --------------------------------------------------------------------- QR ---

def _qr_householder(A, full: bool, positive: bool = True, blocksize: int = 0,
                    compute_r: bool = True):
    """``qr_householder!(::LAPACK, A, Q, R; positive, blocksize)``
    (src/implementations/qr.jl:132-188): ``geqrt`` with nb = min(m, n, 36)
    (qr.jl:137, yalapack.jl:88-89), ``gemqrt('L','N', V, T, one!(Q))``
    (qr.jl:163), ``copyto!(R, uppertriangular!(A))`` (qr.jl:179-181) and
    ``gaugefix!(qr_householder!, Q, R, diagview(A))`` (src/common/gauge.jl:16-25).
    """
    A = np.array(A, order="F", copy=True)
    dtype = A.dtype
    m, n = A.shape
    k = min(m, n)
    qcols = m if full else k
    Q = np.zeros((m, qcols), dtype=dtype, order="F")
    Q[np.arange(qcols), np.arange(qcols)] = 1  # one!(Q)
    if k == 0:
        R = np.zeros((qcols, n), dtype=dtype, order="F")
        return Q, R
    nb = blocksize if blocksize > 0 else default_qr_blocksize(m, n)
    nb = min(k, nb)
    Apk, T, info = _lp("geqrt", dtype)(nb, A)
    assert info == 0, f"?geqrt info={info}"
    V = np.asfortranarray(Apk[:, :k])
    Q, info = _lp("gemqrt", dtype)(V, T, Q, side="L", trans="N")
    assert info == 0, f"?gemqrt info={info}"
    Q = np.asfortranarray(Q)
    R = np.triu(Apk[:qcols, :]) if compute_r else None
    if R is not None:
        R = np.asfortranarray(R)
    if positive:
        s = sign_safe(np.diagonal(Apk)[:k].copy())
        Q[:, :k] *= s[None, :]
        if R is not None:
            R[:k, :] *= np.conj(s)[:, None]
    return Q, R


def qr_compact(A, positive: bool = True, blocksize: int = 0):
    """``qr_compact!(A, (Q, R), Householder(; positive))`` with the LAPACK
    driver (src/implementations/qr.jl:110-113,132-188): Q is m x min(m,n),
    R is min(m,n) x n."""
    return _qr_householder(A, full=False, positive=positive, blocksize=blocksize)


def qr_r(A, positive: bool = True, blocksize: int = 0):
    """R alone of ``qr_compact!(A, (Q, R))`` with the LAPACK driver: the same
    ``geqrt`` (nb = min(m, n, 36)), ``uppertriangular!`` copy and the R half
    of ``gaugefix!`` (src/implementations/qr.jl:132-188,
    src/common/gauge.jl:16-25) as :func:`qr_compact`, without forming Q
    (the geqrt call and R's values are identical)."""
    A = np.array(A, order="F", copy=True)
    m, n = A.shape
    k = min(m, n)
    if k == 0:
        return np.zeros((k, n), dtype=A.dtype, order="F")
    nb = blocksize if blocksize > 0 else default_qr_blocksize(m, n)
    Apk, T, info = _lp("geqrt", A.dtype)(min(k, nb), A)
    assert info == 0, f"?geqrt info={info}"
    R = np.asfortranarray(np.triu(Apk[:k, :]))
    if positive:
        s = sign_safe(np.diagonal(Apk)[:k].copy())
        R *= np.conj(s)[:, None]
    return R


def qr_full(A, positive: bool = True, blocksize: int = 0):
    """``qr_full!`` (src/implementations/qr.jl:106-109,132-188): Q is m x m,
    R is m x n."""
    return _qr_householder(A, full=True, positive=positive, blocksize=blocksize)


def qr_null(A, positive: bool = True):
    """``qr_null!`` (src/implementations/qr.jl:236-295): the last m - min(m,n)
    columns of the full Q (``unmqr`` of ``[0; I]``)."""
    m, n = np.shape(A)
    Q, _ = qr_full(A, positive=positive)
    return np.asfortranarray(Q[:, min(m, n):])


# --------------------------------------------------------------------- LQ ---

def lq_via_qr(A, full: bool = False, positive: bool = True, blocksize: int = 0):
    """``lq_via_qr!(A, L, Q, qr_alg)`` (src/implementations/lq.jl:303-318), the
    LQ the reference computes for its GPU drivers (lq.jl:130-131) and for
    ``LQViaTransposedQR`` (src/interface/decompositions.jl:340-353): the QR of
    ``A^H`` (``qr_full!`` when Q is n x n, else ``qr_compact!``), then
    ``Q = Qt^H`` and ``L = Rt^H``.  Returns ``(L, Q)``: compact L m x min(m,n),
    Q min(m,n) x n; full L m x n, Q n x n."""
    A = np.asarray(A)
    At = np.asfortranarray(A.conj().T)
    Qt, Rt = (qr_full if full else qr_compact)(At, positive=positive, blocksize=blocksize)
    return np.asfortranarray(Rt.conj().T), np.asfortranarray(Qt.conj().T)


def lq_compact(A, positive: bool = True, blocksize: int = 0):
    """``lq_compact!`` through the transposed QR (see ``lq_via_qr``)."""
    return lq_via_qr(A, full=False, positive=positive, blocksize=blocksize)


def lq_full(A, positive: bool = True, blocksize: int = 0):
    """``lq_full!`` through the transposed QR (see ``lq_via_qr``)."""
    return lq_via_qr(A, full=True, positive=positive, blocksize=blocksize)


def lq_null(A, positive: bool = True):
    """``lq_null!`` through ``lq_null_via_qr!`` (src/implementations/lq.jl:
    320-326): the conjugate transpose of ``qr_null`` of A^H."""
    return np.asfortranarray(qr_null(np.asarray(A).conj().T, positive=positive).conj().T)


def _householder_vec(v):
    """``_householder!(v, 1)`` (src/common/householder.jl:35-67): returns
    ``(beta, v, nu)`` with ``v[0] = 1`` so that ``(I - beta v v^H) x = nu e_1``
    for the input x (nu = ||x|| >= 0)."""
    v = np.array(v, copy=True)
    sigma = float(np.sum(np.abs(v[1:]) ** 2))
    vi = v[0]
    nu = math.sqrt(abs(vi) ** 2 + sigma)
    if sigma == 0 and vi == nu:
        return v.dtype.type(0), v, nu
    if vi.real < 0:
        vi = vi - nu
    else:
        vi = ((vi - np.conj(vi)) * nu - sigma) / (np.conj(vi) + nu)
    v[1:] = v[1:] / vi
    v[0] = 1
    beta = -np.conj(vi) / nu
    return beta, v, nu


def lq_householder_native(A, full: bool = False):
    """``lq_householder!(::Native, A, L, Q)`` (src/implementations/lq.jl:
    177-219): unblocked Householder LQ, one reflector per row from
    ``_householder!(conj(A[i, i:n]))``, applied from the right to the rows
    below; Q accumulated backwards from ``one!(Q)``.  diag(L) = nu >= 0, so
    this is the positive gauge.  Pure-Python loop over rows: small cases only."""
    A = np.array(A, copy=True)
    if not np.issubdtype(A.dtype, np.inexact):
        A = A.astype(np.float64)
    m, n = A.shape
    k = min(m, n)
    lcols = n if full else k
    qrows = n if full else k
    L = np.zeros((m, lcols), dtype=A.dtype)
    refl = []
    for i in range(k):
        L[i, :i] = A[i, :i]
        beta, v, nu = _householder_vec(np.conj(A[i, i:]))
        L[i, i] = nu
        if i + 1 < m:
            B = A[i + 1:, i:]
            # rmul!(A, H) with H = HouseholderReflection(conj(beta), v): A (I - conj(beta) v v^H)
            A[i + 1:, i:] = B - np.conj(beta) * np.outer(B @ v, v.conj())
        refl.append((beta, v))
    if m > k:
        L[k:, :k] = A[k:, :k]
    Q = np.zeros((qrows, n), dtype=A.dtype)
    Q[np.arange(qrows), np.arange(qrows)] = 1
    for i in range(k - 1, -1, -1):
        beta, v = refl[i]
        # rmul!(Q, H^H) with H^H = I - beta v v^H
        Qi = Q[:, i:]
        Q[:, i:] = Qi - beta * np.outer(Qi @ v, v.conj())
    return np.asfortranarray(L), np.asfortranarray(Q)


# ----------------------------------------------------------------- polar ---

def project_hermitian(A):
    """``project_hermitian!`` (src/implementations/projections.jl:61-108):
    ``(A + A^H)/2`` with a real diagonal."""
    A = np.asarray(A)
    B = (A + A.conj().T) / 2
    if is_complex(B.dtype):
        d = np.arange(B.shape[0])
        B[d, d] = B[d, d].real
    return np.asfortranarray(B.astype(A.dtype, copy=False))


def svd_compact(A):
    """``svd_compact!(A, SafeDivideAndConquer())`` (src/implementations/svd.jl:
    169-200): ``?gesdd`` with ``?gesvd`` fallback (src/yalapack.jl:2173-2200),
    then ``gaugefix!(svd_compact!, U, Vh)`` (src/common/gauge.jl:69-77)."""
    A = np.array(A, order="F", copy=True)
    dtype = A.dtype
    u, s, vh, info = _lp("gesdd", dtype)(A, compute_uv=1, full_matrices=0)
    if info > 0:
        u, s, vh, info = _lp("gesvd", dtype)(A, compute_uv=1, full_matrices=0)
    assert info == 0, f"svd info={info}"
    # signs: the entry of largest modulus per column of U, first one on ties
    # (``_largest`` keeps the earlier element unless the later is strictly larger)
    idx = np.argmax(np.abs(u), axis=0)
    piv = u[idx, np.arange(u.shape[1])]
    sg = np.where(piv == 0, 0, piv / np.where(piv == 0, 1, np.abs(piv)))
    u = u * np.conj(sg)[None, :]
    vh = sg[:, None] * vh
    return np.asfortranarray(u), s, np.asfortranarray(vh)


def left_polar_svd(A):
    """``left_polar!(A, (W, P), PolarViaSVD(...))`` (src/implementations/polar.jl:
    59-70,87-95): ``W = U Vh`` and ``P = (sqrt(S) Vh)^H (sqrt(S) Vh)``."""
    A = np.asarray(A)
    m, n = A.shape
    if m < n:
        raise ValueError(f"input matrix needs at least as many rows ({m}) as columns ({n})")
    U, S, Vh = svd_compact(A)
    W = U @ Vh
    SV = np.sqrt(S)[:, None] * Vh
    P = SV.conj().T @ SV
    return np.asfortranarray(W), np.asfortranarray(P.astype(A.dtype, copy=False))


def left_polar_newton(A, tol: float | None = None, maxiter: int = 10,
                      compute_p: bool = True):
    """``left_polar!(A, (W, P), PolarNewton(; tol, maxiter))``
    (src/implementations/polar.jl:99-111) with ``left_polar_newton!``
    (polar.jl:128-166) and ``_avgdiff!`` (polar.jl:209-220).

    Returns ``(W, P, info)`` with ``info = {"iterations", "residual", "converged"}``.
    ``norm(X, Inf)`` of a Julia matrix is its largest absolute entry.
    """
    A0 = np.array(A, order="F", copy=True)
    dtype = A0.dtype
    m, n = A0.shape
    if m < n:
        raise ValueError(f"input matrix needs at least as many rows ({m}) as columns ({n})")
    if tol is None:
        tol = defaulttol(dtype)
    eye = np.eye(n, dtype=dtype)
    if m > n:
        Q, R = qr_compact(A0)
        X = R.copy()
        # ldiv!(UpperTriangular(Rc)', one!(Rinvh)) = R^{-H}
        Xinvh = sla.solve_triangular(R, eye, trans="C", lower=False)
    else:
        Q = None
        X = A0.copy()
        lu = sla.lu_factor(X)
        Xinvh = sla.lu_solve(lu, eye, trans=2)
    gamma = math.sqrt(np.linalg.norm(Xinvh) / np.linalg.norm(X))
    X = X * gamma
    Xinvh = Xinvh / gamma
    X, Xinvh = (X + Xinvh) / 2, Xinvh - X
    it = 1
    conv = float(np.max(np.abs(Xinvh))) if Xinvh.size else 0.0
    while it < maxiter and conv > tol:
        lu = sla.lu_factor(X)
        Xinvh = sla.lu_solve(lu, eye, trans=2)
        gamma = math.sqrt(np.linalg.norm(Xinvh) / np.linalg.norm(X))
        X = X * gamma
        Xinvh = Xinvh / gamma
        X, Xinvh = (X + Xinvh) / 2, Xinvh - X
        conv = float(np.max(np.abs(Xinvh)))
        it += 1
    W = Q @ X if m > n else X
    W = np.asfortranarray(W.astype(dtype, copy=False))
    P = project_hermitian(W.conj().T @ A0) if compute_p else None
    return W, P, {"iterations": it, "residual": conv, "converged": conv <= tol}


def right_polar_newton(A, tol: float | None = None, maxiter: int = 10,
                       compute_p: bool = True):
    """``right_polar!(A, (P, Wh), PolarNewton(; tol, maxiter))``
    (src/implementations/polar.jl:113-125) with ``right_polar_newton!``
    (polar.jl:168-206): for m < n an initial LQ, then the scaled Newton
    iteration on the lower-triangular (or square) factor; ``Wh = Lc Q`` and
    ``P = project_hermitian(A Wh^H)``.  Returns ``(P, Wh, info)``."""
    A0 = np.array(A, order="F", copy=True)
    dtype = A0.dtype
    m, n = A0.shape
    if n < m:
        raise ValueError(f"input matrix needs at least as many columns ({n}) as rows ({m})")
    if tol is None:
        tol = defaulttol(dtype)
    eye = np.eye(m, dtype=dtype)
    if m < n:
        Lf, Q = lq_compact(A0)
        X = Lf.copy()
        # ldiv!(LowerTriangular(Lc)', one!(Linvh)) = L^{-H}
        Xinvh = sla.solve_triangular(Lf, eye, trans="C", lower=True)
    else:
        Q = None
        X = A0.copy()
        Xinvh = sla.lu_solve(sla.lu_factor(X), eye, trans=2)
    gamma = math.sqrt(np.linalg.norm(Xinvh) / np.linalg.norm(X))
    X = X * gamma
    Xinvh = Xinvh / gamma
    X, Xinvh = (X + Xinvh) / 2, Xinvh - X
    it = 1
    conv = float(np.max(np.abs(Xinvh))) if Xinvh.size else 0.0
    while it < maxiter and conv > tol:
        Xinvh = sla.lu_solve(sla.lu_factor(X), eye, trans=2)
        gamma = math.sqrt(np.linalg.norm(Xinvh) / np.linalg.norm(X))
        X = X * gamma
        Xinvh = Xinvh / gamma
        X, Xinvh = (X + Xinvh) / 2, Xinvh - X
        conv = float(np.max(np.abs(Xinvh)))
        it += 1
    Wh = X @ Q if m < n else X
    Wh = np.asfortranarray(Wh.astype(dtype, copy=False))
    P = project_hermitian(A0 @ Wh.conj().T) if compute_p else None
    return P, Wh, {"iterations": it, "residual": conv, "converged": conv <= tol}


def right_polar_svd(A):
    """``right_polar!(A, (P, Wh), PolarViaSVD(...))`` (src/implementations/
    polar.jl:71-83): ``Wh = U Vh`` and ``P = (U sqrt(S)) (U sqrt(S))^H``."""
    A = np.asarray(A)
    m, n = A.shape
    if n < m:
        raise ValueError(f"input matrix needs at least as many columns ({n}) as rows ({m})")
    U, S, Vh = svd_compact(A)
    US = U * np.sqrt(S)[None, :]
    return np.asfortranarray((US @ US.conj().T).astype(A.dtype, copy=False)), \
        np.asfortranarray(U @ Vh)


# ------------------------------------------------------------- pullbacks ---

def qr_rank(R, rank_atol: float | None = None) -> int:
    """``qr_rank`` (src/pullbacks/qr.jl:1-2): index of the last diagonal entry of
    R with ``|R_jj| >= rank_atol``; default ``eps(norm(R, Inf))^(3/4)``
    (src/common/defaults.jl:36)."""
    R = np.asarray(R)
    if rank_atol is None:
        rank_atol = default_atol(R)
    d = np.abs(np.diagonal(R))
    idx = np.nonzero(d >= rank_atol)[0]
    return int(idx[-1] + 1) if idx.size else 0


def default_atol(X) -> float:
    """``eps(norm(X, Inf))^(3/4)`` (src/common/defaults.jl:18-36)."""
    X = np.asarray(X)
    nrm = float(np.max(np.abs(X))) if X.size else 0.0
    return _eps_of(nrm, X.dtype) ** 0.75


def qr_pullback(dA, A, Q, R, dQ, dR, rank_atol=None, gauge_atol=None):
    """``qr_pullback!(dA, A, (Q, R), (dQ, dR))`` (src/pullbacks/qr.jl:73-120) with
    ``check_and_prepare_qr_cotangents`` (qr.jl:4-53).  ``dQ``/``dR`` may be
    ``None`` (a zero tangent).  Returns ``(dA, info)`` where ``info`` holds the
    rank ``p`` and the gauge measure ``dgauge`` that the reference warns on."""
    dA = np.array(dA, order="F", copy=True)
    Q = np.asarray(Q)
    R = np.asarray(R)
    m, n = Q.shape[0], R.shape[1]
    k = min(m, n)
    if rank_atol is None:
        rank_atol = default_atol(R)
    if gauge_atol is None:
        gauge_atol = default_atol(dQ) if dQ is not None else 0.0
    p = qr_rank(R, rank_atol)
    if dA.shape != (m, n):
        raise ValueError("size of dA does not match size of Q*R")
    Q1 = Q[:, :p]
    R11 = np.triu(R[:p, :p])
    R12 = R[:p, p:n]
    dgauge = 0.0
    dQ1 = np.zeros((m, p), dtype=Q.dtype)
    if dQ is not None:
        dQ = np.asarray(dQ)
        dQ1[:] = dQ[:, :p]
        if p == k:
            dQ3 = dQ[:, k:Q.shape[1]].copy()
            Q3 = Q[:, k:Q.shape[1]]
            Q1hdQ3 = Q1.conj().T @ dQ3
            dQ3 = dQ3 - Q1 @ Q1hdQ3
            dgauge_q = float(np.max(np.abs(dQ3))) if dQ3.size else 0.0
            dQ1 = dQ1 - Q3 @ Q1hdQ3.conj().T
        else:
            dQ23 = dQ[:, p:Q.shape[1]]
            dgauge_q = float(np.max(np.abs(dQ23))) if dQ23.size else 0.0
        dgauge = max(dgauge, dgauge_q)
    if dR is not None:
        dR = np.asarray(dR)
        dR11 = np.triu(dR[:p, :p])
        dR12 = dR[:p, p:n]
        if p < k:
            dR22 = dR[p:k, p:n]
            dgauge = max(dgauge, float(np.max(np.abs(np.triu(dR22)))))
    if dgauge > gauge_atol:
        pass  # the reference emits a warning here (qr.jl:50-51)
    if dR is not None and n > p:
        dQ1 = dQ1 - Q1 @ (dR12 @ R12.conj().T)
        dA[:, p:n] += Q1 @ dR12
    M = np.zeros((p, p), dtype=Q.dtype)
    if dR is not None:
        M += dR11 @ R11.conj().T
    M -= Q1.conj().T @ dQ1
    iu = np.triu_indices(p, 1)
    M[iu[1], iu[0]] = np.conj(M[iu[0], iu[1]])
    if is_complex(M.dtype):
        d = np.arange(p)
        M[d, d] = M[d, d].real
    dQ1 = dQ1 + Q1 @ M
    # _rdiv!(dQ1, dQ1, R11'): dQ1 * R11^{-H}
    if p:
        X = sla.solve_triangular(R11, dQ1.conj().T, trans="N", lower=False).conj().T
        dA[:, :p] += X
    return dA, {"rank": p, "dgauge": dgauge, "gauge_atol": gauge_atol,
                "warn": bool(dgauge > gauge_atol)}


def remove_qr_gauge_dependence(dQ, dR, A, Q, R, rank_atol=None):
    """``remove_qr_gauge_dependence!`` (src/pullbacks/qr.jl:162-189)."""
    dQ = np.array(dQ, copy=True)
    dR = np.array(dR, copy=True)
    A = np.asarray(A)
    m, n = A.shape
    k = min(m, n)
    r = qr_rank(R, rank_atol)
    Q1 = Q[:, :r]
    dQ[:, r:k] = 0
    if r == k:
        Q1hdQ3 = Q1.conj().T @ dQ[:, k:]
        dQ[:, k:] = Q1 @ Q1hdQ3
    else:
        dQ[:, k:] = 0
    if r < k:
        sub = dR[r:k, r:n]
        sub[np.triu_indices(k - r, 0, n - r)] = 0
        dR[r:k, r:n] = sub
    else:
        d = np.arange(k - r)
        dR[r + d, r + d] = 0
    return dQ, dR


def qr_null_pullback(dA, A, N, dN, gauge_atol=None):
    """``qr_null_pullback!(dA, A, N, dN)`` (src/pullbacks/qr.jl:141-152) with
    ``check_qr_null_cotangents`` (qr.jl:122-128).  Returns ``(dA, info)``."""
    dA = np.array(dA, order="F", copy=True)
    N = np.asarray(N)
    info = {"dgauge": 0.0, "gauge_atol": 0.0, "warn": False}
    if dN is None or N.shape[1] == 0:
        return dA, info
    dN = np.asarray(dN)
    if gauge_atol is None:
        gauge_atol = default_atol(dN)
    S = N.conj().T @ dN
    dgauge = float(np.linalg.norm((S - S.conj().T) / 2))
    info = {"dgauge": dgauge, "gauge_atol": gauge_atol, "warn": dgauge > gauge_atol}
    Q, R = qr_compact(A, positive=True)
    # rdiv!(dN^H Q, UpperTriangular(R)') = (dN^H Q) R^{-H}
    G = dN.conj().T @ Q
    X = sla.solve_triangular(R, G.conj().T, trans="N", lower=False).conj().T \
        if R.size else G
    dA -= N @ X
    return dA, info


def remove_qr_null_gauge_dependence(dN, A, N):
    """``remove_qr_null_gauge_dependence!`` (src/pullbacks/qr.jl:198-200):
    dN - N (N^H dN)."""
    N = np.asarray(N)
    return np.asarray(dN) - N @ (N.conj().T @ np.asarray(dN))


def lq_pullback(dA, A, L, Q, dL, dQ, rank_atol=None, gauge_atol=None):
    """``lq_pullback!(dA, A, (L, Q), (dL, dQ))`` (src/pullbacks/lq.jl:71-112)
    with ``check_and_prepare_lq_cotangents`` (lq.jl:3-55), restated directly on
    the rows of Q (not through the transposed QR rule).  ``dL``/``dQ`` may be
    ``None``.  Returns ``(dA, info)``."""
    dA = np.array(dA, order="F", copy=True)
    L = np.asarray(L)
    Q = np.asarray(Q)
    m, n = L.shape[0], Q.shape[1]
    k = min(m, n)
    if rank_atol is None:
        rank_atol = default_atol(L)
    if gauge_atol is None:
        gauge_atol = default_atol(dQ) if dQ is not None else 0.0
    p = qr_rank(L, rank_atol)  # lq_rank = qr_rank of L (the diagonal of L)
    if dA.shape != (m, n):
        raise ValueError("size of dA does not match size of L*Q")
    L11 = np.tril(L[:p, :p])
    L21 = L[p:m, :p]
    Q1 = Q[:p, :]
    dgauge = 0.0
    dQ1 = np.zeros((p, n), dtype=Q.dtype)
    if dQ is not None:
        dQ = np.asarray(dQ)
        dQ1[:] = dQ[:p, :n]
        if p == k:
            dQ3 = dQ[k:Q.shape[0], :].copy()
            Q3 = Q[k:Q.shape[0], :]
            dQ3Q1h = dQ3 @ Q1.conj().T
            dQ3 = dQ3 - dQ3Q1h @ Q1
            dgauge_q = float(np.max(np.abs(dQ3))) if dQ3.size else 0.0
            dQ1 = dQ1 - dQ3Q1h.conj().T @ Q3
        else:
            dQ2 = dQ[p:Q.shape[0], :]
            dgauge_q = float(np.max(np.abs(dQ2))) if dQ2.size else 0.0
        dgauge = max(dgauge, dgauge_q)
    if dL is not None:
        dL = np.asarray(dL)
        dL11 = np.tril(dL[:p, :p])
        dL21 = dL[p:m, :p]
        if p < k:
            dL22 = dL[p:m, p:k]
            dgauge = max(dgauge, float(np.max(np.abs(np.tril(dL22)))))
    if dL is not None and m > p:
        dQ1 = dQ1 - (L21.conj().T @ dL21) @ Q1
        dA[p:m, :] += dL21 @ Q1
    M = np.zeros((p, p), dtype=Q.dtype)
    if dL is not None:
        M += L11.conj().T @ dL11
    M -= dQ1 @ Q1.conj().T
    il = np.tril_indices(p, -1)
    M[il[1], il[0]] = np.conj(M[il[0], il[1]])
    if is_complex(M.dtype):
        d = np.arange(p)
        M[d, d] = M[d, d].real
    dQ1 = dQ1 + M @ Q1
    # ldiv!(L11', dQ1): L11^{-H} dQ1
    if p:
        dA[:p, :] += sla.solve_triangular(L11, dQ1, trans="C", lower=True)
    return dA, {"rank": p, "dgauge": dgauge, "gauge_atol": gauge_atol,
                "warn": bool(dgauge > gauge_atol)}


def remove_lq_gauge_dependence(dL, dQ, A, L, Q, rank_atol=None):
    """``remove_lq_gauge_dependence!`` (src/pullbacks/lq.jl:155-186)."""
    dL = np.array(dL, copy=True)
    dQ = np.array(dQ, copy=True)
    m, n = np.shape(A)
    k = min(m, n)
    r = qr_rank(L, rank_atol)
    Q1 = Q[:r, :]
    dQ[r:k, :] = 0
    if r == k and dQ.shape[0] > k:
        dQ[k:, :] = (dQ[k:, :] @ Q1.conj().T) @ Q1
    else:
        dQ[k:, :] = 0
    sub = dL[r:, r:k]
    d = np.arange(min(sub.shape))
    sub[d, d] = 0
    if r < k:
        sub[np.tril_indices(sub.shape[0], 0, sub.shape[1])] = 0
    dL[r:, r:k] = sub
    return dL, dQ


def lq_null_pullback(dA, A, Nh, dNh, gauge_atol=None):
    """``lq_null_pullback!(dA, A, Nh, dNh)`` (src/pullbacks/lq.jl:133-145) with
    ``check_lq_null_cotangents`` (lq.jl:114-120).  Returns ``(dA, info)``."""
    dA = np.array(dA, order="F", copy=True)
    Nh = np.asarray(Nh)
    info = {"dgauge": 0.0, "gauge_atol": 0.0, "warn": False}
    if dNh is None or Nh.shape[0] == 0:
        return dA, info
    dNh = np.asarray(dNh)
    if gauge_atol is None:
        gauge_atol = default_atol(dNh)
    S = Nh @ dNh.conj().T
    dgauge = float(np.linalg.norm((S - S.conj().T) / 2))
    info = {"dgauge": dgauge, "gauge_atol": gauge_atol, "warn": dgauge > gauge_atol}
    L, Q = lq_compact(A, positive=True)
    # ldiv!(LowerTriangular(L)', Q dNh^H) = L^{-H} (Q dNh^H)
    G = Q @ dNh.conj().T
    X = sla.solve_triangular(L, G, trans="C", lower=True) if L.size else G
    dA -= X @ Nh
    return dA, info


def remove_lq_null_gauge_dependence(dNh, A, Nh):
    """``remove_lq_null_gauge_dependence!`` (src/pullbacks/lq.jl:194-196):
    dNh - (dNh Nh^H) Nh."""
    Nh = np.asarray(Nh)
    return np.asarray(dNh) - (np.asarray(dNh) @ Nh.conj().T) @ Nh


def sylvester(A, B, C):
    """Julia ``LinearAlgebra.sylvester(A, B, C)``, which solves ``A X + X B + C = 0``
    (src/common/pullbacks.jl:15).  scipy's ``solve_sylvester`` solves
    ``A X + X B = Q``, so it is handed ``-C``."""
    return sla.solve_sylvester(A, B, -np.asarray(C))


def left_polar_pullback(dA, A, W, P, dW, dP):
    """``left_polar_pullback!(dA, A, (W, P), (dW, dP))`` (src/pullbacks/polar.jl:
    7-29).  ``dW``/``dP`` may be ``None`` (a zero tangent)."""
    dA = np.array(dA, order="F", copy=True)
    W = np.asarray(W)
    P = np.asarray(P)
    if dP is not None:
        dP = project_hermitian(dP)
    M = np.zeros_like(P)
    if dW is not None:
        M = M + W.conj().T @ dW
    if dP is not None:
        M = M - dP @ P
    C = sylvester(P, P, M.conj().T - M)
    if dP is not None:
        C = C + dP
    dA += W @ C
    if dW is not None:
        dWP = np.linalg.solve(P.T, np.asarray(dW).T).T  # dW / P
        dWP = dWP - W @ (W.conj().T @ dWP)
        dA += dWP
    return dA


def right_polar_pullback(dA, A, P, Wh, dP, dWh):
    """``right_polar_pullback!(dA, A, (P, Wh), (dP, dWh))`` (src/pullbacks/
    polar.jl:37-59).  ``dP``/``dWh`` may be ``None`` (a zero tangent)."""
    dA = np.array(dA, order="F", copy=True)
    P = np.asarray(P)
    Wh = np.asarray(Wh)
    if dP is not None:
        dP = project_hermitian(dP)
    M = np.zeros_like(P)
    if dWh is not None:
        M = M + np.asarray(dWh) @ Wh.conj().T
    if dP is not None:
        M = M - P @ dP
    C = sylvester(P, P, M.conj().T - M)
    if dP is not None:
        C = C + dP
    dA += C @ Wh
    if dWh is not None:
        PdWh = np.linalg.solve(P, np.asarray(dWh))
        PdWh = PdWh - (PdWh @ Wh.conj().T) @ Wh
        dA += PdWh
    return dA


def left_polar_pushforward(dA, A, W, P):
    """``left_polar_pushforward!(dA, A, (W, P), (dW, dP))`` (src/pushforwards/
    polar.jl:1-12): returns ``(dW, dP)``."""
    dA = np.asarray(dA)
    W = np.asarray(W)
    P = np.asarray(P)
    dP = W.conj().T @ dA
    K = sylvester(P, P, dP.conj().T - dP)
    dW = dA @ np.linalg.inv(P)
    dW = dW - W @ (W.conj().T @ dW)
    dW = dW + W @ K
    dP = dP - K @ P
    return np.asfortranarray(dW), np.asfortranarray(dP)


def right_polar_pushforward(dA, A, P, Wh):
    """``right_polar_pushforward!(dA, A, (P, Wh), (dP, dWh))`` (src/pushforwards/
    polar.jl:14-26): returns ``(dWh, dP)`` in the reference's order."""
    dA = np.asarray(dA)
    P = np.asarray(P)
    Wh = np.asarray(Wh)
    dP = dA @ Wh.conj().T
    K = sylvester(P, P, dP.conj().T - dP)
    dWh = np.linalg.inv(P) @ dA
    dWh = dWh - (dWh @ Wh.conj().T) @ Wh
    dWh = dWh + K @ Wh
    dP = dP - P @ K
    return np.asfortranarray(dWh), np.asfortranarray(dP)


# ------------------------------------------------------------ generators ---

def gaussian(rng, m, n, dtype=np.float64):
    """iid N(0,1) entries; complex: real and imaginary parts iid N(0,1)."""
    if is_complex(dtype):
        a = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    else:
        a = rng.standard_normal((m, n))
    return np.asfortranarray(a.astype(dtype))


def haar(rng, n, dtype=np.float64):
    """Haar-distributed unitary: QR of a Gaussian with ``Q diag(sign(diag R))``."""
    G = gaussian(rng, n, n, np.complex128 if is_complex(dtype) else np.float64)
    Qh, Rh = np.linalg.qr(G)
    d = np.diagonal(Rh)
    s = d / np.abs(d)
    return np.asfortranarray((Qh * s[None, :]).astype(dtype))


def polar_test_matrix(rng, n, dtype=np.float64, smax=1.0, smin=1e-6):
    """``A = U diag(s) V^H``, U and V Haar, s log-spaced from smax to smin."""
    U = haar(rng, n, dtype)
    V = haar(rng, n, dtype)
    s = np.logspace(math.log10(smax), math.log10(smin), n)
    return np.asfortranarray(((U * s[None, :]) @ V.conj().T).astype(dtype))


def rank_deficient(rng, m, n, r, dtype=np.complex128):
    """``A = B C`` with B m x r and C r x n Gaussian (rank r)."""
    return np.asfortranarray((gaussian(rng, m, r, dtype) @ gaussian(rng, r, n, dtype)).astype(dtype))


def batched_blocks(rng, nblocks=300, mmin=8, mmax=1024, nmin=4,
                   dtypes=(np.float64, np.complex128)):
    """Uneven blocks: m_i ~ U{mmin..mmax}, n_i ~ U{nmin..m_i}; the first half
    of the blocks take ``dtypes[0]``, the second half ``dtypes[1]``."""
    out = []
    for i in range(nblocks):
        m = int(rng.integers(mmin, mmax + 1))
        n = int(rng.integers(nmin, m + 1))
        dt = dtypes[0] if i < nblocks // 2 else dtypes[1]
        out.append(gaussian(rng, m, n, dt))
    return out


# --------------------------------------------------------------- metrics ---

def rel_err(X, Y) -> float:
    X = np.asarray(X, dtype=np.complex128 if is_complex(np.asarray(X).dtype) else np.float64)
    Y = np.asarray(Y, dtype=X.dtype)
    d = np.linalg.norm(Y)
    return float(np.linalg.norm(X - Y) / (d if d else 1.0))


def qr_residual(A, Q, R) -> float:
    """||A - Q R||_F / ||A||_F in float64."""
    A = np.asarray(A).astype(np.complex128 if is_complex(np.asarray(A).dtype) else np.float64)
    Q = np.asarray(Q).astype(A.dtype)
    R = np.asarray(R).astype(A.dtype)
    k = min(Q.shape[1], R.shape[0])
    d = np.linalg.norm(A)
    return float(np.linalg.norm(A - Q[:, :k] @ R[:k, :]) / (d if d else 1.0))


def orth_error(Q) -> float:
    """||Q^H Q - I||_F in float64."""
    Q = np.asarray(Q).astype(np.complex128 if is_complex(np.asarray(Q).dtype) else np.float64)
    return float(np.linalg.norm(Q.conj().T @ Q - np.eye(Q.shape[1])))


def qr_flops(m, n, complex_=False) -> float:
    """geqrf + orgqr (Q with min(m,n) columns) minimal counts (LAPACK working
    note 41); equals ``4mn^2 - 4n^3/3`` for m >= n.  x4 for complex."""
    k = min(m, n)
    if m >= n:
        geqrf = 2.0 * m * n * n - 2.0 * n ** 3 / 3.0
    else:
        geqrf = 2.0 * n * m * m - 2.0 * m ** 3 / 3.0
    orgqr = 2.0 * m * k * k - 2.0 * k ** 3 / 3.0
    return (4.0 if complex_ else 1.0) * (geqrf + orgqr)


def polar_flops(m, n, k_ref, complex_=False) -> float:
    """Reference ``PolarNewton`` count: [m > n: QR + W = Q X (2mn^2)] +
    k_ref * 8n^3/3 (LU + inverse) + 2mn^2 (P = W^H A)."""
    c = 4.0 if complex_ else 1.0
    f = 0.0
    if m > n:
        f += qr_flops(m, n, complex_) + c * 2.0 * m * n * n
    f += c * k_ref * 8.0 * n ** 3 / 3.0
    f += c * 2.0 * m * n * n
    return f
