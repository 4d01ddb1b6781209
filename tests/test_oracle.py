"""CPU tests of the oracle (the checker), against known answers and the
reference's own property tests (test/testsuite/decompositions/{qr,polar}.jl,
test/testsuite/chainrules.jl)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
DTYPES = [np.float64, np.complex128, np.float32, np.complex64]


def prec(dt):
    """``TestSuite.precision(T) = sqrt(eps(real(T)))`` (test/testsuite/TestSuite.jl:45)."""
    return np.sqrt(O.eps(dt))


@pytest.mark.parametrize("path", sorted(GOLD.glob("qr_kat_*.npz")), ids=lambda p: p.stem)
def test_oracle_qr_known_answer(path):
    d = np.load(path)
    Q, R = O.qr_compact(d["A"])
    assert O.rel_err(R, d["R"]) < 1e-12
    assert O.rel_err(Q, d["Q"]) < 1e-12


@pytest.mark.parametrize("path", sorted(GOLD.glob("polar_kat_*.npz")), ids=lambda p: p.stem)
def test_oracle_polar_known_answer(path):
    d = np.load(path)
    for W, P in (O.left_polar_svd(d["A"]), O.left_polar_newton(d["A"])[:2]):
        assert O.rel_err(W, d["W"]) < 1e-11
        assert O.rel_err(P, d["P"]) < 1e-11


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", [37, 54, 63])
def test_oracle_qr_properties(dt, n):
    """test/testsuite/decompositions/qr.jl:22-113 at m = 54."""
    rng = np.random.default_rng(123)
    A = O.gaussian(rng, 54, n, dt)
    for full in (False, True):
        Q, R = (O.qr_full if full else O.qr_compact)(A)
        assert O.qr_residual(A, Q, R) < prec(dt)
        assert O.orth_error(Q) < prec(dt) * np.sqrt(Q.shape[1])
        assert np.allclose(R, np.triu(R))
        d = np.diagonal(R)
        assert np.all(d.real >= 0) and np.all(np.abs(d.imag) == 0)
    Qn, Rn = O.qr_compact(A, positive=False)
    assert O.qr_residual(A, Qn, Rn) < prec(dt)
    for bs in (1, 8):
        Qb, Rb = O.qr_compact(A, blocksize=bs)
        assert O.qr_residual(A, Qb, Rb) < prec(dt)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_polar_newton_vs_svd(dt):
    rng = np.random.default_rng(5)
    for (m, n) in ((54, 37), (54, 54), (120, 40)):
        A = O.gaussian(rng, m, n, dt)
        W1, P1 = O.left_polar_svd(A)
        W2, P2, info = O.left_polar_newton(A)
        assert info["converged"]
        assert O.rel_err(W1, W2) < 1e-12 and O.rel_err(P1, P2) < 1e-12
        assert O.orth_error(W2) < 1e-13 * n
        assert np.linalg.norm(A - W2 @ P2) / np.linalg.norm(A) < 1e-13


def test_oracle_newton_iteration_count_illconditioned():
    rng = np.random.default_rng(2)
    A = O.polar_test_matrix(rng, 128, np.float64)
    W, P, info = O.left_polar_newton(A)
    assert info["converged"] and 5 <= info["iterations"] <= 10
    assert np.linalg.norm(A - W @ P) / np.linalg.norm(A) < 1e-12


def test_oracle_sylvester_sign_convention():
    """Julia sylvester(A,B,C) solves AX + XB + C = 0 (scipy: AX + XB = Q)."""
    rng = np.random.default_rng(3)
    A = rng.standard_normal((6, 6)) + 6 * np.eye(6)
    B = rng.standard_normal((6, 6)) + 6 * np.eye(6)
    Cm = rng.standard_normal((6, 6))
    X = O.sylvester(A, B, Cm)
    assert np.allclose(A @ X + X @ B + Cm, 0, atol=1e-12)


def _fd(f, A, E, h=1e-6):
    return (f(A + h * E) - f(A - h * E)) / (2 * h)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("n", [17, 19, 23])
def test_oracle_qr_pullback_fd(dt, n):
    """Central finite differences, step 1e-6 (test/testsuite/chainrules.jl:53-145)."""
    rng = np.random.default_rng(11)
    m = 19
    A = O.gaussian(rng, m, n, dt)
    Q, R = O.qr_compact(A)
    dQ, dR = O.gaussian(rng, *Q.shape, dt), O.gaussian(rng, *R.shape, dt)
    dQ, dR = O.remove_qr_gauge_dependence(dQ, dR, A, Q, R)
    dA, info = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, dR)
    assert not info["warn"]
    E = O.gaussian(rng, m, n, dt)

    def loss(X):
        Qx, Rx = O.qr_compact(X)
        return np.real(np.vdot(dQ, Qx) + np.vdot(dR, Rx))

    assert abs(_fd(loss, A, E) - np.real(np.vdot(dA, E))) < 1e-7 * max(1, abs(_fd(loss, A, E)))


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_qr_pullback_rank_deficient_fd(dt):
    """Rank-deficient A with a gauge-invariant cotangent
    (test/testsuite/chainrules.jl:125-143)."""
    rng = np.random.default_rng(12)
    A = O.rank_deficient(rng, 30, 20, 14, dt)
    Q, R = O.qr_compact(A)
    dQ, dR = O.gaussian(rng, *Q.shape, dt), O.gaussian(rng, *R.shape, dt)
    dQ, dR = O.remove_qr_gauge_dependence(dQ, dR, A, Q, R)
    dA, info = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, dR)
    assert info["rank"] == 14
    # FD along directions that keep the rank (E = B1 C + B C1)
    B = rng.standard_normal((30, 14)); Cm = rng.standard_normal((14, 20))
    E = A @ np.linalg.pinv(A) @ O.gaussian(rng, 30, 20, dt) @ np.linalg.pinv(A) @ A

    def loss(X):
        Qx, Rx = O.qr_compact(X)
        return np.real(np.vdot(dQ, Qx) + np.vdot(dR, Rx))

    fd = _fd(loss, A, E)
    assert abs(fd - np.real(np.vdot(dA, E))) < 1e-6 * max(1, abs(fd))


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_polar_pullback_fd(dt):
    rng = np.random.default_rng(13)
    A = O.gaussian(rng, 19, 17, dt)
    W, P = O.left_polar_svd(A)
    dW, dP = O.gaussian(rng, 19, 17, dt), O.gaussian(rng, 17, 17, dt)
    dA = O.left_polar_pullback(np.zeros_like(A), A, W, P, dW, dP)
    E = O.gaussian(rng, 19, 17, dt)

    def loss(X):
        Wx, Px = O.left_polar_svd(X)
        return np.real(np.vdot(dW, Wx) + np.vdot(dP, Px))

    fd = _fd(loss, A, E)
    assert abs(fd - np.real(np.vdot(dA, E))) < 1e-7 * max(1, abs(fd))


def test_oracle_flop_counts():
    assert abs(O.qr_flops(512, 256) - 0.1118e9) / 0.1118e9 < 1e-3
    assert abs(O.qr_flops(16384, 8192) - 3.665e12) / 3.665e12 < 1e-3


# ----------------------------------------------- LQ, right polar, pushforwards ---

@pytest.mark.parametrize("path", sorted(GOLD.glob("qr_kat_*.npz")), ids=lambda p: p.stem)
def test_oracle_lq_known_answer(path):
    """A^H = R0^H Q0^H is the positive-diagonal LQ of A^H (the QR known
    answers, conjugate-transposed); both LQ routes must return it."""
    d = np.load(path)
    Ah = d["A"].conj().T
    for L, Q in (O.lq_compact(Ah), O.lq_householder_native(Ah)):
        assert O.rel_err(L, d["R"].conj().T) < 1e-12
        assert O.rel_err(Q, d["Q"].conj().T) < 1e-12


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("shape", [(37, 54), (54, 54), (54, 37), (1, 9)])
def test_oracle_lq_properties(dt, shape):
    """test/testsuite/decompositions/lq.jl:21-160: L Q = A, Q has orthonormal
    rows (unitary for lq_full), L lower triangular with a positive diagonal;
    the transposed-QR route agrees with the native row-Householder LQ."""
    rng = np.random.default_rng(321)
    m, n = shape
    A = O.gaussian(rng, m, n, dt)
    k = min(m, n)
    for full in (False, True):
        L, Q = (O.lq_full if full else O.lq_compact)(A)
        assert L.shape == ((m, n) if full else (m, k))
        assert Q.shape == ((n, n) if full else (k, n))
        assert O.qr_residual(A.T, Q.T, L.T) < prec(dt)
        assert O.orth_error(Q.conj().T) < prec(dt) * np.sqrt(Q.shape[0])
        assert np.allclose(L, np.tril(L))
        dg = np.diagonal(L)
        assert np.all(dg.real >= 0) and np.all(np.abs(dg.imag) == 0)
        Ln, Qn = O.lq_householder_native(A, full=full)
        tol = 1e-11 if O.eps(dt) < 1e-10 else 1e-4
        assert O.rel_err(Ln, L) < tol
        assert O.rel_err(Qn[:k], Q[:k]) < tol


@pytest.mark.parametrize("path", sorted(GOLD.glob("polar_kat_*.npz")), ids=lambda p: p.stem)
def test_oracle_right_polar_known_answer(path):
    """A^H = P W^H: the right polar factors of A^H are the left factors of A,
    conjugate-transposed."""
    d = np.load(path)
    Ah = d["A"].conj().T
    for P, Wh in (O.right_polar_svd(Ah), O.right_polar_newton(Ah)[:2]):
        assert O.rel_err(Wh, d["W"].conj().T) < 1e-11
        assert O.rel_err(P, d["P"]) < 1e-11


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_right_polar_newton_vs_svd(dt):
    """test/testsuite/decompositions/polar.jl:47-80."""
    rng = np.random.default_rng(6)
    for (m, n) in ((37, 54), (54, 54), (40, 120)):
        A = O.gaussian(rng, m, n, dt)
        P1, Wh1 = O.right_polar_svd(A)
        P2, Wh2, info = O.right_polar_newton(A)
        assert info["converged"]
        assert O.rel_err(Wh1, Wh2) < 1e-12 and O.rel_err(P1, P2) < 1e-12
        assert O.orth_error(Wh2.conj().T) < 1e-13 * m
        assert np.linalg.norm(A - P2 @ Wh2) / np.linalg.norm(A) < 1e-13
    with pytest.raises(ValueError):
        O.right_polar_newton(O.gaussian(rng, 5, 4, dt))


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_right_polar_pullback_fd(dt):
    """Central finite differences of Re<dP, P(A)> + Re<dWh, Wh(A)>, and the
    conjugate-transpose identity with the left pullback of A^H."""
    rng = np.random.default_rng(14)
    A = O.gaussian(rng, 17, 19, dt)
    P, Wh = O.right_polar_svd(A)
    dP, dWh = O.gaussian(rng, 17, 17, dt), O.gaussian(rng, 17, 19, dt)
    dA = O.right_polar_pullback(np.zeros_like(A), A, P, Wh, dP, dWh)
    E = O.gaussian(rng, 17, 19, dt)

    def loss(X):
        Px, Whx = O.right_polar_svd(X)
        return np.real(np.vdot(dP, Px) + np.vdot(dWh, Whx))

    fd = _fd(loss, A, E)
    assert abs(fd - np.real(np.vdot(dA, E))) < 1e-7 * max(1, abs(fd))
    dAt = O.left_polar_pullback(np.zeros_like(A.T), A.conj().T, Wh.conj().T, P,
                                dWh.conj().T, dP)
    assert O.rel_err(dAt.conj().T, dA) < 1e-12
    for zdP, zdWh in ((None, dWh), (dP, None)):
        d1 = O.right_polar_pullback(np.zeros_like(A), A, P, Wh, zdP, zdWh)
        d2 = O.right_polar_pullback(np.zeros_like(A), A, P, Wh,
                                    np.zeros_like(dP) if zdP is None else zdP,
                                    np.zeros_like(dWh) if zdWh is None else zdWh)
        assert O.rel_err(d1, d2) < 1e-13


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_polar_pushforward_fd(dt):
    """Both pushforwards against central differences of the SVD-based polar
    decomposition, and the pairing <dA_pullback, E> = <cotangent, tangent>."""
    rng = np.random.default_rng(15)
    A = O.gaussian(rng, 19, 17, dt)
    E = O.gaussian(rng, 19, 17, dt)
    W, P = O.left_polar_svd(A)
    dW, dP = O.left_polar_pushforward(E, A, W, P)
    fW = _fd(lambda X: O.left_polar_svd(X)[0], A, E)
    fP = _fd(lambda X: O.left_polar_svd(X)[1], A, E)
    assert O.rel_err(dW, fW) < 1e-7 and O.rel_err(dP, fP) < 1e-7
    cW, cP = O.gaussian(rng, 19, 17, dt), O.project_hermitian(O.gaussian(rng, 17, 17, dt))
    dA = O.left_polar_pullback(np.zeros_like(A), A, W, P, cW, cP)
    lhs = np.real(np.vdot(dA, E))
    rhs = np.real(np.vdot(cW, dW) + np.vdot(cP, dP))
    assert abs(lhs - rhs) < 1e-10 * max(1, abs(lhs))

    B = A.conj().T.copy()
    F = E.conj().T.copy()
    Pb, Whb = O.right_polar_svd(B)
    dWh, dPb = O.right_polar_pushforward(F, B, Pb, Whb)
    fWh = _fd(lambda X: O.right_polar_svd(X)[1], B, F)
    fPb = _fd(lambda X: O.right_polar_svd(X)[0], B, F)
    assert O.rel_err(dWh, fWh) < 1e-7 and O.rel_err(dPb, fPb) < 1e-7
    # conjugate-transpose duality: right pushforward of A^H = (left pushforward of A)^H
    assert O.rel_err(dWh, dW.conj().T) < 1e-12 and O.rel_err(dPb, dP.conj().T) < 1e-12


# ------------------------------------------------- null-space and LQ pullbacks ---

@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_qr_null_pullback_fd(dt):
    """FD of Re<dN, qr_null(A)> with a gauge-invariant cotangent
    (remove_qr_null_gauge_dependence!, src/pullbacks/qr.jl:198-200)."""
    rng = np.random.default_rng(16)
    A = O.gaussian(rng, 23, 9, dt)
    N = O.qr_null(A)
    dN = O.remove_qr_null_gauge_dependence(O.gaussian(rng, *N.shape, dt), A, N)
    dA, info = O.qr_null_pullback(np.zeros_like(A), A, N, dN)
    assert not info["warn"]
    E = O.gaussian(rng, 23, 9, dt)
    fd = _fd(lambda X: np.real(np.vdot(dN, O.qr_null(X))), A, E)
    assert abs(fd - np.real(np.vdot(dA, E))) < 1e-7 * max(1, abs(fd))
    # a gauge-dependent cotangent trips the check
    _, info2 = O.qr_null_pullback(np.zeros_like(A), A, N, N @ (1j * np.eye(N.shape[1]) if
                                  O.is_complex(dt) else np.triu(np.ones((14, 14)), 1)))
    assert info2["warn"]


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_lq_null_pullback_fd(dt):
    rng = np.random.default_rng(17)
    A = O.gaussian(rng, 9, 23, dt)
    Nh = O.lq_null(A)
    assert Nh.shape == (14, 23) and np.linalg.norm(A @ Nh.conj().T) < 1e-12
    dNh = O.remove_lq_null_gauge_dependence(O.gaussian(rng, *Nh.shape, dt), A, Nh)
    dA, info = O.lq_null_pullback(np.zeros_like(A), A, Nh, dNh)
    assert not info["warn"]
    E = O.gaussian(rng, 9, 23, dt)
    fd = _fd(lambda X: np.real(np.vdot(dNh, O.lq_null(X))), A, E)
    assert abs(fd - np.real(np.vdot(dA, E))) < 1e-7 * max(1, abs(fd))
    # conjugate-transpose duality with the QR null-space rule
    dAt, _ = O.qr_null_pullback(np.zeros_like(A.T), A.conj().T, Nh.conj().T, dNh.conj().T)
    assert O.rel_err(dAt.conj().T, dA) < 1e-12


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("shape", [(17, 19), (19, 19), (19, 17)])
def test_oracle_lq_pullback_fd(dt, shape):
    """test/testsuite/chainrules.jl pattern for lq_compact and lq_full."""
    rng = np.random.default_rng(18)
    A = O.gaussian(rng, *shape, dt)
    E = O.gaussian(rng, *shape, dt)
    for full in (False, True):
        f = O.lq_full if full else O.lq_compact
        L, Q = f(A)
        dL, dQ = O.gaussian(rng, *L.shape, dt), O.gaussian(rng, *Q.shape, dt)
        dL, dQ = O.remove_lq_gauge_dependence(dL, dQ, A, L, Q)
        dA, info = O.lq_pullback(np.zeros_like(A), A, L, Q, dL, dQ)
        assert not info["warn"] and info["rank"] == min(shape)

        def loss(X):
            Lx, Qx = f(X)
            return np.real(np.vdot(dL, Lx) + np.vdot(dQ, Qx))

        fd = _fd(loss, A, E)
        assert abs(fd - np.real(np.vdot(dA, E))) < 1e-7 * max(1, abs(fd))
        dAt, _ = O.qr_pullback(np.zeros_like(A.T), A.conj().T, Q.conj().T, L.conj().T,
                               dQ.conj().T, dL.conj().T)
        assert O.rel_err(dAt.conj().T, dA) < 1e-12


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_oracle_lq_pullback_rank_deficient_fd(dt):
    rng = np.random.default_rng(19)
    A = O.rank_deficient(rng, 20, 30, 14, dt)
    L, Q = O.lq_compact(A)
    dL, dQ = O.gaussian(rng, *L.shape, dt), O.gaussian(rng, *Q.shape, dt)
    dL, dQ = O.remove_lq_gauge_dependence(dL, dQ, A, L, Q)
    dA, info = O.lq_pullback(np.zeros_like(A), A, L, Q, dL, dQ)
    assert info["rank"] == 14 and not info["warn"]
    E = A @ np.linalg.pinv(A) @ O.gaussian(rng, 20, 30, dt) @ np.linalg.pinv(A) @ A

    def loss(X):
        Lx, Qx = O.lq_compact(X)
        return np.real(np.vdot(dL, Lx) + np.vdot(dQ, Qx))

    fd = _fd(loss, A, E)
    assert abs(fd - np.real(np.vdot(dA, E))) < 1e-6 * max(1, abs(fd))
