"""GPU parity tests of the transposed duals and forward rules through the C ABI:
lq_compact! / lq_full! / lq_null! (LQViaTransposedQR), right_polar!
(PolarNewton), right_polar_pullback!, left_polar_pushforward! and
right_polar_pushforward!.

Oracle: the reference's algorithms restated on the CPU (lq_via_qr!,
right_polar_newton!, src/pullbacks/polar.jl, src/pushforwards/polar.jl), the
known-answer fixtures conjugate-transposed, and central finite differences
of the GPU factorizations.  Tolerances follow the QR / polar tests:
factors 1e-12 (Float64 QR-type), 1e-10 (polar factors), 1e-4 (Float32);
||A - L Q||/||A|| and ||A - P Wh||/||A|| <= 1e-12 in Float64.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
DTS = [np.float64, np.complex128]
ALL = [np.float64, np.complex128, np.float32, np.complex64]


def _tol(dt, tight=1e-12):
    return tight if O.eps(dt) < 1e-10 else 1e-4


def _lq_res(A, L, Q):
    k = min(L.shape[1], Q.shape[0])
    return np.linalg.norm(A - L[:, :k] @ Q[:k]) / max(np.linalg.norm(A), 1e-300)


# -------------------------------------------------------------------- LQ ---

@pytest.mark.parametrize("dt", ALL, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(37, 54), (54, 54), (54, 37), (100, 257), (1, 9), (9, 1)])
def test_lq_parity(mak, cuda, dt, shape):
    rng = np.random.default_rng(61)
    A = O.gaussian(rng, *shape, dt)
    Ad = to_dev(A, cuda)
    A_before = Ad.clone()
    for full in (False, True):
        L, Q = (mak.lq_full if full else mak.lq_compact)(Ad)
        Lo, Qo = (O.lq_full if full else O.lq_compact)(A)
        Lh, Qh = to_host(L), to_host(Q)
        assert Lh.shape == Lo.shape and Qh.shape == Qo.shape
        assert O.rel_err(Lh, Lo) <= _tol(dt)
        assert O.rel_err(Qh, Qo) <= _tol(dt)
        assert np.array_equal(Lh, np.tril(Lh))
        d = np.diagonal(Lh)
        assert np.all(d.real >= 0) and np.all(d.imag == 0)
        assert _lq_res(A, Lh, Qh) <= _tol(dt, 1e-13)
        assert O.orth_error(Qh.conj().T) <= _tol(dt, 1e-13) * np.sqrt(Qh.shape[0])
    assert torch.equal(Ad, A_before)  # lq_compact(A) leaves A unmodified


@pytest.mark.parametrize("path", sorted(GOLD.glob("qr_kat_*.npz")), ids=lambda p: p.stem)
def test_lq_known_answer(mak, cuda, path):
    """A^H = R0^H Q0^H is the positive-diagonal LQ of A^H."""
    d = np.load(path)
    L, Q = mak.lq_compact(to_dev(d["A"].conj().T.copy(), cuda))
    assert O.rel_err(to_host(L), d["R"].conj().T) <= 1e-12
    assert O.rel_err(to_host(Q), d["Q"].conj().T) <= 1e-12


@pytest.mark.parametrize("shape", [(0, 5), (5, 0), (1, 1), (2, 2)])
def test_lq_edge_shapes(mak, cuda, shape):
    rng = np.random.default_rng(62)
    A = O.gaussian(rng, *shape, np.float64)
    for full in (False, True):
        L, Q = (mak.lq_full if full else mak.lq_compact)(to_dev(A, cuda))
        Lo, Qo = (O.lq_full if full else O.lq_compact)(A)
        assert tuple(L.shape) == Lo.shape and tuple(Q.shape) == Qo.shape
        if Qo.size:
            assert O.rel_err(to_host(Q), Qo) <= 1e-12
        if Lo.size:
            assert O.rel_err(to_host(L), Lo) <= 1e-12


def test_lq_bang_outputs_null_and_checks(mak, cuda):
    rng = np.random.default_rng(63)
    A = O.gaussian(rng, 30, 70, np.complex128)
    Ad = to_dev(A, cuda)
    L = torch.empty((30, 30), dtype=Ad.dtype, device=cuda).t().contiguous().t()
    Q = torch.empty((30, 70), dtype=Ad.dtype, device=cuda).t().contiguous().t()
    L2, Q2 = mak.lq_compact_(Ad.clone(), (L, Q))
    assert L2 is L and Q2 is Q
    # empty L: only Q is computed
    Le = torch.empty((0, 0), dtype=Ad.dtype, device=cuda)
    _, Qe = mak.lq_compact_(Ad.clone(), (Le, torch.empty_like(Q)))
    assert O.rel_err(to_host(Qe), to_host(Q)) <= 1e-14
    # null space rows: orthonormal, orthogonal to the rows of A
    Nh = to_host(mak.lq_null(Ad))
    assert Nh.shape == (40, 70)
    assert np.linalg.norm(A @ Nh.conj().T) <= 1e-12 * np.linalg.norm(A)
    assert O.orth_error(Nh.conj().T) <= 1e-12
    with pytest.raises(mak.DimensionMismatch):
        mak.lq_compact_(Ad.clone(), (torch.empty((30, 31), dtype=Ad.dtype, device=cuda), Q))
    with pytest.raises(mak.ArgumentError):
        mak.lq_compact_(Ad.clone(), (L, Q.to(torch.complex64)))


def test_lq_mixed_precision_wide(mak, cuda):
    """A 512 x 4096 ComplexF64 LQ takes the split tensor-core blocking of the
    transposed QR (products of 4 * 4096 * 512 * 128 multiply-adds >= 2^26)."""
    rng = np.random.default_rng(64)
    A = O.gaussian(rng, 512, 4096, np.complex128)
    L, Q = mak.lq_compact(to_dev(A, cuda), precision="mixed")
    Lh, Qh = to_host(L), to_host(Q)
    assert _lq_res(A, Lh, Qh) <= 1e-12
    assert O.orth_error(Qh.conj().T) <= 1e-13 * np.sqrt(512)  # as the mixed QR tests
    Lo, Qo = O.lq_compact(A)
    assert O.rel_err(Lh, Lo) <= 1e-11 and O.rel_err(Qh, Qo) <= 1e-11


# ----------------------------------------------------------- right polar ---

@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(37, 54), (54, 54), (128, 300), (257, 257)])
def test_right_polar_parity(mak, cuda, dt, shape):
    rng = np.random.default_rng(65)
    A = O.gaussian(rng, *shape, dt)
    Ad = to_dev(A, cuda)
    A_before = Ad.clone()
    info = {}
    P, Wh = mak.right_polar_(Ad, None, None, _info=info)
    Ph, Whh = to_host(P), to_host(Wh)
    Po, Who, oinfo = O.right_polar_newton(A)
    assert info["converged"] and abs(info["iterations"] - oinfo["iterations"]) <= 1
    assert O.rel_err(Whh, Who) <= 1e-10 and O.rel_err(Ph, Po) <= 1e-10
    assert np.linalg.norm(A - Ph @ Whh) / np.linalg.norm(A) <= 1e-12
    assert O.orth_error(Whh.conj().T) <= 1e-12
    assert np.array_equal(Ph, Ph.conj().T) and np.all(np.diagonal(Ph).imag == 0)
    assert torch.equal(Ad, A_before)


@pytest.mark.parametrize("path", sorted(GOLD.glob("polar_kat_*.npz")), ids=lambda p: p.stem)
def test_right_polar_known_answer(mak, cuda, path):
    d = np.load(path)
    P, Wh = mak.right_polar(to_dev(d["A"].conj().T.copy(), cuda))
    assert O.rel_err(to_host(Wh), d["W"].conj().T) <= 1e-11
    assert O.rel_err(to_host(P), d["P"]) <= 1e-11


@pytest.mark.parametrize("dt", [np.float32, np.complex64], ids=lambda d: np.dtype(d).name)
def test_right_polar_single(mak, cuda, dt):
    rng = np.random.default_rng(66)
    A = O.gaussian(rng, 60, 120, dt)
    P, Wh = mak.right_polar(to_dev(A, cuda))
    Po, Who, _ = O.right_polar_newton(A.astype(np.complex128 if O.is_complex(dt) else np.float64))
    assert O.rel_err(to_host(Wh), Who) <= 1e-4 and O.rel_err(to_host(P), Po) <= 1e-4


def test_right_polar_empty_p_and_checks(mak, cuda):
    rng = np.random.default_rng(67)
    A = O.gaussian(rng, 40, 90, np.float64)
    Ad = to_dev(A, cuda)
    Pe = torch.empty((0, 0), dtype=Ad.dtype, device=cuda)
    Wh = torch.empty((90, 40), dtype=Ad.dtype, device=cuda).t()
    P2, Wh2 = mak.right_polar_(Ad, (Pe, Wh))
    assert P2 is Pe and Wh2 is Wh and P2.numel() == 0
    assert O.rel_err(to_host(Wh), O.right_polar_svd(A)[1]) <= 1e-10
    with pytest.raises(mak.ArgumentError):
        mak.right_polar(to_dev(O.gaussian(rng, 9, 8, np.float64), cuda))


def test_right_polar_mixed(mak, cuda):
    """Wide ComplexF64 right polar with the split tensor-core products."""
    rng = np.random.default_rng(68)
    A = O.gaussian(rng, 768, 1536, np.complex128)
    P, Wh = mak.right_polar(to_dev(A, cuda), precision="mixed")
    Ph, Whh = to_host(P), to_host(Wh)
    assert np.linalg.norm(A - Ph @ Whh) / np.linalg.norm(A) <= 1e-12
    assert O.orth_error(Whh.conj().T) <= 1e-12 * np.sqrt(768)  # as the mixed left polar tests
    Po, Who = O.right_polar_svd(A)
    assert O.rel_err(Whh, Who) <= 1e-10 and O.rel_err(Ph, Po) <= 1e-10


# ------------------------------------------------ pullback / pushforwards ---

@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(17, 19), (19, 19), (50, 120)])
def test_right_polar_pullback_vs_oracle_and_fd(mak, cuda, dt, shape):
    rng = np.random.default_rng(69)
    A = O.gaussian(rng, *shape, dt)
    m, n = shape
    P, Wh = O.right_polar_svd(A)
    dP, dWh = O.gaussian(rng, m, m, dt), O.gaussian(rng, m, n, dt)
    dA0 = O.gaussian(rng, m, n, dt)
    ref = O.right_polar_pullback(dA0, A, P, Wh, dP, dWh)
    dA = to_dev(dA0, cuda)
    mak.right_polar_pullback_(dA, to_dev(A, cuda), (to_dev(P, cuda), to_dev(Wh, cuda)),
                              (to_dev(dP, cuda), to_dev(dWh, cuda)))
    got = to_host(dA)
    assert O.rel_err(got - dA0, ref - dA0) <= 1e-10
    E = O.gaussian(rng, m, n, dt)
    h = 1e-6

    def loss(X):
        Px, Whx = mak.right_polar(to_dev(X, cuda))
        return float(np.real(np.vdot(dP, to_host(Px)) + np.vdot(dWh, to_host(Whx))))

    fd = (loss(A + h * E) - loss(A - h * E)) / (2 * h)
    an = float(np.real(np.vdot(got - dA0, E)))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_right_polar_pullback_zero_tangents(mak, cuda, dt):
    rng = np.random.default_rng(70)
    A = O.gaussian(rng, 20, 33, dt)
    P, Wh = O.right_polar_svd(A)
    dP, dWh = O.gaussian(rng, 20, 20, dt), O.gaussian(rng, 20, 33, dt)
    for cot in ((None, dWh), (dP, None)):
        ref = O.right_polar_pullback(np.zeros_like(A), A, P, Wh, *cot)
        dA = to_dev(np.zeros_like(A), cuda)
        mak.right_polar_pullback_(dA, None, (to_dev(P, cuda), to_dev(Wh, cuda)),
                                  tuple(None if c is None else to_dev(c, cuda) for c in cot))
        assert O.rel_err(to_host(dA), ref) <= 1e-10


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(19, 17), (19, 19), (120, 50)])
def test_left_polar_pushforward_vs_oracle_and_fd(mak, cuda, dt, shape):
    rng = np.random.default_rng(71)
    A = O.gaussian(rng, *shape, dt)
    E = O.gaussian(rng, *shape, dt)
    W, P = O.left_polar_svd(A)
    dWo, dPo = O.left_polar_pushforward(E, A, W, P)
    dW, dP = mak.left_polar_pushforward_(to_dev(E, cuda), None,
                                         (to_dev(W, cuda), to_dev(P, cuda)))
    dWh, dPh = to_host(dW), to_host(dP)
    assert O.rel_err(dWh, dWo) <= 1e-10 and O.rel_err(dPh, dPo) <= 1e-10
    h = 1e-6
    Wp, Pp = (to_host(x) for x in mak.left_polar(to_dev(A + h * E, cuda)))
    Wm, Pm = (to_host(x) for x in mak.left_polar(to_dev(A - h * E, cuda)))
    assert O.rel_err(dWh, (Wp - Wm) / (2 * h)) <= 1e-6
    assert O.rel_err(dPh, (Pp - Pm) / (2 * h)) <= 1e-6


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(17, 19), (19, 19), (50, 120)])
def test_right_polar_pushforward_vs_oracle(mak, cuda, dt, shape):
    rng = np.random.default_rng(72)
    A = O.gaussian(rng, *shape, dt)
    E = O.gaussian(rng, *shape, dt)
    P, Wh = O.right_polar_svd(A)
    dWho, dPo = O.right_polar_pushforward(E, A, P, Wh)
    m, n = shape
    dP = torch.empty((m, m), dtype=to_dev(A, cuda).dtype, device=cuda).t()
    dWh = torch.empty((n, m), dtype=dP.dtype, device=cuda).t()
    r1, r2 = mak.right_polar_pushforward_(to_dev(E, cuda), None,
                                          (to_dev(P, cuda), to_dev(Wh, cuda)), (dP, dWh))
    assert r1 is dWh and r2 is dP  # the reference's return order (dWh, dP)
    assert O.rel_err(to_host(dWh), dWho) <= 1e-10 and O.rel_err(to_host(dP), dPo) <= 1e-10
    # pairing with the pullback: <pullback(c), E> = <c, pushforward(E)>
    cP = O.project_hermitian(O.gaussian(rng, m, m, dt))
    cWh = O.gaussian(rng, m, n, dt)
    dA = to_dev(np.zeros_like(A), cuda)
    mak.right_polar_pullback_(dA, None, (to_dev(P, cuda), to_dev(Wh, cuda)),
                              (to_dev(cP, cuda), to_dev(cWh, cuda)))
    lhs = float(np.real(np.vdot(to_host(dA), E)))
    rhs = float(np.real(np.vdot(cP, to_host(dP)) + np.vdot(cWh, to_host(dWh))))
    assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(lhs))


def test_pushforward_mixed_precision(mak, cuda):
    """ComplexF64 1024 x 512 left pushforward with the split products."""
    rng = np.random.default_rng(73)
    A = O.gaussian(rng, 1024, 512, np.complex128)
    E = O.gaussian(rng, 1024, 512, np.complex128)
    W, P = O.left_polar_svd(A)
    dWo, dPo = O.left_polar_pushforward(E, A, W, P)
    dW, dP = mak.left_polar_pushforward_(to_dev(E, cuda), None,
                                         (to_dev(W, cuda), to_dev(P, cuda)), precision="mixed")
    assert O.rel_err(to_host(dW), dWo) <= 1e-9 and O.rel_err(to_host(dP), dPo) <= 1e-9


# ------------------------------------------------- null-space and LQ pullbacks ---

@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(23, 9), (80, 30)])
def test_qr_null_pullback_vs_oracle_and_fd(mak, cuda, dt, shape):
    rng = np.random.default_rng(74)
    A = O.gaussian(rng, *shape, dt)
    N = O.qr_null(A)
    dN = O.remove_qr_null_gauge_dependence(O.gaussian(rng, *N.shape, dt), A, N)
    dA0 = O.gaussian(rng, *shape, dt)
    ref, oinfo = O.qr_null_pullback(dA0, A, N, dN)
    dA = to_dev(dA0, cuda)
    info = {}
    mak.qr_null_pullback_(dA, to_dev(A, cuda), to_dev(N, cuda), to_dev(dN, cuda), _info=info)
    got = to_host(dA)
    assert O.rel_err(got - dA0, ref - dA0) <= 1e-11
    assert info["gauge"] <= info["gauge_atol"] and not oinfo["warn"]
    E = O.gaussian(rng, *shape, dt)
    h = 1e-6

    def loss(X):
        return float(np.real(np.vdot(dN, to_host(mak.qr_null(to_dev(X, cuda))))))

    fd = (loss(A + h * E) - loss(A - h * E)) / (2 * h)
    an = float(np.real(np.vdot(got - dA0, E)))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd))


def test_qr_null_pullback_gauge_warning_and_empty(mak, cuda):
    rng = np.random.default_rng(75)
    A = O.gaussian(rng, 30, 10, np.complex128)
    N = O.qr_null(A)
    dN = N @ (1j * np.eye(20))  # N^H dN = i I: purely gauge
    dA = to_dev(np.zeros_like(A), cuda)
    with pytest.warns(RuntimeWarning, match="gauge"):
        mak.qr_null_pullback_(dA, to_dev(A, cuda), to_dev(N, cuda), to_dev(dN, cuda))
    # square A: the null space is empty and nothing is added
    B = O.gaussian(rng, 12, 12, np.float64)
    dB0 = O.gaussian(rng, 12, 12, np.float64)
    dB = to_dev(dB0, cuda)
    Ne = torch.empty((12, 0), dtype=torch.float64, device=cuda)
    mak.qr_null_pullback_(dB, to_dev(B, cuda), Ne, Ne)
    assert np.array_equal(to_host(dB), dB0)


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_lq_null_pullback_vs_oracle_and_fd(mak, cuda, dt):
    rng = np.random.default_rng(76)
    A = O.gaussian(rng, 9, 23, dt)
    Nh = O.lq_null(A)
    dNh = O.remove_lq_null_gauge_dependence(O.gaussian(rng, *Nh.shape, dt), A, Nh)
    ref, _ = O.lq_null_pullback(np.zeros_like(A), A, Nh, dNh)
    dA = to_dev(np.zeros_like(A), cuda)
    mak.lq_null_pullback_(dA, to_dev(A, cuda), to_dev(Nh, cuda), to_dev(dNh, cuda))
    got = to_host(dA)
    assert O.rel_err(got, ref) <= 1e-11
    E = O.gaussian(rng, 9, 23, dt)
    h = 1e-6

    def loss(X):
        return float(np.real(np.vdot(dNh, to_host(mak.lq_null(to_dev(X, cuda))))))

    fd = (loss(A + h * E) - loss(A - h * E)) / (2 * h)
    assert abs(fd - float(np.real(np.vdot(got, E)))) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(17, 19), (19, 19), (19, 17), (50, 120)])
def test_lq_pullback_vs_oracle_and_fd(mak, cuda, dt, shape):
    rng = np.random.default_rng(77)
    A = O.gaussian(rng, *shape, dt)
    E = O.gaussian(rng, *shape, dt)
    for full in (False, True):
        f = O.lq_full if full else O.lq_compact
        L, Q = f(A)
        dL, dQ = O.gaussian(rng, *L.shape, dt), O.gaussian(rng, *Q.shape, dt)
        dL, dQ = O.remove_lq_gauge_dependence(dL, dQ, A, L, Q)
        dA0 = O.gaussian(rng, *shape, dt)
        ref, oinfo = O.lq_pullback(dA0, A, L, Q, dL, dQ)
        dA = to_dev(dA0, cuda)
        info = {}
        mak.lq_pullback_(dA, to_dev(A, cuda), (to_dev(L, cuda), to_dev(Q, cuda)),
                         (to_dev(dL, cuda), to_dev(dQ, cuda)), _info=info)
        got = to_host(dA)
        assert info["rank"] == oinfo["rank"] == min(shape)
        assert O.rel_err(got - dA0, ref - dA0) <= 1e-11
        g = mak.lq_full if full else mak.lq_compact
        h = 1e-6

        def loss(X):
            Lx, Qx = g(to_dev(X, cuda))
            return float(np.real(np.vdot(dL, to_host(Lx)) + np.vdot(dQ, to_host(Qx))))

        fd = (loss(A + h * E) - loss(A - h * E)) / (2 * h)
        an = float(np.real(np.vdot(got - dA0, E)))
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_lq_pullback_rank_deficient_and_zero_tangents(mak, cuda, dt):
    rng = np.random.default_rng(78)
    A = O.rank_deficient(rng, 40, 60, 25, dt)
    L, Q = O.lq_compact(A)
    dL, dQ = O.gaussian(rng, *L.shape, dt), O.gaussian(rng, *Q.shape, dt)
    dL, dQ = O.remove_lq_gauge_dependence(dL, dQ, A, L, Q)
    for cot in ((dL, dQ), (None, dQ), (dL, None)):
        ref, oinfo = O.lq_pullback(np.zeros_like(A), A, L, Q, *cot)
        dA = to_dev(np.zeros_like(A), cuda)
        info = {}
        mak.lq_pullback_(dA, None, (to_dev(L, cuda), to_dev(Q, cuda)),
                         tuple(None if c is None else to_dev(c, cuda) for c in cot), _info=info)
        assert info["rank"] == oinfo["rank"] == 25
        assert O.rel_err(to_host(dA), ref) <= 1e-9
