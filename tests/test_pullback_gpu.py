"""GPU tests of the reverse rules through the C ABI against the CPU oracle
(the reference's qr_pullback! / left_polar_pullback! restated) and central
finite differences (step 1e-6) of the GPU factorization itself, in
ComplexF64 and Float64, including the rank-deficient case with a
gauge-invariant cotangent (test/testsuite/chainrules.jl:125-143)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu
DTS = [np.float64, np.complex128]


def _loss_qr(mak, cuda, X, dQ, dR):
    Q, R = mak.qr_compact(to_dev(X, cuda))
    return float(np.real(np.vdot(dQ, to_host(Q)) + np.vdot(dR, to_host(R))))


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(19, 17), (19, 19), (19, 23), (120, 50)])
def test_qr_pullback_vs_oracle_and_fd(mak, cuda, dt, shape):
    rng = np.random.default_rng(51)
    A = O.gaussian(rng, *shape, dt)
    Q, R = O.qr_compact(A)
    dQ, dR = O.gaussian(rng, *Q.shape, dt), O.gaussian(rng, *R.shape, dt)
    dQ, dR = O.remove_qr_gauge_dependence(dQ, dR, A, Q, R)
    dA0 = O.gaussian(rng, *shape, dt)
    ref, oinfo = O.qr_pullback(dA0, A, Q, R, dQ, dR)
    dA = to_dev(dA0, cuda)
    info = {}
    mak.qr_pullback_(dA, to_dev(A, cuda), (to_dev(Q, cuda), to_dev(R, cuda)),
                     (to_dev(dQ, cuda), to_dev(dR, cuda)), _info=info)
    got = to_host(dA)
    assert info["rank"] == oinfo["rank"]
    assert O.rel_err(got - dA0, ref - dA0) <= 1e-11
    E = O.gaussian(rng, *shape, dt)
    h = 1e-6
    fd = (_loss_qr(mak, cuda, A + h * E, dQ, dR) - _loss_qr(mak, cuda, A - h * E, dQ, dR)) / (2 * h)
    an = float(np.real(np.vdot(got - dA0, E)))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_qr_pullback_rank_deficient(mak, cuda, dt):
    rng = np.random.default_rng(52)
    A = O.rank_deficient(rng, 60, 40, 25, dt)
    Q, R = O.qr_compact(A)
    dQ, dR = O.gaussian(rng, *Q.shape, dt), O.gaussian(rng, *R.shape, dt)
    dQ, dR = O.remove_qr_gauge_dependence(dQ, dR, A, Q, R)
    ref, oinfo = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, dR)
    dA = to_dev(np.zeros_like(A), cuda)
    info = {}
    mak.qr_pullback_(dA, to_dev(A, cuda), (to_dev(Q, cuda), to_dev(R, cuda)),
                     (to_dev(dQ, cuda), to_dev(dR, cuda)), _info=info)
    assert info["rank"] == oinfo["rank"] == 25
    assert O.rel_err(to_host(dA), ref) <= 1e-9


def test_qr_pullback_zero_tangents_and_gauge_warning(mak, cuda):
    rng = np.random.default_rng(53)
    A = O.gaussian(rng, 30, 20, np.float64)
    Q, R = O.qr_compact(A)
    dR = O.gaussian(rng, *R.shape, np.float64)
    ref, _ = O.qr_pullback(np.zeros_like(A), A, Q, R, None, dR)
    dA = to_dev(np.zeros_like(A), cuda)
    mak.qr_pullback_(dA, None, (to_dev(Q, cuda), to_dev(R, cuda)), (None, to_dev(dR, cuda)))
    assert O.rel_err(to_host(dA), ref) <= 1e-11
    dQ = O.gaussian(rng, *Q.shape, np.float64)
    refq, _ = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, None)
    dA = to_dev(np.zeros_like(A), cuda)
    mak.qr_pullback_(dA, None, (to_dev(Q, cuda), to_dev(R, cuda)), (to_dev(dQ, cuda), None))
    assert O.rel_err(to_host(dA), refq) <= 1e-11
    # rank-deficient A with a cotangent that is NOT gauge invariant -> warning
    B = O.rank_deficient(rng, 30, 20, 12, np.float64)
    Qb, Rb = O.qr_compact(B)
    with pytest.warns(RuntimeWarning, match="gauge"):
        mak.qr_pullback_(to_dev(np.zeros_like(B), cuda), None, (to_dev(Qb, cuda), to_dev(Rb, cuda)),
                         (to_dev(O.gaussian(rng, 30, 20, np.float64), cuda), None))


def _loss_polar(mak, cuda, X, dW, dP):
    W, P = mak.left_polar(to_dev(X, cuda))
    return float(np.real(np.vdot(dW, to_host(W)) + np.vdot(dP, to_host(P))))


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(19, 17), (19, 19), (200, 80)])
def test_polar_pullback_vs_oracle_and_fd(mak, cuda, dt, shape):
    rng = np.random.default_rng(61)
    A = O.gaussian(rng, *shape, dt)
    W, P = O.left_polar_svd(A)
    dW, dP = O.gaussian(rng, *W.shape, dt), O.gaussian(rng, *P.shape, dt)
    dA0 = O.gaussian(rng, *shape, dt)
    ref = O.left_polar_pullback(dA0, A, W, P, dW, dP)
    dA = to_dev(dA0, cuda)
    info = {}
    mak.left_polar_pullback_(dA, None, (to_dev(W, cuda), to_dev(P, cuda)),
                             (to_dev(dW, cuda), to_dev(dP, cuda)), _info=info)
    got = to_host(dA)
    assert 1 <= info["iterations"] <= 40
    assert O.rel_err(got - dA0, ref - dA0) <= 1e-10
    E = O.gaussian(rng, *shape, dt)
    h = 1e-6
    fd = (_loss_polar(mak, cuda, A + h * E, dW, dP) - _loss_polar(mak, cuda, A - h * E, dW, dP)) / (2 * h)
    an = float(np.real(np.vdot(got - dA0, E)))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd))


def test_polar_pullback_one_sided(mak, cuda):
    rng = np.random.default_rng(62)
    A = O.gaussian(rng, 40, 25, np.complex128)
    W, P = O.left_polar_svd(A)
    for dW, dP in ((O.gaussian(rng, 40, 25, np.complex128), None),
                   (None, O.gaussian(rng, 25, 25, np.complex128))):
        ref = O.left_polar_pullback(np.zeros_like(A), A, W, P, dW, dP)
        dA = to_dev(np.zeros_like(A), cuda)
        mak.left_polar_pullback_(dA, None, (to_dev(W, cuda), to_dev(P, cuda)),
                                 (None if dW is None else to_dev(dW, cuda),
                                  None if dP is None else to_dev(dP, cuda)))
        assert O.rel_err(to_host(dA), ref) <= 1e-10
