"""GPU parity tests of left_polar! (GB300_PolarNewton) through the C ABI.

Oracle: the reference's PolarNewton restated (and PolarViaSVD, the
reference's default) on the CPU.  The polar factor of a matrix with
condition number k is itself only determined to ~k * eps, so W and P are
compared at 1e-10 relative (well-conditioned inputs) and the accuracy
bounds are checked directly: ||A - W P||/||A|| <= 1e-12 and
||W^H W - I|| <= 1e-12 in Float64.  Float32: 1e-4 relative.
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


def back_err(A, W, P):
    return np.linalg.norm(A - W @ P) / np.linalg.norm(A)


@pytest.mark.parametrize("dt", [np.float64, np.complex128], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(54, 37), (54, 54), (300, 128), (257, 257)])
def test_left_polar_parity(mak, cuda, dt, shape):
    rng = np.random.default_rng(21)
    A = O.gaussian(rng, *shape, dt)
    Ad = to_dev(A, cuda)
    info = {}
    W, P = mak.left_polar_(mak_copy(Ad), None, None, _info=info)
    Wh, Ph = to_host(W), to_host(P)
    Wo, Po, oinfo = O.left_polar_newton(A)
    assert info["converged"] and abs(info["iterations"] - oinfo["iterations"]) <= 1
    assert O.rel_err(Wh, Wo) <= 1e-10
    assert O.rel_err(Ph, Po) <= 1e-10
    assert back_err(A, Wh, Ph) <= 1e-12
    assert O.orth_error(Wh) <= 1e-12
    assert np.allclose(Ph, Ph.conj().T, atol=0, rtol=0)  # exactly Hermitian
    assert np.all(np.diagonal(Ph).imag == 0)
    assert np.all(np.linalg.eigvalsh(Ph) > 0)


def mak_copy(X):
    return X.t().contiguous().t()


@pytest.mark.parametrize("path", sorted(GOLD.glob("polar_kat_*.npz")), ids=lambda p: p.stem)
def test_left_polar_known_answer(mak, cuda, path):
    d = np.load(path)
    W, P = mak.left_polar(to_dev(d["A"], cuda))
    assert O.rel_err(to_host(W), d["W"]) <= 1e-11
    assert O.rel_err(to_host(P), d["P"]) <= 1e-11


def test_left_polar_ill_conditioned(mak, cuda):
    """kappa = 1e6 (log-spaced singular values 1..1e-6), square."""
    rng = np.random.default_rng(22)
    A = O.polar_test_matrix(rng, 256, np.float64)
    info = {}
    W, P = mak.left_polar_(to_dev(A, cuda), None, None, _info=info)
    Wh, Ph = to_host(W), to_host(P)
    oinfo = O.left_polar_newton(A)[2]
    assert info["converged"] and abs(info["iterations"] - oinfo["iterations"]) <= 1
    assert back_err(A, Wh, Ph) <= 1e-12
    assert O.orth_error(Wh) <= 1e-12
    Ws, Ps = O.left_polar_svd(A)
    assert O.rel_err(Wh, Ws) <= 1e-8  # forward error ~ kappa * eps


@pytest.mark.parametrize("dt", [np.float32, np.complex64], ids=lambda d: np.dtype(d).name)
def test_left_polar_single(mak, cuda, dt):
    rng = np.random.default_rng(23)
    A = O.gaussian(rng, 120, 60, dt)
    W, P = mak.left_polar(to_dev(A, cuda))
    Wh, Ph = to_host(W).astype(np.complex128), to_host(P).astype(np.complex128)
    Wo, Po = O.left_polar_svd(A.astype(np.complex128))
    assert O.rel_err(Wh, Wo) <= 1e-4 and O.rel_err(Ph, Po) <= 1e-4


def test_left_polar_bang_semantics(mak, cuda):
    rng = np.random.default_rng(24)
    A = O.gaussian(rng, 40, 30, np.float64)
    Ad = to_dev(A, cuda)
    A2 = mak_copy(Ad)
    W, P = mak.left_polar(Ad)
    assert np.array_equal(to_host(Ad), A)  # non-bang leaves A untouched
    W2 = torch.empty_like(W)
    P2 = torch.empty_like(P)
    Wr, Pr = mak.left_polar_(A2, (W2, P2))
    assert Wr is W2 and Pr is P2
    # empty P: returned as the same (empty) object, W still computed
    Pe = torch.empty((0, 0), dtype=torch.float64, device=cuda)
    We = torch.empty_like(W)
    Wr, Pr = mak.left_polar_(mak_copy(to_dev(A, cuda)), (We, Pe))
    assert Pr is Pe and Pe.numel() == 0
    assert O.rel_err(to_host(We), to_host(W)) <= 1e-14


def test_left_polar_errors_and_warning(mak, cuda):
    A = to_dev(np.random.default_rng(1).standard_normal((10, 20)), cuda)
    with pytest.raises(mak.ArgumentError):
        mak.left_polar(A)  # m < n
    B = to_dev(O.polar_test_matrix(np.random.default_rng(2), 64, np.float64), cuda)
    with pytest.warns(RuntimeWarning, match="did not converge"):
        mak.left_polar(B, maxiter=2)


@pytest.mark.parametrize("dt", [np.float64, np.complex128], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(300, 300), (700, 260), (512, 512), (768, 768)])
def test_left_polar_mixed(mak, cuda, dt, shape):
    """precision="mixed": 128-wide Gauss-Jordan blocks and the Newton/QR
    products on the split-precision tensor-core GEMM (with the Newton-Schulz
    finish); the 1e-12 accuracy bounds."""
    rng = np.random.default_rng(25)
    A = O.polar_test_matrix(rng, shape[0], dt) if shape[0] == shape[1] else O.gaussian(rng, *shape, dt)
    info = {}
    W, P = mak.left_polar_(to_dev(A, cuda), None, None, precision="mixed", _info=info)
    Wh, Ph = to_host(W), to_host(P)
    assert info["converged"]
    assert back_err(A, Wh, Ph) <= 1e-12
    assert O.orth_error(Wh) <= 1e-12 * np.sqrt(shape[1])
    Wo, Po, _ = O.left_polar_newton(A)
    assert O.rel_err(Wh, Wo) <= 1e-8 and O.rel_err(Ph, Po) <= 1e-8


@pytest.mark.parametrize("dt", [np.float64, np.complex128], ids=lambda d: np.dtype(d).name)
def test_left_polar_mixed_lookahead(mak, cuda, dt):
    """n >= 2048 in mixed precision: the Gauss-Jordan inverse factors block
    column K+1 on the look-ahead side stream while block K updates the other
    columns.  A = U diag(s) V^H with known polar factors W = U V^H and
    P = V diag(s) V^H (s log-spaced 1 .. 1e-6)."""
    rng = np.random.default_rng(29)
    n = 2304
    U, V = O.haar(rng, n, dt), O.haar(rng, n, dt)
    s = np.logspace(0, -6, n)
    A = np.asfortranarray(((U * s[None, :]) @ V.conj().T).astype(dt))
    info = {}
    W, P = mak.left_polar_(to_dev(A, cuda), None, None, precision="mixed", _info=info)
    Wh, Ph = to_host(W), to_host(P)
    assert info["converged"]
    assert back_err(A, Wh, Ph) <= 1e-12
    assert O.orth_error(Wh) <= 1e-12 * np.sqrt(n)
    assert O.rel_err(Wh, U @ V.conj().T) <= 1e-8
    assert O.rel_err(Ph, (V * s[None, :]) @ V.conj().T) <= 1e-8
