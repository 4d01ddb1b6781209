"""GPU parity at the sizes of the workloads the benchmark measures, in both
precisions, through the C ABI:

* the batch of uneven blocks of a block-sparse tensor: 300 blocks with
  m_i ~ U{8..1024}, n_i ~ U{4..m_i}, the first half Float64 and the second
  half ComplexF64; batched qr_compact! and left_polar! (PolarNewton), every
  block against the oracle (the reference's LAPACK_HouseholderQR and
  PolarNewton restated, src/implementations/qr.jl:132-188,
  src/implementations/polar.jl:128-166);
* the differentiation workload: ComplexF64 1024 x 512 with iid complex
  Gaussian cotangents, qr_pullback! and left_polar_pullback! against the
  oracle's pullbacks (src/pullbacks/qr.jl:73-120, src/pullbacks/polar.jl:7-29)
  and against central finite differences (step 1e-6) of the GPU
  factorization in the same precision; and the rank-deficient A = B C
  (1024 x 400 times 400 x 512) with a gauge-invariant cotangent, as the
  reference's test/testsuite/chainrules.jl:125-143 does.

Tolerances: R within 1e-12 relative of the oracle's positive-diagonal R and
||A - QR||/||A|| <= 1e-13 (Float64 and ComplexF64, both precisions); the
polar factor of a matrix of condition number kappa is only determined to
about kappa * eps, so W and P are compared at max(1e-11, 1e-14 kappa) and
the bounds ||A - WP||/||A|| <= 1e-12 and ||W^H W - I||_2 <= 1e-12 are
checked directly; Newton iteration counts within one of the oracle's.  The
isometry bound is taken in the spectral norm: the Frobenius norm of the
n x n error matrix grows like n times the entries' rounding (W^H W itself,
formed in Float64 by the check, carries about sqrt(m) eps per entry), so
for n in the hundreds a Frobenius bound of 1e-12 measures the check's own
rounding rather than W.
Pullbacks: 1e-10 relative to the oracle (1e-9 for the rank-deficient
case), and the directional derivative of the scalar loss
real<dQ, Q(A)> + real<dR, R(A)> within 1e-6 relative of the finite
difference.  The finite difference is taken of the native GPU
factorization for both precisions' pullbacks: a central difference with
step h carries the forward's rounding divided by h, and near the rank-400
matrix the mixed forward's slightly larger rounding alone reaches about
1e-6 of the derivative; the mixed forwards are checked against the oracle
directly elsewhere.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu
PRECISIONS = ["native", "mixed"]
C4_SHAPE = (1024, 512)


# ---------------------------------------------------- the 300-block batch ---

def _orth_error_2(W):
    """||W^H W - I||_2 in float64"""
    G = W.conj().T @ W - np.eye(W.shape[1])
    return float(np.linalg.norm(G, 2))


@pytest.fixture(scope="module")
def batch():
    """The 300 blocks and the oracle's factors of each (computed once)."""
    rng = np.random.default_rng(20260101 + 11)
    blocks = O.batched_blocks(rng, nblocks=300, mmin=8, mmax=1024, nmin=4)
    assert sum(A.dtype == np.complex128 for A in blocks) == 150
    qr = [O.qr_compact(A) for A in blocks]
    polar = [O.left_polar_newton(A) for A in blocks]
    kappa = []
    for A in blocks:
        s = np.linalg.svd(A, compute_uv=False)
        kappa.append(float(s[0] / s[-1]))
    return {"blocks": blocks, "qr": qr, "polar": polar, "kappa": kappa}


@pytest.mark.parametrize("precision", PRECISIONS)
def test_batched_qr_300_blocks_vs_oracle(mak, cuda, batch, precision):
    blocks = batch["blocks"]
    outs = mak.batched_qr_compact([to_dev(A, cuda) for A in blocks], precision=precision)
    worst_r, worst_res = 0.0, 0.0
    for A, (Q, R), (Qo, Ro) in zip(blocks, outs, batch["qr"]):
        Qh, Rh = to_host(Q), to_host(R)
        worst_r = max(worst_r, O.rel_err(Rh, Ro))
        worst_res = max(worst_res, O.qr_residual(A, Qh, Rh))
        assert np.all(np.diagonal(Rh).real >= 0) and np.all(np.diagonal(Rh).imag == 0)
    assert worst_r <= 1e-12, worst_r
    assert worst_res <= 1e-13, worst_res


@pytest.mark.parametrize("precision", PRECISIONS)
def test_batched_polar_300_blocks_vs_oracle(mak, cuda, batch, precision):
    blocks = batch["blocks"]
    iters = []
    outs = mak.batched_left_polar([to_dev(A, cuda) for A in blocks], precision=precision,
                                  maxiter=10, _info=iters)
    assert len(iters) == len(blocks)
    for i, (A, (W, P), (Wo, Po, oinfo), kap) in enumerate(
            zip(blocks, outs, batch["polar"], batch["kappa"])):
        Wh, Ph = to_host(W), to_host(P)
        tol = max(1e-11, 1e-14 * kap)
        assert abs(iters[i] - oinfo["iterations"]) <= 1, (i, iters[i], oinfo["iterations"])
        assert O.rel_err(Wh, Wo) <= tol, (i, A.shape, kap)
        assert O.rel_err(Ph, Po) <= tol, (i, A.shape, kap)
        assert np.linalg.norm(A - Wh @ Ph) / np.linalg.norm(A) <= 1e-12, (i, A.shape)
        assert _orth_error_2(Wh) <= 1e-12, (i, A.shape)
        assert np.array_equal(Ph, Ph.conj().T)


# ------------------------------------------ the differentiation workload ---

def _qr_loss(mak, cuda, X, dQ, dR, precision):
    Q, R = mak.qr_compact(to_dev(X, cuda), precision=precision)
    return float(np.real(np.vdot(dQ, to_host(Q)) + np.vdot(dR, to_host(R))))


def _polar_loss(mak, cuda, X, dW, dP, precision):
    W, P = mak.left_polar(to_dev(X, cuda), precision=precision)
    return float(np.real(np.vdot(dW, to_host(W)) + np.vdot(dP, to_host(P))))


def _fd_check(loss, A, G, rng):
    """central difference of `loss` along a random direction against <G, E>"""
    E = O.gaussian(rng, *A.shape, A.dtype)
    h = 1e-6
    fd = (loss(A + h * E) - loss(A - h * E)) / (2 * h)
    an = float(np.real(np.vdot(G, E)))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (fd, an)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_qr_pullback_1024x512_complex(mak, cuda, precision):
    rng = np.random.default_rng(41)
    A = O.gaussian(rng, *C4_SHAPE, np.complex128)
    Q, R = O.qr_compact(A)
    dQ, dR = O.gaussian(rng, *Q.shape, np.complex128), O.gaussian(rng, *R.shape, np.complex128)
    ref, oinfo = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, dR)
    dA = to_dev(np.zeros_like(A), cuda)
    info = {}
    mak.qr_pullback_(dA, to_dev(A, cuda), (to_dev(Q, cuda), to_dev(R, cuda)),
                     (to_dev(dQ, cuda), to_dev(dR, cuda)), precision=precision, _info=info)
    got = to_host(dA)
    assert info["rank"] == oinfo["rank"] == 512
    assert O.rel_err(got, ref) <= 1e-10
    _fd_check(lambda X: _qr_loss(mak, cuda, X, dQ, dR, "native"), A, got, rng)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_qr_pullback_rank_deficient_1024x512(mak, cuda, precision):
    rng = np.random.default_rng(42)
    A = O.rank_deficient(rng, 1024, 512, 400, np.complex128)
    Q, R = O.qr_compact(A)
    dQ, dR = O.gaussian(rng, *Q.shape, np.complex128), O.gaussian(rng, *R.shape, np.complex128)
    dQ, dR = O.remove_qr_gauge_dependence(dQ, dR, A, Q, R)
    ref, oinfo = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, dR)
    dA = to_dev(np.zeros_like(A), cuda)
    info = {}
    mak.qr_pullback_(dA, to_dev(A, cuda), (to_dev(Q, cuda), to_dev(R, cuda)),
                     (to_dev(dQ, cuda), to_dev(dR, cuda)), precision=precision, _info=info)
    got = to_host(dA)
    assert info["rank"] == oinfo["rank"] == 400
    assert info["gauge"] <= info["gauge_atol"]
    assert O.rel_err(got, ref) <= 1e-9
    _fd_check(lambda X: _qr_loss(mak, cuda, X, dQ, dR, "native"), A, got, rng)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_polar_pullback_1024x512_complex(mak, cuda, precision):
    rng = np.random.default_rng(43)
    A = O.gaussian(rng, *C4_SHAPE, np.complex128)
    W, P = O.left_polar_svd(A)
    dW, dP = O.gaussian(rng, *W.shape, np.complex128), O.gaussian(rng, *P.shape, np.complex128)
    ref = O.left_polar_pullback(np.zeros_like(A), A, W, P, dW, dP)
    dA = to_dev(np.zeros_like(A), cuda)
    mak.left_polar_pullback_(dA, None, (to_dev(W, cuda), to_dev(P, cuda)),
                             (to_dev(dW, cuda), to_dev(dP, cuda)), precision=precision)
    got = to_host(dA)
    assert O.rel_err(got, ref) <= 1e-10
    _fd_check(lambda X: _polar_loss(mak, cuda, X, dW, dP, "native"), A, got, rng)


def test_qr_pullback_zero_matrix(mak, cuda):
    """R = 0: the rank tolerance eps(0)^(3/4) is positive (Julia's eps(0.0)
    is the smallest subnormal), so the rank is 0 and the pullback is finite
    (only the gauge-invariant dR12 term of a rank-0 factorization is left)."""
    rng = np.random.default_rng(44)
    for dt in (np.float64, np.complex128):
        A = np.zeros((40, 24), dtype=dt, order="F")
        Q, R = O.qr_compact(A)
        assert O.qr_rank(R) == 0
        dQ = O.gaussian(rng, *Q.shape, dt)
        dR = O.gaussian(rng, *R.shape, dt)
        ref, oinfo = O.qr_pullback(np.zeros_like(A), A, Q, R, dQ, dR)
        dA = to_dev(np.zeros_like(A), cuda)
        info = {}
        with pytest.warns(RuntimeWarning, match="gauge"):
            mak.qr_pullback_(dA, to_dev(A, cuda), (to_dev(Q, cuda), to_dev(R, cuda)),
                             (to_dev(dQ, cuda), to_dev(dR, cuda)), _info=info)
        got = to_host(dA)
        assert info["rank"] == oinfo["rank"] == 0
        assert np.all(np.isfinite(got))
        assert O.rel_err(got, ref) <= 1e-12
