"""GPU tests of the reverse-mode front-end (``autodiff``: torch.autograd
Functions over the device pullbacks), the counterpart of the reference's
ChainRulesCore rules (ext/MatrixAlgebraKitChainRulesCoreExt.jl:26-43,
249-261), checked the way the reference's test_rrule does
(test/testsuite/chainrules.jl:53-145): against finite differences of the
factorization itself.

* ``torch.autograd.gradcheck`` (central differences, eps 1e-6) on small
  Float64 and ComplexF64 inputs for qr_compact, qr_full, lq_compact,
  left_polar and right_polar, with every output used;
* the differentiation workload at its own size (ComplexF64 1024 x 512):
  the autograd gradient of real<D_Q, Q> + real<D_R, R> (and of the polar
  loss) against a central difference along a random direction, in both
  precisions (1e-6 relative), and against the oracle's pullback (1e-10).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu
DTS = [torch.float64, torch.complex128]


def _input(shape, dtype, cuda, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn(shape, dtype=dtype, generator=g)
    return A.to(cuda).requires_grad_(True)


@pytest.mark.parametrize("dtype", DTS, ids=str)
@pytest.mark.parametrize("fname,shape", [("qr_compact", (9, 6)), ("qr_compact", (6, 9)),
                                         ("qr_full", (9, 6)), ("lq_compact", (6, 9)),
                                         ("left_polar", (9, 6)), ("left_polar", (7, 7)),
                                         ("right_polar", (6, 9))])
def test_gradcheck(mak, cuda, dtype, fname, shape):
    f = getattr(mak.autodiff, fname)
    A = _input(shape, dtype, cuda, 11)
    k = min(shape)
    if fname == "qr_full":
        # the last m - k columns of the full Q are a gauge choice (any
        # orthonormal basis of the complement): only (Q[:, :k], R) is a
        # differentiable function of A, as in the reference's gauge-invariant
        # qr_full cotangents (src/pullbacks/qr.jl:162-189)
        def fn(X):
            Q, R = f(X)
            return Q[:, :k], R
    else:
        fn = f
    assert torch.autograd.gradcheck(fn, (A,), eps=1e-6, atol=1e-5, rtol=1e-4, fast_mode=True)


def test_forward_leaves_input_and_matches_bang_form(mak, cuda):
    A = _input((40, 24), torch.complex128, cuda, 12)
    A0 = A.detach().clone()
    Q, R = mak.autodiff.qr_compact(A)
    assert torch.equal(A.detach(), A0)
    Q1, R1 = mak.qr_compact(A0)
    assert torch.equal(Q.detach(), Q1) and torch.equal(R.detach(), R1)


def test_unused_output_is_a_zero_tangent(mak, cuda):
    A = _input((30, 20), torch.float64, cuda, 13)
    Q, R = mak.autodiff.qr_compact(A)
    (R.diagonal().sum()).backward()
    An, Qn, Rn = (to_host(x.detach()) for x in (A, Q, R))
    dR = np.eye(20)
    ref, _ = O.qr_pullback(np.zeros_like(An), An, Qn, Rn, None, dR)
    assert O.rel_err(to_host(A.grad), ref) <= 1e-11


@pytest.mark.parametrize("precision", ["native", "mixed"])
@pytest.mark.parametrize("which", ["qr", "polar"])
def test_autograd_1024x512_complex(mak, cuda, precision, which):
    rng = np.random.default_rng(91)
    An = O.gaussian(rng, 1024, 512, np.complex128)
    D1 = O.gaussian(rng, 1024, 512, np.complex128)
    D2 = O.gaussian(rng, 512, 512, np.complex128)
    d1, d2 = to_dev(D1, cuda), to_dev(D2, cuda)
    f = mak.autodiff.qr_compact if which == "qr" else mak.autodiff.left_polar

    def loss(X):
        U, S = f(X, precision=precision)
        return (torch.vdot(d1.flatten(), U.flatten()) + torch.vdot(d2.flatten(), S.flatten())).real

    A = to_dev(An, cuda).requires_grad_(True)
    loss(A).backward()
    G = to_host(A.grad)
    if which == "qr":
        Q, R = O.qr_compact(An)
        ref, _ = O.qr_pullback(np.zeros_like(An), An, Q, R, D1, D2)
    else:
        W, P = O.left_polar_svd(An)
        ref = O.left_polar_pullback(np.zeros_like(An), An, W, P, D1, D2)
    assert O.rel_err(G, ref) <= 1e-10
    E = O.gaussian(rng, 1024, 512, np.complex128)
    h = 1e-6
    with torch.no_grad():
        fp = float(loss(to_dev(An + h * E, cuda)))
        fm = float(loss(to_dev(An - h * E, cuda)))
    fd = (fp - fm) / (2 * h)
    an = float(np.real(np.vdot(G, E)))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (fd, an)
