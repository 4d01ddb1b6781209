"""Reverse-mode front-end: ``torch.autograd.Function`` wrappers of the
factorizations over the device pullbacks.

These are the counterparts of the reference's ChainRulesCore rules
(ext/MatrixAlgebraKitChainRulesCoreExt.jl:26-43 for qr_compact / qr_full,
249-261 for left_polar / right_polar): the forward pass copies A (the
factorization itself runs on the copy, so the caller's A is untouched, as
``copy_input`` does), and the backward pass calls the pullback on the
device (``qr_pullback!``, ``left_polar_pullback!``, ``right_polar_pullback!``,
``lq_pullback!``) with the incoming cotangents.  An output whose gradient is
not needed arrives as ``None`` and is passed on as a zero tangent.

Complex convention: PyTorch's gradient of a real loss L with respect to a
complex z is conj(dL/dz) * 2 = dL/d(re z) + i dL/d(im z), i.e. the cotangent
C with dL = Re <C, dz> = Re sum(conj(C) dz) -- the same convention
ChainRules uses for the reference's pullbacks, so cotangents pass through
unchanged.
"""

from __future__ import annotations

import torch

from .algorithms import select_algorithm
from .core import check_cuda_tensor, empty_cm, to_cm
from .lq import lq_compact_
from .polar import left_polar_, right_polar_
from .pullbacks import left_polar_pullback_, lq_pullback_, qr_pullback_, right_polar_pullback_
from .qr import qr_compact_, qr_full_


def _cm_or_none(X):
    return None if X is None else to_cm(X)


def _zeros_cm(A):
    m, n = A.shape
    return empty_cm(m, n, A.dtype, A.device).zero_()


class _QR(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, alg, full):
        ctx.set_materialize_grads(False)
        Q, R = (qr_full_ if full else qr_compact_)(to_cm(A.detach()), None, alg)
        ctx.save_for_backward(Q, R)
        ctx.alg = alg
        return Q, R

    @staticmethod
    def backward(ctx, dQ, dR):
        Q, R = ctx.saved_tensors
        if dQ is None and dR is None:
            return None, None, None
        dA = _zeros_cm(torch.empty(Q.shape[0], R.shape[1], dtype=Q.dtype, device=Q.device))
        qr_pullback_(dA, None, (Q, R), (_cm_or_none(dQ), _cm_or_none(dR)),
                     precision=ctx.alg.precision)
        return dA, None, None


class _LeftPolar(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, alg):
        ctx.set_materialize_grads(False)
        W, P = left_polar_(to_cm(A.detach()), None, alg)
        ctx.save_for_backward(W, P)
        ctx.alg = alg
        return W, P

    @staticmethod
    def backward(ctx, dW, dP):
        W, P = ctx.saved_tensors
        if dW is None and dP is None:
            return None, None
        dA = _zeros_cm(W)
        left_polar_pullback_(dA, None, (W, P), (_cm_or_none(dW), _cm_or_none(dP)),
                             precision=ctx.alg.precision)
        return dA, None


class _RightPolar(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, alg):
        ctx.set_materialize_grads(False)
        P, Wh = right_polar_(to_cm(A.detach()), None, alg)
        ctx.save_for_backward(P, Wh)
        ctx.alg = alg
        return P, Wh

    @staticmethod
    def backward(ctx, dP, dWh):
        P, Wh = ctx.saved_tensors
        if dP is None and dWh is None:
            return None, None
        dA = _zeros_cm(Wh)
        right_polar_pullback_(dA, None, (P, Wh), (_cm_or_none(dP), _cm_or_none(dWh)),
                              precision=ctx.alg.precision)
        return dA, None


class _LQ(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, alg):
        ctx.set_materialize_grads(False)
        L, Q = lq_compact_(to_cm(A.detach()), None, alg)
        ctx.save_for_backward(L, Q)
        ctx.alg = alg
        return L, Q

    @staticmethod
    def backward(ctx, dL, dQ):
        L, Q = ctx.saved_tensors
        if dL is None and dQ is None:
            return None, None
        dA = _zeros_cm(torch.empty(L.shape[0], Q.shape[1], dtype=L.dtype, device=L.device))
        precision = getattr(getattr(ctx.alg, "alg", ctx.alg), "precision", "native")
        lq_pullback_(dA, None, (L, Q), (_cm_or_none(dL), _cm_or_none(dQ)), precision=precision)
        return dA, None


def qr_compact(A, alg=None, **kwargs):
    """Differentiable ``qr_compact(A)``: returns (Q, R); gradients flow to A
    through ``qr_pullback!`` on the device."""
    check_cuda_tensor(A, "A")
    return _QR.apply(A, select_algorithm("qr_compact", A, alg, **kwargs), False)


def qr_full(A, alg=None, **kwargs):
    """Differentiable ``qr_full(A)``."""
    check_cuda_tensor(A, "A")
    return _QR.apply(A, select_algorithm("qr_full", A, alg, **kwargs), True)


def left_polar(A, alg=None, **kwargs):
    """Differentiable ``left_polar(A)``: returns (W, P); gradients through
    ``left_polar_pullback!`` (device Sylvester solve)."""
    check_cuda_tensor(A, "A")
    return _LeftPolar.apply(A, select_algorithm("left_polar", A, alg, **kwargs))


def right_polar(A, alg=None, **kwargs):
    """Differentiable ``right_polar(A)``: returns (P, Wh)."""
    check_cuda_tensor(A, "A")
    return _RightPolar.apply(A, select_algorithm("right_polar", A, alg, **kwargs))


def lq_compact(A, alg=None, **kwargs):
    """Differentiable ``lq_compact(A)``: returns (L, Q)."""
    check_cuda_tensor(A, "A")
    return _LQ.apply(A, select_algorithm("lq_compact", A, alg, **kwargs))
