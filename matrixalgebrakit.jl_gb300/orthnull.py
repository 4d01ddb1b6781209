"""Orthonormal bases and null spaces: ``left_orth``, ``right_orth``,
``left_null``, ``right_null``, ``project_isometric`` and their batched forms.

Mirrors src/interface/orthnull.jl (selection by ``alg``: ``None`` or a kind
symbol -- ``"qr"`` / ``"polar"`` for left_orth, ``"lq"`` / ``"polar"`` for
right_orth, ``"qr"`` for left_null, ``"lq"`` for right_null -- or an
algorithm instance) and src/implementations/orthnull.jl:79-125, where each
kind forwards to one decomposition:

* ``left_orth!(A, VC, LeftOrthViaQR)``     = ``qr_compact!``   (orthnull.jl:80)
* ``left_orth!(A, VC, LeftOrthViaPolar)``  = ``left_polar!``   (orthnull.jl:81)
* ``right_orth!(A, CVh, RightOrthViaLQ)``  = ``lq_compact!``   (orthnull.jl:91)
* ``right_orth!(A, CVh, RightOrthViaPolar)`` = ``right_polar!`` (orthnull.jl:92)
* ``left_null!`` = ``qr_null!``, ``right_null!`` = ``lq_null!`` (orthnull.jl:104,113)
* ``project_isometric!(A, W, alg)`` = ``left_polar!`` without P
  (src/implementations/projections.jl:70-75)

The SVD kinds and truncation (``trunc``) need a GPU SVD, which is not on this
library's path: they raise ``ArgumentError``.  The batched forms run one
stream-ordered call over a list of blocks (the symmetry sectors of a
block-sparse tensor) through the batched driver.
"""

from __future__ import annotations

from .algorithms import (ArgumentError, GB300_HouseholderQR, GB300_PolarNewton, LeftOrthViaPolar,
                         LeftOrthViaQR, LQViaTransposedQR, RightOrthViaLQ, RightOrthViaPolar)
from .batched import batched_left_polar, batched_qr_compact
from .core import check_cuda_tensor, empty_cm, to_cm
from .lq import lq_compact_, lq_null_
from .polar import left_polar_, right_polar_
from .qr import qr_compact_, qr_null_

_NO_SVD = ("the SVD kinds and truncation are not provided by the GB300 library "
           "(no GPU SVD on this path)")


def left_orth_alg(alg=None, **kwargs):
    """``left_orth_alg`` (src/interface/orthnull.jl:414-456): the
    LeftOrth{ViaQR,ViaPolar} wrapper of a kind symbol or an algorithm."""
    if alg is None or alg == "qr":
        return LeftOrthViaQR(GB300_HouseholderQR(**kwargs))
    if alg == "polar":
        return LeftOrthViaPolar(GB300_PolarNewton(**kwargs))
    if kwargs:
        raise ArgumentError("Additional keyword arguments are not allowed when algorithm "
                            "parameters are specified.")
    if isinstance(alg, (LeftOrthViaQR, LeftOrthViaPolar)):
        return alg
    if isinstance(alg, GB300_HouseholderQR):
        return LeftOrthViaQR(alg)
    if isinstance(alg, GB300_PolarNewton):
        return LeftOrthViaPolar(alg)
    if alg == "svd":
        raise ArgumentError(_NO_SVD)
    raise ArgumentError(f"Unknown alg {alg}")


def right_orth_alg(alg=None, **kwargs):
    """``right_orth_alg`` (src/interface/orthnull.jl): RightOrthViaLQ / ViaPolar."""
    if alg is None or alg == "lq":
        return RightOrthViaLQ(LQViaTransposedQR(GB300_HouseholderQR(**kwargs)))
    if alg == "polar":
        return RightOrthViaPolar(GB300_PolarNewton(**kwargs))
    if kwargs:
        raise ArgumentError("Additional keyword arguments are not allowed when algorithm "
                            "parameters are specified.")
    if isinstance(alg, (RightOrthViaLQ, RightOrthViaPolar)):
        return alg
    if isinstance(alg, GB300_HouseholderQR):
        return RightOrthViaLQ(LQViaTransposedQR(alg))
    if isinstance(alg, LQViaTransposedQR):
        return RightOrthViaLQ(alg)
    if isinstance(alg, GB300_PolarNewton):
        return RightOrthViaPolar(alg)
    if alg == "svd":
        raise ArgumentError(_NO_SVD)
    raise ArgumentError(f"Unknown alg {alg}")


def _no_trunc(trunc):
    if trunc is not None:
        raise ArgumentError(_NO_SVD)


def left_orth_(A, VC=None, alg=None, trunc=None, **kwargs):
    """``left_orth!(A, [VC], [alg]; trunc, kwargs...)``: A = V C with V an
    isometry; destroys A."""
    _no_trunc(trunc)
    alg = left_orth_alg(alg, **kwargs)
    if isinstance(alg, LeftOrthViaQR):
        return qr_compact_(A, VC, alg.alg)
    return left_polar_(A, VC, alg.alg)


def left_orth(A, alg=None, trunc=None, **kwargs):
    """``left_orth(A; alg, trunc, kwargs...) -> V, C``; A is left unmodified."""
    check_cuda_tensor(A, "A")
    return left_orth_(to_cm(A), None, alg, trunc, **kwargs)


def right_orth_(A, CVh=None, alg=None, trunc=None, **kwargs):
    """``right_orth!(A, [CVh], [alg]; trunc, kwargs...)``: A = C Vh with Vh
    having orthonormal rows."""
    _no_trunc(trunc)
    alg = right_orth_alg(alg, **kwargs)
    if isinstance(alg, RightOrthViaLQ):
        return lq_compact_(A, CVh, alg.alg)
    return right_polar_(A, CVh, alg.alg)


def right_orth(A, alg=None, trunc=None, **kwargs):
    """``right_orth(A; alg, trunc, kwargs...) -> C, Vh``; A is left unmodified."""
    check_cuda_tensor(A, "A")
    return right_orth_(to_cm(A), None, alg, trunc, **kwargs)


def left_null_(A, N=None, alg=None, trunc=None, **kwargs):
    """``left_null!``: an orthonormal basis of the null space of A^H (qr_null!)."""
    _no_trunc(trunc)
    if alg not in (None, "qr") and not isinstance(alg, GB300_HouseholderQR):
        raise ArgumentError(_NO_SVD if alg == "svd" else f"Unknown alg {alg}")
    return qr_null_(A, N, None if alg in (None, "qr") else alg, **kwargs)


def left_null(A, alg=None, trunc=None, **kwargs):
    check_cuda_tensor(A, "A")
    return left_null_(to_cm(A), None, alg, trunc, **kwargs)


def right_null_(A, Nh=None, alg=None, trunc=None, **kwargs):
    """``right_null!``: orthonormal rows spanning the null space of A (lq_null!)."""
    _no_trunc(trunc)
    if alg not in (None, "lq") and not isinstance(alg, (GB300_HouseholderQR, LQViaTransposedQR)):
        raise ArgumentError(_NO_SVD if alg == "svd" else f"Unknown alg {alg}")
    return lq_null_(A, Nh, None if alg in (None, "lq") else alg, **kwargs)


def right_null(A, alg=None, trunc=None, **kwargs):
    check_cuda_tensor(A, "A")
    return right_null_(to_cm(A), None, alg, trunc, **kwargs)


def project_isometric_(A, W=None, alg=None, **kwargs):
    """``project_isometric!(A, W, alg)`` (src/implementations/projections.jl:70-75):
    the closest isometry to A, the W of ``left_polar!`` with P not computed."""
    check_cuda_tensor(A, "A")
    if W is None:
        W = empty_cm(A.shape[0], A.shape[1], A.dtype, A.device)
    noP = empty_cm(0, 0, A.dtype, A.device)
    W, _ = left_polar_(A, (W, noP), alg, **kwargs)
    return W


def project_isometric(A, alg=None, **kwargs):
    check_cuda_tensor(A, "A")
    return project_isometric_(to_cm(A), None, alg, **kwargs)


# ----------------------------------------------------------------- batched ---

def batched_left_orth(As, alg=None, copy_inputs=True, outs=None, **kwargs):
    """``left_orth`` of every block of a block-sparse tensor in one call:
    [(V_i, C_i)] via the batched QR (default) or the batched polar driver."""
    a = left_orth_alg(alg, **kwargs)
    if isinstance(a, LeftOrthViaQR):
        return batched_qr_compact(As, a.alg, copy_inputs=copy_inputs, outs=outs)
    return batched_left_polar(As, a.alg, copy_inputs=copy_inputs, outs=outs)


def batched_project_isometric(As, alg=None, copy_inputs=True, **kwargs):
    """``project_isometric`` of every block: [W_i], the batched polar driver
    with P not computed."""
    outs = [(empty_cm(A.shape[0], A.shape[1], A.dtype, A.device),
             empty_cm(0, 0, A.dtype, A.device)) for A in As]
    res = batched_left_polar(As, alg, copy_inputs=copy_inputs, outs=outs, **kwargs)
    return [W for W, _ in res]
