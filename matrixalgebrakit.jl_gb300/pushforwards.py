"""Forward rules: ``left_polar_pushforward_`` and ``right_polar_pushforward_``.

Mirror ``left_polar_pushforward!(ΔA, A, (W, P), (ΔW, ΔP))`` and
``right_polar_pushforward!(ΔA, A, (P, Wᴴ), (ΔP, ΔWᴴ))`` (src/pushforwards/
polar.jl:1-26): the tangent outputs are overwritten and returned in the
reference's order, ``(ΔW, ΔP)`` for the left and ``(ΔWᴴ, ΔP)`` for the right
form.  These are what the package's Enzyme forward rules call
(ext/MatrixAlgebraKitEnzymeExt/MatrixAlgebraKitEnzymeExt.jl:13,120-121).  The Sylvester equation
``P K + K P = ΔP0 - ΔP0^H`` is solved on the device by the sign-function
Newton iteration of the pullbacks; the right form runs the left one on the
conjugate transposes.
"""

from __future__ import annotations

import ctypes as ct

import torch

from .algorithms import ArgumentError, DimensionMismatch
from .core import (DTYPE_CODE, SUFFIX, check_cuda_tensor, check_rc, check_status, empty_cm,
                   ld_or_raise, lib, new_info, ptr, read_info, stream_handle, workspace)
from .pullbacks import _chk, _opts


def left_polar_pushforward_(dA, A, WP, dWP=None, precision="native", _info=None):
    """``left_polar_pushforward!``: writes (dW, dP), the tangent of
    ``left_polar`` at A = W P along dA; returns ``(dW, dP)``."""
    W, P = WP
    check_cuda_tensor(dA, "dA")
    m, n = W.shape
    if m < n:
        raise ArgumentError(f"W must have at least as many rows ({m}) as columns ({n})")
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"dA must have size {(m, n)}")
    if dWP is None:
        dWP = (empty_cm(m, n, dA.dtype, dA.device), empty_cm(n, n, dA.dtype, dA.device))
    dW, dP = dWP
    _chk(W, (m, n), dA.dtype, "W")
    _chk(P, (n, n), dA.dtype, "P")
    _chk(dW, (m, n), dA.dtype, "dW")
    _chk(dP, (n, n), dA.dtype, "dP")
    opts = _opts(None, None, precision)
    L = lib()
    nbytes = ct.c_size_t(0)
    check_rc(L.mak_left_polar_pushforward_workspace(DTYPE_CODE[dA.dtype], m, n, opts.precision,
                                                    ct.byref(nbytes)),
             "mak_left_polar_pushforward_workspace")
    dev = dA.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_left_polar_pushforward_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, ptr(dA), ld_or_raise(dA, "dA"), ptr(W), ld_or_raise(W, "W"), ptr(P),
                ld_or_raise(P, "P"), ptr(dW), ld_or_raise(dW, "dW"), ptr(dP),
                ld_or_raise(dP, "dP"), ct.byref(opts), ptr(work), nbytes.value, ptr(info),
                stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if _info is not None:
        _info.update(iterations=inf.iterations)
    return dW, dP


def right_polar_pushforward_(dA, A, PWh, dPWh=None, precision="native", _info=None):
    """``right_polar_pushforward!``: writes (dP, dWh), the tangent of
    ``right_polar`` at A = P Wh along dA; returns ``(dWh, dP)`` like the
    reference."""
    P, Wh = PWh
    check_cuda_tensor(dA, "dA")
    m, n = Wh.shape
    if n < m:
        raise ArgumentError(f"Wh must have at least as many columns ({n}) as rows ({m})")
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"dA must have size {(m, n)}")
    if dPWh is None:
        dPWh = (empty_cm(m, m, dA.dtype, dA.device), empty_cm(m, n, dA.dtype, dA.device))
    dP, dWh = dPWh
    _chk(P, (m, m), dA.dtype, "P")
    _chk(Wh, (m, n), dA.dtype, "Wh")
    _chk(dP, (m, m), dA.dtype, "dP")
    _chk(dWh, (m, n), dA.dtype, "dWh")
    opts = _opts(None, None, precision)
    L = lib()
    nbytes = ct.c_size_t(0)
    check_rc(L.mak_right_polar_pushforward_workspace(DTYPE_CODE[dA.dtype], m, n, opts.precision,
                                                     ct.byref(nbytes)),
             "mak_right_polar_pushforward_workspace")
    dev = dA.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_right_polar_pushforward_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, ptr(dA), ld_or_raise(dA, "dA"), ptr(P), ld_or_raise(P, "P"), ptr(Wh),
                ld_or_raise(Wh, "Wh"), ptr(dP), ld_or_raise(dP, "dP"), ptr(dWh),
                ld_or_raise(dWh, "dWh"), ct.byref(opts), ptr(work), nbytes.value, ptr(info),
                stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if _info is not None:
        _info.update(iterations=inf.iterations)
    return dWh, dP
