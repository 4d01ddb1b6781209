"""Reverse rules on CUDA tensors: ``qr_pullback_``, ``qr_null_pullback_``,
``lq_pullback_``, ``lq_null_pullback_``, ``left_polar_pullback_`` and
``right_polar_pullback_``.

Mirror ``qr_pullback!(ΔA, A, (Q, R), (ΔQ, ΔR); rank_atol, gauge_atol)``
(src/pullbacks/qr.jl:73-120) and ``left_polar_pullback!(ΔA, A, (W, P),
(ΔW, ΔP))`` (src/pullbacks/polar.jl:7-29): ``ΔA`` is accumulated into and
returned; a cotangent given as ``None`` is a zero tangent
(``iszerotangent``, src/common/pullbacks.jl:9-12); a gauge-dependent
cotangent emits the reference's warning (qr.jl:50-51).  These are the
functions the package's ChainRulesCore and Mooncake rules call
(ext/MatrixAlgebraKitChainRulesCoreExt.jl:34,254), so the Julia extension
specialises these for CuMatrix.  The right polar rule (polar.jl:37-59) is
the conjugate transpose of the left one.
"""

from __future__ import annotations

import ctypes as ct
import warnings

import torch

from . import _lib
from .algorithms import ArgumentError, DimensionMismatch
from .core import (DTYPE_CODE, SUFFIX, check_cuda_tensor, check_rc, check_status, ld_or_raise,
                   lib, new_info, ptr, read_info, stream_handle, workspace)
from .qr import PRECISION_CODE


def _opts(rank_atol, gauge_atol, precision):
    return _lib.mak_pullback_opts(-1.0 if rank_atol is None else float(rank_atol),
                                  -1.0 if gauge_atol is None else float(gauge_atol),
                                  PRECISION_CODE[precision], 0)


def _chk(X, shape, dtype, name):
    if X is None:
        return
    check_cuda_tensor(X, name)
    if tuple(X.shape) != tuple(shape):
        raise DimensionMismatch(f"{name} must have size {tuple(shape)}, got {tuple(X.shape)}")
    if X.dtype != dtype:
        raise ArgumentError(f"{name} has element type {X.dtype}, expected {dtype}")


def qr_pullback_(dA, A, QR, dQR, rank_atol=None, gauge_atol=None, precision="native",
                 _info=None):
    """``qr_pullback!``: dA += (pullback of qr_compact / qr_full at (Q, R))."""
    Q, R = QR
    dQ, dR = dQR
    check_cuda_tensor(dA, "dA")
    m, n = Q.shape[0], R.shape[1]
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"size of dA ({tuple(dA.shape)}) does not match size of Q*R "
                                f"({m}, {n})")
    # qr_full and qr_compact only differ when m > n (Q m x m, R m x n)
    full = int(m > n and Q.shape[1] == m)
    k = min(m, n)
    qc = m if full else k
    _chk(Q, (m, qc), dA.dtype, "Q")
    _chk(R, (m if full else k, n), dA.dtype, "R")
    _chk(dQ, Q.shape, dA.dtype, "dQ")
    _chk(dR, R.shape, dA.dtype, "dR")
    opts = _opts(rank_atol, gauge_atol, precision)
    L = lib()
    nbytes = ct.c_size_t(0)
    check_rc(L.mak_qr_pullback_workspace(DTYPE_CODE[dA.dtype], m, n, full, opts.precision,
                                         ct.byref(nbytes)), "mak_qr_pullback_workspace")
    dev = dA.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_qr_pullback_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, full, ptr(dA), ld_or_raise(dA, "dA"), ptr(Q), ld_or_raise(Q, "Q"), ptr(R),
                ld_or_raise(R, "R"), ptr(dQ), ld_or_raise(dQ, "dQ") if dQ is not None else 1,
                ptr(dR), ld_or_raise(dR, "dR") if dR is not None else 1, ct.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if inf.gauge > inf.gauge_atol:
        warnings.warn(f"`qr` cotangents sensitive to gauge choice: (|Δgauge| = {inf.gauge})",
                      RuntimeWarning, stacklevel=2)
    if _info is not None:
        _info.update(rank=inf.rank, gauge=inf.gauge, gauge_atol=inf.gauge_atol)
    return dA


def left_polar_pullback_(dA, A, WP, dWP, precision="native", _info=None):
    """``left_polar_pullback!``: dA += (pullback of left_polar at (W, P))."""
    W, P = WP
    dW, dP = dWP
    check_cuda_tensor(dA, "dA")
    m, n = W.shape
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"dA must have size {(m, n)}")
    _chk(W, (m, n), dA.dtype, "W")
    _chk(P, (n, n), dA.dtype, "P")
    _chk(dW, (m, n), dA.dtype, "dW")
    _chk(dP, (n, n), dA.dtype, "dP")
    opts = _opts(None, None, precision)
    L = lib()
    nbytes = ct.c_size_t(0)
    check_rc(L.mak_left_polar_pullback_workspace(DTYPE_CODE[dA.dtype], m, n, opts.precision,
                                                 ct.byref(nbytes)),
             "mak_left_polar_pullback_workspace")
    dev = dA.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_left_polar_pullback_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, ptr(dA), ld_or_raise(dA, "dA"), ptr(W), ld_or_raise(W, "W"), ptr(P),
                ld_or_raise(P, "P"), ptr(dW), ld_or_raise(dW, "dW") if dW is not None else 1,
                ptr(dP), ld_or_raise(dP, "dP") if dP is not None else 1, ct.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if _info is not None:
        _info.update(iterations=inf.iterations)
    return dA


def right_polar_pullback_(dA, A, PWh, dPWh, precision="native", _info=None):
    """``right_polar_pullback!(ΔA, A, (P, Wᴴ), (ΔP, ΔWᴴ))`` (src/pullbacks/polar.jl:
    37-59): dA += (pullback of right_polar at (P, Wh)).  On the device this is
    the conjugate transpose of the left pullback of A^H at (Wh^H, P) with
    cotangents (dWh^H, dP): the same Sylvester solve, transposed."""
    P, Wh = PWh
    dP, dWh = dPWh
    check_cuda_tensor(dA, "dA")
    m, n = Wh.shape
    if n < m:
        raise ArgumentError(f"Wh must have at least as many columns ({n}) as rows ({m})")
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"dA must have size {(m, n)}")
    _chk(P, (m, m), dA.dtype, "P")
    _chk(Wh, (m, n), dA.dtype, "Wh")
    _chk(dP, (m, m), dA.dtype, "dP")
    _chk(dWh, (m, n), dA.dtype, "dWh")
    opts = _opts(None, None, precision)
    L = lib()
    nbytes = ct.c_size_t(0)
    check_rc(L.mak_right_polar_pullback_workspace(DTYPE_CODE[dA.dtype], m, n, opts.precision,
                                                  ct.byref(nbytes)),
             "mak_right_polar_pullback_workspace")
    dev = dA.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_right_polar_pullback_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, ptr(dA), ld_or_raise(dA, "dA"), ptr(P), ld_or_raise(P, "P"), ptr(Wh),
                ld_or_raise(Wh, "Wh"), ptr(dP), ld_or_raise(dP, "dP") if dP is not None else 1,
                ptr(dWh), ld_or_raise(dWh, "dWh") if dWh is not None else 1, ct.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if _info is not None:
        _info.update(iterations=inf.iterations)
    return dA


def _null_pullback(kind, dA, A, X, dX, gauge_atol, precision, _info):
    """Shared driver of qr_null_pullback_ / lq_null_pullback_."""
    check_cuda_tensor(dA, "dA")
    check_cuda_tensor(A, "A")
    m, n = A.shape
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"dA must have size {(m, n)}")
    k = min(m, n)
    shape = (m, m - k) if kind == "qr_null" else (n - k, n)
    _chk(A, (m, n), dA.dtype, "A")
    _chk(X, shape, dA.dtype, "N" if kind == "qr_null" else "Nh")
    _chk(dX, shape, dA.dtype, "dN" if kind == "qr_null" else "dNh")
    opts = _opts(None, gauge_atol, precision)
    L = lib()
    nbytes = ct.c_size_t(0)
    check_rc(getattr(L, f"mak_{kind}_pullback_workspace")(DTYPE_CODE[dA.dtype], m, n,
                                                          opts.precision, ct.byref(nbytes)),
             f"mak_{kind}_pullback_workspace")
    dev = dA.device
    ldx = ld_or_raise(X, "N") if X.numel() else max(1, shape[0])
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_{kind}_pullback_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, ptr(dA), ld_or_raise(dA, "dA"), ptr(A), ld_or_raise(A, "A"),
                ptr(X) if X.numel() else None, ldx, ptr(dX) if dX is not None else None,
                ld_or_raise(dX, "dN") if dX is not None and dX.numel() else max(1, shape[0]),
                ct.byref(opts), ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if inf.gauge > inf.gauge_atol:
        warnings.warn(f"`{kind}` cotangent sensitive to gauge choice: (|Δgauge| = {inf.gauge})",
                      RuntimeWarning, stacklevel=3)
    if _info is not None:
        _info.update(gauge=inf.gauge, gauge_atol=inf.gauge_atol)
    return dA


def qr_null_pullback_(dA, A, N, dN, gauge_atol=None, precision="native", _info=None):
    """``qr_null_pullback!(ΔA, A, N, ΔN; gauge_atol)`` (src/pullbacks/qr.jl:141-152):
    dA -= N (ΔN^H Q) R^{-H} with (Q, R) = qr_compact(A; positive = true)
    recomputed on the device; warns on a gauge-dependent cotangent (qr.jl:122-128)."""
    return _null_pullback("qr_null", dA, A, N, dN, gauge_atol, precision, _info)


def lq_null_pullback_(dA, A, Nh, dNh, gauge_atol=None, precision="native", _info=None):
    """``lq_null_pullback!(ΔA, A, Nᴴ, ΔNᴴ; gauge_atol)`` (src/pullbacks/lq.jl:133-145):
    dA -= L^{-H} (Q ΔNᴴ^H) Nᴴ with (L, Q) = lq_compact(A; positive = true)."""
    return _null_pullback("lq_null", dA, A, Nh, dNh, gauge_atol, precision, _info)


def lq_pullback_(dA, A, LQ, dLQ, rank_atol=None, gauge_atol=None, precision="native",
                 _info=None):
    """``lq_pullback!(ΔA, A, (L, Q), (ΔL, ΔQ); rank_atol, gauge_atol)``
    (src/pullbacks/lq.jl:71-112): dA += (pullback of lq_compact / lq_full at
    (L, Q)), computed as the conjugate transpose of the QR rule on A^H."""
    L_, Q = LQ
    dL, dQ = dLQ
    check_cuda_tensor(dA, "dA")
    m, n = L_.shape[0], Q.shape[1]
    if tuple(dA.shape) != (m, n):
        raise DimensionMismatch(f"size of dA ({tuple(dA.shape)}) does not match size of L*Q "
                                f"({m}, {n})")
    full = int(n > m and Q.shape[0] == n)
    k = min(m, n)
    qr_ = n if full else k
    _chk(L_, (m, qr_), dA.dtype, "L")
    _chk(Q, (qr_, n), dA.dtype, "Q")
    _chk(dL, L_.shape, dA.dtype, "dL")
    _chk(dQ, Q.shape, dA.dtype, "dQ")
    opts = _opts(rank_atol, gauge_atol, precision)
    lb = lib()
    nbytes = ct.c_size_t(0)
    check_rc(lb.mak_lq_pullback_workspace(DTYPE_CODE[dA.dtype], m, n, full, opts.precision,
                                          ct.byref(nbytes)), "mak_lq_pullback_workspace")
    dev = dA.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(lb, f"mak_lq_pullback_{SUFFIX[dA.dtype]}")
        rc = fn(m, n, full, ptr(dA), ld_or_raise(dA, "dA"), ptr(L_), ld_or_raise(L_, "L"),
                ptr(Q), ld_or_raise(Q, "Q"), ptr(dL),
                ld_or_raise(dL, "dL") if dL is not None else 1, ptr(dQ),
                ld_or_raise(dQ, "dQ") if dQ is not None else 1, ct.byref(opts), ptr(work),
                nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if inf.gauge > inf.gauge_atol:
        warnings.warn(f"`lq` cotangents sensitive to gauge choice: (|Δgauge| = {inf.gauge})",
                      RuntimeWarning, stacklevel=2)
    if _info is not None:
        _info.update(rank=inf.rank, gauge=inf.gauge, gauge_atol=inf.gauge_atol)
    return dA
