"""Polar entry points: ``left_polar(!)`` on CUDA tensors.

Mirrors ``@functiondef left_polar`` (src/interface/polar.jl:20) and
``left_polar!(A, (W, P), ::PolarNewton)`` (src/implementations/polar.jl:99-111):
m >= n is required (ArgumentError otherwise, polar.jl:6-17); an empty P is
returned unchanged and not computed; the bang form returns the same W and P
objects; non-convergence within ``maxiter`` emits a warning, not an error
(polar.jl:159-161).
"""

from __future__ import annotations

import ctypes as C
import warnings

import torch

from . import _lib
from .algorithms import ArgumentError, DimensionMismatch, select_algorithm
from .core import (DTYPE_CODE, SUFFIX, check_cuda_tensor, check_rc, check_status, empty_cm,
                   ld_or_raise, lib, new_info, ptr, read_info, stream_handle, to_cm, workspace)
from .qr import PRECISION_CODE

_ARGNAMES = ("m", "n", "A", "lda", "W", "ldw", "P", "ldp", "opts", "work", "work_bytes", "info",
             "stream")


class SingularException(ArithmeticError):
    """Julia's ``LinearAlgebra.SingularException`` (an exactly singular iterate)."""


def _opts(alg) -> _lib.mak_polar_opts:
    return _lib.mak_polar_opts(int(alg.maxiter), PRECISION_CODE[alg.precision],
                               float(alg.tol) if alg.tol is not None else 0.0)


def _check_input(A, W, P):
    check_cuda_tensor(A, "A")
    m, n = A.shape
    if m < n:
        raise ArgumentError(f"input matrix needs at least as many rows ({m}) as columns ({n})")
    if tuple(W.shape) != (m, n):
        raise DimensionMismatch(f"W has size {tuple(W.shape)}, expected {(m, n)}")
    if W.dtype != A.dtype:
        raise ArgumentError(f"W has element type {W.dtype}, expected {A.dtype}")
    if P is not None and P.numel() > 0 and tuple(P.shape) != (n, n):
        raise DimensionMismatch(f"P has size {tuple(P.shape)}, expected {(n, n)}")
    if P is not None and P.dtype != A.dtype:
        raise ArgumentError(f"P has element type {P.dtype}, expected {A.dtype}")


def initialize_output(A):
    m, n = A.shape
    return empty_cm(m, n, A.dtype, A.device), empty_cm(n, n, A.dtype, A.device)


def left_polar_(A, WP=None, alg=None, _info=None, **kwargs):
    """``left_polar!(A, (W, P), alg)``: destroys A, returns the passed W, P."""
    alg = select_algorithm("left_polar_", A, alg, **kwargs)
    if WP is None:
        check_cuda_tensor(A, "A")
        WP = initialize_output(A)
    W, P = WP
    _check_input(A, W, P)
    m, n = A.shape
    want_p = P is not None and P.numel() > 0
    lda = ld_or_raise(A, "A")
    ldw = ld_or_raise(W, "W")
    ldp = ld_or_raise(P, "P") if want_p else 1
    opts = _opts(alg)
    L = lib()
    nbytes = C.c_size_t(0)
    check_rc(L.mak_left_polar_workspace(DTYPE_CODE[A.dtype], m, n, int(want_p), C.byref(opts),
                                        C.byref(nbytes)), "mak_left_polar_workspace")
    dev = A.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_left_polar_newton_{SUFFIX[A.dtype]}")
        rc = fn(m, n, ptr(A), lda, ptr(W), ldw, ptr(P) if want_p else None, ldp, C.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__, _ARGNAMES)
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if inf.singular:
        raise SingularException("left_polar!: Newton iterate is exactly singular")
    if n > 0 and not inf.converged:
        warnings.warn(f"`left_polar!` via Newton iteration did not converge within {alg.maxiter} "
                      f"iterations (final residual: {inf.residual})", RuntimeWarning, stacklevel=2)
    if _info is not None:
        _info.update(iterations=inf.iterations, residual=inf.residual, converged=bool(inf.converged))
    return W, P


def left_polar(A, alg=None, **kwargs):
    """``left_polar(A; kwargs...)``: A is left unmodified."""
    check_cuda_tensor(A, "A")
    return left_polar_(to_cm(A), None, alg, **kwargs)


def _check_input_right(A, P, Wh):
    """``check_input(right_polar!, ...)`` (src/implementations/polar.jl:18-30)."""
    check_cuda_tensor(A, "A")
    m, n = A.shape
    if n < m:
        raise ArgumentError(f"input matrix needs at least as many columns ({n}) as rows ({m})")
    if P is not None and P.numel() > 0 and tuple(P.shape) != (m, m):
        raise DimensionMismatch(f"P has size {tuple(P.shape)}, expected {(m, m)}")
    if P is not None and P.dtype != A.dtype:
        raise ArgumentError(f"P has element type {P.dtype}, expected {A.dtype}")
    if tuple(Wh.shape) != (m, n):
        raise DimensionMismatch(f"Wh has size {tuple(Wh.shape)}, expected {(m, n)}")
    if Wh.dtype != A.dtype:
        raise ArgumentError(f"Wh has element type {Wh.dtype}, expected {A.dtype}")


def initialize_output_right(A):
    """``initialize_output(right_polar!, ...)`` (src/implementations/polar.jl:39-44)."""
    m, n = A.shape
    return empty_cm(m, m, A.dtype, A.device), empty_cm(m, n, A.dtype, A.device)


def right_polar_(A, PWh=None, alg=None, _info=None, **kwargs):
    """``right_polar!(A, (P, Wh), alg)`` (src/implementations/polar.jl:113-125):
    A = P Wh for n >= m, computed on the device as the conjugate transpose of
    the left polar decomposition of A^H.  A is read, not written; an empty P is
    returned unchanged and not computed; returns the passed P and Wh."""
    alg = select_algorithm("right_polar_", A, alg, **kwargs)
    if PWh is None:
        check_cuda_tensor(A, "A")
        PWh = initialize_output_right(A)
    P, Wh = PWh
    _check_input_right(A, P, Wh)
    m, n = A.shape
    want_p = P is not None and P.numel() > 0
    lda = ld_or_raise(A, "A")
    ldwh = ld_or_raise(Wh, "Wh")
    ldp = ld_or_raise(P, "P") if want_p else 1
    opts = _opts(alg)
    L = lib()
    nbytes = C.c_size_t(0)
    check_rc(L.mak_right_polar_workspace(DTYPE_CODE[A.dtype], m, n, int(want_p), C.byref(opts),
                                         C.byref(nbytes)), "mak_right_polar_workspace")
    dev = A.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(L, f"mak_right_polar_newton_{SUFFIX[A.dtype]}")
        rc = fn(m, n, ptr(A), lda, ptr(P) if want_p else None, ldp, ptr(Wh), ldwh, C.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__, ("m", "n", "A", "lda", "P", "ldp", "Wh", "ldwh", "opts",
                                   "work", "work_bytes", "info", "stream"))
        inf = read_info(info)
    check_status(inf, fn.__name__)
    if inf.singular:
        raise SingularException("right_polar!: Newton iterate is exactly singular")
    if m > 0 and not inf.converged:
        warnings.warn(f"`right_polar!` via Newton iteration did not converge within {alg.maxiter} "
                      f"iterations (final residual: {inf.residual})", RuntimeWarning, stacklevel=2)
    if _info is not None:
        _info.update(iterations=inf.iterations, residual=inf.residual, converged=bool(inf.converged))
    return P, Wh


def right_polar(A, alg=None, **kwargs):
    """``right_polar(A; kwargs...)``: A is left unmodified."""
    check_cuda_tensor(A, "A")
    return right_polar_(to_cm(A), None, alg, **kwargs)
