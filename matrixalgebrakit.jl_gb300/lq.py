"""LQ entry points: ``lq_compact(!)``, ``lq_full(!)``, ``lq_null(!)`` on CUDA tensors.

Mirrors the reference's LQ interface (src/interface/lq.jl) and its
implementation through the transposed QR, ``lq_via_qr!``
(src/implementations/lq.jl:303-318), which is what the reference runs for
its GPU drivers (lq.jl:130-131) and for ``LQViaTransposedQR``:

* ``check_input`` (lq.jl:9-28): L is m x n (full) or m x min(m,n) (compact),
  or empty (not computed); Q is n x n (full) or min(m,n) x n (compact);
  DimensionMismatch / ArgumentError otherwise.
* ``initialize_output`` (lq.jl:63-74).
* ``lq_compact(A)`` leaves A unmodified (``copy_input``, lq.jl:3-4); the bang
  form returns the same L and Q objects.  The device path reads A and does
  not write it.
"""

from __future__ import annotations

import ctypes as C

import torch

from .algorithms import ArgumentError, DimensionMismatch, LQViaTransposedQR, select_algorithm
from .core import (DTYPE_CODE, SUFFIX, check_cuda_tensor, check_rc, check_status, empty_cm,
                   ld_or_raise, lib, new_info, ptr, read_info, stream_handle, to_cm, workspace)
from .qr import _opts as _qr_opts

_ARGNAMES = ("m", "n", "A", "lda", "L", "ldl", "Q", "ldq", "opts", "work", "work_bytes", "info",
             "stream")


def _check_input(A, L, Q, full: bool):
    check_cuda_tensor(A, "A")
    m, n = A.shape
    k = min(m, n)
    lshape = (m, n) if full else (m, k)
    qshape = (n, n) if full else (k, n)
    if not isinstance(Q, torch.Tensor) or Q.dim() != 2:
        raise ArgumentError("Q must be a matrix")
    if tuple(Q.shape) != qshape:
        raise DimensionMismatch(f"Q has size {tuple(Q.shape)}, expected {qshape}")
    if Q.dtype != A.dtype:
        raise ArgumentError(f"Q has element type {Q.dtype}, expected {A.dtype}")
    if L is not None and L.numel() > 0 and tuple(L.shape) != lshape:
        raise DimensionMismatch(f"L has size {tuple(L.shape)}, expected {lshape}")
    if L is not None and L.dtype != A.dtype:
        raise ArgumentError(f"L has element type {L.dtype}, expected {A.dtype}")
    for X, nm in ((Q, "Q"), (L, "L")):
        if X is not None and X.numel() > 0 and X.device != A.device:
            raise ArgumentError(f"{nm} must be on {A.device}")


def initialize_output(f, A):
    """``initialize_output`` (src/implementations/lq.jl:63-74)."""
    m, n = A.shape
    k = min(m, n)
    if f in ("lq_full_", "lq_full"):
        return empty_cm(m, n, A.dtype, A.device), empty_cm(n, n, A.dtype, A.device)
    return empty_cm(m, k, A.dtype, A.device), empty_cm(k, n, A.dtype, A.device)


def _lq_bang(A, LQ, alg: LQViaTransposedQR, full: bool):
    L_, Q = LQ
    _check_input(A, L_, Q, full)
    m, n = A.shape
    want_l = L_ is not None and L_.numel() > 0
    lda = ld_or_raise(A, "A")
    ldq = ld_or_raise(Q, "Q")
    ldl = ld_or_raise(L_, "L") if want_l else 1
    dev = A.device
    opts = _qr_opts(alg.alg)
    lb = lib()
    nbytes = C.c_size_t(0)
    check_rc(lb.mak_lq_workspace(DTYPE_CODE[A.dtype], m, n, int(full), C.byref(opts),
                                 C.byref(nbytes)), "mak_lq_workspace")
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        fn = getattr(lb, f"mak_lq_{'full' if full else 'compact'}_{SUFFIX[A.dtype]}")
        rc = fn(m, n, ptr(A), lda, ptr(L_) if want_l else None, ldl, ptr(Q), ldq, C.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__, _ARGNAMES)
        check_status(read_info(info), fn.__name__)
    return L_, Q


def lq_compact_(A, LQ=None, alg=None, **kwargs):
    """``lq_compact!(A, (L, Q), alg)``: returns the passed L (m x min(m,n)), Q."""
    alg = select_algorithm("lq_compact_", A, alg, **kwargs)
    if LQ is None:
        check_cuda_tensor(A, "A")
        LQ = initialize_output("lq_compact_", A)
    return _lq_bang(A, LQ, alg, full=False)


def lq_full_(A, LQ=None, alg=None, **kwargs):
    """``lq_full!(A, (L, Q), alg)``: L is m x n, Q is n x n."""
    alg = select_algorithm("lq_full_", A, alg, **kwargs)
    if LQ is None:
        check_cuda_tensor(A, "A")
        LQ = initialize_output("lq_full_", A)
    return _lq_bang(A, LQ, alg, full=True)


def lq_compact(A, alg=None, **kwargs):
    """``lq_compact(A; kwargs...)``: A is left unmodified."""
    check_cuda_tensor(A, "A")
    return lq_compact_(to_cm(A), None, alg, **kwargs)


def lq_full(A, alg=None, **kwargs):
    """``lq_full(A; kwargs...)``: A is left unmodified."""
    check_cuda_tensor(A, "A")
    return lq_full_(to_cm(A), None, alg, **kwargs)


def lq_null_(A, Nh=None, alg=None, **kwargs):
    """``lq_null!(A, Nh, alg)`` through ``lq_null_via_qr!`` (src/implementations/
    lq.jl:320-326): the last n - min(m,n) rows of the full Q, an orthonormal
    basis (as rows) of the null space of A."""
    check_cuda_tensor(A, "A")
    m, n = A.shape
    k = min(m, n)
    if Nh is None:
        Nh = empty_cm(n - k, n, A.dtype, A.device)
    if tuple(Nh.shape) != (n - k, n):
        raise DimensionMismatch(f"Nh has size {tuple(Nh.shape)}, expected {(n - k, n)}")
    _, Q = lq_full_(A, (None, empty_cm(n, n, A.dtype, A.device)), alg, **kwargs)
    Nh.copy_(Q[k:, :])
    return Nh


def lq_null(A, alg=None, **kwargs):
    check_cuda_tensor(A, "A")
    return lq_null_(to_cm(A), None, alg, **kwargs)
