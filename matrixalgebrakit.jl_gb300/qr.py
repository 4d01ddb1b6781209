"""QR entry points: ``qr_compact(!)``, ``qr_full(!)`` on CUDA tensors.

Mirrors the reference's ``@functiondef`` pairs (src/interface/qr.jl:20,44)
and their implementations (src/implementations/qr.jl):

* ``qr_compact(A; alg, kwargs...)`` -- copies A (``copy_input``, qr.jl:3-4),
  allocates Q (m x min(m,n)) and R (min(m,n) x n) (``initialize_output``,
  qr.jl:69-75) and calls the bang form; A is not modified.
* ``qr_compact_(A, (Q, R), alg)`` -- ``qr_compact!``: validates sizes and
  element types (``check_input``, qr.jl:19-29, raising DimensionMismatch /
  ArgumentError), destroys A and returns the *same* Q and R objects.  An
  empty R (0 elements) means R is not computed (qr.jl:149).
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .algorithms import ArgumentError, DimensionMismatch, select_algorithm
from .core import (DTYPE_CODE, SUFFIX, check_cuda_tensor, check_rc, check_status, empty_cm,
                   ld_or_raise, lib, new_info, ptr, read_info, stream_handle, to_cm, workspace)

_QR_ARGNAMES = ("m", "n", "A", "lda", "Q", "ldq", "R", "ldr", "opts", "work", "work_bytes",
                "info", "stream")
PRECISION_CODE = {"native": _lib.MAK_PREC_NATIVE, "mixed": _lib.MAK_PREC_MIXED}


def _opts(alg) -> _lib.mak_qr_opts:
    return _lib.mak_qr_opts(int(bool(alg.positive)), int(alg.blocksize),
                            PRECISION_CODE[alg.precision], 0)


def _check_input(A, Q, R, full: bool):
    check_cuda_tensor(A, "A")
    m, n = A.shape
    k = min(m, n)
    qshape = (m, m) if full else (m, k)
    rshape = (m, n) if full else (k, n)
    if not isinstance(Q, torch.Tensor) or Q.dim() != 2:
        raise ArgumentError("Q must be a matrix")
    if tuple(Q.shape) != qshape:
        raise DimensionMismatch(f"Q has size {tuple(Q.shape)}, expected {qshape}")
    if Q.dtype != A.dtype:
        raise ArgumentError(f"Q has element type {Q.dtype}, expected {A.dtype}")
    if R is not None and R.numel() > 0:
        if tuple(R.shape) != rshape:
            raise DimensionMismatch(f"R has size {tuple(R.shape)}, expected {rshape}")
    if R is not None and R.dtype != A.dtype:
        raise ArgumentError(f"R has element type {R.dtype}, expected {A.dtype}")
    for X, nm in ((Q, "Q"), (R, "R")):
        if X is not None and X.numel() > 0 and X.device != A.device:
            raise ArgumentError(f"{nm} must be on {A.device}")


def _qr_bang(A, QR, alg, full: bool, info_out=None):
    Q, R = QR
    _check_input(A, Q, R, full)
    m, n = A.shape
    want_r = R is not None and R.numel() > 0
    lda = ld_or_raise(A, "A")
    ldq = ld_or_raise(Q, "Q")
    ldr = ld_or_raise(R, "R") if want_r else 1
    dev = A.device
    code = DTYPE_CODE[A.dtype]
    opts = _opts(alg)
    L = lib()
    nbytes = C.c_size_t(0)
    check_rc(L.mak_qr_workspace(code, m, n, int(full), C.byref(opts), C.byref(nbytes)),
             "mak_qr_workspace")
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev) if info_out is None else info_out
        fn = getattr(L, f"mak_qr_{'full' if full else 'compact'}_{SUFFIX[A.dtype]}")
        rc = fn(m, n, ptr(A), lda, ptr(Q), ldq, ptr(R) if want_r else None, ldr, C.byref(opts),
                ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, fn.__name__, _QR_ARGNAMES)
        if info_out is None:
            check_status(read_info(info), fn.__name__)
    return Q, R


def qr_compact_(A, QR=None, alg=None, info=None, **kwargs):
    """``qr_compact!(A, (Q, R), alg)``: destroys A, returns the passed Q, R.

    Like the reference, the call checks the device's outcome record before
    it returns (one host synchronization).  With ``info`` (a record from
    ``new_info(device)``) it returns as soon as the work is queued on the
    current stream, as the C ABI does, and the caller checks the record
    later with ``check_info`` (so that copies and the next calls overlap)."""
    alg = select_algorithm("qr_compact_", A, alg, **kwargs)
    if QR is None:
        QR = initialize_output("qr_compact_", A)
    return _qr_bang(A, QR, alg, full=False, info_out=info)


def qr_full_(A, QR=None, alg=None, info=None, **kwargs):
    """``qr_full!(A, (Q, R), alg)``: Q is m x m, R is m x n (``info`` as for
    ``qr_compact_``)."""
    alg = select_algorithm("qr_full_", A, alg, **kwargs)
    if QR is None:
        QR = initialize_output("qr_full_", A)
    return _qr_bang(A, QR, alg, full=True, info_out=info)


def qr_compact(A, alg=None, **kwargs):
    """``qr_compact(A; kwargs...)``: A is left unmodified."""
    check_cuda_tensor(A, "A")
    return qr_compact_(to_cm(A), None, alg, **kwargs)


def qr_full(A, alg=None, **kwargs):
    """``qr_full(A; kwargs...)``: A is left unmodified."""
    check_cuda_tensor(A, "A")
    return qr_full_(to_cm(A), None, alg, **kwargs)


def qr_null_(A, N=None, alg=None, **kwargs):
    """``qr_null!(A, N, alg)`` (src/implementations/qr.jl:236-295): the last
    m - min(m,n) columns of the full Q, an orthonormal basis of the left null
    space of A."""
    check_cuda_tensor(A, "A")
    m, n = A.shape
    k = min(m, n)
    if N is None:
        N = empty_cm(m, m - k, A.dtype, A.device)
    if tuple(N.shape) != (m, m - k):
        raise DimensionMismatch(f"N has size {tuple(N.shape)}, expected {(m, m - k)}")
    Q, _ = qr_full_(A, (empty_cm(m, m, A.dtype, A.device), None), alg, **kwargs)
    N.copy_(Q[:, k:])
    return N


def qr_null(A, alg=None, **kwargs):
    check_cuda_tensor(A, "A")
    return qr_null_(to_cm(A), None, alg, **kwargs)


def initialize_output(f, A):
    """``initialize_output`` (src/implementations/qr.jl:63-81)."""
    m, n = A.shape
    k = min(m, n)
    if f in ("qr_full_", "qr_full"):
        return empty_cm(m, m, A.dtype, A.device), empty_cm(m, n, A.dtype, A.device)
    return empty_cm(m, k, A.dtype, A.device), empty_cm(k, n, A.dtype, A.device)
