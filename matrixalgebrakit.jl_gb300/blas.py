"""``gemm``: the library's product kernel (native SIMT or split-precision
tensor core), exposed for callers' own contractions and for tests."""

from __future__ import annotations

import ctypes as ct

import torch

from .algorithms import ArgumentError, DimensionMismatch
from .core import (DTYPE_CODE, check_cuda_tensor, check_rc, check_status, empty_cm, ld_or_raise,
                   lib, new_info, ptr, read_info, stream_handle, workspace)
from .qr import PRECISION_CODE

_OPS = {"N": 0, "T": 1, "C": 2}
_ARGNAMES = ("opA", "opB", "m", "n", "k", "alpha", "A", "lda", "B", "ldb", "beta", "C", "ldc",
             "precision", "work", "work_bytes", "info", "stream")


def gemm(A, B, opA="N", opB="N", alpha=1.0, beta=0.0, C=None, precision="native"):
    """C = alpha op(A) op(B) + beta C for Float64 / ComplexF64 column-major
    CUDA tensors; returns C (allocated when not given)."""
    check_cuda_tensor(A, "A")
    check_cuda_tensor(B, "B")
    if A.dtype != B.dtype or A.dtype not in (torch.float64, torch.complex128):
        raise ArgumentError("gemm supports Float64 and ComplexF64 operands of one type")
    oa, ob = _OPS[opA], _OPS[opB]
    m, k = A.shape if oa == 0 else A.shape[::-1]
    k2, n = B.shape if ob == 0 else B.shape[::-1]
    if k != k2:
        raise DimensionMismatch(f"inner dimensions {k} and {k2} differ")
    if C is None:
        C = empty_cm(m, n, A.dtype, A.device)
        beta = 0.0
    elif tuple(C.shape) != (m, n):
        raise DimensionMismatch(f"C has size {tuple(C.shape)}, expected {(m, n)}")
    L = lib()
    prec = PRECISION_CODE[precision]
    nbytes = _size_t(0)
    check_rc(L.mak_gemm_workspace(DTYPE_CODE[A.dtype], oa, ob, m, n, k, prec, _byref(nbytes)),
             "mak_gemm_workspace")
    dev = A.device
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        info = new_info(dev)
        head = (oa, ob, m, n, k)
        lda, ldb, ldc = ld_or_raise(A, "A"), ld_or_raise(B, "B"), ld_or_raise(C, "C")
        if A.dtype == torch.float64:
            rc = L.mak_gemm_d(*head, float(alpha), ptr(A), lda, ptr(B), ldb, float(beta), ptr(C),
                              ldc, prec, ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        else:
            al = (_double * 2)(complex(alpha).real, complex(alpha).imag)
            be = (_double * 2)(complex(beta).real, complex(beta).imag)
            rc = L.mak_gemm_z(*head, al, ptr(A), lda, ptr(B), ldb, be, ptr(C), ldc, prec,
                              ptr(work), nbytes.value, ptr(info), stream_handle(dev))
        check_rc(rc, "mak_gemm", _ARGNAMES)
        check_status(read_info(info), "mak_gemm")
    return C


_size_t = ct.c_size_t
_double = ct.c_double
_byref = ct.byref
