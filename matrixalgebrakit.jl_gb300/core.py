"""Host-side plumbing: column-major CUDA tensors, workspace, streams, status.

PyTorch is used only for device memory and streams.  Matrices follow the
reference's (Julia) column-major layout: a torch tensor of shape (m, n) is
accepted as-is when its strides are (1, ld) with ld >= m, i.e. the
transpose view of a row-major (n, ld) buffer -- exactly the memory of a
CuMatrix.  Non-mutating entry points copy their input into that layout
(the reference's ``copy_input``).
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .algorithms import ArgumentError, DimensionMismatch

DTYPE_CODE = {torch.float64: _lib.MAK_F64, torch.complex128: _lib.MAK_C64,
              torch.float32: _lib.MAK_F32, torch.complex64: _lib.MAK_C32}
SUFFIX = {torch.float64: "d", torch.complex128: "z", torch.float32: "s", torch.complex64: "c"}
REAL_OF = {torch.float64: torch.float64, torch.complex128: torch.float64,
           torch.float32: torch.float32, torch.complex64: torch.float32}
INFO_BYTES = C.sizeof(_lib.mak_info)


def lib():
    return _lib.load()


def check_cuda_tensor(X, name="A"):
    if not isinstance(X, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor on a CUDA device")
    if X.device.type != "cuda":
        raise ArgumentError(f"{name} must live on a CUDA device (no CPU fallback exists)")
    if X.dtype not in DTYPE_CODE:
        raise ArgumentError(f"{name} has unsupported element type {X.dtype}")
    if X.dim() != 2:
        raise DimensionMismatch(f"{name} must be a matrix")


def leading_dim(X) -> int | None:
    """ld if X (m x n) is column-major with unit row stride, else None."""
    m, n = X.shape
    s0, s1 = X.stride()
    if m <= 1 and n <= 1:
        return max(1, m)
    if n == 1:
        return max(1, m) if (s0 == 1 or m <= 1) else None
    if m == 1:
        return s1 if s1 >= 1 else None
    if s0 == 1 and s1 >= m:
        return s1
    return None


def empty_cm(m, n, dtype, device):
    """Uninitialised column-major m x n tensor (strides (1, m))."""
    return torch.empty((n, m), dtype=dtype, device=device).t()


def zeros_cm(m, n, dtype, device):
    return torch.zeros((n, m), dtype=dtype, device=device).t()


def to_cm(X, dtype=None):
    """Column-major copy of X (the reference's ``copy_input``)."""
    dtype = dtype or X.dtype
    Y = empty_cm(X.shape[0], X.shape[1], dtype, X.device)
    Y.copy_(X)
    return Y


def ld_or_raise(X, name):
    ld = leading_dim(X)
    if ld is None:
        raise ArgumentError(f"{name} must be column-major (strides (1, ld) with ld >= rows); "
                            f"got strides {tuple(X.stride())}")
    return ld


def stream_handle(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def workspace(nbytes: int, device):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


def new_info(device):
    """A device outcome record (``mak_info``) for a call to write."""
    return torch.zeros(INFO_BYTES, dtype=torch.uint8, device=device)


def read_info(info_t) -> _lib.mak_info:
    """Copy the device outcome record to the host (synchronizes the stream)."""
    raw = bytes(info_t.cpu().numpy().tobytes())
    return _lib.mak_info.from_buffer_copy(raw)


def ptr(X) -> int | None:
    return None if X is None else X.data_ptr()


def check_rc(rc: int, fname: str, argnames=()):
    if rc == 0:
        return
    if rc < 0:
        idx = -rc
        nm = argnames[idx - 1] if 0 < idx <= len(argnames) else f"#{idx}"
        raise ArgumentError(f"{fname}: argument {idx} ({nm}) is invalid")
    msg = _lib.status_string(rc)
    if rc == _lib.MAK_ERR_UNSUPPORTED:
        raise ArgumentError(f"{fname}: {msg}")
    raise RuntimeError(f"{fname}: {msg} (code {rc})")


def check_info(info_t, fname: str = "mak_gb300"):
    """Read a device outcome record (synchronizes its stream) and raise if
    the call that wrote it failed on the device."""
    check_status(read_info(info_t), fname)


def check_status(info: _lib.mak_info, fname: str):
    if info.status != 0:
        raise RuntimeError(f"{fname}: device status {info.status}: {_lib.status_string(info.status)}")
