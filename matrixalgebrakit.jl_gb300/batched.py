"""Batched entry points over many uneven blocks (block-sparse symmetry sectors).

The reference has no batched API -- a caller loops ``qr_compact!`` /
``left_polar!`` over the blocks (the symmetry sectors of a block-sparse tensor,
the tensors of an orthogonalisation sweep).  ``batched_qr_compact`` and
``batched_left_polar`` take the whole list in one stream-ordered call
(mak_batched_*), with longest-first scheduling over internal streams; the
result is identical to the per-block calls.
"""

from __future__ import annotations

import ctypes as ct

import torch

from . import _lib
from .algorithms import ArgumentError, select_algorithm
from .core import (DTYPE_CODE, INFO_BYTES, check_cuda_tensor, check_rc, empty_cm, ld_or_raise,
                   lib, stream_handle, to_cm, workspace)
from .qr import PRECISION_CODE


def _items(As, outs):
    arr = (_lib.mak_batch_item * len(As))()
    for i, (A, (Q, R)) in enumerate(zip(As, outs)):
        m, n = A.shape
        arr[i] = _lib.mak_batch_item(DTYPE_CODE[A.dtype], 0, m, n, A.data_ptr(),
                                     ld_or_raise(A, "A"), Q.data_ptr(), ld_or_raise(Q, "Q"),
                                     R.data_ptr() if R is not None and R.numel() else None,
                                     ld_or_raise(R, "R") if R is not None and R.numel() else 1)
    return arr


def _read_infos(infos, n):
    raw = bytes(infos.cpu().numpy().tobytes())
    sz = ct.sizeof(_lib.mak_info)
    return [_lib.mak_info.from_buffer_copy(raw[i * sz:(i + 1) * sz]) for i in range(n)]


def _run(kind, As, outs, opts, copy_inputs, capturing=False):
    if not As:
        return []
    dev = As[0].device
    for A in As:
        check_cuda_tensor(A, "A")
        if A.device != dev:
            raise ArgumentError("all blocks must live on one device")
    work_As = [to_cm(A) for A in As] if copy_inputs else list(As)
    items = _items(work_As, outs)
    L = lib()
    nbytes = ct.c_size_t(0)
    wsfn = L.mak_batched_qr_workspace if kind == "qr" else L.mak_batched_left_polar_workspace
    runfn = L.mak_batched_qr_compact if kind == "qr" else L.mak_batched_left_polar
    check_rc(wsfn(items, len(As), ct.byref(opts), ct.byref(nbytes)), wsfn.__name__)
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        infos = torch.zeros(len(As) * INFO_BYTES, dtype=torch.uint8, device=dev)
        rc = runfn(items, len(As), ct.byref(opts), work.data_ptr(), nbytes.value,
                   infos.data_ptr(), stream_handle(dev))
        check_rc(rc, runfn.__name__)
        if capturing:  # inside CUDA-graph capture: no host reads
            return None
        res = _read_infos(infos, len(As))
    for i, inf in enumerate(res):
        if inf.status != 0:
            raise RuntimeError(f"{runfn.__name__}: block {i}: device status {inf.status}")
    return res


def batched_qr_compact(As, alg=None, copy_inputs=True, outs=None, _capturing=False, **kwargs):
    """qr_compact of every block; returns [(Q_i, R_i)].  With
    ``copy_inputs=False`` the blocks are destroyed (bang semantics)."""
    alg = select_algorithm("qr_compact_", None, alg, **kwargs)
    if outs is None:
        outs = []
        for A in As:
            m, n = A.shape
            k = min(m, n)
            outs.append((empty_cm(m, k, A.dtype, A.device), empty_cm(k, n, A.dtype, A.device)))
    opts = _lib.mak_qr_opts(int(alg.positive), int(alg.blocksize), PRECISION_CODE[alg.precision], 0)
    _run("qr", As, outs, opts, copy_inputs, _capturing)
    return outs


def batched_left_polar(As, alg=None, copy_inputs=True, outs=None, _capturing=False, _info=None,
                       **kwargs):
    """left_polar of every block; returns [(W_i, P_i)].  Without host
    synchronization (CUDA-graph capturable): alg.maxiter Newton iterations
    are launched per block and each block stops on the device once it meets
    the tolerance.  ``_info`` (a list) receives the steps each block took."""
    alg = select_algorithm("left_polar_", None, alg, **kwargs)
    for A in As:
        if A.shape[0] < A.shape[1]:
            raise ArgumentError("every block needs at least as many rows as columns")
    if outs is None:
        outs = [(empty_cm(A.shape[0], A.shape[1], A.dtype, A.device),
                 empty_cm(A.shape[1], A.shape[1], A.dtype, A.device)) for A in As]
    opts = _lib.mak_polar_opts(int(alg.maxiter), PRECISION_CODE[alg.precision],
                               float(alg.tol) if alg.tol is not None else 0.0)
    res = _run("polar", As, outs, opts, copy_inputs, _capturing)
    if _info is not None and res is not None:
        _info.extend(int(r.iterations) for r in res)
    return outs
