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
import warnings

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


def small_qr_max_bytes() -> int:
    """Shared memory (bytes) a block may take in the one-CTA small-block QR:
    m n + 2 min(m, n) elements (0: the kernel is switched off)."""
    return int(lib().mak_small_qr_max_bytes())


def batch_items_device(As, outs):
    """The work list of ``As`` / ``outs`` as a DEVICE array of
    ``mak_batch_item`` records (a uint8 tensor), the layout a caller's own
    kernel may also write."""
    items = _items(As, outs)
    raw = torch.frombuffer(bytearray(bytes(items)), dtype=torch.uint8)
    return raw.to(As[0].device)


def batched_qr_compact_device(As, alg=None, copy_inputs=True, outs=None, items=None,
                              _capturing=False, **kwargs):
    """qr_compact of every block from a work list in DEVICE memory
    (``mak_batched_qr_compact_device``): one persistent launch in which each
    CTA factors whole blocks in shared memory; every block must fit
    ``small_qr_max_bytes()``.  ``items`` (from ``batch_items_device``) may be
    passed to reuse a list; returns [(Q_i, R_i)]."""
    alg = select_algorithm("qr_compact_", None, alg, **kwargs)
    if not As:
        return []
    dev = As[0].device
    for A in As:
        check_cuda_tensor(A, "A")
        if A.device != dev:
            raise ArgumentError("all blocks must live on one device")
    if outs is None:
        outs = []
        for A in As:
            m, n = A.shape
            k = min(m, n)
            outs.append((empty_cm(m, k, A.dtype, A.device), empty_cm(k, n, A.dtype, A.device)))
    work_As = [to_cm(A) for A in As] if copy_inputs else list(As)
    if items is None:
        items = batch_items_device(work_As, outs)
    opts = _lib.mak_qr_opts(int(alg.positive), int(alg.blocksize), PRECISION_CODE[alg.precision], 0)
    L = lib()
    with torch.cuda.device(dev):
        infos = torch.zeros(len(As) * INFO_BYTES, dtype=torch.uint8, device=dev)
        rc = L.mak_batched_qr_compact_device(items.data_ptr(), len(As), ct.byref(opts),
                                             infos.data_ptr(), stream_handle(dev))
        check_rc(rc, "mak_batched_qr_compact_device")
        if _capturing:
            return outs
        res = _read_infos(infos, len(As))
    for i, inf in enumerate(res):
        if inf.status != 0:
            raise RuntimeError(f"mak_batched_qr_compact_device: block {i}: device status "
                               f"{inf.status}")
    return outs


def small_polar_max_bytes() -> int:
    """Shared memory (bytes) a block may take in the one-CTA small-block
    polar: m n + 2 n^2 + 2 n elements and n pivot indices (0: off)."""
    return int(lib().mak_small_polar_max_bytes())


def batched_left_polar_device(As, alg=None, copy_inputs=True, outs=None, items=None,
                              _capturing=False, _info=None, **kwargs):
    """left_polar of every block (m >= n) from a work list in DEVICE memory
    (``mak_batched_left_polar_device``): one persistent launch in which each
    CTA runs the whole Newton iteration of its blocks in shared memory;
    every block must fit ``small_polar_max_bytes()``.  Returns [(W_i, P_i)];
    ``_info`` (a list) receives the steps each block took."""
    alg = select_algorithm("left_polar_", None, alg, **kwargs)
    if not As:
        return []
    dev = As[0].device
    for A in As:
        check_cuda_tensor(A, "A")
        if A.device != dev:
            raise ArgumentError("all blocks must live on one device")
        if A.shape[0] < A.shape[1]:
            raise ArgumentError("every block needs at least as many rows as columns")
    if outs is None:
        outs = [(empty_cm(A.shape[0], A.shape[1], A.dtype, A.device),
                 empty_cm(A.shape[1], A.shape[1], A.dtype, A.device)) for A in As]
    work_As = [to_cm(A) for A in As] if copy_inputs else list(As)
    if items is None:
        items = batch_items_device(work_As, outs)
    opts = _lib.mak_polar_opts(int(alg.maxiter), PRECISION_CODE[alg.precision],
                               float(alg.tol) if alg.tol is not None else 0.0)
    L = lib()
    with torch.cuda.device(dev):
        infos = torch.zeros(len(As) * INFO_BYTES, dtype=torch.uint8, device=dev)
        rc = L.mak_batched_left_polar_device(items.data_ptr(), len(As), ct.byref(opts),
                                             infos.data_ptr(), stream_handle(dev))
        check_rc(rc, "mak_batched_left_polar_device")
        if _capturing:
            return outs
        res = _read_infos(infos, len(As))
    for i, inf in enumerate(res):
        if inf.status != 0:
            raise RuntimeError(f"mak_batched_left_polar_device: block {i}: device status "
                               f"{inf.status}")
    if _info is not None:
        _info.extend((int(r.iterations), int(r.singular)) for r in res)
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


def _pb_items(dAs, F1s, F2s, dF1s, dF2s):
    arr = (_lib.mak_batch_pullback_item * len(dAs))()
    for i, (dA, F1, F2, d1, d2) in enumerate(zip(dAs, F1s, F2s, dF1s, dF2s)):
        m, n = dA.shape
        arr[i] = _lib.mak_batch_pullback_item(
            DTYPE_CODE[dA.dtype], 0, m, n, dA.data_ptr(), ld_or_raise(dA, "dA"),
            F1.data_ptr(), ld_or_raise(F1, "F1"), F2.data_ptr(), ld_or_raise(F2, "F2"),
            d1.data_ptr() if d1 is not None else None,
            ld_or_raise(d1, "dF1") if d1 is not None else 1,
            d2.data_ptr() if d2 is not None else None,
            ld_or_raise(d2, "dF2") if d2 is not None else 1)
    return arr


def _run_pb(kind, dAs, F1s, F2s, dF1s, dF2s, precision, rank_atol=None, gauge_atol=None,
            capturing=False):
    from .pullbacks import _opts

    if not dAs:
        return []
    dev = dAs[0].device
    for lst, nm in ((dAs, "dA"), (F1s, "F1"), (F2s, "F2")):
        for X in lst:
            check_cuda_tensor(X, nm)
            if X.device != dev:
                raise ArgumentError("all blocks must live on one device")
    for dA, F1 in zip(dAs, F1s):
        if dA.dtype != F1.dtype:
            raise ArgumentError("element types of dA and the factors differ")
    items = _pb_items(dAs, F1s, F2s, dF1s, dF2s)
    opts = _opts(rank_atol, gauge_atol, precision)
    L = lib()
    wsfn = getattr(L, f"mak_batched_{kind}_pullback_workspace")
    runfn = getattr(L, f"mak_batched_{kind}_pullback")
    nbytes = ct.c_size_t(0)
    check_rc(wsfn(items, len(dAs), ct.byref(opts), ct.byref(nbytes)), wsfn.__name__)
    with torch.cuda.device(dev):
        work = workspace(nbytes.value, dev)
        infos = torch.zeros(len(dAs) * INFO_BYTES, dtype=torch.uint8, device=dev)
        rc = runfn(items, len(dAs), ct.byref(opts), work.data_ptr(), nbytes.value,
                   infos.data_ptr(), stream_handle(dev))
        check_rc(rc, runfn.__name__)
        if capturing:
            return None
        res = _read_infos(infos, len(dAs))
    for i, inf in enumerate(res):
        if inf.status != 0:
            raise RuntimeError(f"{runfn.__name__}: block {i}: device status {inf.status}")
    return res


def batched_qr_pullback(dAs, QRs, dQRs, precision="native", rank_atol=None, gauge_atol=None,
                        _info=None):
    """``qr_pullback!`` of every block (qr_compact factors): ``dA_i +=`` the
    pullback of ``(dQ_i, dR_i)`` at ``(Q_i, R_i)``; one host synchronization
    for the whole batch (the blocks' ranks).  ``_info`` (a list) receives
    each block's rank."""
    res = _run_pb("qr", dAs, [q for q, _ in QRs], [r for _, r in QRs],
                  [d for d, _ in dQRs], [d for _, d in dQRs], precision, rank_atol, gauge_atol)
    if _info is not None:
        _info.extend(int(r.rank) for r in res)
    for i, r in enumerate(res):
        if r.gauge > r.gauge_atol:
            warnings.warn(f"block {i}: `qr` cotangents sensitive to gauge choice: "
                          f"(|Δgauge| = {r.gauge})", RuntimeWarning, stacklevel=2)
    return dAs


def batched_left_polar_pullback(dAs, WPs, dWPs, precision="native", _capturing=False,
                                _info=None):
    """``left_polar_pullback!`` of every block: ``dA_i +=`` the pullback of
    ``(dW_i, dP_i)`` at ``(W_i, P_i)``; no host synchronization (the
    Sylvester sign iterations stop on the device), so the call can be
    captured in a CUDA graph.  ``_info`` (a list) receives each block's sign
    iteration count."""
    res = _run_pb("left_polar", dAs, [w for w, _ in WPs], [p for _, p in WPs],
                  [d for d, _ in dWPs], [d for _, d in dWPs], precision, capturing=_capturing)
    if res is None:
        return dAs
    if _info is not None:
        _info.extend(int(r.iterations) for r in res)
    for i, r in enumerate(res):
        if not r.converged and dAs[i].shape[1] > 0:
            raise RuntimeError(f"mak_batched_left_polar_pullback: block {i}: the Sylvester "
                               f"sign iteration did not converge in {r.iterations} steps")
    return dAs
