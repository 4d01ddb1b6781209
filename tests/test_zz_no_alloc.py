"""GPU test of mak_qr_compact_d_noalloc, the Float64 qr_compact! entry point
that takes its scratch from a fixed array inside the library instead of a
caller workspace.  Called through the C ABI and compared with the workspace
entry point mak_qr_compact_d on the same inputs, for two calls in a row.

The file name sorts last so that the suite also exercises the entry after
every other test has run; it passes on its own in a fresh process as well.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, Float64 (the same bound as the qr_compact! parity tests)


def _cm(m, n, device):
    return torch.zeros((n, m), dtype=torch.float64, device=device).t()


def _opts(_lib, precision):
    return _lib.mak_qr_opts(1, 0, precision, 0)


def _run_workspace_entry(lib, _lib, A, precision, device):
    m, n = A.shape
    k = min(m, n)
    Ad = to_dev(A, device)
    Q, R = _cm(m, k, device), _cm(k, n, device)
    info = torch.zeros(C.sizeof(_lib.mak_info), dtype=torch.uint8, device=device)
    nb = C.c_size_t(0)
    opts = _opts(_lib, precision)
    assert lib.mak_qr_workspace(_lib.MAK_F64, m, n, 0, C.byref(opts), C.byref(nb)) == 0
    work = torch.empty(nb.value, dtype=torch.uint8, device=device)
    st = torch.cuda.current_stream(device).cuda_stream
    rc = lib.mak_qr_compact_d(m, n, Ad.data_ptr(), m, Q.data_ptr(), m, R.data_ptr(), k,
                              C.byref(opts), work.data_ptr(), nb.value, info.data_ptr(), st)
    assert rc == 0
    torch.cuda.synchronize()
    return to_host(Q), to_host(R)


@pytest.mark.parametrize("precision", [0, 1], ids=["native", "mixed"])
def test_noalloc_matches_workspace_entry_twice(mak, cuda, precision):
    from mak_gb300 import _lib

    lib = mak.library()
    rng = np.random.default_rng(2024)
    A = O.gaussian(rng, 300, 200, np.float64)
    m, n = A.shape
    Qw, Rw = _run_workspace_entry(lib, _lib, A, precision, cuda)

    opts = _opts(_lib, precision)
    st = torch.cuda.current_stream(cuda).cuda_stream
    outs = []
    for _ in range(2):  # two calls in a row on one stream, no host sync between
        Ad = to_dev(A, cuda)
        Q, R = _cm(m, n, cuda), _cm(n, n, cuda)
        info = torch.zeros(C.sizeof(_lib.mak_info), dtype=torch.uint8, device=cuda)
        rc = lib.mak_qr_compact_d_noalloc(m, n, Ad.data_ptr(), m, Q.data_ptr(), m, R.data_ptr(),
                                          n, C.byref(opts), info.data_ptr(), st)
        assert rc == 0, lib.mak_status_string(rc)
        outs.append((Q, R, info))
    torch.cuda.synchronize()
    for Q, R, info in outs:
        assert _lib.mak_info.from_buffer_copy(bytes(info.cpu().numpy().tobytes())).status == 0
        Qh, Rh = to_host(Q), to_host(R)
        assert O.rel_err(Rh, Rw) <= TOL
        assert O.rel_err(Qh, Qw) <= TOL
        assert O.qr_residual(A, Qh, Rh) <= TOL


def test_noalloc_second_call_leaves_device_memory_unchanged(mak, cuda):
    from mak_gb300 import _lib

    lib = mak.library()
    rng = np.random.default_rng(7)
    A = O.gaussian(rng, 256, 128, np.float64)
    m, n = A.shape
    opts = _opts(_lib, 0)
    st = torch.cuda.current_stream(cuda).cuda_stream
    Ad = to_dev(A, cuda)
    Q, R = _cm(m, n, cuda), _cm(n, n, cuda)
    info = torch.zeros(C.sizeof(_lib.mak_info), dtype=torch.uint8, device=cuda)
    args = (m, n, Ad.data_ptr(), m, Q.data_ptr(), m, R.data_ptr(), n, C.byref(opts),
            info.data_ptr(), st)
    assert lib.mak_qr_compact_d_noalloc(*args) == 0  # set-up on this device
    torch.cuda.synchronize()
    Ad.copy_(to_dev(A, cuda))
    free0, _ = torch.cuda.mem_get_info(cuda)
    assert lib.mak_qr_compact_d_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(cuda)
    assert free1 == free0
    assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= TOL


def test_noalloc_rejects_problems_beyond_the_scratch(mak, cuda):
    from mak_gb300 import _lib

    lib = mak.library()
    m = n = 4096
    opts = _opts(_lib, 0)
    nb = C.c_size_t(0)
    assert lib.mak_qr_workspace(_lib.MAK_F64, m, n, 0, C.byref(opts), C.byref(nb)) == 0
    assert nb.value > _lib.MAK_QR_NOALLOC_SCRATCH_BYTES
    # correctly sized operands, so nothing could go out of bounds either way
    A, Q, R = _cm(m, n, cuda), _cm(m, n, cuda), _cm(n, n, cuda)
    info = torch.zeros(C.sizeof(_lib.mak_info), dtype=torch.uint8, device=cuda)
    before = lib.mak_kernel_launches()
    rc = lib.mak_qr_compact_d_noalloc(m, n, A.data_ptr(), m, Q.data_ptr(), m, R.data_ptr(), n,
                                      C.byref(opts), info.data_ptr(),
                                      torch.cuda.current_stream(cuda).cuda_stream)
    assert rc == _lib.MAK_ERR_WORKSPACE
    assert lib.mak_kernel_launches() == before  # rejected before any work was queued
