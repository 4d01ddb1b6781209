"""GPU test of the failure path of the bounded device-side waits: a grid
barrier told to expect one more CTA than was launched gives up after its
poll limit, reports MAK_ERR_TIMEOUT in the device status word, and the
context stays usable (a factorization right after it is correct).  No GPU
fault, trap or hang is involved: the wait is bounded by construction."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ctas,missing", [(1, 1), (4, 1), (2, 0)])
def test_grid_barrier_wait_runs_out(mak, cuda, ctas, missing):
    from mak_gb300 import _lib

    lib = mak.library()
    work = torch.zeros(64, dtype=torch.uint8, device=cuda)
    status = torch.full((1,), -7, dtype=torch.int32, device=cuda)
    st = torch.cuda.current_stream(cuda).cuda_stream
    rc = lib.mak_selftest_barrier(ctas, missing, 1 << 14, work.data_ptr(), 64,
                                  status.data_ptr(), st)
    assert rc == 0, lib.mak_status_string(rc)
    torch.cuda.synchronize()
    assert int(status.item()) == (_lib.MAK_ERR_TIMEOUT if missing else 0)
    # the context is still usable
    rng = np.random.default_rng(3)
    A = O.gaussian(rng, 96, 40, np.float64)
    Q, R = mak.qr_compact(to_dev(A, cuda))
    assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12


def test_selftest_rejects_bad_arguments(mak, cuda):
    lib = mak.library()
    work = torch.zeros(64, dtype=torch.uint8, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    st = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.mak_selftest_barrier(0, 1, 100, work.data_ptr(), 64, status.data_ptr(), st) == -1
    assert lib.mak_selftest_barrier(1, 1, 0, work.data_ptr(), 64, status.data_ptr(), st) == -3
    assert lib.mak_selftest_barrier(1, 1, 100, work.data_ptr(), 4, status.data_ptr(), st) == -5
