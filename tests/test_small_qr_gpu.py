"""GPU tests of the one-CTA small-block QR and polar (csrc/small.cu): blocks
factored in shared memory by one persistent launch over a work list -- in
DEVICE memory (mak_batched_qr_compact_device / mak_batched_left_polar_device)
or taken by the batched driver -- each compared with the CPU oracle's
qr_compact (positive gauge) and left_polar_newton / left_polar_svd."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (5, 1), (1, 5), (7, 3), (3, 7), (40, 40), (64, 17), (17, 64), (100, 48),
          (130, 31), (33, 90)]
DTYPES = [np.float64, np.complex128, np.float32, np.complex64]


def _tol(dt):
    return 1e-12 if dt in (np.float64, np.complex128) else 2e-5


@pytest.mark.parametrize("dt", DTYPES, ids=lambda d: np.dtype(d).name)
def test_small_qr_device_list(mak, cuda, dt):
    rng = np.random.default_rng(81)
    blocks = [O.gaussian(rng, m, n, dt) for (m, n) in SHAPES]
    outs = mak.batched_qr_compact_device([to_dev(A, cuda) for A in blocks])
    t = _tol(dt)
    for A, (Q, R) in zip(blocks, outs):
        Qh, Rh = to_host(Q), to_host(R)
        Qo, Ro = O.qr_compact(A)
        assert O.rel_err(Rh, Ro) <= t, A.shape
        assert O.rel_err(Qh, Qo) <= 10 * t, A.shape
        assert np.all(np.diagonal(Rh).real >= 0) and np.allclose(np.diagonal(Rh).imag, 0)
        assert np.array_equal(np.triu(Rh), Rh)


def test_small_qr_mixed_types_one_list(mak, cuda):
    """One device list holding all four element types (one launch)."""
    rng = np.random.default_rng(82)
    blocks = [O.gaussian(rng, m, n, DTYPES[i % 4]) for i, (m, n) in enumerate(SHAPES * 2)]
    dev = [to_dev(A, cuda) for A in blocks]
    outs = mak.batched_qr_compact_device(dev)
    for A, (Q, R) in zip(blocks, outs):
        assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= _tol(A.dtype.type)


def test_small_qr_degenerate_and_scaled_columns(mak, cuda):
    """Zero and repeated columns (tau = 0, sign_safe(0) = +1) and columns far
    outside the range of a plain sum of squares (the rescaled norm)."""
    rng = np.random.default_rng(83)
    A = O.gaussian(rng, 60, 20, np.float64)
    A[:, 3] = 0.0
    A[:, 7] = A[:, 2]
    B = O.gaussian(rng, 50, 12, np.complex128)
    d = np.array([1e250, 1e-250, 1.0] * 4)
    B = B * d[None, :]
    outs = mak.batched_qr_compact_device([to_dev(A, cuda), to_dev(B, cuda)])
    (Qa, Ra), (Qb, Rb) = [(to_host(Q), to_host(R)) for Q, R in outs]
    assert O.qr_residual(A, Qa, Ra) <= 1e-14 and O.orth_error(Qa) <= 1e-13
    assert np.all(np.diagonal(Ra) >= 0)
    assert np.all(np.isfinite(Rb)) and O.orth_error(Qb) <= 1e-13
    Ro = O.qr_compact(B)[1]
    for j in range(B.shape[1]):
        assert np.linalg.norm(Rb[:, j] - Ro[:, j]) <= 1e-12 * np.linalg.norm(Ro[:, j])


def test_small_qr_positive_false(mak, cuda):
    rng = np.random.default_rng(84)
    A = O.gaussian(rng, 45, 30, np.complex128)
    (Q, R), = mak.batched_qr_compact_device([to_dev(A, cuda)], positive=False)
    Qh, Rh = to_host(Q), to_host(R)
    assert O.qr_residual(A, Qh, Rh) <= 1e-14 and O.orth_error(Qh) <= 1e-13
    # the raw Householder R: beta = -sign(Re alpha) |column|, real diagonal
    assert np.allclose(np.diagonal(Rh).imag, 0)


def test_small_qr_oversize_item_reports(mak, cuda):
    """An item beyond the shared-memory limit reports MAK_ERR_UNSUPPORTED in
    its record (the device list is not inspected on the host)."""
    cap = mak.small_qr_max_bytes()
    assert cap > 0
    rng = np.random.default_rng(85)
    n = 8
    m = cap // (8 * n) + 8  # m n doubles > cap
    A = O.gaussian(rng, m, n, np.float64)
    B = O.gaussian(rng, 20, 10, np.float64)
    with pytest.raises(RuntimeError, match="block 0: device status 1002"):
        mak.batched_qr_compact_device([to_dev(A, cuda), to_dev(B, cuda)])


def test_batched_routes_small_blocks(mak, cuda):
    """The batched driver sends the blocks that fit to the one-CTA launch and
    the others to its streams; every block matches the oracle."""
    rng = np.random.default_rng(86)
    shapes = [(20, 10), (600, 300), (64, 64), (900, 450), (5, 3), (256, 40)]
    blocks = [O.gaussian(rng, m, n, np.float64 if i % 2 else np.complex128)
              for i, (m, n) in enumerate(shapes)]
    for prec in ("native", "mixed"):
        outs = mak.batched_qr_compact([to_dev(A, cuda) for A in blocks], precision=prec)
        for A, (Q, R) in zip(blocks, outs):
            assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12
            assert O.qr_residual(A, to_host(Q), to_host(R)) <= 5e-13


def test_small_qr_graph_capture(mak, cuda):
    rng = np.random.default_rng(87)
    blocks = [O.gaussian(rng, m, n, np.float64) for (m, n) in SHAPES]
    srcs = [to_dev(A, cuda) for A in blocks]
    work = [s.clone() for s in srcs]
    outs = mak.batched_qr_compact_device(work, copy_inputs=False)
    items = mak.batch_items_device(work, outs)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            for w, a in zip(work, srcs):
                w.copy_(a)
            mak.batched_qr_compact_device(work, copy_inputs=False, outs=outs, items=items,
                                          _capturing=True)
    torch.cuda.current_stream().wait_stream(s)
    for o in outs:
        o[0].zero_()
        o[1].zero_()
    g.replay()
    torch.cuda.synchronize()
    for A, (Q, R) in zip(blocks, outs):
        assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12


POLAR_SHAPES = [(1, 1), (5, 1), (7, 3), (40, 40), (64, 17), (100, 48), (130, 31), (33, 33)]


@pytest.mark.parametrize("dt", DTYPES, ids=lambda d: np.dtype(d).name)
def test_small_polar_device_list(mak, cuda, dt):
    rng = np.random.default_rng(91)
    blocks = [O.gaussian(rng, m, n, dt) for (m, n) in POLAR_SHAPES]
    steps = []
    outs = mak.batched_left_polar_device([to_dev(A, cuda) for A in blocks], _info=steps)
    dbl = dt in (np.float64, np.complex128)
    for A, (W, P), (k, sing) in zip(blocks, outs, steps):
        Wh, Ph = to_host(W), to_host(P)
        n = A.shape[1]
        assert sing == 0
        assert np.array_equal(Ph, Ph.conj().T)  # exactly Hermitian
        back = np.linalg.norm(A - Wh @ Ph) / np.linalg.norm(A)
        assert back <= (1e-12 if dbl else 2e-5), (A.shape, back)
        assert O.orth_error(Wh) <= (1e-12 if dbl else 2e-5) * np.sqrt(n)
        Wo, Po = O.left_polar_svd(A.astype(np.complex128 if np.iscomplexobj(A) else np.float64))
        assert O.rel_err(Wh, Wo) <= (1e-9 if dbl else 1e-3), A.shape
        if dbl:
            ko = O.left_polar_newton(A)[2]["iterations"]
            assert abs(k - ko) <= 1, (A.shape, k, ko)


def test_small_polar_ill_conditioned_and_singular(mak, cuda):
    """kappa = 1e6 (several Newton steps) and an exactly singular block (a
    zero column: the Gauss-Jordan inverse meets a zero pivot)."""
    rng = np.random.default_rng(92)
    n = 40
    U = np.linalg.qr(rng.standard_normal((96, n)))[0]
    V = np.linalg.qr(rng.standard_normal((n, n)))[0]
    A = np.asfortranarray((U * np.logspace(0, -6, n)[None, :]) @ V.T)
    S = O.gaussian(rng, 50, 10, np.float64)
    S[:, 4] = 0.0
    steps = []
    outs = mak.batched_left_polar_device([to_dev(A, cuda), to_dev(S, cuda)], _info=steps)
    Wh, Ph = to_host(outs[0][0]), to_host(outs[0][1])
    assert np.linalg.norm(A - Wh @ Ph) / np.linalg.norm(A) <= 1e-12
    assert O.orth_error(Wh) <= 1e-12 * np.sqrt(n)
    ko = O.left_polar_newton(A)[2]["iterations"]
    assert abs(steps[0][0] - ko) <= 1 and steps[0][1] == 0
    assert steps[1][1] == 1  # singular reported in the record


def test_batched_polar_routes_small_blocks(mak, cuda):
    """The batched polar sends the blocks that fit to the one-CTA launch and
    the others to its streams; every block meets the reference's accuracy."""
    rng = np.random.default_rng(93)
    shapes = [(20, 10), (600, 300), (64, 64), (700, 350), (5, 3), (256, 40)]
    blocks = [O.gaussian(rng, m, n, np.float64 if i % 2 else np.complex128)
              for i, (m, n) in enumerate(shapes)]
    for prec in ("native", "mixed"):
        outs = mak.batched_left_polar([to_dev(A, cuda) for A in blocks], precision=prec)
        for A, (W, P) in zip(blocks, outs):
            Wh, Ph = to_host(W), to_host(P)
            assert np.linalg.norm(A - Wh @ Ph) / np.linalg.norm(A) <= 1e-12
            assert O.orth_error(Wh) <= 1e-12 * np.sqrt(A.shape[1])
