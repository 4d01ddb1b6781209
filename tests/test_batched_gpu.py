"""GPU tests of the batched entry points (mak_batched_*): uneven blocks of
mixed element types in one stream-ordered call, each compared with the
CPU oracle -- the result must equal the per-block factorizations."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


def _blocks(seed, nblocks, mmax):
    rng = np.random.default_rng(seed)
    return O.batched_blocks(rng, nblocks=nblocks, mmin=8, mmax=mmax, nmin=4)


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_batched_qr_compact(mak, cuda, precision):
    blocks = _blocks(71, 24, 300)
    outs = mak.batched_qr_compact([to_dev(A, cuda) for A in blocks], precision=precision)
    for A, (Q, R) in zip(blocks, outs):
        Qo, Ro = O.qr_compact(A)
        assert O.rel_err(to_host(R), Ro) <= 1e-12
        assert O.qr_residual(A, to_host(Q), to_host(R)) <= 5e-13


def test_batched_qr_matches_single_calls(mak, cuda):
    """The streams run the single-call kernels in the same order (the
    one-CTA small-block launch switched off): bit-identical factors; with it
    on, the small blocks agree to rounding."""
    blocks = _blocks(72, 10, 200)
    mak.autotune.set_tuning(MAK_SMALL_QR_BYTES=0)
    try:
        outs = mak.batched_qr_compact([to_dev(A, cuda) for A in blocks])
    finally:
        mak.autotune.set_tuning(MAK_SMALL_QR_BYTES=None)
    outs_small = mak.batched_qr_compact([to_dev(A, cuda) for A in blocks])
    for A, (Q, R), (Qs, Rs) in zip(blocks, outs, outs_small):
        Q1, R1 = mak.qr_compact(to_dev(A, cuda))
        assert torch.equal(R, R1) and torch.equal(Q, Q1)  # same kernels, same order
        assert O.rel_err(to_host(Rs), to_host(R1)) <= 1e-13
        assert O.rel_err(to_host(Qs), to_host(Q1)) <= 1e-13


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_batched_left_polar(mak, cuda, precision):
    blocks = _blocks(73, 16, 200)
    outs = mak.batched_left_polar([to_dev(A, cuda) for A in blocks], precision=precision)
    for A, (W, P) in zip(blocks, outs):
        Wh, Ph = to_host(W), to_host(P)
        assert np.linalg.norm(A - Wh @ Ph) / np.linalg.norm(A) <= 1e-12
        assert O.orth_error(Wh) <= 1e-12 * np.sqrt(A.shape[1])


def test_batched_graph_capture(mak, cuda):
    """The batch is one stream-ordered unit: capture it in a CUDA graph and replay."""
    blocks = _blocks(74, 12, 160)
    srcs = [to_dev(A, cuda) for A in blocks]
    work = [s.clone() for s in srcs]
    outs = mak.batched_qr_compact(work, copy_inputs=False)  # first call creates the streams
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for w, a in zip(work, srcs):
            w.copy_(a)
        with torch.cuda.graph(g, stream=s):
            for w, a in zip(work, srcs):
                w.copy_(a)
            mak.batched_qr_compact(work, copy_inputs=False, outs=outs, _capturing=True)
    torch.cuda.current_stream().wait_stream(s)
    for o in outs:
        o[0].zero_(); o[1].zero_()
    g.replay()
    torch.cuda.synchronize()
    for A, (Q, R) in zip(blocks, outs):
        assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_batched_polar_stops_on_device(mak, cuda, precision):
    """The batch launches maxiter iterations per block without a host
    synchronization, and each block stops on the device at the reference's
    criterion (conv <= tol), switching to the Newton-Schulz finish in mixed
    precision: it takes the same number of steps, and gives the same
    factors, as the host-checked single-block call (mixed: the batch caps
    the split product's grid, which changes its K-split rounding, so +-1
    step and 1e-13)."""
    blocks = _blocks(76, 12, 240)
    iters = []
    alg = mak.GB300_PolarNewton(maxiter=30, precision=precision)
    outs = mak.batched_left_polar([to_dev(A, cuda) for A in blocks], alg, _info=iters)
    assert len(iters) == len(blocks)
    exact = precision == "native"
    for A, (W, P), k in zip(blocks, outs, iters):
        info = {}
        W1, P1 = mak.left_polar_(to_dev(A, cuda), None, alg, _info=info)
        assert info["converged"] and info["iterations"] < 30
        assert (k == info["iterations"]) if exact else abs(k - info["iterations"]) <= 1
        tol = 1e-14 if exact else 1e-13
        assert O.rel_err(to_host(W), to_host(W1)) <= tol
        assert O.rel_err(to_host(P), to_host(P1)) <= tol
        assert np.linalg.norm(A - to_host(W) @ to_host(P)) / np.linalg.norm(A) <= 1e-13
        assert O.orth_error(to_host(W)) <= 1e-12


def test_batched_two_threads_two_streams(mak, cuda):
    """Two host threads call the batched QR at the same time, each on its
    own stream: the internal streams and events belong to the calling thread
    (and device), so neither call waits on or runs ahead of the other's
    inputs, and both results equal the oracle's."""
    import threading

    sets = {"a": _blocks(81, 14, 300), "b": _blocks(82, 14, 300)}
    results, errors = {}, []
    gate = threading.Barrier(2)

    def run(name):
        try:
            s = torch.cuda.Stream(device=cuda)
            with torch.cuda.stream(s):
                devs = [to_dev(A, cuda) for A in sets[name]]
                gate.wait()
                for _ in range(3):
                    outs = mak.batched_qr_compact(devs, precision="mixed")
                s.synchronize()
                results[name] = [(to_host(Q), to_host(R)) for Q, R in outs]
        except Exception as e:  # reported on the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in sets]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for name, blocks in sets.items():
        for A, (Q, R) in zip(blocks, results[name]):
            assert O.rel_err(R, O.qr_compact(A)[1]) <= 1e-12
            assert O.qr_residual(A, Q, R) <= 5e-13
