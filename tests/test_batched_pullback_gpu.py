"""GPU tests of the batched reverse rules (mak_batched_qr_pullback,
mak_batched_left_polar_pullback): uneven blocks of mixed element types in
one call, each block's accumulated dA against the oracle's pullback (the
reference's qr_pullback! / left_polar_pullback! restated,
src/pullbacks/qr.jl:73-120, src/pullbacks/polar.jl:7-29) and against the
single-block entry point; the polar batch is also captured in a CUDA graph
and replayed (it synchronizes nothing)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


def _blocks(seed, nblocks, mmax):
    rng = np.random.default_rng(seed)
    return rng, O.batched_blocks(rng, nblocks=nblocks, mmin=8, mmax=mmax, nmin=4)


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_batched_qr_pullback_vs_oracle(mak, cuda, precision):
    rng, blocks = _blocks(301, 20, 400)
    blocks.append(O.rank_deficient(rng, 120, 60, 35, np.complex128))  # rank 35 of 60
    facs = [O.qr_compact(A) for A in blocks]
    cots = []
    for A, (Q, R) in zip(blocks, facs):
        dQ, dR = O.gaussian(rng, *Q.shape, A.dtype), O.gaussian(rng, *R.shape, A.dtype)
        cots.append(O.remove_qr_gauge_dependence(dQ, dR, A, Q, R))
    dA0 = [O.gaussian(rng, *A.shape, A.dtype) for A in blocks]
    dAs = [to_dev(d, cuda) for d in dA0]
    ranks = []
    mak.batched_qr_pullback(dAs, [(to_dev(Q, cuda), to_dev(R, cuda)) for Q, R in facs],
                            [(to_dev(a, cuda), to_dev(b, cuda)) for a, b in cots],
                            precision=precision, _info=ranks)
    for i, (A, (Q, R), (dQ, dR), d0, dA) in enumerate(zip(blocks, facs, cots, dA0, dAs)):
        ref, oinfo = O.qr_pullback(d0, A, Q, R, dQ, dR)
        assert ranks[i] == oinfo["rank"]
        tol = 1e-9 if oinfo["rank"] < min(A.shape) else 1e-10
        assert O.rel_err(to_host(dA) - d0, ref - d0) <= tol, i
        # the same as the single-block entry point
        d1 = to_dev(d0, cuda)
        mak.qr_pullback_(d1, None, (to_dev(Q, cuda), to_dev(R, cuda)),
                         (to_dev(dQ, cuda), to_dev(dR, cuda)), precision=precision)
        assert O.rel_err(to_host(dA), to_host(d1)) <= (0 if precision == "native" else 1e-13)


def test_batched_qr_pullback_zero_tangents(mak, cuda):
    rng, blocks = _blocks(302, 6, 200)
    facs = [O.qr_compact(A) for A in blocks]
    dAs = [to_dev(np.zeros_like(A), cuda) for A in blocks]
    dRs = [O.gaussian(rng, *R.shape, A.dtype) for A, (Q, R) in zip(blocks, facs)]
    mak.batched_qr_pullback(dAs, [(to_dev(Q, cuda), to_dev(R, cuda)) for Q, R in facs],
                            [(None, to_dev(d, cuda)) for d in dRs])
    for A, (Q, R), dR, dA in zip(blocks, facs, dRs, dAs):
        ref, _ = O.qr_pullback(np.zeros_like(A), A, Q, R, None, dR)
        assert O.rel_err(to_host(dA), ref) <= 1e-10


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_batched_polar_pullback_vs_oracle(mak, cuda, precision):
    rng, blocks = _blocks(303, 16, 320)
    facs = [O.left_polar_svd(A) for A in blocks]
    cots = [(O.gaussian(rng, *W.shape, A.dtype), O.gaussian(rng, *P.shape, A.dtype))
            for A, (W, P) in zip(blocks, facs)]
    dA0 = [O.gaussian(rng, *A.shape, A.dtype) for A in blocks]
    dAs = [to_dev(d, cuda) for d in dA0]
    iters = []
    mak.batched_left_polar_pullback(dAs, [(to_dev(W, cuda), to_dev(P, cuda)) for W, P in facs],
                                    [(to_dev(a, cuda), to_dev(b, cuda)) for a, b in cots],
                                    precision=precision, _info=iters)
    for i, (A, (W, P), (dW, dP), d0, dA) in enumerate(zip(blocks, facs, cots, dA0, dAs)):
        ref = O.left_polar_pullback(d0, A, W, P, dW, dP)
        assert O.rel_err(to_host(dA) - d0, ref - d0) <= 1e-10, i
        d1 = to_dev(d0, cuda)
        info = {}
        mak.left_polar_pullback_(d1, None, (to_dev(W, cuda), to_dev(P, cuda)),
                                 (to_dev(dW, cuda), to_dev(dP, cuda)), precision=precision,
                                 _info=info)
        # the device-stopped sign iteration takes the host-checked loop's steps
        assert iters[i] == info["iterations"], i
        assert O.rel_err(to_host(dA), to_host(d1)) <= (0 if precision == "native" else 1e-13)


def test_batched_polar_pullback_graph_capture(mak, cuda):
    rng, blocks = _blocks(304, 10, 256)
    facs = [O.left_polar_svd(A) for A in blocks]
    cots = [(O.gaussian(rng, *W.shape, A.dtype), O.gaussian(rng, *P.shape, A.dtype))
            for A, (W, P) in zip(blocks, facs)]
    WPs = [(to_dev(W, cuda), to_dev(P, cuda)) for W, P in facs]
    dWPs = [(to_dev(a, cuda), to_dev(b, cuda)) for a, b in cots]
    dAs = [to_dev(np.zeros_like(A), cuda) for A in blocks]
    mak.batched_left_polar_pullback(dAs, WPs, dWPs)  # creates the internal streams
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            for d in dAs:
                d.zero_()
            mak.batched_left_polar_pullback(dAs, WPs, dWPs, _capturing=True)
    torch.cuda.current_stream().wait_stream(s)
    for d in dAs:
        d.fill_(7.0)
    g.replay()
    torch.cuda.synchronize()
    for A, (W, P), (dW, dP), dA in zip(blocks, facs, cots, dAs):
        ref = O.left_polar_pullback(np.zeros_like(A), A, W, P, dW, dP)
        assert O.rel_err(to_host(dA), ref) <= 1e-10
