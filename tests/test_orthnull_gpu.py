"""GPU tests of left_orth / right_orth / left_null / right_null /
project_isometric and their batched (block-sparse) forms, against the
oracle's QR / LQ / polar factors (test/testsuite/decompositions/orthnull.jl
properties: A = V C, V isometric, A^H N = 0, N isometric; idempotent
projection)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu
DTS = [np.float64, np.complex128]


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_left_and_right_orth(mak, cuda, dt):
    rng = np.random.default_rng(81)
    A = O.gaussian(rng, 70, 30, dt)
    V, C = mak.left_orth(to_dev(A, cuda))
    Qo, Ro = O.qr_compact(A)
    assert O.rel_err(to_host(V), Qo) <= 1e-12 and O.rel_err(to_host(C), Ro) <= 1e-12
    V, C = mak.left_orth(to_dev(A, cuda), alg="polar")
    Wo, Po, _ = O.left_polar_newton(A)
    assert O.rel_err(to_host(V), Wo) <= 1e-10 and O.rel_err(to_host(C), Po) <= 1e-10
    B = A.conj().T.copy()
    C, Vh = mak.right_orth(to_dev(B, cuda))
    Lo, Qlo = O.lq_compact(B)
    assert O.rel_err(to_host(C), Lo) <= 1e-12 and O.rel_err(to_host(Vh), Qlo) <= 1e-12
    C, Vh = mak.right_orth(to_dev(B, cuda), alg="polar")
    Pr, Whr, _ = O.right_polar_newton(B)
    assert O.rel_err(to_host(C), Pr) <= 1e-10 and O.rel_err(to_host(Vh), Whr) <= 1e-10
    with pytest.raises(mak.ArgumentError):
        mak.left_orth(to_dev(A, cuda), trunc={"atol": 1e-3})
    with pytest.raises(mak.ArgumentError):
        mak.right_orth(to_dev(B, cuda), alg="svd")


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_left_and_right_null(mak, cuda, dt):
    rng = np.random.default_rng(82)
    A = O.gaussian(rng, 50, 20, dt)
    N = to_host(mak.left_null(to_dev(A, cuda)))
    assert N.shape == (50, 30)
    assert np.linalg.norm(A.conj().T @ N) <= 1e-12 * np.linalg.norm(A)
    assert O.orth_error(N) <= 1e-12
    assert O.rel_err(N, O.qr_null(A)) <= 1e-12
    B = A.conj().T.copy()
    Nh = to_host(mak.right_null(to_dev(B, cuda)))
    assert Nh.shape == (30, 50)
    assert np.linalg.norm(B @ Nh.conj().T) <= 1e-12 * np.linalg.norm(B)
    assert O.rel_err(Nh, O.lq_null(B)) <= 1e-12


@pytest.mark.parametrize("dt", DTS, ids=lambda d: np.dtype(d).name)
def test_project_isometric(mak, cuda, dt):
    rng = np.random.default_rng(83)
    A = O.gaussian(rng, 90, 40, dt)
    W = mak.project_isometric(to_dev(A, cuda))
    assert O.rel_err(to_host(W), O.left_polar_svd(A)[0]) <= 1e-10
    W2 = mak.project_isometric(W)  # idempotent on isometries
    assert O.rel_err(to_host(W2), to_host(W)) <= 1e-13


def test_batched_left_orth_and_projection(mak, cuda):
    rng = np.random.default_rng(84)
    blocks = O.batched_blocks(rng, nblocks=24, mmin=8, mmax=300, nmin=2)
    Ad = [to_dev(b, cuda) for b in blocks]
    outs = mak.batched_left_orth(Ad)
    for b, (V, C) in zip(blocks, outs):
        Qo, Ro = O.qr_compact(b)
        assert O.rel_err(to_host(V), Qo) <= 1e-12 and O.rel_err(to_host(C), Ro) <= 1e-12
    outs = mak.batched_left_orth(Ad, alg="polar", maxiter=20)
    Ws = mak.batched_project_isometric(Ad, maxiter=20)
    for b, (V, C), W in zip(blocks, outs, Ws):
        Wo, Po = O.left_polar_svd(b)
        assert O.rel_err(to_host(V), Wo) <= 1e-9 and O.rel_err(to_host(C), Po) <= 1e-9
        assert O.rel_err(to_host(W), Wo) <= 1e-9
