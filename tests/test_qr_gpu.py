"""GPU parity tests of qr_compact! / qr_full! through the C ABI against the
CPU oracle (the reference's LAPACK_HouseholderQR restated) and against the
analytic known-answer fixtures.

Tolerances: Float64/ComplexF64 R within 1e-12 relative of the oracle R
(the positive-diagonal R is unique for full-rank A); Float32/ComplexF32
within 2e-5 relative.  Residual and isometry bounds mirror
test/testsuite/decompositions/qr.jl (rtol = precision(T) = sqrt(eps)).
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
DTYPES = [np.float64, np.complex128, np.float32, np.complex64]
TOL_R = {np.float64: 1e-12, np.complex128: 1e-12, np.float32: 2e-5, np.complex64: 2e-5}


def tol(dt):
    return TOL_R[dt]


@pytest.mark.parametrize("dt", DTYPES, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(54, 37), (54, 54), (54, 63), (512, 256), (1000, 33), (33, 1000)])
def test_qr_compact_parity(mak, cuda, dt, shape):
    rng = np.random.default_rng(123)
    A = O.gaussian(rng, *shape, dt)
    Ad = to_dev(A, cuda)
    Q, R = mak.qr_compact(Ad)
    torch.cuda.synchronize()
    assert np.array_equal(to_host(Ad), A)  # non-bang leaves A untouched
    Qh, Rh = to_host(Q), to_host(R)
    Qo, Ro = O.qr_compact(A)
    assert O.rel_err(Rh, Ro) <= tol(dt)
    assert O.rel_err(Qh, Qo) <= 50 * tol(dt)
    assert O.qr_residual(A, Qh, Rh) <= tol(dt)
    assert O.orth_error(Qh) <= 10 * tol(dt) * np.sqrt(Qh.shape[1])
    assert np.array_equal(np.triu(Rh), Rh)
    d = np.diagonal(Rh)
    assert np.all(d.real >= 0) and np.all(d.imag == 0)


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.float32], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(54, 37), (54, 63), (300, 128)])
def test_qr_full_parity(mak, cuda, dt, shape):
    rng = np.random.default_rng(7)
    A = O.gaussian(rng, *shape, dt)
    Q, R = mak.qr_full(to_dev(A, cuda))
    Qh, Rh = to_host(Q), to_host(R)
    Qo, Ro = O.qr_full(A)
    assert Qh.shape == (shape[0], shape[0]) and Rh.shape == shape
    assert O.rel_err(Rh, Ro) <= tol(dt)
    assert O.orth_error(Qh) <= 10 * tol(dt) * np.sqrt(shape[0])
    assert O.qr_residual(A, Qh, Rh) <= tol(dt)
    # the first min(m,n) columns are unique; the rest must span the complement
    k = min(shape)
    assert O.rel_err(Qh[:, :k], Qo[:, :k]) <= 50 * tol(dt)


@pytest.mark.parametrize("path", sorted(GOLD.glob("qr_kat_*.npz")), ids=lambda p: p.stem)
def test_qr_known_answer(mak, cuda, path):
    d = np.load(path)
    Q, R = mak.qr_compact(to_dev(d["A"], cuda))
    assert O.rel_err(to_host(R), d["R"]) <= 1e-12
    assert O.rel_err(to_host(Q), d["Q"]) <= 1e-12


def test_qr_bang_returns_same_objects_and_empty_r(mak, cuda):
    rng = np.random.default_rng(1)
    A = O.gaussian(rng, 80, 30, np.float64)
    Ad = to_dev(A, cuda)
    Q, R = mak.initialize_output("qr_compact_", Ad)
    Q2, R2 = mak.qr_compact_(Ad, (Q, R))
    assert Q2 is Q and R2 is R
    assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12
    # empty R: only Q is computed (src/implementations/qr.jl:149)
    Ae = to_dev(A, cuda)
    Re = torch.empty((0, 0), dtype=torch.float64, device=cuda)
    Qe = mak.initialize_output("qr_compact_", Ae)[0]
    Q3, R3 = mak.qr_compact_(Ae, (Qe, Re))
    assert R3 is Re and R3.numel() == 0
    assert O.rel_err(to_host(Q3), O.qr_compact(A)[0]) <= 1e-12


def test_qr_bang_deferred_info(mak, cuda):
    """info=: the calls return once queued; a stream of factorizations into
    the same outputs matches the oracle, and the records read back clean."""
    rng = np.random.default_rng(3)
    As = [O.gaussian(rng, 300, 200, np.float64) for _ in range(3)]
    infos = [mak.new_info(cuda) for _ in As]
    Q, R = mak.initialize_output("qr_compact_", to_dev(As[0], cuda))
    Rs = []
    for A, inf in zip(As, infos):
        mak.qr_compact_(to_dev(A, cuda), (Q, R), info=inf, precision="mixed")
        Rs.append(R.clone())
    for A, Rd, inf in zip(As, Rs, infos):
        mak.check_info(inf, "qr_compact_")
        assert O.rel_err(to_host(Rd), O.qr_compact(A)[1]) <= 1e-12
    Qf, Rf = mak.qr_full_(to_dev(As[0], cuda), info=infos[0])
    mak.check_info(infos[0])
    assert O.qr_residual(As[0], to_host(Qf), to_host(Rf)) <= 1e-13


def test_qr_positive_false_and_blocksizes(mak, cuda):
    rng = np.random.default_rng(2)
    A = O.gaussian(rng, 70, 45, np.complex128)
    Ro = O.qr_compact(A)[1]
    Q, R = mak.qr_compact(to_dev(A, cuda), positive=False)
    Qh, Rh = to_host(Q), to_host(R)
    assert O.qr_residual(A, Qh, Rh) <= 1e-14
    assert O.rel_err(np.abs(Rh), np.abs(Ro)) <= 1e-12
    for bs in (1, 3, 8, 32):
        Q, R = mak.qr_compact(to_dev(A, cuda), blocksize=bs)
        assert O.rel_err(to_host(R), Ro) <= 1e-12, bs


def test_qr_strided_input(mak, cuda):
    rng = np.random.default_rng(3)
    A = O.gaussian(rng, 60, 40, np.float64)
    big = torch.zeros((40, 77), dtype=torch.float64, device=cuda)  # ld = 77
    Av = big.t()[:60, :]
    Av.copy_(to_dev(A, cuda))
    assert Av.stride() == (1, 77)
    Q, R = mak.initialize_output("qr_compact_", Av)
    mak.qr_compact_(Av, (Q, R))
    assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12


@pytest.mark.parametrize("shape", [(0, 5), (5, 0), (1, 1), (7, 1), (1, 7), (2, 2)])
def test_qr_edge_shapes(mak, cuda, shape):
    rng = np.random.default_rng(4)
    A = O.gaussian(rng, *shape, np.float64)
    Q, R = mak.qr_compact(to_dev(A, cuda))
    Qo, Ro = O.qr_compact(A)
    assert tuple(Q.shape) == Qo.shape and tuple(R.shape) == Ro.shape
    if A.size:
        assert O.rel_err(to_host(R), Ro) <= 1e-12
        assert O.rel_err(to_host(Q), Qo) <= 1e-12


def test_qr_zero_and_rank_deficient_columns(mak, cuda):
    rng = np.random.default_rng(5)
    A = O.gaussian(rng, 50, 20, np.float64)
    A[:, 3] = 0.0            # a zero column: tau = 0, sign_safe(0) = +1
    A[:, 7] = A[:, 2]        # a dependent column
    Q, R = mak.qr_compact(to_dev(A, cuda))
    Qh, Rh = to_host(Q), to_host(R)
    assert O.qr_residual(A, Qh, Rh) <= 1e-14
    assert O.orth_error(Qh) <= 1e-13
    assert np.all(np.diagonal(Rh) >= 0)


@pytest.mark.parametrize("dt,big", [(np.float64, 1e250), (np.complex128, 1e250),
                                    (np.float32, 1e20), (np.complex64, 1e20)],
                         ids=["float64", "complex128", "float32", "complex64"])
def test_qr_extreme_column_scales(mak, cuda, dt, big):
    """Columns scaled far outside the range where a plain sum of squares is
    safe (squares overflow or underflow): the panel's column norms take the
    rescaled pass.  QR is column-scale equivariant, A D = Q (R D) for a
    positive diagonal D, so the scaled factorization must reproduce the
    unscaled one column by column; R is also checked against the oracle."""
    rng = np.random.default_rng(17)
    m, n = 300, 40
    A = O.gaussian(rng, m, n, dt)
    rdt = np.float64 if dt in (np.float64, np.complex128) else np.float32
    d = np.array([big, 1.0 / big, 1.0, big, 1.0 / big] * (n // 5), dtype=rdt)
    AD = (A * d[None, :]).astype(dt)
    Q1, R1 = mak.qr_compact(to_dev(A, cuda))
    Q2, R2 = mak.qr_compact(to_dev(AD, cuda))
    Q1h, R1h, Q2h, R2h = to_host(Q1), to_host(R1), to_host(Q2), to_host(R2)
    assert np.all(np.isfinite(R2h)) and np.all(np.isfinite(Q2h))
    t = tol(dt)
    assert O.rel_err(Q2h, Q1h) <= 50 * t
    for j in range(n):
        col = R1h[:, j] * d[j]
        assert np.linalg.norm(R2h[:, j] - col) <= 50 * t * np.linalg.norm(col)
    Ro = O.qr_compact(AD)[1]
    for j in range(n):
        assert np.linalg.norm(R2h[:, j] - Ro[:, j]) <= 50 * t * np.linalg.norm(Ro[:, j])


def test_qr_dimension_errors(mak, cuda):
    A = torch.zeros((10, 4), dtype=torch.float64, device=cuda).t().contiguous().t()
    Q = torch.zeros((4, 10), dtype=torch.float64, device=cuda).t()
    R = torch.zeros((3, 4), dtype=torch.float64, device=cuda).t()
    with pytest.raises(mak.DimensionMismatch):
        mak.qr_compact_(A, (Q, torch.zeros((4, 3), dtype=torch.float64, device=cuda).t()))
    with pytest.raises(mak.DimensionMismatch):
        mak.qr_compact_(A, (torch.zeros((10, 10), dtype=torch.float64, device=cuda), R))
    with pytest.raises(mak.ArgumentError):
        mak.qr_compact_(A, (Q.to(torch.float32), R))
    with pytest.raises(mak.ArgumentError):
        mak.qr_compact(A.cpu())


@pytest.mark.parametrize("dt", [np.float64, np.complex128], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("shape", [(512, 256), (700, 650), (300, 900), (2048, 512)])
def test_qr_compact_mixed_parity(mak, cuda, dt, shape):
    """precision="mixed": 128-wide block reflectors applied with the split-
    precision tensor-core GEMM; the same 1e-12 bound on R vs the oracle."""
    rng = np.random.default_rng(41)
    A = O.gaussian(rng, *shape, dt)
    Q, R = mak.qr_compact(to_dev(A, cuda), precision="mixed")
    Qh, Rh = to_host(Q), to_host(R)
    Qo, Ro = O.qr_compact(A)
    assert O.rel_err(Rh, Ro) <= 1e-12
    assert O.qr_residual(A, Qh, Rh) <= 5e-13  # within the 1e-12 accuracy bound
    # isometry in the reference's relative form (is_left_isometric,
    # src/common/matrixproperties.jl:49-54): ||Q^H Q - I|| <= rtol ||Q^H Q||
    assert O.orth_error(Qh) <= 1e-13 * np.sqrt(Qh.shape[1])
    d = np.diagonal(Rh)
    assert np.all(d.real >= 0) and np.all(d.imag == 0)


def test_qr_full_mixed(mak, cuda):
    rng = np.random.default_rng(42)
    A = O.gaussian(rng, 400, 150, np.float64)
    Q, R = mak.qr_full(to_dev(A, cuda), precision="mixed")
    Qh, Rh = to_host(Q), to_host(R)
    assert O.rel_err(Rh, O.qr_full(A)[1]) <= 1e-12
    assert O.orth_error(Qh) <= 1e-13 * np.sqrt(Qh.shape[1])


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_qr_lookahead_path(mak, cuda, precision):
    """Large enough (m n >= 4e6) for the look-ahead side stream: block b+1 is
    factored while block b updates the far columns."""
    rng = np.random.default_rng(43)
    A = O.gaussian(rng, 2560, 1664, np.float64)
    Q, R = mak.qr_compact(to_dev(A, cuda), precision=precision)
    Qh, Rh = to_host(Q), to_host(R)
    Ro = O.qr_compact(A)[1]
    assert O.rel_err(Rh, Ro) <= 1e-12
    assert O.qr_residual(A, Qh, Rh) <= 5e-13
    assert O.orth_error(Qh) <= 1e-13 * np.sqrt(Qh.shape[1])
