"""GPU tests of the product kernel through mak_gemm_{d,z}: the native SIMT
path and the split-precision tcgen05 path (Ozaki scheme) against a float64
numpy product.  Bound for both: max|C - C_ref| <= 1e-13 * max(|A||B|)
(the split path keeps ~2^-46 of sum |a||b|)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


def opx(X, op):
    return X if op == "N" else (X.T if op == "T" else X.conj().T)


@pytest.mark.parametrize("precision", ["native", "mixed"])
@pytest.mark.parametrize("dt", [np.float64, np.complex128], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("ops", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "T")])
@pytest.mark.parametrize("mnk", [(128, 64, 32), (300, 200, 700), (37, 129, 1000), (1, 5, 3),
                                 (256, 256, 4096)])
def test_gemm(mak, cuda, precision, dt, ops, mnk):
    rng = np.random.default_rng(31)
    m, n, k = mnk
    A = O.gaussian(rng, *((m, k) if ops[0] == "N" else (k, m)), dt)
    B = O.gaussian(rng, *((k, n) if ops[1] == "N" else (n, k)), dt)
    C0 = O.gaussian(rng, m, n, dt)
    ref = 1.5 * opx(A, ops[0]) @ opx(B, ops[1]) - 0.5 * C0
    Cd = to_dev(C0, cuda)
    mak.gemm(to_dev(A, cuda), to_dev(B, cuda), ops[0], ops[1], 1.5, -0.5, Cd, precision)
    got = to_host(Cd)
    scale = np.max(np.abs(opx(A, ops[0])) @ np.abs(opx(B, ops[1])))
    assert np.max(np.abs(got - ref)) <= 1e-13 * scale


def test_gemm_mixed_wide_dynamic_range(mak, cuda):
    """Rows and columns scaled over 1e-8..1e8: per-row / per-column exponents."""
    rng = np.random.default_rng(32)
    m, n, k = 200, 150, 513
    A = rng.standard_normal((m, k)) * np.logspace(-8, 8, m)[:, None]
    B = rng.standard_normal((k, n)) * np.logspace(8, -8, n)[None, :]
    C = mak.gemm(to_dev(A, cuda), to_dev(B, cuda), precision="mixed")
    ref = A @ B
    rel = np.abs(to_host(C) - ref) / (np.abs(A) @ np.abs(B))
    assert rel.max() <= 1e-13
