"""GPU parity of the orthogonalisation-sweep composite: for ComplexF64
1024 x 256 tensors (bond dimension 256, physical dimension 4), left_orth via
QR and left_polar of every tensor (batched calls), then the pullback of
sum_i real(tr(D_i^H Q_i)) + real(tr(D_i^H W_i)) through both (batched QR and
polar pullbacks), against the oracle (the reference's qr_pullback! and
left_polar_pullback! restated, src/pullbacks/qr.jl:73-120,
src/pullbacks/polar.jl:7-29).  The Float32-class run converts the tensors
to ComplexF32 and is held to the reference's precision(ComplexF32) =
sqrt(eps(Float32)) (test/testsuite/TestSuite.jl:45); the FP64 runs (native
and split tensor-core products) to 1e-10."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["fp64", "mixed", "fp32"])
def test_orth_sweep_composite_vs_oracle(mak, cuda, mode):
    rng = np.random.default_rng(401)
    As = [O.gaussian(rng, 1024, 256, np.complex128) for _ in range(6)]
    Ds = [O.gaussian(rng, 1024, 256, np.complex128) for _ in range(6)]
    prec = "mixed" if mode == "mixed" else "native"
    dt = torch.complex64 if mode == "fp32" else torch.complex128
    X = [to_dev(A, cuda).to(dt) for A in As]
    D = [to_dev(d, cuda).to(dt) for d in Ds]
    QR = mak.batched_qr_compact(X, precision=prec)
    WP = mak.batched_left_polar(X, precision=prec, maxiter=10)
    dA = [torch.zeros_like(x) for x in X]
    mak.batched_qr_pullback(dA, QR, [(d, None) for d in D], precision=prec)
    mak.batched_left_polar_pullback(dA, WP, [(d, None) for d in D], precision=prec)
    tol = float(np.sqrt(np.finfo(np.float32).eps)) if mode == "fp32" else 1e-10
    for A, d, (Q, R), (W, P), g in zip(As, Ds, QR, WP, dA):
        Qo, Ro = O.qr_compact(A)
        Wo, Po = O.left_polar_svd(A)
        ref, _ = O.qr_pullback(np.zeros_like(A), A, Qo, Ro, d, None)
        ref = O.left_polar_pullback(ref, A, Wo, Po, d, None)
        assert O.rel_err(to_host(Q).astype(np.complex128), Qo) <= tol
        assert O.rel_err(to_host(W).astype(np.complex128), Wo) <= tol
        assert O.rel_err(to_host(g).astype(np.complex128), ref) <= tol
