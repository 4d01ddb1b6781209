"""Generate the analytic known-answer fixtures in this folder.

The reference ships no golden vectors for QR / polar and Julia is not
available, so these fixtures are known answers by construction instead:

* ``qr_kat_<t>.npz``   A = Q0 R0 with Q0 an m x n isometry (Haar) and R0
  upper triangular with a real positive diagonal.  Because the
  positive-diagonal QR of a full-rank matrix is unique (the convention the
  reference enforces with ``positive=true``), ``qr_compact(A)`` must return
  exactly (Q0, R0) up to rounding.
* ``polar_kat_<t>.npz``  A = U diag(s) V^H with U (m x n) an isometry, V
  unitary and s > 0: the left polar factors are W = U V^H, P = V diag(s) V^H.

Run:  python tests/golden/make_golden.py   (seeded; rewrites the .npz files)
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def haar(rng, m, n, cpx):
    G = rng.standard_normal((m, n)) + (1j * rng.standard_normal((m, n)) if cpx else 0)
    Q, R = np.linalg.qr(G)
    d = np.diagonal(R)
    return Q * (d / np.abs(d))[None, :]


def main():
    rng = np.random.default_rng(20240601)
    for tag, cpx in (("d", False), ("z", True)):
        for (m, n) in ((54, 37), (54, 54), (100, 40)):
            Q0 = haar(rng, m, n, cpx)
            # well-conditioned upper triangle: small off-diagonal part
            R0 = np.triu(rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if cpx else 0))
            R0 *= 0.3 / np.sqrt(n)
            R0[np.arange(n), np.arange(n)] = 1.0 + rng.random(n)  # real, positive
            A = Q0 @ R0
            np.savez_compressed(HERE / f"qr_kat_{tag}_{m}x{n}.npz", A=A, Q=Q0, R=R0)
        for (m, n) in ((54, 37), (64, 64)):
            U = haar(rng, m, n, cpx)
            V = haar(rng, n, n, cpx)
            s = np.logspace(0, -3, n)
            A = (U * s[None, :]) @ V.conj().T
            W = U @ V.conj().T
            P = (V * s[None, :]) @ V.conj().T
            P = (P + P.conj().T) / 2
            np.savez_compressed(HERE / f"polar_kat_{tag}_{m}x{n}.npz", A=A, W=W, P=P)


if __name__ == "__main__":
    main()
