"""CPU oracle for the orthogonal-factorization path (test infrastructure only).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference legs
may import it.  The product path (``matrixalgebrakit.jl_gb300``) never calls
into it and fails loudly when its CUDA library is missing.

It restates, with numpy + scipy's bundled LAPACK (the same ``?geqrt``,
``?gemqrt``, ``?gesdd``/``?gesvd`` routines the reference ``ccall``s through
libblastrampoline), the reference's CPU algorithms:

* ``LAPACK_HouseholderQR``  -- src/implementations/qr.jl:132-188
* ``PolarViaSVD``           -- src/implementations/polar.jl:59-95
* ``PolarNewton``           -- src/implementations/polar.jl:99-166,209-220
* ``qr_pullback!``          -- src/pullbacks/qr.jl:1-120
* ``qr_null_pullback!``     -- src/pullbacks/qr.jl:122-152,198-200
* ``left_polar_pullback!``  -- src/pullbacks/polar.jl:7-29
* ``right_polar_pullback!`` -- src/pullbacks/polar.jl:37-59
* polar pushforwards        -- src/pushforwards/polar.jl:1-26
* LQ via the transposed QR  -- src/implementations/lq.jl:303-326, and the
  Native row-Householder LQ (lq.jl:177-219) as its independent check
* ``lq_pullback!``, ``lq_null_pullback!`` -- src/pullbacks/lq.jl:1-196
* ``right_polar!(::PolarNewton)`` -- src/implementations/polar.jl:113-125,168-206

Parity status: the reference ships no golden vectors for this path (its tests
are property based, test/testsuite/decompositions/{qr,polar}.jl) and Julia is
not available to generate any, so parity is *unpinned* in the strict sense.
The restatement is pinned instead against (a) analytic known-answer cases
whose positive-diagonal QR / polar factors are unique by construction, and
(b) the reference's own property tests, both in ``tests/test_oracle.py``.
"""

from .mak_oracle import *  # noqa: F401,F403
