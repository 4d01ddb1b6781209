"""Algorithm types and selection, mirroring MatrixAlgebraKit's plugin API.

``GB300_HouseholderQR`` and ``GB300_PolarNewton`` play the role of the new
``@algdef`` types a Julia extension registers (reference pattern
src/algorithms.jl:342-353); ``select_algorithm`` / ``default_algorithm``
follow src/algorithms.jl:106-145 (``alg`` may be None, a name, a type, a
dict of keyword arguments, or an instance; keyword arguments next to an
instance are an error).
"""

from __future__ import annotations

from dataclasses import dataclass, field, fields


class ArgumentError(ValueError):
    """Julia's ``ArgumentError``."""


class DimensionMismatch(ValueError):
    """Julia's ``DimensionMismatch``."""


_PRECISIONS = ("native", "mixed")


@dataclass(frozen=True)
class GB300_HouseholderQR:
    """Blocked Householder QR on one GB300 (``Householder``'s keyword set,
    src/interface/decompositions.jl:80-86).

    positive  -- make diag(R) real and >= 0 (``sign_safe`` gauge; default True)
    blocksize -- panel width, 0 = library default (32), otherwise 1..32
    pivoted   -- not provided: True raises ``ArgumentError`` like the
                 reference's non-LAPACK drivers (src/implementations/qr.jl:139-145)
    precision -- "native": every flop in the element type; "mixed": the large
                 products as split bf16 tensor-core GEMMs (Ozaki scheme)
    """

    positive: bool = True
    blocksize: int = 0
    pivoted: bool = False
    precision: str = "native"

    def __post_init__(self):
        if self.pivoted:
            raise ArgumentError("GB300_HouseholderQR does not provide a pivoted QR decomposition")
        if not (0 <= int(self.blocksize) <= 32):
            raise ArgumentError(f"blocksize must be 0 (default) or in 1..32, got {self.blocksize}")
        if self.precision not in _PRECISIONS:
            raise ArgumentError(f"precision must be one of {_PRECISIONS}")


@dataclass(frozen=True)
class GB300_PolarNewton:
    """Scaled Newton iteration for the left polar decomposition
    (``PolarNewton(; maxiter=10, tol=defaulttol)``, src/implementations/polar.jl:128)."""

    maxiter: int = 10
    tol: float | None = None
    precision: str = "native"

    def __post_init__(self):
        if int(self.maxiter) < 1:
            raise ArgumentError("maxiter must be >= 1")
        if self.precision not in _PRECISIONS:
            raise ArgumentError(f"precision must be one of {_PRECISIONS}")


@dataclass(frozen=True)
class LQViaTransposedQR:
    """``LQViaTransposedQR(qr_alg)`` (src/interface/decompositions.jl:340-353):
    the LQ of A as the conjugate transpose of the QR of A^H.  A bare
    ``GB300_HouseholderQR`` given to an ``lq_*`` function is wrapped in it, as
    the reference routes its GPU Householder drivers through ``lq_via_qr!``
    (src/implementations/lq.jl:130-131)."""

    alg: GB300_HouseholderQR = field(default_factory=GB300_HouseholderQR)

    @property
    def positive(self) -> bool:
        return self.alg.positive


@dataclass(frozen=True)
class LeftOrthViaQR:
    """``left_orth`` through a QR algorithm (src/interface/decompositions.jl:556-577)."""

    alg: GB300_HouseholderQR = field(default_factory=GB300_HouseholderQR)


@dataclass(frozen=True)
class LeftOrthViaPolar:
    """``left_orth`` through a polar algorithm."""

    alg: GB300_PolarNewton = field(default_factory=GB300_PolarNewton)


@dataclass(frozen=True)
class RightOrthViaLQ:
    """``right_orth`` through an LQ algorithm (src/interface/orthnull.jl,
    implementations/orthnull.jl:91)."""

    alg: LQViaTransposedQR = field(default_factory=LQViaTransposedQR)


@dataclass(frozen=True)
class RightOrthViaPolar:
    """``right_orth`` through a (right) polar algorithm (orthnull.jl:92)."""

    alg: GB300_PolarNewton = field(default_factory=GB300_PolarNewton)


ALGORITHMS = {c.__name__: c for c in (GB300_HouseholderQR, GB300_PolarNewton)}

_QR_FUNCS = ("qr_compact", "qr_compact_", "qr_full", "qr_full_", "qr_null", "qr_null_")
_LQ_FUNCS = ("lq_compact", "lq_compact_", "lq_full", "lq_full_", "lq_null", "lq_null_")
_POLAR_FUNCS = ("left_polar", "left_polar_", "right_polar", "right_polar_")


def _fname(f) -> str:
    return f if isinstance(f, str) else getattr(f, "__name__", str(f))


def default_algorithm(f, A=None, **kwargs):
    """``default_algorithm(f, A; kwargs...)``: GB300 QR for the qr_* family
    (reference default Householder, src/interface/qr.jl:71-87) and GB300 Newton
    for left_polar (the GPU default the extension registers)."""
    name = _fname(f)
    if name in _QR_FUNCS:
        return GB300_HouseholderQR(**kwargs)
    if name in _LQ_FUNCS:
        return LQViaTransposedQR(GB300_HouseholderQR(**kwargs))
    if name in _POLAR_FUNCS:
        return GB300_PolarNewton(**kwargs)
    if name in ("left_orth", "left_orth_"):
        return LeftOrthViaQR(GB300_HouseholderQR(**kwargs))
    raise TypeError(f"no default algorithm for {name}")


def select_algorithm(f, A=None, alg=None, **kwargs):
    """``select_algorithm(f, A, alg; kwargs...)`` (src/algorithms.jl:106-124)."""
    if alg is None:
        return default_algorithm(f, A, **kwargs)
    if isinstance(alg, str):
        if alg not in ALGORITHMS:
            raise ArgumentError(f"Unknown alg {alg}")
        return _lq_wrap(f, ALGORITHMS[alg](**kwargs))
    if isinstance(alg, type):
        return _lq_wrap(f, alg(**kwargs))
    if isinstance(alg, dict):
        if kwargs:
            raise ArgumentError("Additional keyword arguments are not allowed when algorithm "
                                "parameters are specified.")
        return default_algorithm(f, A, **alg)
    if isinstance(alg, (GB300_HouseholderQR, GB300_PolarNewton, LeftOrthViaQR, LeftOrthViaPolar,
                        LQViaTransposedQR)):
        if kwargs:
            raise ArgumentError("Additional keyword arguments are not allowed when algorithm "
                                "parameters are specified.")
        return _lq_wrap(f, alg)
    raise ArgumentError(f"Unknown alg {alg}")


def _lq_wrap(f, alg):
    """A QR algorithm given to an lq_* function means the transposed QR."""
    if _fname(f) in _LQ_FUNCS and isinstance(alg, GB300_HouseholderQR):
        return LQViaTransposedQR(alg)
    return alg


def is_positive(alg) -> bool:
    """TestSuite trait ``is_positive`` (test/testsuite/TestSuite.jl:63-74)."""
    return bool(getattr(alg, "positive", False))


def algorithm_kwargs(alg) -> dict:
    return {f.name: getattr(alg, f.name) for f in fields(alg)}
