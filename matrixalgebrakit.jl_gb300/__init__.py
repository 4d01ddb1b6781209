"""mak_gb300 -- GB300-native dense orthogonal factorizations (QR, polar, pullbacks).

Python host mirror of the Julia extension: the same entry points and
algorithm types MatrixAlgebraKit users call, backed by libmak_gb300.so
(hand-written sm_103a CUDA behind a C ABI).  Bang functions end in ``_``
(``qr_compact_`` is ``qr_compact!``).

The directory name carries a dot, so load it with::

    import importlib.util, sys
    spec = importlib.util.spec_from_file_location(
        "mak_gb300", "<repo>/matrixalgebrakit.jl_gb300/__init__.py",
        submodule_search_locations=["<repo>/matrixalgebrakit.jl_gb300"])
    mak = importlib.util.module_from_spec(spec); sys.modules["mak_gb300"] = mak
    spec.loader.exec_module(mak)

(``__graft_entry__.load_package()`` does exactly this.)
"""

from . import _lib
from .algorithms import (ArgumentError, DimensionMismatch, GB300_HouseholderQR,
                         GB300_PolarNewton, LeftOrthViaPolar, LeftOrthViaQR, LQViaTransposedQR,
                         default_algorithm, is_positive, select_algorithm)
from .blas import gemm
from .core import check_info, new_info
from .lq import lq_compact, lq_compact_, lq_full, lq_full_, lq_null, lq_null_
from .polar import SingularException, left_polar, left_polar_, right_polar, right_polar_
from .qr import (initialize_output, qr_compact, qr_compact_, qr_full, qr_full_, qr_null,
                 qr_null_)

__all__ = [
    "ArgumentError", "DimensionMismatch", "SingularException", "GB300_HouseholderQR",
    "GB300_PolarNewton", "LeftOrthViaQR", "LeftOrthViaPolar", "default_algorithm",
    "select_algorithm", "is_positive", "qr_compact", "qr_compact_", "qr_full", "qr_full_",
    "qr_null", "qr_null_", "left_polar", "left_polar_", "initialize_output", "library", "gemm",
    "LQViaTransposedQR", "lq_compact", "lq_compact_", "lq_full", "lq_full_", "lq_null",
    "lq_null_", "right_polar", "right_polar_", "new_info", "check_info",
]


def library():
    """The loaded ctypes handle of libmak_gb300.so (raises if unavailable)."""
    return _lib.load()

from .pullbacks import (left_polar_pullback_, lq_null_pullback_, lq_pullback_,  # noqa: E402
                        qr_null_pullback_, qr_pullback_, right_polar_pullback_)
from .pushforwards import left_polar_pushforward_, right_polar_pushforward_  # noqa: E402

__all__ += ["qr_pullback_", "left_polar_pullback_", "right_polar_pullback_", "qr_null_pullback_",
            "lq_pullback_", "lq_null_pullback_",
            "left_polar_pushforward_", "right_polar_pushforward_"]

from .batched import (batch_items_device, batched_left_polar,  # noqa: E402
                      batched_left_polar_device, batched_left_polar_pullback, batched_qr_compact,
                      batched_qr_compact_device, batched_qr_pullback, small_polar_max_bytes,
                      small_qr_max_bytes)

__all__ += ["batched_qr_compact", "batched_left_polar", "batched_qr_pullback",
            "batched_left_polar_pullback", "batched_qr_compact_device", "batch_items_device",
            "small_qr_max_bytes", "batched_left_polar_device", "small_polar_max_bytes"]

from .algorithms import RightOrthViaLQ, RightOrthViaPolar  # noqa: E402
from .orthnull import (batched_left_orth, batched_project_isometric, left_null,  # noqa: E402
                       left_null_, left_orth, left_orth_, left_orth_alg, project_isometric,
                       project_isometric_, right_null, right_null_, right_orth, right_orth_,
                       right_orth_alg)

__all__ += ["RightOrthViaLQ", "RightOrthViaPolar", "left_orth", "left_orth_", "right_orth",
            "right_orth_", "left_null", "left_null_", "right_null", "right_null_",
            "project_isometric", "project_isometric_", "left_orth_alg", "right_orth_alg",
            "batched_left_orth", "batched_project_isometric"]

from . import autodiff  # noqa: E402  (torch.autograd front-end over the device pullbacks)

__all__ += ["autodiff"]

from . import autotune  # noqa: E402  (tuning table of the drivers and its autotuner)

__all__ += ["autotune"]
