"""ctypes binding of libmak_gb300.so -- the same C ABI Julia reaches via ``ccall``.

The library is built in-tree by ``build.py``.  There is no CPU fallback: if
the shared object is missing or fails to load, every entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libmak_gb300.so"

MAK_F64, MAK_C64, MAK_F32, MAK_C32 = 0, 1, 2, 3
MAK_PREC_NATIVE, MAK_PREC_MIXED = 0, 1
MAK_OK = 0
MAK_ERR_CUDA, MAK_ERR_TIMEOUT, MAK_ERR_UNSUPPORTED, MAK_ERR_WORKSPACE = 1000, 1001, 1002, 1003


class mak_info(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("rank", C.c_int32),
                ("converged", C.c_int32), ("residual", C.c_double), ("gauge", C.c_double),
                ("gauge_atol", C.c_double), ("singular", C.c_int32), ("pad", C.c_int32)]


class mak_qr_opts(C.Structure):
    _fields_ = [("positive", C.c_int32), ("blocksize", C.c_int32), ("precision", C.c_int32),
                ("reserved", C.c_int32)]


class mak_polar_opts(C.Structure):
    _fields_ = [("maxiter", C.c_int32), ("precision", C.c_int32), ("tol", C.c_double)]


class mak_pullback_opts(C.Structure):
    _fields_ = [("rank_atol", C.c_double), ("gauge_atol", C.c_double), ("precision", C.c_int32),
                ("reserved", C.c_int32)]


_i64 = C.c_int64
_p = C.c_void_p
_sz = C.c_size_t

# name -> (restype, argtypes); every symbol declared in include/mak_gb300.h
SIGNATURES = {
    "mak_version": (C.c_char_p, []),
    "mak_status_string": (C.c_char_p, [C.c_int]),
    "mak_kernel_launches": (C.c_uint64, []),
    "mak_profile_start": (C.c_int, []),
    "mak_profile_stop": (C.c_int, []),
    "mak_profile_read": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_uint64)]),
    "mak_qr_workspace": (C.c_int, [C.c_int, _i64, _i64, C.c_int, C.POINTER(mak_qr_opts),
                                   C.POINTER(_sz)]),
}
_QR_ARGS = [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, C.POINTER(mak_qr_opts), _p, _sz, _p, _p]
for _kind in ("compact", "full"):
    for _s in "dzsc":
        SIGNATURES[f"mak_qr_{_kind}_{_s}"] = (C.c_int, _QR_ARGS)
# Float64 qr_compact! with a fixed in-library scratch array (no workspace)
MAK_QR_NOALLOC_SCRATCH_BYTES = 32 << 20
SIGNATURES["mak_qr_compact_d_noalloc"] = (C.c_int, [_i64, _i64, _p, _i64, _p, _i64, _p, _i64,
                                                    C.POINTER(mak_qr_opts), _p, _p])
SIGNATURES["mak_gemm_workspace"] = (C.c_int, [C.c_int, C.c_int, C.c_int, _i64, _i64, _i64, C.c_int,
                                              C.POINTER(_sz)])
SIGNATURES["mak_gemm_d"] = (C.c_int, [C.c_int, C.c_int, _i64, _i64, _i64, C.c_double, _p, _i64, _p,
                                      _i64, C.c_double, _p, _i64, C.c_int, _p, _sz, _p, _p])
SIGNATURES["mak_gemm_z"] = (C.c_int, [C.c_int, C.c_int, _i64, _i64, _i64, C.POINTER(C.c_double), _p,
                                      _i64, _p, _i64, C.POINTER(C.c_double), _p, _i64, C.c_int, _p,
                                      _sz, _p, _p])
SIGNATURES["mak_qr_pullback_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int, C.c_int,
                                                     C.POINTER(_sz)])
SIGNATURES["mak_left_polar_pullback_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                             C.POINTER(_sz)])
for _s in "dzsc":
    SIGNATURES[f"mak_qr_pullback_{_s}"] = (C.c_int, [_i64, _i64, C.c_int, _p, _i64, _p, _i64, _p,
                                                     _i64, _p, _i64, _p, _i64,
                                                     C.POINTER(mak_pullback_opts), _p, _sz, _p,
                                                     _p])
    SIGNATURES[f"mak_left_polar_pullback_{_s}"] = (C.c_int, [_i64, _i64, _p, _i64, _p, _i64, _p,
                                                             _i64, _p, _i64, _p, _i64,
                                                             C.POINTER(mak_pullback_opts), _p,
                                                             _sz, _p, _p])
SIGNATURES["mak_left_polar_workspace"] =(C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                    C.POINTER(mak_polar_opts), C.POINTER(_sz)])
_POLAR_ARGS = [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, C.POINTER(mak_polar_opts), _p, _sz, _p,
               _p]
for _s in "dzsc":
    SIGNATURES[f"mak_left_polar_newton_{_s}"] = (C.c_int, _POLAR_ARGS)

# LQ via the transposed QR and the right polar decomposition (transposed duals)
SIGNATURES["mak_lq_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int, C.POINTER(mak_qr_opts),
                                            C.POINTER(_sz)])
SIGNATURES["mak_right_polar_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                     C.POINTER(mak_polar_opts), C.POINTER(_sz)])
for _s in "dzsc":
    for _kind in ("compact", "full"):
        SIGNATURES[f"mak_lq_{_kind}_{_s}"] = (C.c_int, _QR_ARGS)
    SIGNATURES[f"mak_right_polar_newton_{_s}"] = (C.c_int, _POLAR_ARGS)
# right polar pullback and left polar pushforward
_PB_ARGS = [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64,
            C.POINTER(mak_pullback_opts), _p, _sz, _p, _p]
SIGNATURES["mak_right_polar_pullback_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                              C.POINTER(_sz)])
SIGNATURES["mak_left_polar_pushforward_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                                C.POINTER(_sz)])
for _s in "dzsc":
    SIGNATURES[f"mak_right_polar_pullback_{_s}"] = (C.c_int, _PB_ARGS)
    SIGNATURES[f"mak_left_polar_pushforward_{_s}"] = (C.c_int, _PB_ARGS)
    SIGNATURES[f"mak_right_polar_pushforward_{_s}"] = (C.c_int, _PB_ARGS)
# null-space pullbacks and the LQ pullback
_NULLPB_ARGS = [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, C.POINTER(mak_pullback_opts),
                _p, _sz, _p, _p]
for _nm in ("qr_null", "lq_null"):
    SIGNATURES[f"mak_{_nm}_pullback_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                             C.POINTER(_sz)])
    for _s in "dzsc":
        SIGNATURES[f"mak_{_nm}_pullback_{_s}"] = (C.c_int, _NULLPB_ARGS)
SIGNATURES["mak_lq_pullback_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int, C.c_int,
                                                     C.POINTER(_sz)])
for _s in "dzsc":
    SIGNATURES[f"mak_lq_pullback_{_s}"] = SIGNATURES[f"mak_qr_pullback_{_s}"]
SIGNATURES["mak_right_polar_pushforward_workspace"] = (C.c_int, [C.c_int, _i64, _i64, C.c_int,
                                                                 C.POINTER(_sz)])
# tuning table of the drivers
SIGNATURES["mak_tuning_set"] = (C.c_int, [C.c_char_p, C.c_double])
SIGNATURES["mak_tuning_get"] = (C.c_int, [C.c_char_p, C.POINTER(C.c_double)])
SIGNATURES["mak_tuning_name"] = (C.c_char_p, [C.c_int])
# self-test of the bounded device waits (failure path)
SIGNATURES["mak_selftest_barrier"] = (C.c_int, [C.c_int, C.c_int, _i64, _p, _sz, _p, _p])

_lib = None
_load_error = None


def load():
    """Load the shared library once; raise with the reason if unavailable."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    if _load_error is not None:
        raise RuntimeError(_load_error)
    path = Path(os.environ.get("MAK_GB300_LIB", LIB_PATH))
    if not path.exists():
        _load_error = (f"libmak_gb300.so not found at {path}; build it with "
                       f"`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        raise RuntimeError(_load_error)
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        if not hasattr(lib, name):
            continue
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(code: int) -> str:
    return load().mak_status_string(code).decode()


class mak_batch_item(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("reserved", C.c_int32), ("m", C.c_int64),
                ("n", C.c_int64), ("A", C.c_void_p), ("lda", C.c_int64), ("Q", C.c_void_p),
                ("ldq", C.c_int64), ("R", C.c_void_p), ("ldr", C.c_int64)]


SIGNATURES["mak_batched_qr_workspace"] = (C.c_int, [C.POINTER(mak_batch_item), C.c_int,
                                                    C.POINTER(mak_qr_opts), C.POINTER(_sz)])
SIGNATURES["mak_batched_qr_compact"] = (C.c_int, [C.POINTER(mak_batch_item), C.c_int,
                                                  C.POINTER(mak_qr_opts), _p, _sz, _p, _p])
SIGNATURES["mak_batched_qr_compact_device"] = (C.c_int, [_p, C.c_int, C.POINTER(mak_qr_opts), _p,
                                                         _p])
SIGNATURES["mak_small_qr_max_bytes"] = (C.c_int, [])
SIGNATURES["mak_batched_left_polar_device"] = (C.c_int, [_p, C.c_int, C.POINTER(mak_polar_opts),
                                                         _p, _p])
SIGNATURES["mak_small_polar_max_bytes"] = (C.c_int, [])
SIGNATURES["mak_batched_left_polar_workspace"] = (C.c_int, [C.POINTER(mak_batch_item), C.c_int,
                                                            C.POINTER(mak_polar_opts),
                                                            C.POINTER(_sz)])
SIGNATURES["mak_batched_left_polar"] = (C.c_int, [C.POINTER(mak_batch_item), C.c_int,
                                                  C.POINTER(mak_polar_opts), _p, _sz, _p, _p])


class mak_batch_pullback_item(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("reserved", C.c_int32), ("m", C.c_int64),
                ("n", C.c_int64), ("dA", C.c_void_p), ("ldda", C.c_int64), ("F1", C.c_void_p),
                ("ld1", C.c_int64), ("F2", C.c_void_p), ("ld2", C.c_int64),
                ("dF1", C.c_void_p), ("ldd1", C.c_int64), ("dF2", C.c_void_p),
                ("ldd2", C.c_int64)]


for _nm in ("qr", "left_polar"):
    SIGNATURES[f"mak_batched_{_nm}_pullback_workspace"] = (
        C.c_int, [C.POINTER(mak_batch_pullback_item), C.c_int, C.POINTER(mak_pullback_opts),
                  C.POINTER(_sz)])
    SIGNATURES[f"mak_batched_{_nm}_pullback"] = (
        C.c_int, [C.POINTER(mak_batch_pullback_item), C.c_int, C.POINTER(mak_pullback_opts),
                  _p, _sz, _p, _p])
