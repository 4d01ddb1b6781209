"""CPU tests of the C-ABI boundary: the library builds, loads, and exports
every symbol declared in include/*.h; host-side argument validation runs
without a GPU (no compute calls)."""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        for m in re.finditer(r"\b(mak_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "mak_qr_compact_d" in syms and "mak_qr_workspace" in syms
    assert len(syms) >= 10


def test_library_exports_every_declared_symbol(mak):
    lib = mak.library()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"not exported: {missing}"


def test_python_signatures_cover_header(mak):
    from mak_gb300 import _lib

    missing = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"


def test_version_and_status_strings(mak):
    lib = mak.library()
    assert b"sm_103a" in lib.mak_version()
    assert lib.mak_status_string(0) == b"ok"
    assert b"invalid" in lib.mak_status_string(-3)


def test_workspace_query_is_host_only(mak):
    from mak_gb300 import _lib

    lib = mak.library()
    nb = C.c_size_t(0)
    opts = _lib.mak_qr_opts(1, 0, 0, 0)
    assert lib.mak_qr_workspace(_lib.MAK_F64, 512, 256, 0, C.byref(opts), C.byref(nb)) == 0
    assert nb.value > 0
    assert lib.mak_qr_workspace(_lib.MAK_F64, -1, 256, 0, C.byref(opts), C.byref(nb)) == -2
    assert lib.mak_qr_workspace(9, 4, 4, 0, C.byref(opts), C.byref(nb)) == -1


def test_argument_validation_is_host_only(mak):
    """Invalid arguments are rejected before any CUDA call (LAPACK -i codes)."""
    from mak_gb300 import _lib

    lib = mak.library()
    opts = _lib.mak_qr_opts(1, 0, 0, 0)
    rc = lib.mak_qr_compact_d(-1, 4, None, 4, None, 4, None, 4, C.byref(opts), None, 0, None, None)
    assert rc == -1
    rc = lib.mak_qr_compact_d(8, 4, 16, 4, 32, 8, None, 4, C.byref(opts), None, 0, None, None)
    assert rc == -4  # lda < m
    bad = _lib.mak_qr_opts(1, 99, 0, 0)
    rc = lib.mak_qr_compact_d(8, 4, 16, 8, 32, 8, None, 4, C.byref(bad), None, 0, None, None)
    assert rc == -9
    rc = lib.mak_qr_compact_d(8, 4, 16, 8, 16, 8, None, 4, C.byref(opts), None, 0, None, None)
    assert rc == -5  # Q aliases A


def test_algorithm_selection(mak):
    """src/algorithms.jl:106-124 semantics."""
    from mak_gb300 import (ArgumentError, GB300_HouseholderQR, GB300_PolarNewton,
                           select_algorithm, default_algorithm)

    assert default_algorithm("qr_compact_") == GB300_HouseholderQR()
    assert default_algorithm("left_polar_") == GB300_PolarNewton()
    assert select_algorithm("qr_compact_", None, None, positive=False) == GB300_HouseholderQR(positive=False)
    assert select_algorithm("qr_compact_", None, "GB300_HouseholderQR", blocksize=8).blocksize == 8
    assert select_algorithm("qr_compact_", None, GB300_HouseholderQR, blocksize=4).blocksize == 4
    assert select_algorithm("qr_compact_", None, {"positive": False}).positive is False
    alg = GB300_HouseholderQR(blocksize=16)
    assert select_algorithm("qr_compact_", None, alg) is alg
    with pytest.raises(ArgumentError):
        select_algorithm("qr_compact_", None, alg, positive=False)
    with pytest.raises(ArgumentError):
        GB300_HouseholderQR(pivoted=True)
    with pytest.raises(ArgumentError):
        select_algorithm("qr_compact_", None, "NoSuchAlgorithm")
