"""CPU tests of the C-ABI boundary: the library builds, loads, and exports
every symbol declared in include/*.h; host-side argument validation runs
without a GPU (no compute calls)."""

from __future__ import annotations

import os

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


def test_dual_entry_points_validate_on_host(mak):
    """LQ, right polar, the right pullback and the pushforwards: workspace
    queries and argument checks run without a GPU (LAPACK -i codes)."""
    from mak_gb300 import _lib

    lib = mak.library()
    nb = C.c_size_t(0)
    qo = _lib.mak_qr_opts(1, 0, 0, 0)
    po = _lib.mak_polar_opts(10, 0, 0.0)
    pb = _lib.mak_pullback_opts(-1.0, -1.0, 0, 0)
    for full in (0, 1):
        assert lib.mak_lq_workspace(_lib.MAK_C64, 300, 700, full, C.byref(qo), C.byref(nb)) == 0
        assert nb.value > 0
    assert lib.mak_lq_workspace(_lib.MAK_F64, -1, 7, 0, C.byref(qo), C.byref(nb)) == -2
    assert lib.mak_right_polar_workspace(_lib.MAK_F64, 30, 70, 1, C.byref(po), C.byref(nb)) == 0
    assert nb.value > 0
    assert lib.mak_right_polar_workspace(_lib.MAK_F64, 70, 30, 1, C.byref(po), C.byref(nb)) == -3
    for fn in ("mak_right_polar_pullback_workspace", "mak_right_polar_pushforward_workspace"):
        assert getattr(lib, fn)(_lib.MAK_C64, 20, 50, 0, C.byref(nb)) == 0 and nb.value > 0
        assert getattr(lib, fn)(_lib.MAK_F64, 50, 20, 0, C.byref(nb)) == -3
    assert lib.mak_left_polar_pushforward_workspace(_lib.MAK_F64, 50, 20, 1, C.byref(nb)) == 0
    assert lib.mak_left_polar_pushforward_workspace(_lib.MAK_F64, 20, 50, 0, C.byref(nb)) == -3

    rc = lib.mak_lq_compact_d(-1, 4, None, 4, None, 4, None, 4, C.byref(qo), None, 0, None, None)
    assert rc == -1
    rc = lib.mak_lq_compact_d(8, 4, 16, 4, None, 8, 32, 4, C.byref(qo), None, 0, None, None)
    assert rc == -4  # lda < m
    rc = lib.mak_lq_full_d(4, 8, 16, 4, None, 4, 32, 4, C.byref(qo), None, 0, None, None)
    assert rc == -8  # ldq < n for the n x n Q
    rc = lib.mak_right_polar_newton_d(8, 4, 16, 8, None, 8, 32, 8, C.byref(po), None, 0, None,
                                      None)
    assert rc == -2  # n >= m required
    bad = _lib.mak_polar_opts(0, 0, 0.0)
    rc = lib.mak_right_polar_newton_d(4, 8, 16, 4, None, 4, 32, 4, C.byref(bad), None, 0, None,
                                      None)
    assert rc == -9
    rc = lib.mak_right_polar_pullback_d(8, 4, 16, 8, 32, 8, 48, 8, None, 8, None, 8, C.byref(pb),
                                        None, 0, None, None)
    assert rc == -2
    rc = lib.mak_left_polar_pushforward_d(8, 4, 16, 8, 32, 8, 48, 4, None, 8, 64, 4, C.byref(pb),
                                          None, 0, None, None)
    assert rc == -9  # dW missing
    rc = lib.mak_right_polar_pushforward_d(4, 8, 16, 4, 32, 4, 48, 4, 64, 4, 80, 2, C.byref(pb),
                                           None, 0, None, None)
    assert rc == -12  # lddwh < m
    rc = lib.mak_lq_compact_z(4, 8, 16, 4, None, 4, 32, 4, C.byref(qo), None, 0, None, None)
    assert rc == -12  # info missing (checked before the workspace)


def test_dual_algorithm_selection(mak):
    from mak_gb300 import (GB300_HouseholderQR, GB300_PolarNewton, LQViaTransposedQR,
                           default_algorithm, select_algorithm)

    assert default_algorithm("lq_compact_") == LQViaTransposedQR(GB300_HouseholderQR())
    assert default_algorithm("right_polar") == GB300_PolarNewton()
    alg = select_algorithm("lq_full_", None, GB300_HouseholderQR(blocksize=8))
    assert isinstance(alg, LQViaTransposedQR) and alg.alg.blocksize == 8
    assert select_algorithm("lq_compact", None, None, positive=False).positive is False
    assert select_algorithm("qr_compact_", None, GB300_HouseholderQR()) == GB300_HouseholderQR()


def test_orth_algorithm_selection(mak):
    """src/interface/orthnull.jl:414-456: kind symbols and algorithm instances."""
    from mak_gb300 import (ArgumentError, GB300_HouseholderQR, GB300_PolarNewton, LeftOrthViaPolar,
                           LeftOrthViaQR, LQViaTransposedQR, RightOrthViaLQ, RightOrthViaPolar,
                           left_orth_alg, right_orth_alg)

    assert left_orth_alg() == LeftOrthViaQR(GB300_HouseholderQR())
    assert left_orth_alg("polar", maxiter=7) == LeftOrthViaPolar(GB300_PolarNewton(maxiter=7))
    assert left_orth_alg(GB300_PolarNewton()) == LeftOrthViaPolar(GB300_PolarNewton())
    assert right_orth_alg() == RightOrthViaLQ(LQViaTransposedQR(GB300_HouseholderQR()))
    assert right_orth_alg(GB300_HouseholderQR(blocksize=4)).alg.alg.blocksize == 4
    assert right_orth_alg("polar") == RightOrthViaPolar(GB300_PolarNewton())
    for bad in ("svd", "nope"):
        with pytest.raises(ArgumentError):
            left_orth_alg(bad)
        with pytest.raises(ArgumentError):
            right_orth_alg(bad)
    with pytest.raises(ArgumentError):
        left_orth_alg(GB300_HouseholderQR(), positive=False)


def test_every_entry_point_refuses_host_tensors(mak):
    """No CPU fallback: each public factorization, rule and GEMM raises on a
    host tensor before any work (the product path is the CUDA library only)."""
    import torch

    A = torch.zeros((6, 4), dtype=torch.float64)
    W = torch.zeros((4, 6), dtype=torch.float64)
    calls = [
        lambda: mak.qr_compact(A), lambda: mak.qr_full(A), lambda: mak.qr_null(A),
        lambda: mak.lq_compact(W), lambda: mak.lq_full(W), lambda: mak.lq_null(W),
        lambda: mak.left_polar(A), lambda: mak.right_polar(W),
        lambda: mak.left_orth(A), lambda: mak.right_orth(W), lambda: mak.left_null(A),
        lambda: mak.right_null(W), lambda: mak.project_isometric(A),
        lambda: mak.gemm(A, W),
        lambda: mak.qr_pullback_(A, A, (A, A[:4]), (None, None)),
        lambda: mak.left_polar_pullback_(A, A, (A, A[:4, :4]), (None, None)),
        lambda: mak.right_polar_pullback_(W, W, (W[:, :4], W), (None, None)),
        lambda: mak.left_polar_pushforward_(A, A, (A, A[:4, :4])),
        lambda: mak.right_polar_pushforward_(W, W, (W[:, :4], W)),
        lambda: mak.qr_null_pullback_(A, A, A[:, :2], A[:, :2]),
        lambda: mak.lq_pullback_(W, W, (W[:, :4], W), (None, None)),
        lambda: mak.lq_null_pullback_(W, W, W[:2], W[:2]),
        lambda: mak.batched_qr_compact([A]), lambda: mak.batched_left_polar([A]),
    ]
    for call in calls:
        with pytest.raises(mak.ArgumentError, match="CUDA device"):
            call()


def test_tuning_table_is_host_only(mak):
    """The drivers' tuning table: every parameter has a value without a GPU,
    setting checks the name and the range, NaN returns to the default."""
    import math

    from mak_gb300 import autotune

    names = autotune.tuning_names()
    assert "MAK_BATCH_STREAMS" in names and "MAK_SPLIT_MIN_MNK" in names
    before = autotune.get_tuning()
    assert set(before) == set(names)
    autotune.set_tuning(MAK_BATCH_STREAMS=8, MAK_SPLIT_MIN_MNK=2.0 ** 20)
    assert autotune.get_tuning("MAK_BATCH_STREAMS") == 8
    assert autotune.get_tuning("MAK_SPLIT_MIN_MNK") == 2.0 ** 20
    with pytest.raises(ValueError):
        autotune.set_tuning(MAK_BATCH_STREAMS=64)
    with pytest.raises(KeyError):
        autotune.set_tuning(MAK_NO_SUCH_PARAMETER=1)
    autotune.reset_tuning()
    assert autotune.get_tuning() == before
    lib = mak.library()
    assert lib.mak_tuning_set(b"MAK_BATCH_STREAMS", math.nan) == 0
    assert lib.mak_tuning_name(len(names)) is None


def test_tuning_switches_and_defaults(mak):
    """The kernel switches and launch-shape parameters are in the table with
    their built-in defaults (no environment override in this process) and
    range checks."""
    from mak_gb300 import autotune

    defaults = {"MAK_PANEL_PAIR": 1, "MAK_OZ_MERGED": 1, "MAK_OZ_NARROW": 1,
                "MAK_LOOKAHEAD_CTAS": 48, "MAK_LOOKAHEAD_TAIL_COLS": 4096,
                "MAK_LOOKAHEAD_TAIL_CTAS": 96, "MAK_SMALL_QR_BYTES": 200704,
                "MAK_SMALL_POLAR_BYTES": 200704, "MAK_PANEL_HIER_C": 0,
                "MAK_QR_PANEL_SPLIT": 1}
    for name, value in defaults.items():
        if name in os.environ:
            continue
        assert autotune.get_tuning(name) == value, name
    for name, bad in (("MAK_PANEL_PAIR", 2), ("MAK_OZ_NARROW", -1),
                      ("MAK_LOOKAHEAD_TAIL_CTAS", 200), ("MAK_SMALL_QR_BYTES", 1 << 20)):
        with pytest.raises(ValueError):
            autotune.set_tuning({name: bad})
    autotune.set_tuning(MAK_PANEL_PAIR=0, MAK_SMALL_QR_BYTES=0)
    try:
        assert autotune.get_tuning("MAK_PANEL_PAIR") == 0
        assert autotune.get_tuning("MAK_SMALL_QR_BYTES") == 0
    finally:
        autotune.reset_tuning(["MAK_PANEL_PAIR", "MAK_SMALL_QR_BYTES"])


def test_tuning_table_json_round_trip(mak, tmp_path):
    from mak_gb300 import autotune

    path = tmp_path / "tune.json"
    autotune.save_tuning({"table": {"MAK_BATCH_STREAMS": 16, "MAK_GJ_SPLIT_MIN": 2.0 ** 27}},
                         path)
    autotune.load_tuning(path, strict=False)
    try:
        assert autotune.get_tuning("MAK_BATCH_STREAMS") == 16
        assert autotune.get_tuning("MAK_GJ_SPLIT_MIN") == 2.0 ** 27
    finally:
        autotune.reset_tuning()
