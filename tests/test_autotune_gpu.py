"""GPU test of the autotuner of the drivers' tuning table
(``autotune.autotune_batched``): on a small batch of uneven blocks it
times each candidate value from a CUDA-graph replay of the batched calls,
keeps the fastest table installed, and the batched results under that
table still match the oracle; the JSON file it writes loads back on the
same device."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


def test_autotune_small_batch(mak, cuda, tmp_path):
    from mak_gb300 import autotune

    rng = np.random.default_rng(501)
    blocks = O.batched_blocks(rng, nblocks=12, mmin=8, mmax=200, nmin=4)
    As = [to_dev(A, cuda) for A in blocks]
    try:
        res = autotune.autotune_batched(
            As, precision="mixed", kinds=("qr", "polar"), reps=1,
            candidates={"MAK_BATCH_STREAMS": [4, 32], "MAK_SPLIT_MIN_MNK": [2.0 ** 20]})
        assert res["ms_after"] <= res["ms_before"]
        assert len(res["trials"]) == 3
        for nm, v in res["table"].items():
            assert autotune.get_tuning(nm) == v
        outs = mak.batched_qr_compact(As, precision="mixed")
        for A, (Q, R) in zip(blocks, outs):
            assert O.rel_err(to_host(R), O.qr_compact(A)[1]) <= 1e-12
        pol = mak.batched_left_polar(As, precision="mixed")
        for A, (W, P) in zip(blocks, pol):
            assert np.linalg.norm(A - to_host(W) @ to_host(P)) / np.linalg.norm(A) <= 1e-12
        path = tmp_path / "tune.json"
        autotune.save_tuning(res, path)
        autotune.reset_tuning()
        table = autotune.load_tuning(path)
        assert table == res["table"]
    finally:
        autotune.reset_tuning()
