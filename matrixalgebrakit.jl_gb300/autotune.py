"""Tuning table of the drivers and an autotuner for it.

The kernels' tiles are fixed at build time; what varies per workload is
which kernels run and how many run side by side: the batched calls' number
of internal streams and per-product CTA cap, the size from which a product
takes the split tensor-core path, the size from which the Gauss-Jordan
inverse blocks by 128, the range of the Newton-Schulz finish, and so on
(the names and defaults are listed with ``mak_tuning_set`` in
``include/mak_gb300.h``).  ``autotune_batched`` measures a caller's own
batch of blocks under candidate values, one parameter at a time
(coordinate descent over the whole batch replayed from a CUDA graph), and
returns the fastest table; ``save_tuning`` / ``load_tuning`` keep it as JSON
keyed by the device it was measured on, and ``set_tuning`` installs a
table for the calls that follow.
"""

from __future__ import annotations

import ctypes as ct
import json
import math
import time
from pathlib import Path

import torch

from .batched import batched_left_polar, batched_qr_compact
from .core import lib


def tuning_names() -> list:
    """Names of every tuning parameter the library knows."""
    L = lib()
    out, i = [], 0
    while True:
        nm = L.mak_tuning_name(i)
        if not nm:
            return out
        out.append(nm.decode())
        i += 1


def get_tuning(name=None):
    """The value in effect of one parameter, or of all as a dict."""
    L = lib()
    if name is None:
        return {nm: get_tuning(nm) for nm in tuning_names()}
    v = ct.c_double()
    rc = L.mak_tuning_get(name.encode(), ct.byref(v))
    if rc != 0:
        raise KeyError(f"unknown tuning parameter {name!r}")
    return v.value


def set_tuning(table=None, **params):
    """Install values (a dict and/or keyword arguments); None resets a
    parameter to its environment / built-in default."""
    L = lib()
    items = dict(table or {})
    items.update(params)
    for name, value in items.items():
        rc = L.mak_tuning_set(name.encode(), math.nan if value is None else float(value))
        if rc == -1:
            raise KeyError(f"unknown tuning parameter {name!r}")
        if rc == -2:
            raise ValueError(f"{name} = {value} is outside the parameter's range")


def reset_tuning(names=None):
    """Every (or the named) parameter back to its environment / default value."""
    set_tuning({nm: None for nm in (names or tuning_names())})


def _device_key(dev):
    p = torch.cuda.get_device_properties(dev)
    return {"device": p.name, "sms": p.multi_processor_count}


def default_candidates(dev, kinds):
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    cand = {"MAK_BATCH_STREAMS": [8, 16, 32],
            "MAK_BATCH_GEMM_CTAS": [max(8, sms // 8), max(8, sms // 4), max(8, sms // 2)],
            "MAK_SPLIT_MIN_MNK": [2.0 ** 20, 2.0 ** 22, 2.0 ** 24]}
    if "polar" in kinds:
        cand["MAK_GJ_SPLIT_MIN"] = [2.0 ** 23, 2.0 ** 25, 2.0 ** 27]
        cand["MAK_NS_FIXED_MIN_N"] = [128, 256, 512]
    return cand


def _timer(As, kinds, precision, maxiter, reps):
    """Time of the batch (the chosen kinds, one after the other) replayed
    from a CUDA graph, the inputs restored inside the graph."""
    work = [A.clone() for A in As]

    def restore():
        for w, a in zip(work, As):
            w.copy_(a)

    outs = {}
    restore()
    if "qr" in kinds:
        outs["qr"] = batched_qr_compact(work, copy_inputs=False, precision=precision)
        restore()
    if "polar" in kinds:
        outs["polar"] = batched_left_polar(work, copy_inputs=False, precision=precision,
                                           maxiter=maxiter)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            if "qr" in kinds:
                restore()
                batched_qr_compact(work, copy_inputs=False, outs=outs["qr"],
                                   precision=precision, _capturing=True)
            if "polar" in kinds:
                restore()
                batched_left_polar(work, copy_inputs=False, outs=outs["polar"],
                                   precision=precision, maxiter=maxiter, _capturing=True)
    torch.cuda.current_stream().wait_stream(s)
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    del g
    return ms


def autotune_batched(As, precision="mixed", kinds=("qr", "polar"), candidates=None, reps=2,
                     maxiter=10, rounds=1):
    """Pick the tuning values that make the batched calls fastest on the
    blocks ``As`` (CUDA tensors, the caller's own batch or a representative
    one).  Coordinate descent: each parameter in turn takes each of its
    candidate values with the others held at the best found so far.
    Returns a dict with the table, the time before and after, every trial,
    and the device it was measured on; the table is left installed."""
    dev = As[0].device
    kinds = tuple(kinds)
    cand = candidates or default_candidates(dev, kinds)
    table = {nm: get_tuning(nm) for nm in cand}
    t0 = time.perf_counter()
    base = _timer(As, kinds, precision, maxiter, reps)
    best_ms = base
    trials = [{"table": dict(table), "ms": round(base, 3)}]
    for _ in range(rounds):
        for nm, values in cand.items():
            for v in values:
                if v == table[nm]:
                    continue
                set_tuning({**table, nm: v})
                ms = _timer(As, kinds, precision, maxiter, reps)
                trials.append({"table": {**table, nm: v}, "ms": round(ms, 3)})
                if ms < best_ms:
                    best_ms, table = ms, {**table, nm: v}
            set_tuning(table)
    return {**_device_key(dev), "precision": precision, "kinds": list(kinds),
            "blocks": len(As), "table": table, "ms_before": round(base, 3),
            "ms_after": round(best_ms, 3), "trials": trials,
            "seconds": round(time.perf_counter() - t0, 1)}


def save_tuning(result, path):
    """Write an autotune result (or a bare table) as JSON."""
    Path(path).write_text(json.dumps(result, indent=1))


def load_tuning(path, device=None, strict=True):
    """Install the table stored at ``path``.  With ``strict`` the file must
    have been measured on a device of the same name and SM count as
    ``device`` (default: the current CUDA device)."""
    data = json.loads(Path(path).read_text())
    table = data.get("table", data)
    if strict and "device" in data:
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        key = _device_key(dev)
        if (data["device"], data.get("sms")) != (key["device"], key["sms"]):
            raise ValueError(f"tuning table measured on {data['device']} ({data.get('sms')} SMs), "
                             f"not on {key['device']} ({key['sms']} SMs)")
    set_tuning(table)
    return table
