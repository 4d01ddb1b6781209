#!/usr/bin/env python3
"""Benchmark of the GB300 orthogonal-factorization hot path.

Default workload (the single large Float64 problem the headline metric is
quoted on): ``qr_compact!(A, (Q, R); positive=true)`` of one 16384 x 8192
Float64 matrix with iid N(0,1) entries (seeded numpy generator; synthetic --
the reference names no dataset).  A step = restore A from a device-resident
master copy (the factorization destroys its input) + the factorization.
The matrix (1.07 GB) is larger than L2 (129 MB), so no flush is needed.

Printed (rank 0, one JSON line): QR TFLOP/s with the minimal
geqrf + orgqr flop count 4mn^2 - 4n^3/3 (``value``), the same through the
public API with host buffers (``e2e``), factorizations/s, accuracy of every
result (||A-QR||/||A||, ||Q^H Q - I||), the dominant kernel's roofline
(device time measured live with CUDA events inside the timed region),
SM clocks sampled during the timed region, the CPU baseline (the
reference's LAPACK_HouseholderQR path restated with scipy/OpenBLAS on the
host cores) and a left_polar! (Newton) measurement on an 8192 x 8192
kappa = 1e6 matrix.

``--impl reference`` times the reference's CPU implementation of the same
path (the oracle restatement of LAPACK_HouseholderQR: ?geqrt + ?gemqrt +
gaugefix, all host threads) and prints the same JSON line with
``"impl": "reference"``.

Multi-GPU: single matrices do not shard (a reduction tree would be needed),
so N GPUs run N independent replicas ("scaling": "weak"); value = total
flops of all ranks / max-over-ranks time.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("QR/polar TFLOP/s + batched solves/s, mixed vs FP64 at "
          "‖A−QR‖/‖A‖≤1e-12")
SEED = 20260101
OZ_PAIRS = 36  # bf16 plane products per FP64 product in the split GEMM (8 slices)
# DRAM traffic of the split GEMM per FP64-equivalent flop, from ncu captures of
# its two trailing-update shapes (dram__bytes_read.sum + dram__bytes_write.sum:
# 0.059 B/flop for C -= V W2 with K = 128, 0.066 B/flop for W = V^H C with
# K = 8192; summary in profiles/oz_gemm_kernel_trailing_update_shapes.md).
# Both grow in proportion to the work, so the per-launch traffic is this
# rate times the launch's FP64-equivalent flops.
OZ_TRAFFIC = {"bytes_per_fp64_flop": 0.0635,
              "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of oz_gemm_kernel on "
                        "16384x8192x128 (2.173 GB) and 128x8192x16384 (2.194 GB), 34.4 GFLOP "
                        "FP64-equivalent each (bench.py --workload gemm), scaled by the "
                        "launch's FP64-equivalent flops"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["native", "mixed"], default="mixed")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="timed steps of the plain FP64 kernels on the same input (0: skip)")
    ap.add_argument("--m", type=int, default=16384)
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--cpu-sample", type=str, default="8192x4096",
                    help="bounded CPU-baseline sample (m x n of the same distribution)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lean", action="store_true",
                    help="timed region only (profiling runs): no accuracy check, peak, e2e, "
                         "polar or CPU baseline")
    ap.add_argument("--no-polar", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--polar-n", type=int, default=8192)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-blocks", type=int, default=300)
    ap.add_argument("--batched-kinds", type=str, default="qr,polar",
                    help="which batched factorizations to measure (comma list of qr, polar)")
    ap.add_argument("--no-batched-loop", action="store_true",
                    help="skip the per-block launch loop the batched QR is compared with")
    ap.add_argument("--no-pullback", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--sweep-tensors", type=int, default=256)
    ap.add_argument("--workload", choices=["qr", "gemm", "polar", "batched", "sweep", "autotune"],
                    default="qr",
                    help="gemm: time the split-precision product alone on --gemm-shapes; "
                         "polar: left_polar! alone on --polar-n; batched: the batch of "
                         "uneven blocks alone (profiling runs)")
    ap.add_argument("--gemm-shapes", type=str, default="16384x8192x128,128x8192x16384",
                    help="MxNxK list for --workload gemm (the trailing-update shapes of the "
                         "16384 x 8192 QR: C -= V W2 and W = V^H C)")
    return ap.parse_args()


def qr_flops(m, n, cpx=False):
    k = min(m, n)
    geqrf = 2.0 * m * n * n - 2.0 * n ** 3 / 3.0 if m >= n else 2.0 * n * m * m - 2.0 * m ** 3 / 3.0
    orgqr = 2.0 * m * k * k - 2.0 * k ** 3 / 3.0
    return (4.0 if cpx else 1.0) * (geqrf + orgqr)


def polar_flops(m, n, k_ref, cpx=False):
    c = 4.0 if cpx else 1.0
    f = (qr_flops(m, n, cpx) + c * 2.0 * m * n * n) if m > n else 0.0
    return f + c * k_ref * 8.0 * n ** 3 / 3.0 + c * 2.0 * m * n * n


def world():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(dist, value, device="cpu"):
    """The largest of the ranks' values (the whole job takes as long as its
    slowest replica); `value` itself with one rank."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_tflops(world_size, flops_per_replica, ms):
    """Whole-job throughput of `world_size` replicas that each factor one
    matrix of `flops_per_replica` flops, the slowest taking `ms`."""
    return world_size * flops_per_replica / (ms / 1e3) / 1e12


# ------------------------------------------------------------- clocks ---
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons (200 ms)."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str):
        self.uuid = uuid.replace("GPU-", "")
        self.proc = None
        self.tmp = None

    def start(self):
        """Start sampling (again: every start/stop pair is its own record)."""
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 8 or self.uuid not in parts[0].replace("GPU-", ""):
                    continue
                rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return float("nan")

        sm = [num(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(num(r[2]) for r in rows),
                "power_w_max": max(num(r[3]) for r in rows), "samples": len(rows),
                "reasons": reasons}


# -------------------------------------------------------- CPU baseline ---
class _blas_threads:
    """All host cores for OpenBLAS: threadpoolctl when installed, otherwise
    OpenBLAS's own default (one thread per available core)."""

    def __init__(self, cores):
        self.cores = cores
        self.ctx = None

    def __enter__(self):
        try:
            import threadpoolctl

            self.ctx = threadpoolctl.threadpool_limits(self.cores)
            self.ctx.__enter__()
        except ImportError:
            self.ctx = None
        return self

    def __exit__(self, *exc):
        if self.ctx is not None:
            self.ctx.__exit__(*exc)

    @staticmethod
    def describe():
        try:
            import threadpoolctl

            return ",".join(f"{d.get('internal_api')} {d.get('version')} "
                            f"threads={d.get('num_threads')}"
                            for d in threadpoolctl.threadpool_info())
        except ImportError:
            return "scipy-bundled OpenBLAS (threadpoolctl absent: default thread count)"


def cpu_qr_rate(m, n, reps=1):
    """The reference's LAPACK_HouseholderQR path (oracle restatement) on all
    host cores; returns (TFLOP/s, seconds per factorization, threads)."""
    import numpy as np

    import oracle

    cores = len(os.sched_getaffinity(0))
    rng = np.random.default_rng(SEED + 1)
    A = oracle.gaussian(rng, m, n, np.float64)
    with _blas_threads(cores):
        oracle.qr_compact(A[: min(m, 512), : min(n, 256)])  # warm the BLAS threads
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            oracle.qr_compact(A)
            ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    return qr_flops(m, n) / t / 1e12, t, cores


def _host_info():
    """CPU model, usable cores and the BLAS library behind scipy's LAPACK."""
    info = {"cores": len(os.sched_getaffinity(0))}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() in ("Model name", "Architecture", "Socket(s)", "Vendor ID"):
                info[k.strip().lower().replace(" ", "_").replace("(s)", "s")] = v.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        import scipy

        cfg = scipy.show_config(mode="dicts")
        b = cfg["Build Dependencies"]["lapack"]
        info["blas"] = f"{b.get('name')} {b.get('version')} (scipy {scipy.__version__})"
    except Exception:  # noqa: BLE001 -- informational only
        info["blas"] = "scipy-bundled OpenBLAS"
    info["blas_threads"] = _blas_threads.describe()
    return info


_ONE_THREAD_SNIPPET = r"""
import json, sys, time
import numpy as np
sys.path.insert(0, {root!r})
import oracle
import bench
kind, m, n = {kind!r}, {m}, {n}
if kind == "qr":
    A = oracle.gaussian(np.random.default_rng({seed}), m, n, np.float64)
    oracle.qr_compact(A[:64, :32])
    t0 = time.perf_counter(); oracle.qr_compact(A); t = time.perf_counter() - t0
    print(json.dumps({{"s": t, "tflops": bench.qr_flops(m, n) / t / 1e12}}))
else:
    A = bench.polar_matrix(n)
    oracle.left_polar_svd(A[:64, :64])
    t0 = time.perf_counter(); oracle.left_polar_svd(A); t = time.perf_counter() - t0
    print(json.dumps({{"s": t}}))
"""


def _one_thread(kind, m, n):
    """The oracle on one host thread (a child process with OpenBLAS limited to
    one thread before it loads)."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1",
               MKL_NUM_THREADS="1")
    code = _ONE_THREAD_SNIPPET.format(root=str(ROOT), kind=kind, m=m, n=n, seed=SEED + 1)
    try:
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                           timeout=600, cwd=str(ROOT))
        return json.loads(r.stdout.strip().splitlines()[-1])
    except (OSError, subprocess.SubprocessError, ValueError, IndexError) as e:
        return {"error": str(e)[:200]}


def host_legs(args, A_np, R_mixed, R_native):
    """The host-side legs of the benchmark (rank 0, after every GPU timing):

    * parity at the full size: R of the oracle (the reference's
      LAPACK_HouseholderQR restated) of the same 16384 x 8192 matrix against
      the GPU's R in both precisions;
    * the reference's PolarNewton on the host on the same polar matrix: its
      iteration count k_ref fixes the polar flop count, and its time is the
      CPU rate of that algorithm;
    * the CPU baseline: the reference's LAPACK_HouseholderQR and default
      PolarViaSVD(SafeDivideAndConquer) (?gesdd, ?gesvd fallback) on all host
      cores over bounded samples, and on one thread over smaller ones."""
    import numpy as np

    import oracle

    res = {"host": _host_info()}
    cores = res["host"]["cores"]
    with _blas_threads(cores):
        t0 = time.perf_counter()
        R_ref = oracle.qr_r(A_np)
        t_r = time.perf_counter() - t0
        res["r_vs_oracle"] = {"size": f"{A_np.shape[0]}x{A_np.shape[1]}",
                              "mixed": oracle.rel_err(R_mixed, R_ref) if R_mixed is not None
                              else None,
                              "native": oracle.rel_err(R_native, R_ref) if R_native is not None
                              else None,
                              "oracle_geqrt_s": round(t_r, 2)}
        del R_ref
        if not args.no_polar:
            P_np = polar_matrix(args.polar_n)
            t0 = time.perf_counter()
            _, _, pinfo = oracle.left_polar_newton(P_np, compute_p=True)
            t_n = time.perf_counter() - t0
            k_ref = int(pinfo["iterations"])
            res["polar_newton_oracle"] = {
                "k_ref": k_ref, "converged": bool(pinfo["converged"]), "s": round(t_n, 2),
                "tflops": round(polar_flops(args.polar_n, args.polar_n, k_ref) / t_n / 1e12, 5),
                "what": f"reference PolarNewton on the host, {args.polar_n}^2, all cores"}
            del P_np
        ms_, ns_ = (int(x) for x in args.cpu_sample.split("x"))
        rate, t, _ = cpu_qr_rate(ms_, ns_)
        res["qr"] = {"value": round(rate, 5), "unit": "TFLOP/s", "threads": cores,
                     "sample": f"qr_compact positive=true {ms_}x{ns_} Float64 (LAPACK ?geqrt "
                               f"nb=36 + ?gemqrt + gaugefix)", "s": round(t, 3)}
        ps = max(256, min(args.polar_n, 2048))
        P_s = polar_matrix(ps)
        oracle.left_polar_svd(P_s[:256, :256])
        t0 = time.perf_counter()
        oracle.left_polar_svd(P_s)
        t_svd = time.perf_counter() - t0
        res["polar"] = {"s": round(t_svd, 3), "threads": cores,
                        "factorizations_per_s": round(1.0 / t_svd, 4),
                        "sample": f"left_polar! PolarViaSVD(SafeDivideAndConquer) (?gesdd, "
                                  f"?gesvd fallback, gaugefix) on the {ps}x{ps} polar matrix"}
        del P_s
    q1 = _one_thread("qr", 2048, 1024)
    p1 = _one_thread("polar", 1024, 1024)
    res["threads_1"] = {"qr": {"sample": "qr_compact 2048x1024 Float64", **q1},
                        "polar": {"sample": "PolarViaSVD 1024x1024 polar matrix", **p1}}
    return res


def run_reference(args):
    rank, ws, _ = world()
    if rank != 0:
        return 0
    ms, ns = (int(x) for x in args.cpu_sample.split("x"))
    import numpy as np

    import oracle

    cores = len(os.sched_getaffinity(0))
    rng = np.random.default_rng(SEED)
    A = oracle.gaussian(rng, ms, ns, np.float64)
    with _blas_threads(cores):
        for _ in range(args.warmup):
            oracle.qr_compact(A)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            Q, R = oracle.qr_compact(A)
        dt = (time.perf_counter() - t0) / args.steps
        blas = _blas_threads.describe()
    val = qr_flops(ms, ns) / dt / 1e12
    sample = (f"qr_compact positive=true {ms}x{ns} Float64 per step (bounded sample of the "
              f"{args.m}x{args.n} workload, same distribution)")
    out = {
        "impl": "reference", "metric": METRIC, "value": round(val, 5), "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic iid N(0,1), seeded",
        "config": config_of(args),
        "cpu_baseline": {"value": round(val, 5), "unit": "TFLOP/s", "cores": cores,
                         "kind": "port", "sample": sample, "blas": blas,
                         "threads_all": cores, "host": _host_info()},
        "e2e": {"value": round(val, 5), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "accuracy": {"qr_residual": oracle.qr_residual(A, Q, R)},
    }
    print(json.dumps(out), flush=True)
    return 0


def config_of(args):
    return {"workload": f"qr_compact! positive=true, one {args.m}x{args.n} Float64 matrix, "
                        f"iid N(0,1)", "m": args.m, "n": args.n, "precision": args.precision,
            "parallelism": f"replicas x{args.gpus}",
            "l2": "inputs larger than L2 (A is %.2f GB > 129 MB L2), no flush needed"
                  % (args.m * args.n * 8 / 1e9),
            "cpu_sample": f"host CPU legs (cpu_baseline, --impl reference) time a bounded "
                          f"{args.cpu_sample} sample of the same distribution per step"}


# ------------------------------------------------------------ GB300 arm ---
def _read_prof(lib, kind):
    ms, work, cnt = C.c_double(), C.c_double(), C.c_uint64()
    lib.mak_profile_read(kind, C.byref(ms), C.byref(work), C.byref(cnt))
    return ms.value, work.value, int(cnt.value)


def measure_qr(mak, lib, args, dev, dist, A_master, precision, steps, warmup, clocks=None):
    """Time `steps` factorizations (after `warmup` untimed ones) of the
    device-resident matrix; returns the timing, accuracy and per-kernel-class
    device time of the timed region."""
    import torch

    alg = mak.GB300_HouseholderQR(positive=True, precision=precision)
    A = torch.empty_like(A_master)
    Q, R = mak.initialize_output("qr_compact_", A_master)

    def step():
        A.copy_(A_master)
        mak.qr_compact_(A, (Q, R), alg)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(warmup):
        step()
    barrier()
    if clocks is not None:
        clocks.start()
    launches0 = lib.mak_kernel_launches()
    lib.mak_profile_start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    barrier()
    lib.mak_profile_stop()
    clk = clocks.stop() if clocks is not None else None
    launches = int(lib.mak_kernel_launches() - launches0)
    ms = max_over_ranks(dist, e0.elapsed_time(e1) / steps, dev)
    prof = {name: _read_prof(lib, kid) for name, kid in
            (("gemm_native", 0), ("gemm_split_tensor", 1), ("qr_panel", 2))}
    acc = {"qr_residual": None, "orth_abs_fro": None, "orth_rel": None,
           "diag_R_nonnegative": None}
    if not args.lean:
        An = torch.linalg.norm(A_master)
        acc["qr_residual"] = float(torch.linalg.norm(A_master - Q @ R) / An)
        G = Q.mT.conj() @ Q
        acc["orth_abs_fro"] = float(torch.linalg.norm(
            G - torch.eye(G.shape[0], dtype=G.dtype, device=dev)))
        acc["orth_rel"] = acc["orth_abs_fro"] / float(torch.linalg.norm(G))
        del G
        acc["diag_R_nonnegative"] = bool((torch.diagonal(R) >= 0).all())
    return {"ms": ms, "launches": launches, "prof": prof, "acc": acc, "clocks": clk,
            "alg": alg, "A": A, "Q": Q, "R": R}


def run_gb300(args):
    import numpy as np
    import torch

    import __graft_entry__ as ge

    rank, ws, lrank = world()
    dist = None
    if ws > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = dist_mod
    dev = torch.device(f"cuda:{lrank}")
    torch.cuda.set_device(dev)
    mak = ge.load_package()
    lib = mak.library()
    m, n = args.m, args.n
    flops = qr_flops(m, n)

    rng = np.random.default_rng(SEED + rank)
    A_host = torch.from_numpy(rng.standard_normal((n, m))).t()  # column-major view
    A_master = torch.empty((n, m), dtype=torch.float64, device=dev).t()
    A_master.copy_(A_host)

    clocks = ClockSampler(str(torch.cuda.get_device_properties(dev).uuid))
    r = measure_qr(mak, lib, args, dev, dist, A_master, args.precision, args.steps, args.warmup,
                   clocks)
    ms = r["ms"]
    value = job_tflops(ws, flops, ms)

    # dominant kernel class, timed live (CUDA events on its own stream) inside
    # the timed region
    mixed = args.precision == "mixed"
    g_ms, g_work, g_cnt = r["prof"]["gemm_split_tensor" if mixed else "gemm_native"]
    p_ms, p_work, p_cnt = r["prof"]["qr_panel"]
    breakdown = {k: {"launches": v[2], "ms_per_step": round(v[0] / args.steps, 3)}
                 for k, v in r["prof"].items()}
    peaks = {}
    pk_path = ROOT / "MEASURED_PEAKS.json"
    if pk_path.exists():
        peaks = json.loads(pk_path.read_text())
    if not mixed and args.lean:
        peak, peak_src = None, "not measured (--lean)"
    elif not mixed:
        peak, peak_src = dgemm_peak(dev), ("cuBLAS DGEMM 8192^3 measured in this run "
                                           "(FP64 has no MEASURED_PEAKS entry)")
    elif peaks:
        peak, peak_src = float(peaks["bf16_tflops_sustained"]), \
            "of measured: MEASURED_PEAKS.json bf16_tflops_sustained"
    else:
        peak, peak_src = 1700.0, "of fallback: 1.7 PFLOP/s sustained bf16"
    # native: FP64 flops of the products; mixed: the bf16 tensor-core flops the
    # split method performs (OZ_PAIRS plane products per FP64 product)
    tensor_work = g_work * (OZ_PAIRS if mixed else 1)
    achieved = tensor_work / (g_ms / 1e3) / 1e12 if g_ms > 0 else 0.0
    fp64_equiv = g_work / (g_ms / 1e3) / 1e12 if g_ms > 0 else 0.0
    traffic = OZ_TRAFFIC if (mixed and OZ_TRAFFIC) else None
    roofline = {"bound": "tensor", "achieved": round(achieved, 4),
                "peak": round(peak, 4) if peak else None,
                "unit": "TFLOP/s", "frac": round(achieved / peak, 4) if peak else None,
                "traffic": round(traffic["bytes_per_fp64_flop"] * g_work / max(1, g_cnt))
                if traffic else None,
                "traffic_unit": "bytes per launch",
                "traffic_source": traffic["source"] if traffic else None,
                "fp64_equivalent_tflops": round(fp64_equiv, 4),
                "kernel": "gemm_kernel<double> (larfb / orgqr products)" if not mixed
                else "oz_gemm_kernel<8> (split-bf16 tcgen05 larfb / orgqr products)",
                "launches": g_cnt, "avg_launch_ms": round(g_ms / max(1, g_cnt), 4),
                "share_of_step": round(g_ms / (ms * args.steps), 4),
                "peak_source": peak_src,
                "panel": {"launches": p_cnt, "ms_total": round(p_ms, 3),
                          "achieved_gbs": round(p_work / (p_ms / 1e3) / 1e9, 2)
                          if p_ms > 0 else None},
                "breakdown": breakdown}

    want_host = rank == 0 and not args.no_cpu_baseline and not args.lean
    R_mixed_h = r["R"].cpu().numpy() if want_host else None
    out = {
        "metric": METRIC, "value": round(value, 5), "unit": "TFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic iid N(0,1) (numpy default_rng, seed %d)" % SEED,
        "config": config_of(args),
        "factorizations_per_s": round(ws * 1e3 / ms, 4),
        "accuracy": r["acc"],
        "gpu_launches": r["launches"],
        "roofline": roofline,
        "clocks": r["clocks"],
    }

    # end-to-end through the public API with host buffers: a stream of
    # independent factorizations, each step copying its input from pinned
    # host memory and its factors back.  Two sets of device buffers let the
    # copies of one step run on the copy engines while the kernels of the
    # next run on the SMs (H2D and D2H on streams of their own, ordered with
    # events), as a caller factoring one matrix after another would.  Each
    # call gets its own device outcome record (``info=``), so the host queues
    # the next step without waiting; every record is checked after the
    # timed region.
    if not args.no_e2e and not args.lean:
        alg = r["alg"]
        A0_ = r["A"]
        Q0_, R0_ = mak.initialize_output("qr_compact_", A0_)
        A_pin = torch.empty((n, m), dtype=torch.float64).pin_memory().t()
        A_pin.copy_(A_host)
        bufs = [(torch.empty_like(A0_),) + tuple(mak.initialize_output("qr_compact_", A0_))
                for _ in range(2)]
        pins = [(torch.empty((Q0_.shape[1], Q0_.shape[0]), dtype=torch.float64).pin_memory().t(),
                 torch.empty((R0_.shape[1], R0_.shape[0]), dtype=torch.float64).pin_memory().t())
                for _ in range(2)]
        s_h2d, s_d2h = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        s_comp = torch.cuda.current_stream(dev)
        ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("h2d", "comp", "d2h")}
        used = [False, False]
        k2 = max(3, min(args.steps, 6))
        w2 = max(3, args.warmup)
        infos = [mak.new_info(dev) for _ in range(k2 + w2)]
        calls = [0]

        def e2e_step(i):
            b = i % 2
            A, Q, R = bufs[b]
            Qp, Rp = pins[b]
            with torch.cuda.stream(s_h2d):
                if used[b]:
                    s_h2d.wait_event(ev["comp"][b])  # the kernels of step i-2 read A
                A.copy_(A_pin, non_blocking=True)
                ev["h2d"][b].record(s_h2d)
            s_comp.wait_event(ev["h2d"][b])
            if used[b]:
                s_comp.wait_event(ev["d2h"][b])  # step i-2's factors are on the host
            mak.qr_compact_(A, (Q, R), alg, info=infos[calls[0]])
            calls[0] += 1
            ev["comp"][b].record(s_comp)
            with torch.cuda.stream(s_d2h):
                s_d2h.wait_event(ev["comp"][b])
                Qp.copy_(Q, non_blocking=True)
                Rp.copy_(R, non_blocking=True)
                ev["d2h"][b].record(s_d2h)
            used[b] = True

        for i in range(w2):
            e2e_step(i)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks.start()
        s0.record(s_comp)
        s_h2d.wait_stream(s_comp)
        s_d2h.wait_stream(s_comp)
        for i in range(k2):
            e2e_step(i)
        s_comp.wait_stream(s_h2d)
        s_comp.wait_stream(s_d2h)
        s1.record(s_comp)
        torch.cuda.synchronize()
        e2e_clk = clocks.stop()
        if dist is not None:
            dist.barrier()
        for inf in infos:
            mak.check_info(inf, "qr_compact_")
        ems = max_over_ranks(dist, s0.elapsed_time(s1) / k2, dev)
        out["e2e"] = {"value": round(job_tflops(ws, flops, ems), 5), "unit": "TFLOP/s",
                      "ms_per_step": round(ems, 3), "steps": k2, "warmup": w2,
                      "h2d_bytes_per_step": int(A0_.numel() * 8),
                      "d2h_bytes_per_step": int((Q0_.numel() + R0_.numel()) * 8),
                      "overlap": "double-buffered: step i's copies overlap the kernels of "
                                 "step i+1 (H2D and D2H streams, event-ordered); each call's "
                                 "device outcome record checked after the timed region",
                      "clocks": e2e_clk}
        del A_pin, pins, bufs
    del r

    # the plain FP64 kernels on the same input: the comparison the metric asks for
    R_native_h = None
    if mixed and not args.lean and args.fp64_steps > 0:
        r64 = measure_qr(mak, lib, args, dev, dist, A_master, "native", args.fp64_steps, 1)
        if want_host:
            R_native_h = r64["R"].cpu().numpy()
        v64 = ws * flops / (r64["ms"] / 1e3) / 1e12
        out["fp64"] = {"value": round(v64, 5), "unit": "TFLOP/s",
                       "ms_per_step": round(r64["ms"], 3), "steps": args.fp64_steps,
                       "warmup": 1, "accuracy": r64["acc"],
                       "gemm_native_ms_per_step":
                           round(r64["prof"]["gemm_native"][0] / args.fp64_steps, 3)}
        out["mixed_over_fp64"] = round(value / v64, 3)
        del r64

    # left_polar! (Newton) on the single large polar problem, both precisions
    if not args.no_polar and not args.lean:
        out["polar"] = polar_measure(mak, args, dev, args.precision)
        if mixed and args.fp64_steps > 0:
            p64 = polar_measure(mak, args, dev, "native")
            out["polar_fp64"] = p64
            out["polar"]["mixed_over_fp64"] = round(p64["ms"] / out["polar"]["ms"], 3)
    if not args.no_batched and not args.lean:
        out["batched"] = batched_measure(mak, args, dev)
    if not args.no_pullback and not args.lean:
        out["pullback"] = pullback_measure(mak, args, dev)
    if not args.no_sweep and not args.lean:
        out["orth_sweep"] = sweep_measure(mak, args, dev)

    if want_host:
        del A_master
        torch.cuda.empty_cache()
        h = host_legs(args, A_host.numpy(), R_mixed_h, R_native_h)
        del R_mixed_h, R_native_h
        out["accuracy"]["r_vs_oracle"] = h["r_vs_oracle"]
        po = h.get("polar_newton_oracle")
        if po and "polar" in out:
            # credit the reference's iteration count, not this run's own
            for key in ("polar", "polar_fp64"):
                if key in out:
                    pm = out[key]
                    pm["k_ref"] = po["k_ref"]
                    pm["tflops"] = round(polar_flops(args.polar_n, args.polar_n, po["k_ref"]) /
                                         (pm["ms"] / 1e3) / 1e12, 4)
                    pm["flop_count"] = ("k_ref*8n^3/3 + 2n^3: the reference PolarNewton count "
                                        "with the oracle's iteration count on the same matrix "
                                        "(Newton-Schulz steps not credited)")
        qr_ = h["qr"]
        out["cpu_baseline"] = {
            "value": qr_["value"], "unit": "TFLOP/s", "cores": h["host"]["cores"], "kind": "port",
            "sample": f"{qr_['sample']}, {qr_['s']:.2f} s per factorization, all cores",
            "qr": qr_, "polar": h["polar"], "polar_newton": po,
            "threads_all": h["host"]["cores"], "threads_1": h["threads_1"],
            "host": h["host"]}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def dgemm_peak(dev):
    """Measured FP64 peak: cuBLAS DGEMM 8192^3, best of 6 (CUDA events)."""
    import torch

    X = torch.randn(8192, 8192, dtype=torch.float64, device=dev)
    best = 1e30
    for _ in range(6):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        X @ X
        s1.record()
        torch.cuda.synchronize()
        best = min(best, s0.elapsed_time(s1))
    del X
    return 2 * 8192 ** 3 / (best / 1e3) / 1e12


def batched_measure(mak, args, dev):
    """Uneven blocks of a block-sparse tensor: m_i ~ U{8..1024}, n_i ~ U{4..m_i},
    first half Float64, second half ComplexF64 (iid N(0,1), re/im).  qr_compact
    and left_polar of all blocks in one batched call, captured in a CUDA graph
    and replayed, against a per-block launch loop of the same factorizations."""
    import numpy as np
    import torch

    rng = np.random.default_rng(SEED + 11)
    nb = args.batched_blocks
    shapes = []
    for i in range(nb):
        m = int(rng.integers(8, 1025))
        n = int(rng.integers(4, m + 1))
        shapes.append((m, n, torch.float64 if i < nb // 2 else torch.complex128))

    def rand(m, n, dt):
        if dt == torch.complex128:
            x = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
        else:
            x = rng.standard_normal((n, m))
        return torch.from_numpy(x).to(dev).t()

    srcs = [rand(m, n, dt) for (m, n, dt) in shapes]
    work = [s.clone() for s in srcs]
    flops_qr = sum(qr_flops(m, n, dt == torch.complex128) for (m, n, dt) in shapes)
    res = {"workload": f"{nb} blocks m~U{{8..1024}} n~U{{4..m}}, half Float64 half ComplexF64",
           "qr_gflop": round(flops_qr / 1e9, 2)}

    def timed(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    kinds = args.batched_kinds.split(",")
    for prec in (("native", "mixed") if "qr" in kinds else ()):
        outs = mak.batched_qr_compact(work, copy_inputs=False, precision=prec)

        def restore():
            for w, s in zip(work, srcs):
                w.copy_(s)

        # graph capture of the whole batch (inputs restored inside the graph)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            restore()
            with torch.cuda.graph(g, stream=s):
                restore()
                mak.batched_qr_compact(work, copy_inputs=False, outs=outs, precision=prec,
                                       _capturing=True)
        torch.cuda.current_stream().wait_stream(s)
        ms_graph = timed(g.replay)

        def loop():
            restore()
            for w, (q, r) in zip(work, outs):
                mak.qr_compact_(w, (q, r), precision=prec)

        res[f"qr_{prec}"] = {"graph_ms": round(ms_graph, 3), "blocks_per_s": round(nb * 1e3 / ms_graph, 1),
                             "tflops": round(flops_qr / (ms_graph / 1e3) / 1e12, 4)}
        if not args.no_batched_loop:
            ms_loop = timed(loop, reps=1)
            res[f"qr_{prec}"].update({"per_block_loop_ms": round(ms_loop, 3),
                                      "speedup_vs_loop": round(ms_loop / ms_graph, 2)})
        del g
    # polar (batched: up to 10 Newton iterations, each block stopped on the
    # device at the default tolerance) in both precisions
    for prec in (("native", "mixed") if "polar" in kinds else ()):
        def restore():
            for w, s_ in zip(work, srcs):
                w.copy_(s_)

        def run_polar(iters=None, outs=None):
            restore()
            return mak.batched_left_polar(work, copy_inputs=False, precision=prec, maxiter=10,
                                          outs=outs, _info=iters)

        iters = []
        outs = run_polar(iters)  # eager: also creates the internal streams
        ms_eager = timed(lambda: run_polar(outs=outs), reps=1)
        # the whole batch (inputs restored inside the graph) as one CUDA graph
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            restore()
            with torch.cuda.graph(g, stream=s):
                restore()
                mak.batched_left_polar(work, copy_inputs=False, outs=outs, precision=prec,
                                       maxiter=10, _capturing=True)
        torch.cuda.current_stream().wait_stream(s)
        ms = timed(g.replay)
        back = max(float(torch.linalg.norm(s_ - W @ P) / torch.linalg.norm(s_))
                   for s_, (W, P) in zip(srcs, outs))
        res[f"polar_{prec}"] = {"graph_ms": round(ms, 3), "eager_ms": round(ms_eager, 3),
                                "blocks_per_s": round(nb * 1e3 / ms, 1),
                                "newton_iterations_max": max(iters) if iters else None,
                                "newton_iterations_mean": round(sum(iters) / len(iters), 2)
                                if iters else None, "maxiter": 10,
                                "max_back_err": back}
        del g
    for kind in kinds:
        a = res[f"{kind}_native"]["graph_ms"]
        b = res[f"{kind}_mixed"]["graph_ms"]
        res[f"{kind}_mixed_over_native"] = round(a / b, 3)
    return res


def _crandn(rng, m, n, dev):
    import torch

    x = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
    return torch.from_numpy(x).to(dev).t()


def pullback_measure(mak, args, dev):
    """Differentiation workload: ComplexF64 1024 x 512 iid complex Gaussian,
    cotangents iid complex Gaussian; forward + pullback of qr_compact and of
    left_polar, both precisions (device-resident, one timed repetition after
    a warm-up each), and the relative difference of the mixed dA from the
    native one."""
    import numpy as np
    import torch

    rng = np.random.default_rng(SEED + 21)
    m, n = 1024, 512
    A0 = _crandn(rng, m, n, dev)
    dQ, dR = _crandn(rng, m, n, dev), _crandn(rng, n, n, dev)
    dW, dP = _crandn(rng, m, n, dev), _crandn(rng, n, n, dev)
    res = {"workload": "ComplexF64 1024x512 iid complex Gaussian, cotangents iid complex Gaussian"}
    dAs = {}
    for prec in ("native", "mixed"):
        def qr_fb():
            A = A0.clone()
            Q, R = mak.qr_compact_(A, None, precision=prec)
            dA = torch.zeros_like(A0)
            mak.qr_pullback_(dA, A0, (Q, R), (dQ, dR), precision=prec)
            return dA

        def polar_fb():
            A = A0.clone()
            W, P = mak.left_polar_(A, None, None, precision=prec)
            dA = torch.zeros_like(A0)
            mak.left_polar_pullback_(dA, A0, (W, P), (dW, dP), precision=prec)
            return dA

        for name, fn in (("qr", qr_fb), ("polar", polar_fb)):
            fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dA = fn()
            torch.cuda.synchronize()
            res[f"{name}_{prec}_ms"] = round((time.perf_counter() - t0) * 1e3, 3)
            dAs[(name, prec)] = dA
    for name in ("qr", "polar"):
        d = dAs[(name, "mixed")] - dAs[(name, "native")]
        res[f"{name}_mixed_vs_native_rel"] = float(torch.linalg.norm(d) /
                                                  torch.linalg.norm(dAs[(name, "native")]))
        res[f"{name}_mixed_over_native"] = round(res[f"{name}_native_ms"] /
                                                 res[f"{name}_mixed_ms"], 3)
    return res


def sweep_measure(mak, args, dev):
    """Orthogonalisation sweep of a matrix-product canonicalisation: N
    ComplexF64 tensors of bond dimension 256 and physical dimension 4, each a
    1024 x 256 matrix (iid complex Gaussian).  One step = left_orth via QR of
    every tensor and left_polar of every tensor (batched calls, at most 10
    Newton iterations stopped on the device), then the full pullback of the
    scalar loss sum_i real(tr(D_i^H Q_i)) + real(tr(D_i^H W_i)) through both
    (batched QR pullback: one host synchronization for all ranks; batched
    polar pullback: none).  Three arithmetic modes on the same inputs:
    "fp32" -- the Float32-class run: the tensors are converted to
    ComplexF32 on the device (inside the timed step) and every kernel runs
    in single precision, results compared with the FP64 ones at
    sqrt(eps(Float32)) (the reference's precision(ComplexF32),
    test/testsuite/TestSuite.jl:45); "mixed" -- ComplexF64 with the split
    tensor-core products; "fp64" -- the plain FP64 kernels.  The forward and
    the polar pullback are captured once as CUDA graphs and replayed every
    step (they synchronize nothing); the QR pullback runs between them (it
    reads all blocks' ranks with one host synchronization).  Wall-clock time
    per step on the host."""
    import numpy as np
    import torch

    rng = np.random.default_rng(SEED + 31)
    N = args.sweep_tensors
    As = [_crandn(rng, 1024, 256, dev) for _ in range(N)]
    Ds = [_crandn(rng, 1024, 256, dev) for _ in range(N)]
    flops_qr = N * qr_flops(1024, 256, True)
    res = {"workload": f"{N} ComplexF64 1024x256 tensors: batched QR + batched polar (<= 10 "
                       f"Newton steps, stopped on the device) + batched pullbacks of "
                       f"sum real(tr(D^H Q)) + real(tr(D^H W)) through both",
           "qr_gflop": round(flops_qr / 1e9, 1)}
    dAs_out = {}
    for mode in ("fp64", "mixed", "fp32"):
        prec = "mixed" if mode == "mixed" else "native"
        dt = torch.complex64 if mode == "fp32" else torch.complex128
        # device buffers of the step; the forward (batched QR + batched polar)
        # and the polar pullback synchronize nothing and are replayed from
        # CUDA graphs, the QR pullback (one host read of all ranks) runs
        # between them
        X = [torch.empty_like(A, dtype=dt) for A in As]
        D = [torch.empty_like(d, dtype=dt) for d in Ds]
        Xw = [torch.empty_like(x) for x in X]
        Xp = [torch.empty_like(x) for x in X]
        dA = [torch.empty_like(x) for x in X]

        def load():
            for x, a, xw, xp in zip(X, As, Xw, Xp):
                x.copy_(a)  # the Float32-class run converts here
                xw.copy_(x)
                xp.copy_(x)
            for d, s_ in zip(D, Ds):
                d.copy_(s_)
            for g in dA:
                g.zero_()

        load()
        QR = mak.batched_qr_compact(Xw, copy_inputs=False, precision=prec)
        WP = mak.batched_left_polar(Xp, copy_inputs=False, precision=prec, maxiter=10)
        mak.batched_left_polar_pullback(dA, WP, [(d, None) for d in D], precision=prec)
        torch.cuda.synchronize()
        g_fwd, g_pb = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream()
        cs.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(cs):
            with torch.cuda.graph(g_fwd, stream=cs):
                load()
                mak.batched_qr_compact(Xw, copy_inputs=False, outs=QR, precision=prec,
                                       _capturing=True)
                mak.batched_left_polar(Xp, copy_inputs=False, outs=WP, precision=prec,
                                       maxiter=10, _capturing=True)
            with torch.cuda.graph(g_pb, stream=cs):
                mak.batched_left_polar_pullback(dA, WP, [(d, None) for d in D],
                                                precision=prec, _capturing=True)
        torch.cuda.current_stream().wait_stream(cs)
        phases = {}

        def step(timed_phases=False):
            t = time.perf_counter()
            g_fwd.replay()
            if timed_phases:
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                phases["forward"] = round((t1 - t) * 1e3, 2)
                t = t1
            mak.batched_qr_pullback(dA, QR, [(d, None) for d in D], precision=prec)
            if timed_phases:
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                phases["qr_pullback"] = round((t1 - t) * 1e3, 2)
                t = t1
            g_pb.replay()
            if timed_phases:
                torch.cuda.synchronize()
                phases["polar_pullback"] = round((time.perf_counter() - t) * 1e3, 2)

        step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize()
        res[f"{mode}_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
        dAs_out[mode] = [g.clone() for g in dA]
        step(timed_phases=True)
        res[f"{mode}_phases_ms"] = phases
        del g_fwd, g_pb
    ref = dAs_out["fp64"]
    for mode in ("mixed", "fp32"):
        err = max(float(torch.linalg.norm(a.to(torch.complex128) - b) / torch.linalg.norm(b))
                  for a, b in zip(dAs_out[mode], ref))
        res[f"{mode}_dA_rel_vs_fp64"] = err
        res[f"{mode}_over_fp64"] = round(res["fp64_ms"] / res[f"{mode}_ms"], 3)
    res["fp32_tolerance"] = float(np.sqrt(np.finfo(np.float32).eps))
    return res


def polar_matrix(n):
    """The single large polar problem: A = U diag(s) V^T with U, V Haar
    (QR of a Gaussian with the sign fix) and s log-spaced from 1 to 1e-6."""
    import numpy as np

    rng = np.random.default_rng(SEED + 7)

    def haar(k):
        G = rng.standard_normal((k, k))
        Qh, Rh = np.linalg.qr(G)
        return Qh * np.sign(np.diagonal(Rh))[None, :]

    U, V = haar(n), haar(n)
    s = np.logspace(0, -6, n)
    return np.asfortranarray((U * s[None, :]) @ V.T)


def polar_measure(mak, args, dev, precision):
    import numpy as np
    import torch

    n = args.polar_n
    A_np = polar_matrix(n)
    A0 = torch.from_numpy(A_np).to(dev)
    A = torch.empty_like(A0)
    W, P = mak.polar.initialize_output(A0)
    alg = mak.GB300_PolarNewton(precision=precision)
    info = {}
    A.copy_(A0)
    mak.left_polar_(A, (W, P), alg, _info=info)  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    A.copy_(A0)
    mak.left_polar_(A, (W, P), alg, _info=info)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    k = info["iterations"]
    back = float(torch.linalg.norm(A0 - W @ P) / torch.linalg.norm(A0))
    G = W.mT @ W
    orth = float(torch.linalg.norm(G - torch.eye(n, dtype=G.dtype, device=dev)))
    return {"workload": f"left_polar! PolarNewton, {n}x{n} Float64, U diag(logspace(0,-6)) V^T",
            "precision": precision, "ms": round(ms, 2), "iterations": k,
            "tflops": round(polar_flops(n, n, k) / (ms / 1e3) / 1e12, 4),
            "flop_count": "k*8n^3/3 + 2n^3 with this run's own k (replaced by the oracle's "
                          "k_ref when the host legs run)",
            "back_err": back, "orth_abs_fro": orth, "orth_rel": orth / math.sqrt(n),
            "steps": 1, "warmup": 1}


def run_gemm(args):
    """The split-precision GEMM alone through the C ABI (mak_gemm_d, mixed):
    C = -op(A) B + C on device-resident operands, the shapes of the QR's
    trailing update; FP64-equivalent and bf16 tensor TFLOP/s per shape."""
    import torch

    import __graft_entry__ as ge

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    mak = ge.load_package()
    lib = mak.library()
    from mak_gb300 import _lib

    out = {"metric": "split-precision GEMM TFLOP/s (FP64-equivalent)", "unit": "TFLOP/s",
           "dtype": "f64", "data": "synthetic iid N(0,1)", "shapes": []}
    gen = torch.Generator(device=dev).manual_seed(SEED)
    st = torch.cuda.current_stream(dev).cuda_stream
    for shape in args.gemm_shapes.split(","):
        m, n, k = (int(x) for x in shape.split("x"))
        opA = 2 if m <= 256 else 0  # W = V^H C reads V transposed
        A = (torch.randn((m, k) if opA == 0 else (k, m), dtype=torch.float64, device=dev,
                         generator=gen).t().contiguous().t())
        B = torch.randn((n, k), dtype=torch.float64, device=dev, generator=gen).t()
        Cm = torch.randn((n, m), dtype=torch.float64, device=dev, generator=gen).t()
        nb = C.c_size_t()
        lib.mak_gemm_workspace(_lib.MAK_F64, opA, 0, m, n, k, _lib.MAK_PREC_MIXED, C.byref(nb))
        work = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        info = torch.zeros(C.sizeof(_lib.mak_info), dtype=torch.uint8, device=dev)
        lda = A.stride(1)

        def call():
            rc = lib.mak_gemm_d(opA, 0, m, n, k, -1.0, A.data_ptr(), lda, B.data_ptr(), k, 1.0,
                                Cm.data_ptr(), m, _lib.MAK_PREC_MIXED, work.data_ptr(), nb.value,
                                info.data_ptr(), st)
            assert rc == 0, lib.mak_status_string(rc)

        for _ in range(max(3, args.warmup)):
            call()
        torch.cuda.synchronize()
        lib.mak_profile_start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            call()
        e1.record()
        torch.cuda.synchronize()
        lib.mak_profile_stop()
        ms = e0.elapsed_time(e1) / args.steps
        k_ms, k_work, k_cnt = _read_prof(lib, 1)
        f64 = 2.0 * m * n * k / (ms / 1e3) / 1e12
        kern = k_work / (k_ms / 1e3) / 1e12 if k_ms > 0 else None
        out["shapes"].append({"m": m, "n": n, "k": k, "op_a": "NTC"[opA], "ms": round(ms, 4),
                              "fp64_equiv_tflops": round(f64, 3),
                              "kernel_ms": round(k_ms / max(1, k_cnt), 4),
                              "kernel_fp64_equiv_tflops": round(kern, 3) if kern else None,
                              "kernel_tensor_tflops": round(kern * OZ_PAIRS, 1) if kern else None})
        del A, B, Cm, work
    print(json.dumps(out), flush=True)
    return 0


def run_polar_only(args):
    """left_polar! alone (one warm-up and one timed factorization of the
    --polar-n test matrix) in the requested precision: the small case the
    Gauss-Jordan panel profiles are captured on."""
    import torch

    import __graft_entry__ as ge

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    mak = ge.load_package()
    print(json.dumps(polar_measure(mak, args, dev, args.precision)), flush=True)
    return 0


def run_batched_only(args):
    """The batch of uneven blocks alone (both precisions, QR and polar): the
    case the batched kernels are profiled on."""
    import torch

    import __graft_entry__ as ge

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    mak = ge.load_package()
    print(json.dumps(batched_measure(mak, args, dev)), flush=True)
    return 0


def run_sweep_only(args):
    """The orthogonalisation sweep alone (all three arithmetic modes)."""
    import torch

    import __graft_entry__ as ge

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    mak = ge.load_package()
    print(json.dumps(sweep_measure(mak, args, dev)), flush=True)
    return 0


def run_autotune(args):
    """The autotuner of the drivers' tuning table on the batch of uneven
    blocks (mixed precision, batched QR then batched polar, both replayed
    from a CUDA graph); prints the table and every trial."""
    import numpy as np
    import torch

    import __graft_entry__ as ge

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    mak = ge.load_package()
    rng = np.random.default_rng(SEED + 11)
    As = []
    for i in range(args.batched_blocks):
        m = int(rng.integers(8, 1025))
        n = int(rng.integers(4, m + 1))
        if i < args.batched_blocks // 2:
            x = rng.standard_normal((n, m))
        else:
            x = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
        As.append(torch.from_numpy(x).to(dev).t())
    res = mak.autotune.autotune_batched(As, precision="mixed",
                                        kinds=tuple(args.batched_kinds.split(",")))
    print(json.dumps(res), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "gemm":
        return run_gemm(args)
    if args.workload == "batched":
        return run_batched_only(args)
    if args.workload == "sweep":
        return run_sweep_only(args)
    if args.workload == "autotune":
        return run_autotune(args)
    if args.workload == "polar":
        return run_polar_only(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
